#!/usr/bin/env python
"""Benchmark: particle-solves/s of the capacitance-tensor solve on one GB300.

Workload (the configuration the metric is quoted on): N = 100,000 unit spheres,
seeded random sequential addition at volume fraction 0.3 (seed 2), contrast
beta = 0.9 (eps = 28), the three unit field directions (3x3 capacitance
tensor), xi = 4/rc with rc = (60/phi)^(1/3) (about 60 neighbours), 192^3 grid,
P = 10, fully periodic.  A step = build the configuration's geometry (cell
list, pair list, grid weights, Green's coefficients and scale tensors: the
process-wide k-space cache is emptied before every step, so each step pays for
its own k-space set-up as the reference does on every call) + solve the three
directions to tolerance.  particle-solves/s = N x 3 / step time.

The default run also reports, as extra keys of the same JSON line, the other
configurations (dipole + quadrupole lattice, 256 polydisperse configurations
with contrast spectra, N = 200,000 adjoint forces with finite-difference and
point-dipole checks and 1000 Brownian-dynamics steps), each with its error
against a float64 solve, and the CPU baseline: the CPU oracle (a NumPy
restatement of the reference's path) at N = 100,000 on the host cores.

Arms:
  default           mixed precision (float32 operator, float64-accurate
                    refinement), the three directions batched into one solve
  --impl reference  the reference algorithm on the host cores (the CPU oracle)
                    at N = 100,000: particles placed by the oracle's pure-Python
                    generator, geometry and one field direction solved in full,
                    then each step one float64 matvec of that solve
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-solves/s at N=1e5 (3-direction capacitance tensor, rel. moment err <= 1e-6 vs FP64)"
UNIT = "particle-solves/s"


def workload_params(n=100_000, phi=0.3, beta=0.9, grid=192, P=10):
    """The workload's parameters without its positions (rc from about 60 neighbours, xi = 4 / rc)."""
    rc = (60.0 / phi) ** (1.0 / 3.0)
    return dict(rc=rc, xi=4.0 / rc, Ngrid=np.array([grid, grid, grid]), P=P, n=n, phi=phi, beta=beta, seed=2)


def workload(n=100_000, phi=0.3, seed=2, beta=0.9, grid=192, P=10, placer=None):
    """Parameters and positions.  ``placer`` places the spheres (default: the package's C generator)."""
    if placer is None:
        from mutual_polarization_slab_gb300.workloads import rsa as placer
    x, box, _ = placer(n, phi, seed)
    w = workload_params(n=n, phi=phi, beta=beta, grid=grid, P=P)
    w.update(x=x, box=box, eps=np.full(n, (1.0 + 2.0 * beta) / (1.0 - beta)), seed=seed)
    return w


def config_dict(w, args, world):
    """The workload's description; both arms print the same one."""
    return {"workload": f"RSA N={w['n']} phi={w['phi']} beta={w['beta']} 3 field directions, "
                        f"{int(w['Ngrid'][0])}^3 grid, P={w['P']}, xi={w['xi']:.4f}, rc={w['rc']:.4f}, "
                        f"fully periodic; per step: geometry + k-space set-up + solve to tol",
            "n_particles": int(w["n"]), "n_rhs": 3, "grid": int(w["Ngrid"][0]), "P": int(w["P"]),
            "tol": args.tol, "restart": args.restart, "parallelism": f"replicas x{world}",
            "l2": "per-step working set (9 x 192^3 double-float residual grids = 510 MB, 3 x 192^3 fp32 grids, "
                  "pair lists) exceeds the 129 MB L2; L2 also flushed (256 MB write) between steps"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        idx = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", idx, f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _rel(a, b):
    import torch
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch

    from mutual_polarization_slab_gb300 import _lib
    from mutual_polarization_slab_gb300 import capacitance as gcap
    from mutual_polarization_slab_gb300.system import SpectralEwaldSystem, clear_kspace_cache

    world, rank = dist_init()
    w = workload(n=args.n, grid=args.grid)
    n = w["n"]
    perp, para, rv = gcap.default_table(w["xi"])
    xd = torch.as_tensor(w["x"], device="cuda")
    epsd = torch.as_tensor(w["eps"], device="cuda")
    phi = 4.0 * math.pi * n / (3.0 * float(np.prod(w["box"])))
    amp = torch.as_tensor(gcap.dilute_guess(w["eps"], phi, [1.0, 0.0, 0.0])[:, 0], device="cuda")
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[:, None, :].expand(3, n, 3).contiguous()
    x0 = torch.stack([amp[:, None] * eye[i] for i in range(3)]).contiguous()
    tol, restart = args.tol, args.restart
    lib = _lib.lib()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def make_system(prof=False, inner=None):
        s = SpectralEwaldSystem(xd, epsd, w["box"], w["xi"], w["rc"], w["Ngrid"], w["P"], perp, para, rv,
                                slab_factor=0.0, max_rhs=3, inner=inner)
        if prof:
            s.profile(True)
        return s

    def step_mixed(prof=False):
        s = make_system(prof, inner=args.inner_grid if args.inner == "grad" else None)
        sol, info = s.solve(b, x0, tol=tol, restart=restart, maxit=args.maxref, precision="mixed",
                            inner_tol=args.inner_tol, inner_maxit=args.inner_maxit,
                            residual_precision=args.resid, inner_operator=args.inner)
        return s, sol, info

    def step_fp64_plain():
        """The drop-in: float64 GMRES, one field direction at a time, reference warm-start order."""
        s = make_system()
        guess = x0[0]
        sols, infos = [], []
        for i in range(3):
            si, inf = s.solve(b[i], guess, tol=tol, restart=restart, maxit=100, precision="fp64")
            sols.append(si)
            infos += inf
            guess = si[:, [2, 0, 1]].contiguous()
        return s, torch.stack(sols), infos

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            clear_kspace_cache()
            s, _, _ = fn()
            s.close()
        torch.cuda.synchronize()
        barrier(world)
        total = 0.0
        launches0 = lib.mps_kernel_launches()
        res = None
        for _ in range(steps):
            # each step recomputes its k-space data (Green's coefficients, gradient-form coefficient,
            # double-float scale tensor): the cache is emptied here, outside the timed region
            clear_kspace_cache()
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            s, sol, info = fn()
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
            res = (sol, info)
            s.close()
        launches = lib.mps_kernel_launches() - launches0
        barrier(world)
        return total / steps, launches, res

    if args.only_mixed:
        ms_only, launches, _ = timed(step_mixed, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({"mode": "only-mixed", "ms_per_step": ms_only, "n": n, "gpu_launches": launches}),
                  flush=True)
        return

    # --- headline: mixed + batched
    clk = Clocks()
    ms_mixed, launches, (sol_m, info_m) = timed(step_mixed, args.steps, args.warmup)
    clocks = clk.stop()
    ms_mixed = max_over_ranks(ms_mixed, world)
    value = world * n * 3 / (ms_mixed / 1e3)

    # --- per-configuration setup alone (geometry, pairs, weights, Green's coefficients, tile binning)
    clear_kspace_cache()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    s_setup = make_system(inner=args.inner_grid if args.inner == "grad" else None)
    # first matvec of a system bins the particles into tiles (the inner operator of the solve)
    s_setup.matvec(b[:1], precision="fp32grad" if args.inner == "grad" else "fp32")
    e1.record()
    torch.cuda.synchronize()
    setup_ms = e0.elapsed_time(e1)
    s_setup.close()

    # --- roofline: stage times of one profiled mixed step (same launches, events on the launching stream)
    clear_kspace_cache()
    s_prof, _, _ = step_mixed(prof=True)
    torch.cuda.synchronize()
    st = s_prof.stage_times()
    tuning = s_prof.tuning()
    inner_disc = s_prof.inner
    s_prof.close()
    roof = roofline(w, st, args.inner, inner_disc)

    # --- plain float64 GMRES drop-in (reference solver structure) + accuracy of the mixed result
    ms_fp64, _, (sol_64, info_64) = timed(step_fp64_plain, max(1, min(args.steps, 2)), 1)
    ms_fp64 = max_over_ranks(ms_fp64, world)
    s_ref = make_system()
    ref_sol, _ = s_ref.solve(b, x0, tol=1e-11, restart=restart, maxit=100, precision="fp64")
    s_ref.close()
    err = [_rel(sol_m[i], ref_sol[i]) for i in range(3)]
    C_m = sol_m.mean(dim=1)
    C_r = ref_sol.mean(dim=1)
    cerr = float(torch.linalg.matrix_norm(C_m - C_r) / torch.linalg.matrix_norm(C_r))
    err64 = [_rel(sol_64[i], ref_sol[i]) for i in range(3)]

    # --- end to end through the public API with host buffers
    e2e = run_e2e(args, w, world)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": f"fp32 inner GMRES ({args.inner} operator, inner tol {args.inner_tol}) + {args.resid} "
                 f"refinement residual, fp64 Arnoldi/Givens",
        "data": "synthetic (seeded RSA)",
        "config": config_dict(w, args, world),
        "e2e": e2e,
        "gpu_launches": int(launches / max(args.steps, 1)),
        "gpu_launches_note": "kernels of libmps_gb300.so per timed step (cuFFT executions not counted)",
        "clocks": clocks,
        "roofline": roof,
        "accuracy": {"rel_moment_error_vs_fp64": err, "capacitance_tensor_rel_error": cerr,
                     "fp64_reference": "GPU float64 GMRES to relative residual 1e-11 (the oracle's operator to "
                                       "1e-12, checked at this size by tests/test_headline_parity.py)",
                     "fp64_plain_rel_moment_error": err64,
                     "mixed_matvecs": {"fp64": info_m[0].matvecs_fp64, "fp32": info_m[0].matvecs_fp32,
                                       "refinement_steps": info_m[0].cycles},
                     "fp64_plain_matvecs": sum(i.matvecs_fp64 for i in info_64)},
        "fp64_plain": {"value": world * n * 3 / (ms_fp64 / 1e3), "ms_per_step": ms_fp64,
                       "what": "float64 GMRES, one direction at a time with the reference's warm start "
                               "(k-space recomputed per step as well)"},
        "speedup_vs_fp64_plain": ms_fp64 / ms_mixed,
        "setup_ms_incl_first_fp32_matvec": setup_ms,
        "autotuned_tiles": tuning,
        "inner_discretisation": ({"grid": [int(v) for v in inner_disc[0]], "P": int(inner_disc[1]),
                                  "what": "grid and support of the float32 gradient-form inner operator; the "
                                          "refinement residuals use the workload's own grid and P"}
                                 if inner_disc is not None else None),
    }
    if not args.no_extra:
        out["quadrupole"] = workload_quadrupole(args)
        out["batch"] = workload_batch(args)
        out["forces"] = workload_forces(args)
    if rank == 0 and not args.no_cpu:
        cb, oracle_acc = cpu_baseline(args, w, sol_m.cpu().numpy())
        out["cpu_baseline"] = cb
        out["accuracy"]["oracle_check"] = oracle_acc
    if rank == 0:
        print(json.dumps(out), flush=True)


def measured_traffic(kernel, n, ngrid):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of ``kernel``
    from the committed ncu capture of this workload (profiles/dram_traffic_*.txt:
    lines "kernel n nx ny nz bytes_per_launch"), or None when no capture matches."""
    import glob
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "dram_traffic_*.txt"))):
        for line in open(path):
            f = line.split()
            if len(f) == 6 and not line.startswith("#") and f[0] == kernel and int(f[1]) == n \
                    and [int(v) for v in f[2:5]] == [int(v) for v in ngrid]:
                return float(f[5])
    return None


def roofline(w, st, inner="grad", inner_disc=None):
    """Dominant kernel (largest stage time of this library's kernels in the fp32 matvec) vs HBM peak.
    Algorithmic bytes per launch, R = 3 vectors, s = 4 bytes: the grids written or read once
    (3R grids for the reference discretisation, R for the gradient form), plus per particle its
    moments / fields (24 R), stencil start (12) and separable factors (3P s; twice for the gradient
    form, which also reads dw/dr).  ``inner_disc`` = (grid, P) of the float32 operator when it runs on
    its own (coarser) grid."""
    n, P = w["n"], w["P"]
    ngrid = w["Ngrid"]
    if inner_disc is not None:
        ngrid, P = inner_disc
    G = int(np.prod(ngrid))
    nx = int(ngrid[0])
    Gc = (nx // 2 + 1) * int(ngrid[1]) * int(ngrid[2])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "6800 GB/s (of fallback)"
    cnt, ms = st["fp32"]
    R = 3
    grids = R if inner == "grad" else 3 * R
    per_particle_geom = (2 if inner == "grad" else 1) * 3 * P * 4 + 12
    algo = {
        "spread": grids * G * 4 + n * (R * 3 * 8 + per_particle_geom),
        "contract": grids * G * 4 + n * (per_particle_geom + R * 3 * 8),
        "scale": 2 * grids * Gc * 8 + Gc * 4,
        "real_space": None,
    }
    cand = {k: v for k, v in ms.items() if k in ("spread", "contract", "scale", "real_space")}
    if not cnt:
        return None
    top = max(cand, key=cand.get)
    avg_ms = cand[top] / cnt
    if algo.get(top) is None:
        top = max((k for k in cand if algo.get(k)), key=cand.get)
        avg_ms = cand[top] / cnt
    achieved = algo[top] / (avg_ms / 1e3) / 1e9
    kname = {"spread": "k_spread_grad_tiled" if inner == "grad" else "k_spread_tiled",
             "contract": "k_contract_grad_home" if inner == "grad" else "k_contract_tiled + gather",
             "scale": "k_scale_cs" if inner == "grad" else "k_scale_half"}.get(top, top)
    traffic = measured_traffic(kname, n, ngrid)
    return {"bound": "hbm", "kernel": f"{kname} (fp32, 3 vectors, {int(ngrid[0])}x{int(ngrid[1])}x{int(ngrid[2])} "
                                      f"grid, P={P})", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
            "algorithmic_bytes_per_launch": algo[top], "avg_launch_ms": avg_ms, "launches": cnt,
            "traffic": traffic,
            "stage_ms_per_matvec_fp32": {k: v / cnt for k, v in ms.items()},
            "stage_ms_per_matvec_fp64": ({k: v / st["fp64"][0] for k, v in st["fp64"][1].items()}
                                         if st["fp64"][0] else None),
            "stage_ms_per_matvec_df": ({k: v / st["df"][0] for k, v in st["df"][1].items()}
                                       if st["df"][0] else None)}


def run_e2e(args, w, world):
    """Same metric through the public API (capacitance_tensor) with host numpy inputs/outputs;
    each call builds its own geometry and k-space data (cache emptied before it, untimed)."""
    import torch

    from mutual_polarization_slab_gb300 import capacitance as gcap
    from mutual_polarization_slab_gb300.system import clear_kspace_cache
    n = w["n"]
    phi = 4.0 * math.pi * n / (3.0 * float(np.prod(w["box"])))
    # the step's inputs in page-locked host memory (torch's pinned allocator), as a caller that streams
    # configurations from the host would keep them
    pinned = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    guess = pinned(gcap.dilute_guess(w["eps"], phi, [1.0, 0.0, 0.0]))
    xh = pinned(w["x"])
    eh = pinned(w["eps"])

    def call():
        C, S, info = gcap.capacitance_tensor(xh, eh, w["box"], guess, w["xi"], args.tol, rc=w["rc"],
                                             Ngrid=w["Ngrid"], P=w["P"], restart=args.restart, maxit=args.maxref,
                                             precision="mixed", inner_tol=args.inner_tol,
                                             inner_maxit=args.inner_maxit, residual_precision=args.resid,
                                             inner_operator=args.inner, inner_grid=args.inner_grid)
        return C, S

    for _ in range(max(1, args.warmup - 1)):
        clear_kspace_cache()
        call()
    steps = max(1, args.steps)
    dt = 0.0
    for _ in range(steps):
        clear_kspace_cache()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        C, S = call()
        torch.cuda.synchronize()
        dt += time.perf_counter() - t0
    dt /= steps
    # capacitance_tensor copies the positions, the permittivities and the guess's x column to the device
    h2d = xh.nbytes + eh.nbytes + guess[:, 0].nbytes
    d2h = S.nbytes + C.nbytes
    return {"value": world * n * 3 / dt, "unit": UNIT, "ms_per_step": dt * 1e3, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "api": "capacitance.capacitance_tensor(numpy in from pinned host memory, numpy out)"}


# ----------------------------------------------------------------------------- CPU legs (the oracle)
def oracle_direction(w, threads, tol, restart, maxit=20):
    """The oracle's float64 path at the workload's full size: geometry (cell list, candidate and
    filtered pair lists, dense grid kernel), then one field direction (x, from the dilute guess)
    solved by its GMRES(restart) with the float64 operator on ``threads`` host threads.
    Returns the geometry and the timings."""
    from oracle import capacitance_oracle as co
    from oracle import ewald_oracle as ew
    n = w["n"]
    perp, para, rv = ew.default_table(w["xi"])
    t0 = time.perf_counter()
    geo = ew.Geometry(w["x"], w["eps"], w["box"], w["xi"], w["rc"], w["Ngrid"], w["P"], perp, para, rv, 0.0)
    t_geom = time.perf_counter() - t0
    phi = 4.0 * math.pi * n / (3.0 * float(np.prod(w["box"])))
    guess = co.dilute_guess(w["eps"], phi, [1.0, 0.0, 0.0]).reshape(-1)
    rhs = np.tile(np.array([1.0, 0.0, 0.0]), n)
    mv_time = [0.0]

    def mv(v):
        t = time.perf_counter()
        r = geo.field_real_many(v.reshape(1, n, 3), threads)[0].reshape(-1)
        mv_time[0] += time.perf_counter() - t
        return r

    t0 = time.perf_counter()
    _, flag, relres, nmv = co.gmres(mv, rhs, guess, tol, restart, maxit)
    t_rhs = time.perf_counter() - t0
    return geo, {"t_geom": t_geom, "t_rhs": t_rhs, "matvecs": nmv, "t_matvecs": mv_time[0], "relres": relres,
                 "converged": flag == 0}


def cpu_baseline(args, w, sol_mixed):
    """The oracle at N = 100,000 on this host's cores: geometry and one field direction measured,
    the three-direction rate extrapolated (x3).  Also, as the checker, the oracle operator's true
    residual of the GPU's mixed-precision moments."""
    from oracle import ewald_oracle as ew
    threads = ew.host_threads()
    n = w["n"]
    geo, r = oracle_direction(w, threads, args.tol, args.restart)
    rhs = np.zeros((3, n, 3))
    for i in range(3):
        rhs[i, :, i] = 1.0
    t0 = time.perf_counter()
    Am = geo.field_real_many(sol_mixed, threads)
    t_mv3 = time.perf_counter() - t0
    relres = [float(np.linalg.norm(rhs[i] - Am[i]) / np.linalg.norm(rhs[i])) for i in range(3)]
    value = n * 3 / (r["t_geom"] + 3 * r["t_rhs"])
    cb = {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": f"the workload's own size N={n} (RSA phi={w['phi']}, beta={w['beta']}, {int(w['Ngrid'][0])}^3, P={w['P']}): "
                    f"geometry measured {r['t_geom']:.1f} s; field direction x solved in full by float64 GMRES("
                    f"{args.restart}) to {args.tol} measured {r['t_rhs']:.1f} s ({r['matvecs']} matvecs, "
                    f"{r['t_matvecs'] / max(r['matvecs'], 1):.2f} s each); 3-direction rate extrapolated as "
                    f"geometry + 3 x the measured direction",
          "measured": r, "extrapolated": "x3 from one measured field direction",
          "note": "NumPy restatement of the reference Python path, operator spread over the host threads "
                  "(grid components and particle chunks, scipy FFTs with workers)"}
    acc = {"oracle_true_relres_of_mixed_moments": relres, "oracle_batched_matvec_s": t_mv3,
           "what": "||b - A_oracle m|| / ||b|| per field direction, A_oracle = the CPU oracle's float64 operator"}
    return cb, acc


def run_reference(args):
    """The reference algorithm on the host cores at the GPU arm's workload (rank 0 only)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import ewald_oracle as ew
    from oracle.rsa_oracle import rsa as py_rsa
    threads = ew.host_threads()
    t0 = time.perf_counter()
    w = workload(n=args.n, grid=args.grid, placer=py_rsa)     # no compiled library of the package on this arm
    t_place = time.perf_counter() - t0
    n = w["n"]
    geo, r = oracle_direction(w, threads, args.tol, args.restart)
    v = np.random.default_rng(0).standard_normal((1, n, 3))
    for _ in range(max(0, args.warmup)):
        geo.field_real_many(v, threads)
    times = []
    for _ in range(max(1, args.steps)):
        t = time.perf_counter()
        geo.field_real_many(v, threads)
        times.append(time.perf_counter() - t)
    t_mv = float(np.mean(times))
    overhead = max(r["t_rhs"] - r["t_matvecs"], 0.0)          # Arnoldi, Givens, updates of the measured solve
    t_dir = overhead + r["matvecs"] * t_mv
    value = n * 3 / (r["t_geom"] + 3 * t_dir)
    sample = (f"N={n} (the workload's own size): particles by the oracle's pure-Python generator ({t_place:.0f} s, untimed); "
              f"geometry {r['t_geom']:.1f} s and field direction x solved in full ({r['t_rhs']:.1f} s, "
              f"{r['matvecs']} matvecs, relres {r['relres']:.2e}) measured once; each step = one float64 matvec "
              f"({t_mv:.2f} s mean); value = N x 3 / (geometry + 3 x (solve overhead + matvecs x step))")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_mv * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded RSA)",
           "impl": "reference",
           "config": config_dict(w, args, world),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "measured_one_direction": {"particle_solves_per_s": n / (r["t_geom"] / 3 + r["t_rhs"]), **r},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------- other configurations
def workload_quadrupole(args):
    """Dipole + quadrupole (8 unknowns per sphere) on the body-centred-tetragonal
    chain lattice: 20 x 20 x 37 face-centred cells (59,200 sites), 15% vacancies,
    jitter 0.02 (seed 3), field (1,1,0)/sqrt(2), beta = 0.95; mixed precision vs
    a tight float64 solve on the same grid."""
    import torch

    from mutual_polarization_slab_gb300 import quadrupole as gq
    from mutual_polarization_slab_gb300.workloads import bct_chain_lattice

    x, box = bct_chain_lattice(20, 20, 37, vacancy=0.15, jitter=0.02, seed=3)
    n = x.shape[0]
    beta = 0.95
    eps = np.full(n, (1 + 2 * beta) / (1 - beta))
    phi = 4 * math.pi * n / (3 * float(np.prod(box)))
    tol_sp = 1e-4
    rc = (60.0 / phi) ** (1.0 / 3.0)
    xi = math.sqrt(-math.log(tol_sp)) / rc
    tables, rv = gq.default_table(xi)
    H0 = np.array([1.0, 1.0, 0.0]) / math.sqrt(2.0)
    b = torch.zeros((n, 8), dtype=torch.float64, device="cuda")
    b[:, :3] = torch.as_tensor(H0, device="cuda")
    # the tolerance rule's grid (89 x 89 x 95 here) rounded up to 5-smooth FFT sizes (90 x 90 x 96): a finer grid,
    # so at least the rule's accuracy, with the rule's support; the float64 comparison solves run on the same grid
    grid_used = []

    def step(precision, tol, stages=None):
        s = gq.QuadrupoleSystem(x, eps, box, xi, tol_sp, tables, rv, max_rhs=1, fft_friendly=True)
        grid_used[:] = [int(v) for v in s.Ngrid]
        if stages is not None:
            s.profile(True)
        sol, info = s.solve(b, None, tol=tol, restart=30, maxit=args.maxref if precision == "mixed" else 200,
                            precision=precision, inner_tol=args.inner_tol, inner_maxit=args.inner_maxit)
        if stages is not None:
            for prec, (cnt, ms) in s.stage_times().items():
                if cnt:
                    stages[prec] = {k: v / cnt for k, v in ms.items()}
        s.close()
        return sol, info

    def timed(precision, tol, steps, warmup):
        for _ in range(warmup):
            step(precision, tol)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            sol, info = step(precision, tol)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, sol, info

    ms_m, sol_m, info_m = timed("mixed", args.tol, max(1, min(args.steps, 5)), 2)
    ms_64, sol_64, info_64 = timed("fp64", args.tol, 1, 1)
    ref, _ = step("fp64", 1e-11)
    stages = {}
    step("mixed", args.tol, stages)       # one profiled step: per-matvec stage times (CUDA events)
    S_ref = ref[:, :3].mean(dim=0)
    return {
        "workload": f"dipole+quadrupole, BCT chain lattice 20x20x37 cells, N={n}, jitter 0.02, 15% vacancies, "
                    f"beta={beta}, field (1,1,0)/sqrt2, xi={xi:.4f}, rc={rc:.3f}, spectral tol {tol_sp}",
        "metric": "particle-solves/s", "value": n / (ms_m / 1e3), "ms_per_step": ms_m,
        "fp64_plain": {"value": n / (ms_64 / 1e3), "ms_per_step": ms_64, "matvecs": info_64[0].matvecs_fp64},
        "speedup_vs_fp64_plain": ms_64 / ms_m,
        "rel_moment_error_vs_fp64": _rel(sol_m, ref), "fp64_plain_rel_error": _rel(sol_64, ref),
        "fp64_reference": "float64 GMRES to relative residual 1e-11 on the same grid",
        "mean_dipole_rel_error": _rel(sol_m[:, :3].mean(dim=0), S_ref),
        "mixed_matvecs": {"fp64": info_m[0].matvecs_fp64, "fp32": info_m[0].matvecs_fp32},
        "stage_ms_per_matvec": stages,
        "tol": args.tol, "grid": grid_used,
        "grid_of_the_rule": [int(v) for v in np.ceil(1 + np.asarray(box) * 2 * xi * math.sqrt(-math.log(tol_sp))
                                                     / math.pi)]}


def workload_batch(args):
    """Many configurations (polydisperse radii 0.7-1.3, per-particle beta in
    {0.3, 0.9}, volume fraction 0.1-0.35, N log-uniform 500-20000, seed 4), each
    with 16 contrast scalings: 48 right-hand sides per configuration in one
    batched mixed-precision solve.  particle-solves/s = sum N x 3 x 16 / time.
    Moment and tensor errors against float64 solves (1e-10) on every 8th
    configuration."""
    import torch

    from mutual_polarization_slab_gb300 import batch

    cfgs = batch.make_configurations(count=args.configs, seed=4)
    scal = np.linspace(0.1, 1.0, 16)
    stol = args.batch_solver_tol
    # one-time cuFFT plan creation is reported separately, not timed (the metric's definition): one solve
    # per distinct grid creates every plan the timed pass uses
    torch.cuda.synchronize()
    tw = time.perf_counter()
    seen = {}
    for c in cfgs:
        lt = math.sqrt(-math.log(args.batch_tol))
        rc = min((60.0 / c.meta["phi"]) ** (1.0 / 3.0), 0.49 * float(np.min(c.box)))
        key = tuple(int(v) for v in batch.grid_for(c.box, lt / rc, args.batch_tol)[0])
        if key not in seen:
            seen[key] = c.index
            batch.solve_configuration(c, scal, tol=args.batch_tol, solver_tol=stol)
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - tw
    t0 = time.perf_counter()
    solver = lambda cfg: batch.solve_configuration(cfg, scal, tol=args.batch_tol, solver_tol=stol)
    res = batch.solve_configurations(cfgs, scal, tol=args.batch_tol, precision="mixed", workers=args.batch_workers,
                                     solver=solver)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    units = sum(c.n for c in cfgs) * 3 * len(scal)
    if args.batch_native:
        # the same configurations through one native call (mps_solve_batched): inputs prepared on the device,
        # then the library's worker threads build, solve and release them; compared with the pass above
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        nat = batch.solve_batched(cfgs, scal, tol=args.batch_tol, solver_tol=stol, precision="mixed",
                                  streams=args.batch_workers)
        torch.cuda.synchronize()
        dtn = time.perf_counter() - t1
        diff = max(float(np.abs(nat[k][0] - res[k][0]).max() / np.abs(res[k][0]).max()) for k in res)
        return {"workload": f"{len(cfgs)} polydisperse configurations, 3 fields x 16 contrast scalings each, "
                            f"spectral tol {args.batch_tol}, solver tol {stol}, {args.batch_workers} workers",
                "python_threads": {"value": units / dt, "seconds": dt,
                                   "converged": sum(1 for v in res.values() if v[1])},
                "native": {"value": units / dtn, "seconds": dtn, "converged": sum(1 for v in nat.values() if v[1])},
                "max_rel_capacitance_difference": diff, "metric": "particle-solves/s",
                "distinct_grids": len(seen), "plan_warmup_seconds_untimed": plan_s}
    # accuracy on a sample of the configurations: mixed vs a tight float64 solve of the same discretisation
    merr, cerr = [], []
    for c in cfgs[::8]:
        Cm, _, Mm = batch.solve_configuration(c, scal, tol=args.batch_tol, solver_tol=stol, return_moments=True)
        C64, _, M64 = batch.solve_configuration(c, scal, tol=args.batch_tol, solver_tol=1e-10, precision="fp64",
                                                return_moments=True)
        merr.append(max(_rel(Mm[k], M64[k]) for k in range(Mm.shape[0])))
        cerr.append(float(np.max(np.linalg.norm((Cm - C64).reshape(len(scal), -1), axis=1)
                                 / np.linalg.norm(C64.reshape(len(scal), -1), axis=1))))
    return {
        "workload": f"{len(cfgs)} polydisperse configurations (N {min(c.n for c in cfgs)}..{max(c.n for c in cfgs)}, "
                    f"sum {sum(c.n for c in cfgs)}), 3 fields x 16 contrast scalings each, spectral tol "
                    f"{args.batch_tol}, solver tol {stol}",
        "metric": "particle-solves/s", "value": units / dt, "seconds": dt,
        "converged": sum(1 for v in res.values() if v[1]), "configs": len(cfgs), "workers": args.batch_workers,
        "distinct_grids": len(seen), "plan_warmup_seconds_untimed": plan_s,
        "rel_moment_error_vs_fp64": {"max": max(merr), "median": float(np.median(merr)), "configs_checked": len(merr),
                                     "per_config_max_over_rhs": merr},
        "capacitance_tensor_rel_error": {"max": max(cerr), "median": float(np.median(cerr))},
        "fp64_reference": "float64 GMRES to 1e-10 on the same discretisation, every 8th configuration"}


def workload_forces(args):
    """N = 200,000 spheres by RSA at volume fraction 0.35 (seed 5), beta = 0.9,
    H0 = (0, 0, 1); E = -1/2 m.H0 with adjoint forces dE/dx and dE/dbeta (mixed
    solve to 1e-8).  240^3 grid (h = 0.557, the headline spacing rounded to an
    FFT-friendly size), P = 10, rc = (60 / phi)^(1/3), xi = 4 / rc, coupling
    tables at dr = 1e-6 (their segment slopes then follow the smooth couplings,
    so finite differences across table nodes agree with the adjoint).

    Checks: central differences (h = 1e-4) of the energy on 64 seeded particles
    (3 coordinates each), re-solving at x +- h; the far-field limit against the
    point-dipole kernel (the reference's compute_forces, prefactor 1/(4 pi)) on
    the same moments; then Brownian-dynamics steps (dt = 1e-4) re-solving every
    step from the previous moments."""
    import torch

    from mutual_polarization_slab_gb300 import ewald as gew
    from mutual_polarization_slab_gb300 import forces as gf
    from mutual_polarization_slab_gb300.dipole_forces import compute_forces
    from mutual_polarization_slab_gb300.system import SpectralEwaldSystem
    from mutual_polarization_slab_gb300.workloads import rsa

    n, phi, beta = 200_000, 0.35, 0.9
    t0 = time.perf_counter()
    x, box, _ = rsa(n, phi, seed=5)
    t_rsa = time.perf_counter() - t0
    rc = (60.0 / phi) ** (1.0 / 3.0)
    xi = 4.0 / rc
    Ngrid, P = [240, 240, 240], 10
    H0 = np.array([0.0, 0.0, 1.0])
    dr = 1e-6
    r = torch.arange(1, int((rc + 0.5) / dr) + 2, dtype=torch.float64, device="cuda") * dr
    tt = gew.real_space_table(r, xi)
    tables = (tt[2].contiguous(), tt[3].contiguous(), torch.cat((torch.zeros(1, dtype=torch.float64,
                                                                             device="cuda"), r)))
    xd = torch.as_tensor(x, device="cuda")
    eps = gf.eps_from_beta(np.full(n, beta))

    def energy(xx=xd, guess=None, tol=1e-8):
        return gf.polarization_energy(xx, beta, box, H0, xi, rc, Ngrid, P, tol=tol, precision="mixed", guess=guess,
                                      tables=tables)

    energy()                                            # warm-up: plans, tuner
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    res = energy()
    e1.record()
    torch.cuda.synchronize()
    ms_force = e0.elapsed_time(e1)
    m0 = res.moments
    F = res.forces.cpu().numpy()

    # --- central differences of the energy, re-solved at x +- h (variational form 1/2 m.A m - m.H0, whose error
    #     is quadratic in the solve's error), on 64 seeded particles.  The energy (about 1.7e6) is kept per
    #     particle and the two configurations' per-particle values are subtracted before the sum, so the
    #     difference (2 h F, about 1e-4) is not lost to the rounding of two sums of that size.
    h0 = torch.as_tensor(H0, device="cuda")
    rhs = h0.repeat(n, 1)

    def e_var(xx):
        s = SpectralEwaldSystem(xx, eps, box, xi, rc, Ngrid, P, *tables, slab_factor=0.0, max_rhs=1)
        try:
            m, _ = s.solve(rhs, m0, tol=1e-11, restart=30, maxit=8, precision="mixed")
            Am = s.matvec(m, precision="fp64")
        finally:
            s.close()
        return (0.5 * Am - rhs).mul_(m).sum(dim=1)

    rng = np.random.default_rng(5)
    picks = rng.choice(n, 64, replace=False)
    h = 1e-4
    fd_err, fd_err_rms = [], []
    f_rms = float(np.sqrt(np.mean(np.sum(F * F, axis=1))))
    t0 = time.perf_counter()
    for k in picks:
        for d in range(3):
            xp, xm = xd.clone(), xd.clone()
            xp[k, d] += h
            xm[k, d] -= h
            fd = -float((e_var(xp) - e_var(xm)).sum()) / (2 * h)
            fd_err.append(abs(F[k, d] - fd) / np.abs(F[k]).max())
            fd_err_rms.append(abs(F[k, d] - fd) / f_rms)
    t_fd = time.perf_counter() - t0

    # --- far-field limit: the reference's point-dipole kernel on the same moments (spheres do not overlap, so
    #     every real-space coupling beyond contact is the point-dipole one); differences come from the periodic
    #     images and the kernel's cutoff, and shrink as the cutoff grows
    far = {}
    for rcut in (10.0, 20.0, 40.0):
        Fpd, _ = compute_forces(xd, m0, box, rcut, 1.0 / (4.0 * math.pi), True)
        diff = torch.linalg.vector_norm(Fpd - res.forces) / torch.linalg.vector_norm(res.forces)
        far[f"r_cut={rcut:g}"] = float(diff)

    # --- Brownian dynamics
    bd = gf.BrownianDynamics(xd, beta, box, H0, xi, rc, Ngrid, P, dt=1e-4, pol_every=1, tol=1e-8, seed=5,
                             tables=tables)
    bd.step()                                           # first step solves from scratch
    steps = max(1, args.bd_steps)
    torch.cuda.synchronize()
    e0.record()
    bd.run(steps)
    e1.record()
    torch.cuda.synchronize()
    ms_bd = e0.elapsed_time(e1) / steps
    return {
        "workload": f"N={n} RSA phi={phi} (seed 5, {t_rsa:.0f} s to place, untimed), beta={beta}, H0=(0,0,1), "
                    f"240^3, P=10, xi={xi:.4f}, rc={rc:.3f}, tables dr={dr:g}; mixed solve to 1e-8 + adjoint",
        "metric": "force evaluations/s", "value": 1e3 / ms_force, "ms_per_force_evaluation": ms_force,
        "relres": res.relres, "energy": res.energy, "max_force": float(np.abs(F).max()),
        "finite_differences": {"h": h, "particles": 64, "components": len(fd_err),
                               "max_rel_error": float(max(fd_err)), "median_rel_error": float(np.median(fd_err)),
                               "error_measure": "|F_kd - FD_kd| / max_d |F_kd|", "bound": 1e-5,
                               "max_error_over_rms_force": float(max(fd_err_rms)), "rms_force": f_rms,
                               "energy": "1/2 m.A m - m.H0, m re-solved at x +- h (mixed, 1e-11), A float64",
                               "seconds": t_fd},
        "point_dipole_kernel_rel_diff": far,
        "brownian_dynamics": {"ms_per_step": ms_bd, "particle_steps_per_s": n / (ms_bd / 1e3), "steps": steps,
                              "warm_started": True, "solves": bd.solves,
                              "final_energy": bd.energy, "finite": bool(torch.isfinite(bd.x).all())}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--grid", type=int, default=192)
    ap.add_argument("--tol", type=float, default=1e-7)
    ap.add_argument("--restart", type=int, default=30)
    ap.add_argument("--maxref", type=int, default=8)
    ap.add_argument("--resid", default="df", choices=["df", "fp64"],
                    help="operator of the refinement residual: double-float FFTs (df) or cuFFT float64")
    ap.add_argument("--inner", default="grad", choices=["reference", "grad"],
                    help="inner float32 operator: the reference discretisation or its gradient form")
    ap.add_argument("--inner-grid", dest="inner_grid", default="auto", type=lambda v: None if v == "same" else v,
                    help="auto: the gradient-form inner operator on a coarser grid when one is cheaper; same: the "
                         "system's grid")
    ap.add_argument("--inner-tol", dest="inner_tol", type=float, default=1e-4)
    ap.add_argument("--inner-maxit", dest="inner_maxit", type=int, default=3)
    ap.add_argument("--no-cpu", dest="no_cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", dest="no_extra", action="store_true",
                    help="skip the other configurations (quadrupole, batch, forces)")
    ap.add_argument("--only-mixed", dest="only_mixed", action="store_true",
                    help="time only the mixed solve (profiling runs); prints a short JSON line")
    ap.add_argument("--workload", default="tensor", choices=["tensor", "quadrupole", "batch", "forces"],
                    help="tensor: the headline line (with the other configurations as extra keys); "
                         "quadrupole / batch / forces: one of the other configurations alone")
    ap.add_argument("--configs", type=int, default=256, help="batch workload: number of configurations")
    ap.add_argument("--batch-tol", dest="batch_tol", type=float, default=1e-4,
                    help="batch workload: spectral tolerance (cutoff, grid, support)")
    ap.add_argument("--batch-solver-tol", dest="batch_solver_tol", type=float, default=1e-7,
                    help="batch workload: GMRES tolerance")
    ap.add_argument("--batch-native", dest="batch_native", action="store_true",
                    help="batch workload: also time the native many-configuration call (mps_solve_batched) "
                         "against the Python-thread pass (no float64 accuracy pass)")
    ap.add_argument("--batch-workers", dest="batch_workers", type=int, default=4,
                    help="batch workload: configurations solved at a time (host threads, one CUDA stream each)")
    ap.add_argument("--bd-steps", dest="bd_steps", type=int, default=1000, help="forces workload: BD steps")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    one = {"quadrupole": workload_quadrupole, "batch": workload_batch, "forces": workload_forces}
    if args.workload in one:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(one[args.workload](args)), flush=True)
        return
    run_gpu(args)


if __name__ == "__main__":
    main()
