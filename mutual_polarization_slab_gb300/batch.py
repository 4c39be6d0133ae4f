"""Many configurations, each with a contrast spectrum, solved as batches.

A configuration is one periodic box of spheres (polydisperse radii, a contrast
beta per particle).  For every configuration the 3 field directions times the
K contrast scalings s_k (beta_i -> s_k beta_i) are 3K right-hand sides of ONE
system: the scalings only change the diagonal, so they are permittivity sets
of one geometry, and all 3K solves share every batched matvec
(``capacitance_tensor_spectrum`` of the polydisperse operator, CS/).

Across configurations the work is independent, so ranks take a static share
(largest configurations first, each to the least loaded rank) and the results
are gathered at the end -- no exchange during the solves.  With
``torch.distributed`` initialised (NCCL on GPUs, gloo in the CPU tests) the
gather is ``all_gather_object``; without it one process does everything.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from .system import fft_size  # noqa: F401  (part of this module's interface)

__all__ = ["Configuration", "make_configurations", "partition", "solve_configuration", "solve_configurations",
           "solve_batched"]


@dataclass
class Configuration:
    x: np.ndarray          # (N, 3) positions
    radii: np.ndarray      # (N,)
    beta: np.ndarray       # (N,) contrast of each particle
    box: np.ndarray        # (3,)
    index: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def n(self):
        return int(self.x.shape[0])


def make_configurations(count=256, seed=4, n_range=(500, 20000), radius_range=(0.7, 1.3), betas=(0.3, 0.9),
                        phi_range=(0.1, 0.35), rsa=None) -> List[Configuration]:
    """Seeded synthetic configurations: N log-uniform in n_range, radii uniform,
    per-particle beta drawn from ``betas`` in equal shares (shuffled), volume
    fraction uniform in phi_range, random sequential addition without overlap
    (largest spheres placed first)."""
    if rsa is None:
        from .workloads import rsa as rsa_fn
        rsa = rsa_fn
    rng = np.random.default_rng(seed)
    out = []
    for c in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        radii = np.sort(rng.uniform(radius_range[0], radius_range[1], n))[::-1].copy()
        phi = float(rng.uniform(*phi_range))
        x, box, _ = rsa(n, phi, seed=int(rng.integers(1 << 31)), radii=radii)
        perm = rng.permutation(n)
        beta = np.resize(np.asarray(betas, dtype=np.float64), n)
        rng.shuffle(beta)
        out.append(Configuration(x[perm], radii[perm], beta, np.asarray(box, dtype=np.float64), c,
                                 {"phi": phi}))
    return out


def partition(sizes: Sequence[int], world: int) -> List[List[int]]:
    """Static longest-processing-time partition of items with the given sizes
    (cost ~ N) over ``world`` ranks; every rank's list is in ascending index order."""
    load = [0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += int(sizes[i])
    return [sorted(p) for p in parts]


def _eps(beta):
    return (1.0 + 2.0 * beta) / (1.0 - beta)




def grid_for(box, xi, tol, fft_friendly=True):
    """(Ngrid, P) of one configuration: the tolerance rule of CS/ComputeField.m:25-31,
    each axis rounded up to an FFT-friendly size when ``fft_friendly`` (a finer
    grid, so at least the rule's accuracy; P follows the finer spacing by the same
    rule).  Configurations then share a few FFT sizes: each new size costs a cuFFT
    plan (tens of ms), which dominated a batch of configurations of distinct sizes."""
    from .sizes import spectral_parameters

    _, ng, _, P, _ = spectral_parameters(box, xi, tol)
    if not fft_friendly:
        return ng, P
    ng = np.array([fft_size(int(v)) for v in ng], dtype=np.int64)
    hm = float(np.mean(np.asarray(box, dtype=np.float64).reshape(3) / ng))
    return ng, int(math.ceil(2 / hm - 2 * math.log(tol) / math.pi))


def _configuration_inputs(cfg: Configuration, s, tol, xi, fft_friendly):
    """Spectral parameters, permittivity sets, right-hand sides, guesses and permittivity-set indices of one
    configuration's 3K solves: (xi, Ngrid, P, eps_sets (K, N), b, x0 (3K, N, 3) on the device, diag_index)."""
    import torch

    K = s.size
    box = np.asarray(cfg.box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(tol))
    if xi is None:
        # real-space cutoff about 60 neighbours' worth, at most just under half the box
        phi = cfg.meta.get("phi", 4 * math.pi * float(np.sum(cfg.radii ** 3)) / (3 * float(np.prod(box))))
        rc = min((60.0 / phi) ** (1.0 / 3.0), 0.49 * float(box.min()))
        xi = lt / rc
    eps_sets = np.stack([_eps(cfg.beta * sk) for sk in s])           # (K, N)
    n = cfg.n
    ng, P = grid_for(box, xi, tol, fft_friendly)
    # right-hand side 3k + i: unit field along i with contrast scaling k; guess 4 pi a^3 beta / (1 - beta phi)
    # along the field (CS/CapacitanceTensorSpectrum.m:45-48), built in a few tensor operations (one
    # assignment per right-hand side costs more host time than a small configuration's solve)
    phi_v = 4 * math.pi * float(np.sum(cfg.radii ** 3)) / (3 * float(np.prod(box)))
    beta = s[:, None] * np.asarray(cfg.beta, dtype=np.float64)[None, :]                  # (K, N)
    amp = torch.as_tensor(4 * math.pi * cfg.radii[None, :] ** 3 * beta / (1 - beta * phi_v), device="cuda")
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[None, :, None, :].expand(K, 3, n, 3).reshape(3 * K, n, 3).contiguous()
    x0 = (amp[:, None, :, None] * eye[None, :, None, :]).reshape(3 * K, n, 3).contiguous()
    diag_index = [k for k in range(K) for _ in range(3)]
    return xi, ng, P, eps_sets, b, x0, diag_index


def solve_configuration(cfg: Configuration, scalings, tol=1e-4, precision="mixed", xi=None, max_rhs_batch=None,
                        fft_friendly=True, return_moments=False, solver_tol=None):
    """C (K, 3, 3) (row i = mean dipole for the unit field along i) of one
    configuration for every contrast scaling, all 3K solves in one batch.
    ``tol`` sets the spectral parameters (cutoff, grid, support) and, unless
    ``solver_tol`` is given, the GMRES tolerance too.  Returns (C, converged), or
    (C, converged, moments (3K, N, 3) on the device) with ``return_moments``."""
    from .sizes import PolydisperseSystem

    s = np.asarray(scalings, dtype=np.float64).reshape(-1)
    K = s.size
    n = cfg.n
    xi, ng, P, eps_sets, b, x0, diag_index = _configuration_inputs(cfg, s, tol, xi, fft_friendly)
    sysm = PolydisperseSystem(cfg.x, cfg.radii, eps_sets, cfg.box, xi, tol, Ngrid=ng, P=P, max_rhs=3 * K)
    try:
        sol, info = sysm.solve(b, x0, tol=tol if solver_tol is None else solver_tol, restart=min(3 * n, 30),
                               maxit=100 if precision != "mixed" else 8,
                               precision=precision, diag_index=diag_index)
        C = sol.reshape(K, 3, n, 3).mean(dim=2).cpu().numpy()
        conv = all(i.converged for i in info)
    finally:
        sysm.close()
    return (C, conv, sol) if return_moments else (C, conv)


def solve_batched(configs: Sequence[Configuration], scalings, tol=1e-4, precision="mixed", xi=None,
                  fft_friendly=True, solver_tol=None, streams=4, return_moments=False):
    """The same results as ``solve_configuration`` for every configuration, solved by one native call
    (``mps_solve_batched``): the library builds, solves and releases the configurations ``streams`` at a
    time, each on a host thread and CUDA stream of its own, with no Python between them.  All inputs are
    prepared on the device first (every configuration's positions, radii, permittivity sets, right-hand
    sides, guesses and solutions are resident at once).  Returns {index: (C, converged)}, with the
    moments as a third entry when ``return_moments``."""
    import ctypes as C

    import torch

    from . import _lib as L
    from .sizes import PolydisperseSystem
    from .system import PRECISIONS

    s = np.asarray(scalings, dtype=np.float64).reshape(-1)
    K = s.size
    specs, keep = [], []
    items = (L.BatchItem * len(configs))()
    for j, cfg in enumerate(configs):
        n = cfg.n
        xi_c, ng, P, eps_sets, b, x0, diag_index = _configuration_inputs(cfg, s, tol, xi, fft_friendly)
        spec = PolydisperseSystem(cfg.x, cfg.radii, eps_sets, cfg.box, xi_c, tol, Ngrid=ng, P=P, max_rhs=3 * K,
                                  create=False)
        x = torch.empty_like(b)
        dix = (C.c_int32 * (3 * K))(*diag_index)
        info = (L.SolveInfo * (3 * K))()
        it = items[j]
        it.desc = spec.desc
        it.b, it.x0, it.x = b.data_ptr(), x0.data_ptr(), x.data_ptr()
        it.nrhs = 3 * K
        it.diag_index = C.cast(dix, C.POINTER(C.c_int32))
        it.info = C.cast(info, C.POINTER(L.SolveInfo))
        specs.append((cfg, spec, x, info))
        keep += [b, x0, dix]
    # solve_configuration's options: restart min(3N, 30), the solver's default inner settings
    restart = min([30] + [3 * c.n for c in configs])
    opts = L.SolveOpts(tol=float(tol if solver_tol is None else solver_tol), restart=restart,
                       maxit=100 if precision != "mixed" else 8, precision=PRECISIONS[precision], inner_tol=1e-4,
                       inner_maxit=4, residual_policy=0, verify=0, residual_precision=PRECISIONS["df"],
                       inner_operator=1)
    lib = L.lib()
    st = lib.mps_solve_batched(items, len(configs), C.byref(opts), int(streams), L.stream_handle())
    if st != L.MPS_NOT_CONVERGED:
        L.check(st, "mps_solve_batched")
    out = {}
    for j, (cfg, spec, x, info) in enumerate(specs):
        n = cfg.n
        Cm = x.reshape(K, 3, n, 3).mean(dim=2).cpu().numpy()
        conv = items[j].status == L.MPS_OK and all(i.converged for i in info)
        out[cfg.index] = (Cm, conv, x) if return_moments else (Cm, conv)
    del keep
    return out


def _solve_concurrently(todo: List[Configuration], solve: Callable, workers: int) -> dict:
    """Solve ``todo`` with ``workers`` host threads, each on its own CUDA stream,
    taking the largest remaining configuration first.  A solve runs in the C
    library with the GIL released, so one thread's host round trips (GMRES
    convergence checks, result read-back) overlap the others' GPU work."""
    import threading

    import torch

    dev = torch.cuda.current_device()
    queue = sorted(todo, key=lambda c: c.n)          # pop() takes the largest
    lock = threading.Lock()
    results: dict = {}
    errors: List[BaseException] = []

    def work():
        try:
            torch.cuda.set_device(dev)
            stream = torch.cuda.Stream()
            with torch.cuda.stream(stream):
                while True:
                    with lock:
                        if not queue or errors:
                            break
                        cfg = queue.pop()
                    out = solve(cfg)
                    with lock:
                        results[cfg.index] = out
            stream.synchronize()
        except BaseException as exc:   # re-raised in the caller
            with lock:
                errors.append(exc)

    threads = [threading.Thread(target=work) for _ in range(min(workers, len(todo)))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return results


def solve_configurations(configs: Sequence[Configuration], scalings, tol=1e-4, precision="mixed",
                         solver: Optional[Callable] = None, gather=True, workers=1):
    """Solve this rank's share of ``configs``; returns {index: (C, converged)} for
    all configurations when gathered, else for this rank's share.  ``workers`` > 1
    solves that many configurations at a time on one GPU (one host thread and CUDA
    stream each)."""
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank() if world > 1 else 0
    parts = partition([c.n for c in configs], world)
    solve = solver or (lambda cfg: solve_configuration(cfg, scalings, tol=tol, precision=precision))
    if workers > 1 and len(parts[rank]) > 1:
        mine = _solve_concurrently([configs[i] for i in parts[rank]], solve, workers)
    else:
        mine = {configs[i].index: solve(configs[i]) for i in parts[rank]}
    if world == 1 or not gather:
        return mine
    everything: List[Optional[dict]] = [None] * world
    dist.all_gather_object(everything, mine)
    merged = {}
    for part in everything:
        merged.update(part)
    return merged
