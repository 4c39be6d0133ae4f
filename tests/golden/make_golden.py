"""Generate golden vectors by running the reference Python module itself.

The reference (``CPU - Ewald test/ewald.py`` and ``capacitance.py``) ships no
golden vectors or known-answer files, so its outputs on seeded synthetic inputs
are recorded here and committed as ``*.npz`` beside this script.  Run it in a
checkout that has the reference tree mounted (it is not needed afterwards):

    python tests/golden/make_golden.py /path/to/reference

The reference is imported read-only (no bytecode written).  Large integer lists
are stored as SHA-256 digests plus their lengths; everything else verbatim.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402


def _import_reference(ref_root):
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(ref_root, "CPU - Ewald test"))
    import ewald  # noqa: F401
    import capacitance  # noqa: F401
    return ewald, capacitance


def digest(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int64))
    return hashlib.sha256(a.tobytes()).hexdigest()


def case_small(ew, cap):
    """N=64 RSA at phi=0.2, parameters derived from errortol=1e-5, xi=0.8."""
    x, box, _ = rsa(64, 0.2, seed=11)
    xi, tol = 0.8, 1e-5
    eps = np.full(64, 4.0)
    rc = float(np.sqrt(-np.log(tol)) / xi)
    kcut = 2.0 * xi * np.sqrt(-np.log(tol))
    Ngrid = np.ceil(1.0 + box * kcut / np.pi).astype(int)
    h = box / Ngrid
    P = int(np.ceil(-2.0 * np.log(tol) / np.pi))
    eta = P * (h * xi) ** 2 / np.pi
    r_table = np.arange(0.001, 10.0 + 1e-12, 0.001, dtype=np.float64)
    tabs = ew.real_space_table(r_table, xi)
    perp, para = tabs[2], tabs[3]
    rvals = np.concatenate(([0.0], r_table))
    cell, Ncell = ew.cell_list(x, box, rc)
    p1, p2 = ew.neighbor_list(cell, Ncell)
    p1f, p2f, rhat, A, B = ew.prepare_real_space_pairs(x, box, p1, p2, rc, perp, para, rvals)
    offset, offsetxyz = ew.pre_calculations(P, h)
    lin, w, wc = ew.prepare_grid_kernel(x, Ngrid, h, xi, eta, P, offset, offsetxyz)
    khat, Hc = ew.precompute_kspace(Ngrid, box, xi, eta)
    rng = np.random.default_rng(5)
    m_real = rng.normal(size=(64, 3))
    m_cplx = rng.normal(size=(64, 3)) + 1j * rng.normal(size=(64, 3))
    kw = dict(real_precomp=(p1f, p2f, rhat, A, B), grid_precomp=(lin, w, wc), k_precomp=(khat, Hc))
    args = (x, None, eps, box, p1, p2, Ngrid, h, P, xi, eta, rc, offset, offsetxyz, perp, para, rvals)
    H_real = ew.magnetic_field(args[0], m_real, *args[2:], **kw, slab_factor=1.0)
    H_cplx = ew.magnetic_field(args[0], m_cplx, *args[2:], **kw, slab_factor=1.0)
    H_loop = ew.magnetic_field(args[0], m_real, *args[2:], slab_factor=0.0)
    Hk, Hr, Hs = ew.magnetic_field_components(args[0], m_real, *args[2:], **kw, slab_factor=1.0)
    grid_spread = ew.spread_fast(m_real, Ngrid, lin, w)
    Ht = ew.contract_fast(grid_spread, Ngrid, lin, wc)
    fH = np.fft.fftshift(np.fft.fftn(grid_spread, axes=(0, 1, 2)), axes=(0, 1, 2))
    scaled = ew.scale_fast(fH, khat, Hc)
    Hr_fast = ew.real_space_fast(m_real, eps, p1f, p2f, rhat, A, B, perp[0])
    C, p = cap.run_capacitance(x, box, eps, xi, np.array([0.0, 0.0, 1.0]), errortol=tol)
    C2, p2sol = cap.run_capacitance(x, box, eps, xi, np.array([1.0, 1.0, 0.0]), errortol=1e-6,
                                    use_scipy_gmres=False)
    tsel = np.r_[0:60, 60:10001:37, 10000]
    return dict(
        x=x, box=box, eps=eps, xi=xi, tol=tol, rc=rc, Ngrid=Ngrid, h=h, P=P, eta=eta,
        cell=cell, Ncell=Ncell, p1=p1, p2=p2, p1f=p1f, p2f=p2f, rhat=rhat, A=A, B=B,
        offset=offset, offsetxyz=offsetxyz, linnode=lin, w_spread=w, w_contract=wc,
        khat=khat.real, Htildecoeff=Hc, m_real=m_real, m_cplx=m_cplx, H_real=H_real, H_cplx=H_cplx,
        H_loop=H_loop, Hk=Hk, Hr=Hr, Hslab=Hs, grid_spread=grid_spread.real, contract_of_spread=Ht,
        scaled=scaled, Hr_fast=Hr_fast, C=C, p=p, C2=C2, p2sol=p2sol,
        table_idx=tsel, tables=np.stack([t[tsel] for t in tabs]), rvals_sel=rvals[tsel],
    )


def case_c1(ew, cap):
    """N=1000 RSA at phi=0.2 (seed 1): xi=0.5, rc=8, 64^3, P=8, GMRES(30) to 1e-8,
    beta=0.5 (eps=4), fully periodic (slab_factor 0), 3-direction tensor."""
    from scipy.sparse.linalg import LinearOperator, gmres
    N = 1000
    x, box, _ = rsa(N, 0.2, seed=1)
    xi, rc, P = 0.5, 8.0, 8
    Ngrid = np.array([64, 64, 64])
    h = box / Ngrid
    eta = P * (h * xi) ** 2 / np.pi
    beta = 0.5
    eps = np.full(N, (1.0 + 2.0 * beta) / (1.0 - beta))
    r_table = np.arange(0.001, 10.0 + 1e-12, 0.001, dtype=np.float64)
    tabs = ew.real_space_table(r_table, xi)
    perp, para = tabs[2], tabs[3]
    rvals = np.concatenate(([0.0], r_table))
    cell, Ncell = ew.cell_list(x, box, rc)
    p1, p2 = ew.neighbor_list(cell, Ncell)
    pre = ew.prepare_real_space_pairs(x, box, p1, p2, rc, perp, para, rvals)
    offset, offsetxyz = ew.pre_calculations(P, h)
    grid = ew.prepare_grid_kernel(x, Ngrid, h, xi, eta, P, offset, offsetxyz)
    kpre = ew.precompute_kspace(Ngrid, box, xi, eta)
    rng = np.random.default_rng(7)
    m_real = rng.normal(size=(N, 3))

    def field(mv):
        return ew.magnetic_field(x, np.asarray(mv).reshape(N, 3), eps, box, p1, p2, Ngrid, h, P, xi, eta, rc,
                                 offset, offsetxyz, perp, para, rvals, real_precomp=pre,
                                 grid_precomp=grid, k_precomp=kpre, slab_factor=0.0).reshape(-1)

    H_real = field(m_real).reshape(N, 3)
    phi = 4.0 * np.pi * N / (3.0 * np.prod(box))
    amp = 4.0 * np.pi * beta / (1.0 - beta * phi)
    guess = np.zeros((N, 3))
    C = np.zeros((3, 3), dtype=np.complex128)
    S = np.zeros((N, 3, 3), dtype=np.complex128)
    op = LinearOperator((3 * N, 3 * N), matvec=field, dtype=np.complex128)
    t0 = time.perf_counter()
    for i in range(3):
        if i == 0:
            guess = np.zeros((N, 3))
            guess[:, 0] = amp
        b = np.tile(np.eye(3)[i], N).astype(np.complex128)
        sol, info = gmres(op, b, x0=guess.reshape(-1).astype(np.complex128), restart=30, maxiter=100,
                          rtol=1e-8, atol=0.0)
        Si = sol.reshape(N, 3)
        S[:, :, i] = Si
        C[i] = Si.mean(axis=0)
        guess = Si[:, [2, 0, 1]]
    wall = time.perf_counter() - t0
    return dict(
        x=x, box=box, eps=eps, xi=xi, rc=rc, Ngrid=Ngrid, P=P, eta=eta, beta=beta,
        Ncell=Ncell, n_cand=p1.size, cand_p1_sha=digest(p1), cand_p2_sha=digest(p2),
        n_pairs=pre[0].size, p1f_sha=digest(pre[0]), p2f_sha=digest(pre[1]),
        pair_A_sel=pre[3][::97], pair_B_sel=pre[4][::97],
        m_real=m_real, H_real=H_real, C=C, S=S, ref_tensor_wall_s=wall,
    )


def case_forces(ew, cap):
    """The reference's compiled point-dipole force extension (built from its own
    source by oracle/build_ref.py) on seeded dipoles, periodic and open z."""
    sys.path.insert(0, ROOT)
    from oracle import build_ref
    ext = build_ref.load()
    if ext is None:
        raise SystemExit("reference force extension unavailable (pybind11 or reference tree missing)")
    rng = np.random.default_rng(17)
    n = 400
    box = np.array([22.0, 22.0, 26.0])
    pos = rng.random((n, 3)) * box - box / 2
    dip = rng.normal(size=(n, 3))
    out = dict(pos=pos, dip=dip, box=box, r_cut=6.5, pref=1.7)
    for pz in (True, False):
        for cl in (True, False):
            F, e = ext.compute_forces(pos, dip, box, 6.5, 1.7, pz, cl)
            out[f"F_pz{int(pz)}_cl{int(cl)}"] = F
            out[f"pe_pz{int(pz)}_cl{int(cl)}"] = e
    return out


def case_gmres(ew, cap):
    """The reference's own restarted GMRES (capacitance.gmres_restarted) on small
    dense problems: a converging solve, one stopped by maxit (the best-iterate
    update of each cycle decides x), and a stagnating one (a cyclic shift: no
    column improves on the cycle's start)."""
    rng = np.random.default_rng(23)
    n = 60
    # real data, as the reference's solver receives it (its complex Givens rotation, c = a / rho with complex
    # a, is not unitary, so genuinely complex systems are outside what it solves)
    A = 4.0 * np.eye(n) + 0.35 * rng.normal(size=(n, n))
    b = rng.normal(size=n)
    x0 = np.zeros(n, dtype=np.complex128)
    out = dict(A=A, b=b, x0=x0)
    for tag, (tol, restart, maxit) in {"conv": (1e-10, 10, 50), "stop": (1e-14, 5, 2)}.items():
        x, flag, relres = cap.gmres_restarted(lambda v: A @ v, b, x0, tol, restart, maxit)
        out[f"x_{tag}"], out[f"flag_{tag}"], out[f"relres_{tag}"] = x, flag, relres
        out[f"ctl_{tag}"] = np.array([tol, restart, maxit])
    m = 12
    S = np.roll(np.eye(m), 1, axis=0)      # S e_i = e_{i+1}
    bs = np.zeros(m, dtype=np.complex128)
    bs[0] = 1.0
    x, flag, relres = cap.gmres_restarted(lambda v: S @ v, bs, np.zeros(m, dtype=np.complex128), 1e-8, 5, 3)
    out.update(S=S, bs=bs, x_stag=x, flag_stag=flag, relres_stag=relres)
    return out


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MPS_REFERENCE_ROOT")
    if not ref_root:
        raise SystemExit("usage: make_golden.py <reference root> [case ...]")
    ew, cap = _import_reference(ref_root)
    cases = (("small", case_small), ("c1", case_c1), ("forces", case_forces), ("gmres", case_gmres))
    wanted = set(sys.argv[2:])
    for name, fn in cases:
        if wanted and name not in wanted:
            continue
        t0 = time.perf_counter()
        d = fn(ew, cap)
        np.savez_compressed(os.path.join(HERE, f"golden_{name}.npz"), **d)
        print(f"{name}: {time.perf_counter() - t0:.1f}s")


if __name__ == "__main__":
    main()
