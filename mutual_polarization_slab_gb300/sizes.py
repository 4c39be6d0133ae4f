"""Drop-in for the polydisperse solver of the MATLAB variant ``Capacitance_Sizes``
(cited ``CS/``): spheres of different radii, one induced dipole each.

Same operator surface as the reference: ``real_space_table`` (RealSpaceTable.m),
``compute_field`` (ComputeField.m), ``compute_dipole`` (ComputeDipole.m),
``capacitance_tensor`` (CapacitanceTensor.m), ``capacitance_tensor_spectrum``
(CapacitanceTensorSpectrum.m), ``dipole`` (Dipole.m), ``dipole_spectrum``
(DipoleSpectrum.m).  The neighbour-list arguments ``n1, n2`` of the reference
are accepted and ignored: the system builds its own list from the same cell
list and keeps exactly the pairs closer than the cutoff.

Couplings: with tables (``r_table``, ``Ep_perp``, ``Ep_para``) every pair
interpolates the column of its two radius classes, as ``CS/RealSpace.m``
does; without tables (``Ep_perp=None``) every pair's couplings are evaluated in
closed form at its exact separation, which is what continuous radius
distributions need (the per-pair-of-radii tables would have N(N+1)/2 columns).

Parameters follow ``CS/ComputeField.m:25-31``: ``r_c = sqrt(-ln tol)/xi``,
``N_grid = ceil(1 + L q_c / pi)``, ``P = ceil(2 / mean(h) - 2 ln(tol) / pi)``,
scalar ``eta = P (mean(h) xi)^2 / pi``.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib as L
from .system import SpectralEwaldSystem, as_device

__all__ = ["unique_radii", "real_space_table", "default_r_table", "spectral_parameters", "PolydisperseSystem",
           "compute_field", "compute_dipole", "capacitance_tensor", "capacitance_tensor_spectrum", "dipole",
           "dipole_spectrum"]


def unique_radii(a, tol=1e-12):
    """Distinct radii and the class of each particle, the ``uniquetol(a)`` of
    ``CS/RealSpace.m:21``: sorted values closer than ``tol * max|a|`` to the
    first member of a group join that group."""
    a = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64).reshape(-1)
    order = np.argsort(a, kind="stable")
    thr = tol * float(np.max(np.abs(a)))
    uniq = []
    cls = np.empty(a.size, dtype=np.int32)
    for i in order:
        if not uniq or a[i] - uniq[-1] > thr:
            uniq.append(float(a[i]))
        cls[i] = len(uniq) - 1
    return np.array(uniq), cls


def default_r_table(dr=1e-3):
    """``[0, 1:dr:10]`` (``CS/CapacitanceTensorSpectrum.m:26``, where the step is
    the driver's tol = 1e-3)."""
    return np.concatenate(([0.0], np.arange(1.0, 10.0 + 1e-12, dr)))


def real_space_table(r, a, xi):
    """``[Ep_perp, Ep_para] = RealSpaceTable(r, a, xi)``: (n, M(M+1)/2) CUDA
    tensors for the distinct radii ``a``; ``r[0]`` must be 0 (its row holds the
    r -> 0 value)."""
    rt = as_device(r).reshape(-1).contiguous()
    if float(rt[0]) != 0.0:
        raise ValueError("first entry of the separation table must be r = 0 (CS/RealSpaceTable.m:14-16)")
    au = as_device(a).reshape(-1).contiguous()
    n, M = int(rt.numel()), int(au.numel())
    m = M * (M + 1) // 2
    perp = torch.empty((m, n), dtype=torch.float64, device="cuda")
    para = torch.empty_like(perp)
    L.check(L.lib().mps_sizes_table(L.dptr(rt), n, L.dptr(au), M, float(xi), L.dptr(perp), L.dptr(para),
                                    L.stream_handle()), "mps_sizes_table")
    return perp.T, para.T


def spectral_parameters(box, xi, tol):
    """r_c, N_grid, h, P, scalar eta (``CS/ComputeField.m:25-31``)."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(tol))
    rc = lt / xi
    Ngrid = np.ceil(1 + box * 2 * xi * lt / math.pi).astype(np.int64)
    h = box / Ngrid
    hm = float(np.mean(h))
    P = int(math.ceil(2 / hm - 2 * math.log(tol) / math.pi))
    eta = P * (hm * xi) ** 2 / math.pi
    return rc, Ngrid, h, P, eta


class PolydisperseSystem(SpectralEwaldSystem):
    """Device-resident geometry of one configuration for the polydisperse operator.

    ``eps_p`` may hold several permittivity sets (K, N) for a spectrum batch."""

    def __init__(self, x, a, eps_p, box, xi, tol, r_table=None, Ep_perp=None, Ep_para=None, *, rc=None,
                 Ngrid=None, P=None, max_rhs=3, create=True):
        box = np.asarray(box, dtype=np.float64).reshape(3)
        rc0, ng0, _, P0, _ = spectral_parameters(box, xi, tol)
        rc = rc0 if rc is None else float(rc)
        Ngrid = ng0 if Ngrid is None else np.asarray(Ngrid, dtype=np.int64).reshape(3)
        P = P0 if P is None else int(P)
        hm = float(np.mean(box / Ngrid))
        eta = P * (hm * xi) ** 2 / math.pi
        if np.any(rc > box / 2):
            raise ValueError("Real space cutoff larger than half the box size (CS/CapacitanceTensor.m:31-33).")
        a_np = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64).reshape(-1)
        kw = {}
        if Ep_perp is not None:
            uniq, cls = unique_radii(a_np)
            M = uniq.size
            perp_t = as_device(Ep_perp)
            para_t = as_device(Ep_para)
            if perp_t.dim() == 1:
                perp_t, para_t = perp_t[:, None], para_t[:, None]
            if perp_t.shape[1] != M * (M + 1) // 2:
                raise ValueError("the tables must have one column per pair of distinct radii")
            kw = dict(radius_class=cls, n_class=M, sizes_tables=torch.stack((perp_t.T, para_t.T)).contiguous())
            rvals = r_table
        else:
            rvals = None
        self.radii = a_np
        super().__init__(x, eps_p, box, xi, rc, Ngrid, P, None, None, rvals, slab_factor=0.0,
                         eta=[eta, eta, eta], max_rhs=max_rhs, radius=a_np, create=create, **kw)
        self.eta_scalar = eta
        self.tol = float(tol)


def _guess_amplitude(a, eps, phi):
    """4 pi a^3 alpha / (1 - alpha phi), alpha = (eps-1)/(eps+2), alpha(inf) = 1
    (``CS/CapacitanceTensorSpectrum.m:45-48``)."""
    with np.errstate(invalid="ignore"):
        alpha = (eps - 1.0) / (eps + 2.0)
    alpha[np.isinf(eps)] = 1.0
    return 4 * np.pi * a ** 3 * alpha / (1 - alpha * phi)


def _np(a):
    return np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64)


def compute_field(x, a, p, eps_p, box, n1, n2, xi, r_table, Ep_perp, Ep_para, tol, *, precision="fp64",
                  system=None):
    """External field E0 (N,3) consistent with dipoles p (``CS/ComputeField.m:1-58``)."""
    asnp = not isinstance(x, torch.Tensor)
    sysm = system or PolydisperseSystem(x, a, eps_p, box, xi, tol, r_table, Ep_perp, Ep_para, max_rhs=1)
    out = sysm.matvec(as_device(_np(p).real if asnp else p).reshape(-1, 3), precision=precision)
    if system is None:
        sysm.close()
    return out.cpu().numpy() if asnp else out


def compute_dipole(x, a, eps_p, E0, box, p_guess, n1, n2, xi, r_table, Ep_perp, Ep_para, tol, *, restart=None,
                   maxit=None, precision="fp64", inner_tol=1e-4, inner_maxit=4, system=None, return_info=False):
    """Dipoles p (N,3) induced by the uniform field E0 (``CS/ComputeDipole.m:20-36``:
    GMRES, restart min(3N,10), maxit min(3N,100), tolerance tol)."""
    asnp = not isinstance(x, torch.Tensor)
    sysm = system or PolydisperseSystem(x, a, eps_p, box, xi, tol, r_table, Ep_perp, Ep_para, max_rhs=1)
    n = sysm.n
    b = torch.as_tensor(_np(E0).reshape(3), device="cuda").repeat(n, 1)
    restart = min(3 * n, 10) if restart is None else int(restart)
    maxit = min(3 * n, 100) if maxit is None else int(maxit)
    sol, info = sysm.solve(b, as_device(_np(p_guess)).reshape(n, 3), tol=float(tol), restart=restart, maxit=maxit,
                           precision=precision, inner_tol=inner_tol, inner_maxit=inner_maxit)
    if system is None:
        sysm.close()
    out = sol.cpu().numpy() if asnp else sol
    return (out, info[0]) if return_info else out


def capacitance_tensor(x, a, eps_p, box, p_guess, xi, tol, r_table=None, Ep_perp=None, Ep_para=None, *,
                       restart=None, maxit=None, precision="fp64", inner_tol=1e-4, inner_maxit=4, batched=True,
                       system=None, return_info=False):
    """``[C, p] = CapacitanceTensor(...)`` (``CS/CapacitanceTensor.m:20-55``): C (9,)
    with C[3i:3i+3] the mean dipole for the unit field along i, p (N, 9).

    ``batched=False`` follows the reference (three sequential solves, warm start
    p_i[:, [z, x, y]]); ``batched=True`` solves the three fields together, field
    i starting from the guess rotated onto axis i."""
    asnp = not isinstance(x, torch.Tensor)
    sysm = system or PolydisperseSystem(x, a, eps_p, box, xi, tol, r_table, Ep_perp, Ep_para, max_rhs=3)
    n = sysm.n
    restart = min(3 * n, 10) if restart is None else int(restart)
    maxit = min(3 * n, 100) if maxit is None else int(maxit)
    kw = dict(tol=float(tol), restart=restart, maxit=maxit, precision=precision, inner_tol=inner_tol,
              inner_maxit=inner_maxit)
    g = as_device(_np(p_guess)).reshape(n, 3)
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    if batched:
        b = eye[:, None, :].expand(3, n, 3).contiguous()
        x0 = torch.stack((g, g[:, [2, 0, 1]], g[:, [1, 2, 0]])).contiguous()
        sol, infos = sysm.solve(b, x0, **kw)
    else:
        sols, infos = [], []
        for i in range(3):
            si, inf = sysm.solve(eye[i].repeat(n, 1), g, **kw)
            sols.append(si)
            infos += inf
            g = si[:, [2, 0, 1]].contiguous()
        sol = torch.stack(sols)
    p = sol.permute(1, 0, 2).reshape(n, 9).contiguous()
    C = sol.mean(dim=1).reshape(9)
    if system is None:
        sysm.close()
    out = (C.cpu().numpy(), p.cpu().numpy()) if asnp else (C, p)
    return (*out, infos) if return_info else out


def capacitance_tensor_spectrum(x, box, a, eps_p, xi, *, tol=1e-3, precision="fp64", tables=True, dr=1e-3):
    """``[C, p] = CapacitanceTensorSpectrum(x, box, a, eps_p, xi)``
    (``CS/CapacitanceTensorSpectrum.m:14-62``): C (N_k, 9) averaged over frames,
    p (N, 9, N_k, N_frames).  The N_k permittivity columns of a frame share one
    geometry and the 3 N_k solves run as one batch.  ``tables=True`` uses the
    reference's table on ``[0, 1:dr:10]`` (the reference's step is its tol,
    1e-3); ``False`` the closed form per pair."""
    xn = _np(x)
    if xn.ndim == 2:
        xn = xn[:, :, None]
    eps = _np(eps_p)
    if eps.ndim == 1:
        eps = eps[:, None]
    a_np = _np(a).reshape(-1)
    N, F, K = xn.shape[0], xn.shape[2], eps.shape[1]
    box = np.asarray(box, dtype=np.float64).reshape(3)
    phi = 4 * np.pi * np.sum(a_np ** 3) / (3 * np.prod(box))
    if tables:
        rt = default_r_table(dr)
        uniq, _ = unique_radii(a_np)
        perp, para = real_space_table(rt, uniq, xi)
    else:
        rt = perp = para = None
    n0 = N
    restart, maxit = min(3 * n0, 10), min(3 * n0, 100)
    C = np.zeros((9, F, K))
    p = np.zeros((N, 9, F, K))
    for f in range(F):
        sysm = PolydisperseSystem(xn[:, :, f], a_np, eps.T.copy(), box, xi, tol, rt, perp, para, max_rhs=3 * K)
        b = torch.zeros((3 * K, N, 3), dtype=torch.float64, device="cuda")
        x0 = torch.zeros_like(b)
        diag_index = []
        for k in range(K):
            amp = torch.as_tensor(_guess_amplitude(a_np, eps[:, k], phi), device="cuda")
            for i in range(3):
                b[3 * k + i, :, i] = 1.0
                x0[3 * k + i, :, i] = amp
                diag_index.append(k)
        sol, _ = sysm.solve(b, x0, tol=tol, restart=restart, maxit=maxit, precision=precision,
                            diag_index=diag_index)
        sol = sol.reshape(K, 3, N, 3).cpu().numpy()
        for k in range(K):
            for i in range(3):
                C[3 * i:3 * i + 3, f, k] = sol[k, i].mean(axis=0)
                p[:, 3 * i:3 * i + 3, f, k] = sol[k, i]
        sysm.close()
    return C.mean(axis=1).T, p.transpose(0, 1, 3, 2)


def dipole(x, a, eps_p, box, E_0, p_guess, xi, tol, r_table=None, Ep_perp=None, Ep_para=None, *, precision="fp64"):
    """``[p_ave, p] = Dipole(...)`` (``CS/Dipole.m:18-39``)."""
    p = compute_dipole(x, a, eps_p, E_0, box, p_guess, None, None, xi, r_table, Ep_perp, Ep_para, tol,
                       precision=precision)
    return p.mean(axis=0) if isinstance(p, np.ndarray) else p.mean(dim=0), p


def dipole_spectrum(x, box, a, eps_p, E_0, xi, p_guess=None, *, tol=1e-3, precision="fp64", tables=True,
                    dr=1e-3):
    """``[p_ave, p] = DipoleSpectrum(x, box, a, eps_p, E_0, xi[, p_guess])``
    (``CS/DipoleSpectrum.m:16-68``): p_ave (N_k, 3) averaged over frames,
    p (N, 3, N_k, N_frames); all N_k columns of a frame solved as one batch.
    ``p_guess`` (N, 3, N_k, N_frames) replaces the dilute guess."""
    xn = _np(x)
    if xn.ndim == 2:
        xn = xn[:, :, None]
    eps = _np(eps_p)
    if eps.ndim == 1:
        eps = eps[:, None]
    a_np = _np(a).reshape(-1)
    E0 = _np(E_0).reshape(3)
    N, F, K = xn.shape[0], xn.shape[2], eps.shape[1]
    box = np.asarray(box, dtype=np.float64).reshape(3)
    phi = 4 * np.pi * np.sum(a_np ** 3) / (3 * np.prod(box))
    if tables:
        rt = default_r_table(dr)
        uniq, _ = unique_radii(a_np)
        perp, para = real_space_table(rt, uniq, xi)
    else:
        rt = perp = para = None
    restart, maxit = min(3 * N, 10), min(3 * N, 100)
    pav = np.zeros((3, F, K))
    p = np.zeros((N, 3, F, K))
    for f in range(F):
        sysm = PolydisperseSystem(xn[:, :, f], a_np, eps.T.copy(), box, xi, tol, rt, perp, para, max_rhs=K)
        b = torch.as_tensor(E0, device="cuda").repeat(K, N, 1).contiguous()
        if p_guess is None:
            x0 = torch.stack([torch.as_tensor(_guess_amplitude(a_np, eps[:, k], phi)[:, None] * E0[None, :],
                                              device="cuda") for k in range(K)])
        else:
            pg = _np(p_guess)
            x0 = torch.as_tensor(np.stack([pg[:, :, k, f] for k in range(K)]), device="cuda")
        sol, _ = sysm.solve(b, x0.contiguous(), tol=tol, restart=restart, maxit=maxit, precision=precision,
                            diag_index=list(range(K)))
        sol = sol.cpu().numpy()
        for k in range(K):
            pav[:, f, k] = sol[k].mean(axis=0)
            p[:, :, f, k] = sol[k]
        sysm.close()
    return pav.mean(axis=1).T, p.transpose(0, 1, 3, 2)
