"""Drop-in for the dipole + quadrupole solver of the MATLAB variant
``Capacitance_Quadrupole`` (cited ``CQ/``): each sphere carries a dipole S and
a traceless quadrupole Q, and the block system

    [M_ES  M_EQ] [S]   [E0]
    [M_GS  M_GQ] [Q] = [ 0]

is solved with GMRES (``CQ/MatrixVectorSolve.m:35-43``).

Layout: the GPU operator keeps the 8 unknowns of a particle together,
(Sx, Sy, Sz, Qxx, Qxy, Qxz, Qyy, Qyz) with Qzz = -(Qxx + Qyy); the functions
below take and return ``S (N,3)`` and ``Q (N,5)`` like the reference.
``matrix_vector_multiply_flat`` works on the reference's flat vector layout
``[S (3N, xyz per particle); Q (5N)]``.

The wave-space part is the real part of the reference's complex pipeline (the
unpaired Nyquist bins of even grids couple symmetrically), as for the dipole
operator.  Tables use separations ``[0, r_1, ...]`` with the r = 0 values
first; the MATLAB spectrum driver evaluates its table on ``[0, 1:1e-4:10]`` and
prepends the self values, which shifts its tables by one entry against the
separations — this module keeps tables and separations aligned.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from . import ewald
from .system import SpectralEwaldSystem, as_device, fft_size, spectral_parameters

__all__ = ["TABLE_ORDER", "real_space_table", "default_table", "QuadrupoleSystem", "matrix_vector_multiply",
           "matrix_vector_multiply_flat", "matrix_vector_solve", "capacitance_tensor",
           "capacitance_tensor_spectrum"]

TABLE_ORDER = ("field_dip_1", "field_dip_2", "field_quad_1", "field_quad_2", "field_quad_3", "grad_quad_1",
               "grad_quad_2", "grad_quad_3", "grad_quad_4")

_TABLE_CACHE: dict = {}


def real_space_table(r, xi):
    """The nine couplings the solve interpolates (``CQ/RealSpaceTable.m:88-378``)
    at separations ``r`` (no zero), each with its r = 0 value first.

    Returns a (9, n+1) float64 CUDA tensor in ``TABLE_ORDER``."""
    rt = as_device(r).reshape(-1).contiguous()
    n = int(rt.numel())
    dip = ewald.real_space_table(rt, float(xi))
    quad = torch.empty((7, n + 1), dtype=torch.float64, device="cuda")
    L.check(L.lib().mps_quad_table(L.dptr(rt), n, float(xi), L.dptr(quad), L.stream_handle()), "mps_quad_table")
    return torch.cat((dip[2].reshape(1, -1), dip[3].reshape(1, -1), quad), dim=0)


def default_table(xi, rmin=0.001, dr=0.001, rmax=10.0):
    """Tables on r = rmin..rmax step dr with 0 prepended, cached per xi and device.
    Returns ((9, n+1) tables, (n+1,) separations) as CUDA tensors on the current device."""
    key = (float(xi), float(rmin), float(dr), float(rmax), torch.cuda.current_device())
    if key not in _TABLE_CACHE:
        r = np.arange(rmin, rmax + 1e-12, dr, dtype=np.float64)
        tabs = real_space_table(r, float(xi))
        rv = torch.cat((torch.zeros(1, dtype=torch.float64, device="cuda"), torch.as_tensor(r, device="cuda")))
        _TABLE_CACHE[key] = (tabs, rv)
    return _TABLE_CACHE[key]


def _params(box, xi, errortol, rc, Ngrid, P, fft_friendly=False):
    rc0, Ng0, _, P0, _ = spectral_parameters(box, xi, errortol)
    rc = rc0 if rc is None else float(rc)
    if Ngrid is None and fft_friendly:
        # each axis of the rule's grid rounded up to a 5-smooth size: a finer grid (at least the rule's accuracy;
        # the support P of the rule does not depend on the spacing) that cuFFT transforms without prime factors
        Ngrid = np.array([fft_size(int(v)) for v in Ng0], dtype=np.int64)
    Ngrid = Ng0 if Ngrid is None else np.asarray(Ngrid, dtype=np.int64).reshape(3)
    P = P0 if P is None else int(P)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    eta = P * (box / Ngrid * xi) ** 2 / math.pi
    if np.any(rc > box / 2.0):
        raise ValueError("Real space cutoff larger than half the box size; accuracy to the error tolerance "
                         "is not guaranteed (CQ/CapacitanceTensor.m:40-42).")
    return rc, Ngrid, P, eta


class QuadrupoleSystem(SpectralEwaldSystem):
    """Device-resident geometry of one configuration for the 8-unknown operator.

    ``tables``/``r_vals`` default to ``default_table(xi)``; ``errortol`` fixes
    rc, grid and support as ``CQ/CapacitanceTensor.m:30-36`` (each may be
    overridden; ``fft_friendly=True`` rounds each axis of that grid up to a
    5-smooth size).  ``lambda_p`` may hold several permittivity sets (K, N)."""

    def __init__(self, x, lambda_p, box, xi, errortol, tables=None, r_vals=None, *, rc=None, Ngrid=None, P=None,
                 max_rhs=3, fft_friendly=False):
        if tables is None:
            tables, r_vals = default_table(xi)
        tables = as_device(tables).reshape(9, -1)
        rc, Ngrid, P, eta = _params(box, xi, errortol, rc, Ngrid, P, fft_friendly)
        super().__init__(x, lambda_p, box, xi, rc, Ngrid, P, tables[0], tables[1], r_vals, slab_factor=0.0,
                         eta=eta, max_rhs=max_rhs, quad_tables=tables[2:])
        self.errortol = float(errortol)

    @staticmethod
    def pack(S, Q):
        """(N,3), (N,5) -> (N,8) (or with a leading batch axis)."""
        return torch.cat((as_device(S), as_device(Q)), dim=-1).contiguous()

    @staticmethod
    def unpack(v):
        return v[..., :3], v[..., 3:]


def _real(a):
    if isinstance(a, torch.Tensor):
        return a.real if a.is_complex() else a
    return np.real(np.asarray(a))


def matrix_vector_multiply(x, S, Q, lambda_p, box, xi, errortol, tables=None, r_vals=None, *, rc=None, Ngrid=None,
                           P=None, precision="fp64", system=None):
    """Field E (N,3) and field gradient G (N,5) induced by dipoles S and
    quadrupoles Q (``CQ/MatrixVectorMultiply.m:31-77``)."""
    asnp = not isinstance(x, torch.Tensor)
    sysm = system or QuadrupoleSystem(x, lambda_p, box, xi, errortol, tables, r_vals, rc=rc, Ngrid=Ngrid, P=P,
                                      max_rhs=1)
    out = sysm.matvec(QuadrupoleSystem.pack(_real(S), _real(Q)), precision=precision)
    E, G = QuadrupoleSystem.unpack(out)
    if system is None:
        sysm.close()
    if asnp:
        return E.cpu().numpy(), G.cpu().numpy()
    return E, G


def matrix_vector_multiply_flat(system, v, precision="fp64"):
    """The operator on the reference's flat layout ``[S (3N); Q (5N)]``
    (the ``fun`` of ``CQ/MatrixVectorSolve.m:53-66``)."""
    n = system.n
    vt = as_device(_real(v)).reshape(-1)
    m = QuadrupoleSystem.pack(vt[:3 * n].reshape(n, 3), vt[3 * n:].reshape(n, 5))
    out = system.matvec(m, precision=precision)
    res = torch.cat((out[:, :3].reshape(-1), out[:, 3:].reshape(-1)))
    return res.cpu().numpy() if not isinstance(v, torch.Tensor) else res


def matrix_vector_solve(x, lambda_p, E0, S_guess, Q_guess, box, xi, errortol, tables=None, r_vals=None, *, rc=None,
                        Ngrid=None, P=None, restart=10, maxit=100, precision="fp64", inner_tol=1e-4, inner_maxit=4,
                        system=None, return_info=False):
    """Dipoles S (N,3) and quadrupoles Q (N,5) for the uniform field E0
    (``CQ/MatrixVectorSolve.m:35-47``: GMRES, restart 10, tolerance errortol,
    100 cycles)."""
    asnp = not isinstance(x, torch.Tensor)
    sysm = system or QuadrupoleSystem(x, lambda_p, box, xi, errortol, tables, r_vals, rc=rc, Ngrid=Ngrid, P=P,
                                      max_rhs=1)
    n = sysm.n
    b = torch.zeros((n, 8), dtype=torch.float64, device="cuda")
    b[:, :3] = torch.as_tensor(np.asarray(_real(E0), dtype=np.float64).reshape(3), device="cuda")
    x0 = QuadrupoleSystem.pack(as_device(_real(S_guess)).reshape(n, 3), as_device(_real(Q_guess)).reshape(n, 5))
    sol, info = sysm.solve(b, x0, tol=float(errortol), restart=restart, maxit=maxit, precision=precision,
                           inner_tol=inner_tol, inner_maxit=inner_maxit)
    S, Q = QuadrupoleSystem.unpack(sol)
    if system is None:
        sysm.close()
    if asnp:
        S, Q = S.cpu().numpy(), Q.cpu().numpy()
    return (S, Q, info[0]) if return_info else (S, Q)


def _q_rotate(Q):
    """Warm start for the next field axis: (xx, xy, xz, yy, yz) -> (zz, yz, xy, xx, xz)
    (``CQ/CapacitanceTensor.m:63``)."""
    return torch.stack((-Q[:, 0] - Q[:, 3], Q[:, 4], Q[:, 1], Q[:, 0], Q[:, 2]), dim=1)


def capacitance_tensor(x, lambda_p, box, S_guess, Q_guess, xi, errortol, tables=None, r_vals=None, *, rc=None,
                       Ngrid=None, P=None, restart=10, maxit=100, precision="fp64", inner_tol=1e-4, inner_maxit=4,
                       batched=True, system=None, return_info=False):
    """C (3,3) with column i the mean dipole for the unit field along i, and the
    moments S (N,3,3), Q (N,5,3) (``CQ/CapacitanceTensor.m:24-67``).

    ``batched=False`` follows the reference: three sequential solves, each
    warm-started from the previous one with S columns [z, x, y] and Q rotated.
    ``batched=True`` solves the three fields as one batch (one batched matvec
    per iteration); field i starts from the given guess rotated onto axis i."""
    asnp = not isinstance(x, torch.Tensor)
    sysm = system or QuadrupoleSystem(x, lambda_p, box, xi, errortol, tables, r_vals, rc=rc, Ngrid=Ngrid, P=P,
                                      max_rhs=3)
    n = sysm.n
    sg = as_device(_real(S_guess)).reshape(n, 3)
    qg = as_device(_real(Q_guess)).reshape(n, 5)
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    kw = dict(tol=float(errortol), restart=restart, maxit=maxit, precision=precision, inner_tol=inner_tol,
              inner_maxit=inner_maxit)
    infos = []
    if batched:
        b = torch.zeros((3, n, 8), dtype=torch.float64, device="cuda")
        x0 = torch.zeros_like(b)
        s_i, q_i = sg, qg
        for i in range(3):
            b[i, :, i] = 1.0
            x0[i] = QuadrupoleSystem.pack(s_i, q_i)
            s_i, q_i = s_i[:, [2, 0, 1]], _q_rotate(q_i)
        sol, infos = sysm.solve(b, x0, **kw)
    else:
        sols = []
        for i in range(3):
            b = torch.zeros((n, 8), dtype=torch.float64, device="cuda")
            b[:, :3] = eye[i]
            si, inf = sysm.solve(b, QuadrupoleSystem.pack(sg, qg), **kw)
            sols.append(si)
            infos += inf
            sg, qg = si[:, [2, 0, 1]].contiguous(), _q_rotate(si[:, 3:]).contiguous()
        sol = torch.stack(sols)
    S = sol[:, :, :3].permute(1, 2, 0).contiguous()     # (N, 3, field)
    Q = sol[:, :, 3:].permute(1, 2, 0).contiguous()     # (N, 5, field)
    Cm = sol[:, :, :3].mean(dim=1).T.contiguous()       # column i = mean dipole for field i
    if system is None:
        sysm.close()
    out = (Cm, S, Q)
    if asnp:
        out = tuple(t.cpu().numpy() for t in out)
    return (*out, infos) if return_info else out


def capacitance_tensor_spectrum(x, box, eps_p, xi, errortol=1e-3, *, rc=None, Ngrid=None, P=None, restart=10,
                                maxit=100, precision="fp64", inner_tol=1e-4, inner_maxit=4, tables=None, r_vals=None):
    """Tensor for every permittivity column of ``eps_p (N, N_k)`` and every frame of
    ``x (N,3[,F])`` (``CQ/CapacitanceTensorSpectrum.m:14-67``, errortol 1e-3).

    The N_k columns of a frame share one geometry (the permittivity enters only
    the diagonal) and all 3 N_k solves run as one batch, each field starting
    from the dilute guess 4 pi beta / (1 - beta phi) along its axis.
    Returns C (3,3,N_k) averaged over frames, p (N,3,3,N_k,F), Q (N,5,3,N_k,F)."""
    xn = x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x, dtype=np.float64)
    if xn.ndim == 2:
        xn = xn[:, :, None]
    eps = np.asarray(eps_p, dtype=np.float64)
    if eps.ndim == 1:
        eps = eps[:, None]
    N, F = xn.shape[0], xn.shape[2]
    K = eps.shape[1]
    box = np.asarray(box, dtype=np.float64).reshape(3)
    phi = 4.0 * np.pi * N / (3.0 * np.prod(box))
    if tables is None:
        tables, r_vals = default_table(xi)
    C = np.zeros((3, 3, F, K))
    p = np.zeros((N, 3, 3, K, F))
    Qo = np.zeros((N, 5, 3, K, F))
    for f in range(F):
        sysm = QuadrupoleSystem(xn[:, :, f], eps.T.copy(), box, xi, errortol, tables, r_vals, rc=rc, Ngrid=Ngrid,
                                P=P, max_rhs=3 * K)
        b = torch.zeros((3 * K, N, 8), dtype=torch.float64, device="cuda")
        x0 = torch.zeros_like(b)
        diag_index = []
        for k in range(K):
            with np.errstate(invalid="ignore"):
                beta = (eps[:, k] - 1.0) / (eps[:, k] + 2.0)
            beta[np.isinf(eps[:, k])] = 1.0
            amp = torch.as_tensor(4 * np.pi * beta / (1 - beta * phi), device="cuda")
            for i in range(3):
                b[3 * k + i, :, i] = 1.0
                x0[3 * k + i, :, i] = amp
                diag_index.append(k)
        sol, _ = sysm.solve(b, x0, tol=errortol, restart=restart, maxit=maxit, precision=precision,
                            inner_tol=inner_tol, inner_maxit=inner_maxit, diag_index=diag_index)
        sol = sol.reshape(K, 3, N, 8).cpu().numpy()
        for k in range(K):
            for i in range(3):
                C[:, i, f, k] = sol[k, i, :, :3].mean(axis=0)
                p[:, :, i, k, f] = sol[k, i, :, :3]
                Qo[:, :, i, k, f] = sol[k, i, :, 3:]
        sysm.close()
    return C.mean(axis=2), p, Qo
