"""Field at probe points from given dipoles (the MATLAB field maps).

Drop-in for ``Compute_Field/FieldMap.m:1-59`` (with ``MagneticField.m``,
``RealSpace.m`` and the typed neighbour list ``NeighborList_Types.m`` of the
same folder): ``E = field_map(x_E, x_p, p, box, xi)`` returns the field at the
probe positions ``x_E`` due to dipoles ``p`` at ``x_p``, with FieldMap's sign
(``E = -MagneticField(...)``) and its fixed spectral tolerance 1e-3.

The whole evaluation runs in ``mps_field_map``: the sources are spread onto
the grid, transformed, scaled by H k^k^ and transformed back, the grid is
contracted at the probes, and the real-space part is summed by one warp per
probe over the sources of the 27 cells around it.  The real-space tables are
``RealSpaceTable.m`` of that folder: the solver's tables without the r < 2
overlap polynomial in field_dip_1 / field_dip_2.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib as L
from .system import as_device

__all__ = ["real_space_table_probe", "field_parameters", "field_map", "quad_tables_probe", "field_map_quadrupole",
           "field_map_sizes"]

ERRORTOL = 1e-3   # FieldMap.m:18


def _is_np(*a):
    return any(not isinstance(v, torch.Tensor) for v in a)


def real_space_table_probe(r, xi):
    """Six tables of ``Compute_Field/RealSpaceTable.m`` (r = 0 self value
    prepended), as CUDA tensors or numpy arrays following ``r``."""
    rd = as_device(r).reshape(-1)
    n = rd.numel()
    out = torch.empty((6, n + 1), dtype=torch.float64, device="cuda")
    L.check(L.lib().mps_real_space_table_probe(L.dptr(rd), n, float(xi), L.dptr(out), L.stream_handle()),
            "real_space_table_probe")
    asnp = _is_np(r)
    return tuple(out[i].cpu().numpy() if asnp else out[i].clone() for i in range(6))


def field_parameters(box, xi, errortol=ERRORTOL):
    """rc, Ngrid, h, P, eta of FieldMap.m:24-30."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(errortol))
    rc = lt / xi
    kcut = 2 * xi * lt
    Ngrid = np.ceil(1 + box * kcut / math.pi).astype(np.int64)
    h = box / Ngrid
    P = int(math.ceil(-2 * math.log(errortol) / math.pi))
    eta = P * (h * xi) ** 2 / math.pi
    return rc, Ngrid, h, P, eta


def _pairs_real(xe, xp, p, box, rc, perp, para, rv, p1, p2):
    """Real-space part over a caller-given probe/particle pair list (FieldMap.m:44-45,
    RealSpace.m:24-58; 1-based indices as MATLAB passes them), on the device."""
    a = as_device(p1, torch.int64).reshape(-1) - 1
    b = as_device(p2, torch.int64).reshape(-1) - 1
    L3 = torch.as_tensor(np.asarray(box, dtype=np.float64).reshape(3), device="cuda")
    r = xe[a] - xp[b]
    r = r - L3 * torch.trunc(2 * r / L3)
    d = torch.linalg.vector_norm(r, dim=1)
    keep = (d < rc) & (d > 0)
    a, b, r, d = a[keep], b[keep], r[keep], d[keep]
    i = torch.searchsorted(rv, d, right=False)
    if i.numel() and (int(i.min()) < 1 or int(i.max()) >= rv.numel()):
        raise ValueError("separation outside the real-space table")
    rh, rl = rv[i], rv[i - 1]
    A = perp[i - 1] * (rh - d) / (rh - rl) + perp[i] * (d - rl) / (rh - rl)
    B = para[i - 1] * (rh - d) / (rh - rl) + para[i] * (d - rl) / (rh - rl)
    rhat = r / d[:, None]
    m = p[b]
    mr = (m * rhat).sum(1, keepdim=True)
    contrib = A[:, None] * (m - mr * rhat) + B[:, None] * mr * rhat
    out = torch.zeros_like(xe)
    out.index_add_(0, a, contrib)
    return out


def field_map(x_E, x_p, p, box, xi, *pairs, errortol=ERRORTOL):
    """Field at the probe points (``FieldMap.m:1-59``).

    x_E (N_E, 3) probe positions, x_p (N_p, 3) particle positions, p (N_p, 3)
    dipoles, box (3,), xi.  ``pairs`` may hold (p1, p2), a probe/particle
    neighbour list with 1-based indices (p1 into x_E, p2 into x_p) as FieldMap's
    varargin; without it the neighbours within rc are found on the device.
    ``errortol`` (keyword only, not in the reference) replaces FieldMap's fixed
    spectral tolerance 1e-3.  Raises ``ValueError`` when rc exceeds half the box
    (FieldMap.m:36-39)."""
    asnp = _is_np(x_E, x_p, p)
    xe = as_device(x_E).reshape(-1, 3).contiguous()
    xp = as_device(x_p).reshape(-1, 3).contiguous()
    pd = as_device(p).reshape(-1, 3).contiguous()
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = field_parameters(box, xi, errortol)
    if np.any(rc > box / 2):
        raise ValueError("Real space cutoff (rc = %.3f) larger than half the box size (%.3f, %.3f, %.3f). "
                         "Accuracy to specified error tolerance not guaranteed." % (rc, *box))
    r_table = torch.arange(1, 10001, dtype=torch.float64, device="cuda") * 1e-3
    _, _, f1, f2, _, _ = real_space_table_probe(r_table, xi)
    rv = torch.cat((torch.zeros(1, dtype=torch.float64, device="cuda"), r_table))
    ne, npart = xe.shape[0], xp.shape[0]
    E = torch.empty((ne, 3), dtype=torch.float64, device="cuda")
    if len(pairs) not in (0, 2):
        raise ValueError("pass both p1 and p2, or neither")
    if ne:
        # with a caller's pair list the device computes the wave part only and the pairs' real part is added here
        L.check(L.lib().mps_field_map(L.dptr(xe), ne, L.dptr(xp), L.dptr(pd), npart, L.host_f64(box), float(xi),
                                      float(rc), L.host_i64(Ngrid), int(P), L.host_f64(eta), L.dptr(f1),
                                      L.dptr(f2), L.dptr(rv), rv.numel(), 0 if pairs else 1, L.dptr(E),
                                      L.stream_handle()),
                "field_map")
        if pairs:
            E = E - _pairs_real(xe, xp, pd, box, rc, f1, f2, rv, pairs[0], pairs[1])
    return E.cpu().numpy() if asnp else E


def quad_tables_probe(r, xi):
    """The 9 couplings of ``Compute_Field_Quadrupole/RealSpaceTable.m`` (no overlap
    polynomials) on separations ``r`` (no zero), r = 0 row prepended: field_dip_1,
    field_dip_2, field_quad_1..3, grad_quad_1..4 as a (9, n+1) CUDA tensor."""
    rd = as_device(r).reshape(-1)
    n = rd.numel()
    dip = real_space_table_probe(rd, xi)
    quad = torch.empty((7, n + 1), dtype=torch.float64, device="cuda")
    L.check(L.lib().mps_quad_table_probe(L.dptr(rd), n, float(xi), L.dptr(quad), L.stream_handle()),
            "quad_table_probe")
    return torch.cat((dip[2].reshape(1, -1), dip[3].reshape(1, -1), quad), dim=0).contiguous()


def field_map_quadrupole(x_E, x_p, p, Q, box, xi, return_gradient=False, *, errortol=ERRORTOL):
    """Field at probe points from dipoles ``p`` (N_p, 3) and quadrupoles ``Q``
    (N_p, 5: xx xy xz yy yz) at ``x_p`` (``Compute_Field_Quadrupole/FieldMap.m:1-58``):
    E (N_E, 3) with FieldMap's sign; with ``return_gradient`` also the field
    gradient G (N_E, 5) its MatrixVectorMultiply computes.  Separation table
    r = 0, 1e-4 .. 10 (FieldMap.m:22); the reference's r = 0 row divides by zero,
    here it holds the solver's r = 0 values (only separations below 1e-4 use it).
    ``errortol`` (keyword only) replaces the fixed spectral tolerance 1e-3."""
    asnp = _is_np(x_E, x_p, p, Q)
    xe = as_device(x_E).reshape(-1, 3).contiguous()
    xp = as_device(x_p).reshape(-1, 3).contiguous()
    sq = torch.cat((as_device(p).reshape(-1, 3), as_device(Q).reshape(-1, 5)), dim=1).contiguous()
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = field_parameters(box, xi, errortol)
    if np.any(rc > box / 2):
        raise ValueError("Real space cutoff (rc = %.3f) larger than half the box size (%.3f, %.3f, %.3f). "
                         "Accuracy to specified error tolerance not guaranteed." % (rc, *box))
    r_table = torch.arange(1, 100001, dtype=torch.float64, device="cuda") * 1e-4
    tab9 = quad_tables_probe(r_table, xi)
    rv = torch.cat((torch.zeros(1, dtype=torch.float64, device="cuda"), r_table))
    ne = xe.shape[0]
    EG = torch.empty((ne, 8), dtype=torch.float64, device="cuda")
    if ne:
        L.check(L.lib().mps_field_map_quad(L.dptr(xe), ne, L.dptr(xp), L.dptr(sq), xp.shape[0], L.host_f64(box),
                                           float(xi), float(rc), L.host_i64(Ngrid), int(P), L.host_f64(eta),
                                           L.dptr(tab9), L.dptr(rv), rv.numel(), 1, L.dptr(EG), L.stream_handle()),
                "field_map_quadrupole")
    E, G = EG[:, :3], EG[:, 3:]
    if asnp:
        E, G = E.cpu().numpy(), G.cpu().numpy()
    return (E, G) if return_gradient else E


def _colon(a, step, b):
    """MATLAB a:step:b."""
    k = int(math.floor((b - a) / step + 1e-10))
    return a + step * np.arange(k + 1, dtype=np.float64)


def field_map_sizes(x_E, x_p, a, p, box, xi, *, errortol=ERRORTOL):
    """Field at probe points from dipoles ``p`` of spheres of radii ``a``
    (``Compute_Field_Sizes/FieldMap.m:1-43``, ``ComputeField.m``, ``RealSpace.m``):
    probes count as spheres of the smallest radius; the real-space table runs over
    r = 0.5 : 1e-3 : rc + 1e-2 (FieldMap.m:31), so a probe closer than 0.5 to a
    sphere centre raises ``ValueError`` as the reference's table lookup fails.
    ``errortol`` (keyword only) replaces the fixed tolerance 1e-3 (also the table step)."""
    from . import sizes as S

    asnp = _is_np(x_E, x_p, p)
    xe = as_device(x_E).reshape(-1, 3).contiguous()
    xp = as_device(x_p).reshape(-1, 3).contiguous()
    pd = as_device(p).reshape(-1, 3).contiguous()
    a_np = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64).reshape(-1)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    tol = float(errortol)
    lt = math.sqrt(-math.log(tol))
    rc = lt / xi
    if np.any(rc > box / 2):
        raise ValueError("Real space cutoff (r_c = %.3f) larger than half the box size (%.3f, %.3f, %.3f)."
                         % (rc, *box))
    a_uniq, cls = S.unique_radii(a_np)
    r_table = _colon(0.5, tol, rc + 10 * tol)
    perp, para = S.real_space_table(np.concatenate(([0.0], r_table)), a_uniq, xi)
    perp = perp.T[:, 1:].contiguous()          # (M(M+1)/2, n) columns, the r = 0 row dropped
    para = para.T[:, 1:].contiguous()
    rv = torch.as_tensor(r_table, device="cuda")
    Ngrid = np.ceil(1 + box * 2 * xi * lt / math.pi).astype(np.int64)   # ComputeField.m:24-29
    hm = float(np.mean(box / Ngrid))
    P = int(math.ceil(2 / hm - 2 * math.log(tol) / math.pi))
    eta = P * (hm * xi) ** 2 / math.pi
    rad = torch.as_tensor(a_np, device="cuda")
    cl = torch.as_tensor(cls, dtype=torch.int32, device="cuda")
    ne = xe.shape[0]
    E = torch.empty((ne, 3), dtype=torch.float64, device="cuda")
    if ne:
        L.check(L.lib().mps_field_map_sizes(L.dptr(xe), ne, L.dptr(xp), L.dptr(rad), L.dptr(cl), int(a_uniq.size),
                                            L.dptr(pd), xp.shape[0], L.host_f64(box), float(xi), float(rc),
                                            L.host_i64(Ngrid), int(P), float(eta), L.dptr(perp), L.dptr(para),
                                            L.dptr(rv), rv.numel(), 1, L.dptr(E), L.stream_handle()),
                "field_map_sizes")
    return E.cpu().numpy() if asnp else E
