"""CPU restatement of the probe-point field map -- test infrastructure only.

Follows ``Compute_Field/FieldMap.m:1-59`` (parameters :18-33, rc guard :36-39,
E = -MagneticField :55), ``MagneticField.m:33-72`` (spread the particle dipoles,
FFT, scale, inverse FFT, contract at the probes, plus the real-space part),
``RealSpace.m:24-58`` (probe/particle pairs within rc, d > 0, table lerp
between the first row with rvals >= d and the row before) and
``RealSpaceTable.m`` of that folder (field_dip_1/2 without the r < 2 overlap
polynomial, lines 80-86 and 102-109).  The wave part uses the reference's
complex pipeline; its real part is what the GPU field map returns.

Parity unpinned for this folder: MATLAB is not runnable here and the folder
ships no golden vectors.  The pieces it shares with the solver (grid weights,
spread, scale, contract, the table polynomials) are the ``ewald_oracle``
functions pinned against the Python reference.
"""
import math

import numpy as np

from . import ewald_oracle as ew

ERRORTOL = 1e-3   # FieldMap.m:18


def real_space_table_probe(r, xi):
    """field_dip_1, field_dip_2 of Compute_Field/RealSpaceTable.m at separations r
    (no zero), r = 0 self value prepended."""
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    t = ew._table_terms(float(xi))
    out = []
    for name in ("field_dip_1", "field_dip_2"):
        spec = list(t[name])
        spec[-1] = lambda rr: 0.0 * rr          # no overlap polynomial
        out.append(ew._eval_table(r, float(xi), tuple(spec)))
    _, s_fd = ew.self_terms(float(xi))
    return np.concatenate(([s_fd], out[0])), np.concatenate(([s_fd], out[1]))


def field_parameters(box, xi, errortol=ERRORTOL):
    """FieldMap.m:24-30."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(errortol))
    rc = lt / xi
    Ngrid = np.ceil(1 + box * 2 * xi * lt / math.pi).astype(np.int64)
    h = box / Ngrid
    P = int(math.ceil(-2 * math.log(errortol) / math.pi))
    eta = P * (h * xi) ** 2 / math.pi
    return rc, Ngrid, h, P, eta


def real_part_pairs(x_E, x_p, p, box, rc, perp, para, rvals, pairs=None):
    """RealSpace.m:24-58 over the given (0-based) pairs, or over every probe/particle pair."""
    x_E = np.asarray(x_E, dtype=np.float64)
    x_p = np.asarray(x_p, dtype=np.float64)
    p = np.asarray(p, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    if pairs is None:
        a, b = np.meshgrid(np.arange(x_E.shape[0]), np.arange(x_p.shape[0]), indexing="ij")
        a, b = a.reshape(-1), b.reshape(-1)
    else:
        a, b = (np.asarray(v, dtype=np.int64).reshape(-1) for v in pairs)
    r = x_E[a] - x_p[b]
    r = r - box * np.trunc(2 * r / box)
    d = np.sqrt(np.sum(r * r, axis=1))
    keep = (d < rc) & (d > 0)
    a, b, r, d = a[keep], b[keep], r[keep], d[keep]
    i = np.searchsorted(rvals, d, side="left")
    rh, rl = rvals[i], rvals[i - 1]
    A = perp[i - 1] * (rh - d) / (rh - rl) + perp[i] * (d - rl) / (rh - rl)
    B = para[i - 1] * (rh - d) / (rh - rl) + para[i] * (d - rl) / (rh - rl)
    rhat = r / d[:, None]
    m = p[b]
    mr = np.sum(m * rhat, axis=1)[:, None]
    contrib = A[:, None] * (m - mr * rhat) + B[:, None] * mr * rhat
    out = np.zeros_like(x_E)
    np.add.at(out, a, contrib)
    return out


def field_map(x_E, x_p, p, box, xi, errortol=ERRORTOL):
    """E = -(Hk + Hr) at the probes (FieldMap.m:1-59); complex (the reference's pipeline).
    errortol: FieldMap's fixed 1e-3 unless given."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = field_parameters(box, xi, errortol)
    if np.any(rc > box / 2):
        raise ValueError("Real space cutoff larger than half the box size")
    r_table = np.arange(1, 10001, dtype=np.float64) * 1e-3
    perp, para = real_space_table_probe(r_table, xi)
    rvals = np.concatenate(([0.0], r_table))
    lin_p, w_p, _ = ew.prepare_grid_kernel(x_p, Ngrid, h, xi, eta, P)
    H = ew.spread_fast(p, Ngrid, lin_p, w_p)
    Ht = ew.wave_space_complex(H, Ngrid, box, xi, eta)
    lin_e, _, wc_e = ew.prepare_grid_kernel(x_E, Ngrid, h, xi, eta, P)
    Hk = ew.contract_fast(Ht, Ngrid, lin_e, wc_e)
    Hr = real_part_pairs(x_E, x_p, p, box, rc, perp, para, rvals)
    return -(Hk + Hr)


# ---------------------------------------------------------------------------
# Quadrupole field map (Compute_Field_Quadrupole/FieldMap.m:1-58, MatrixVectorMultiply.m,
# RealSpace.m, RealSpaceTable.m without any overlap polynomial)
# ---------------------------------------------------------------------------
def quad_tables_probe(r, xi):
    """The 9 couplings of the quadrupole field map on separations r (no zero) with the
    solver's r = 0 values prepended (the reference evaluates r = 0 itself, which
    divides by zero; only separations below the first table step use that row)."""
    from . import quadrupole_oracle as qo
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    f1, f2 = real_space_table_probe(r, xi)
    t = qo._quad_terms(float(xi))
    out = {"field_dip_1": f1, "field_dip_2": f2}
    for k in qo.QUAD_TABLES:
        spec = list(t[k])
        spec[-1] = lambda rr: 0.0 * rr
        head = qo.quad_self(float(xi)) if k == "grad_quad_2" else 0.0
        out[k] = np.concatenate(([head], ew._eval_table(r, float(xi), tuple(spec))))
    return out


def field_map_quadrupole(x_E, x_p, S, Q, box, xi, errortol=ERRORTOL):
    """E (N_E, 3) and G (N_E, 5) at the probes with FieldMap's sign, complex (the
    reference's pipeline)."""
    from . import quadrupole_oracle as qo
    x_E = np.asarray(x_E, dtype=np.float64)
    x_p = np.asarray(x_p, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = field_parameters(box, xi, errortol)
    if np.any(rc > box / 2):
        raise ValueError("Real space cutoff larger than half the box size")
    r_table = np.arange(1, 100001, dtype=np.float64) * 1e-4
    tables = quad_tables_probe(r_table, xi)
    rvals = np.concatenate(([0.0], r_table))
    M = np.concatenate((np.asarray(S, dtype=np.float64), np.asarray(Q, dtype=np.float64)), axis=1)
    lin_p, w_p, _ = ew.prepare_grid_kernel(x_p, Ngrid, h, xi, eta, P)
    G = int(np.prod(Ngrid))
    grids = np.empty((G, 8))
    for c in range(8):
        grids[:, c] = np.bincount(lin_p.reshape(-1), (w_p * M[:, c:c + 1]).reshape(-1), minlength=G)
    nx, ny, nz = (int(v) for v in Ngrid)
    grids = grids.reshape(nz, ny, nx, 8).transpose(2, 1, 0, 3)
    Ht = qo.wave_space_quad(grids, Ngrid, box, xi, eta)
    lin_e, _, wc_e = ew.prepare_grid_kernel(x_E, Ngrid, h, xi, eta, P)
    wave = np.empty((x_E.shape[0], 8), dtype=np.complex128)
    for c in range(8):
        flat = Ht[..., c].transpose(2, 1, 0).reshape(-1)
        wave[:, c] = np.sum(wc_e * flat[lin_e], axis=1)
    a, b = np.meshgrid(np.arange(x_E.shape[0]), np.arange(x_p.shape[0]), indexing="ij")
    a, b = a.reshape(-1), b.reshape(-1)
    r = x_E[a] - x_p[b]
    r = r - box * np.trunc(2 * r / box)
    d = np.sqrt(np.sum(r * r, axis=1))
    keep = (d < rc) & (d > 0)
    a, b, r, d = a[keep], b[keep], r[keep], d[keep]
    dE, dG = qo.quad_pair_terms(r / d[:, None], d, M[b, :3], M[b, 3:], tables, rvals)
    real = np.zeros((x_E.shape[0], 8))
    np.add.at(real, a, np.concatenate((dE, dG), axis=1))
    EG = -(wave + real)
    return EG[:, :3], EG[:, 3:]


# ---------------------------------------------------------------------------
# Polydisperse field map (Compute_Field_Sizes/FieldMap.m:1-43, ComputeField.m:1-40, RealSpace.m:1-77)
# ---------------------------------------------------------------------------
def field_map_sizes(x_E, x_p, a, p, box, xi, errortol=ERRORTOL):
    """E (N_E, 3) with FieldMap's sign; probes are spheres of the smallest radius."""
    from . import polydisperse_oracle as po
    x_E = np.asarray(x_E, dtype=np.float64)
    x_p = np.asarray(x_p, dtype=np.float64)
    p = np.asarray(p, dtype=np.float64)
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    tol = float(errortol)
    rc, Ngrid, h, P, eta = po.spectral_parameters(box, xi, tol)
    if np.any(rc > box / 2):
        raise ValueError("Real space cutoff larger than half the box size")
    a_uniq, cls = po.unique_radii(a)
    k = int(math.floor((rc + 10 * tol - 0.5) / tol + 1e-10))
    r_table = 0.5 + tol * np.arange(k + 1, dtype=np.float64)
    perp, para = po.real_space_table(np.concatenate(([0.0], r_table)), a_uniq, xi)
    perp, para = perp[1:], para[1:]
    # wave space: sources with their radii, probes with the smallest radius
    lin_p, rvec_p = po.stencil(x_p, Ngrid, h, P)
    g_p = np.stack([po.kernel_over_d(np.sqrt(np.sum(rvec_p[j] ** 2, axis=1)), a[j], xi, eta)
                    for j in range(x_p.shape[0])])
    G = int(np.prod(Ngrid))
    vals = g_p * np.einsum("npc,nc->np", rvec_p, p)
    grid = np.bincount(lin_p.reshape(-1), vals.reshape(-1), minlength=G)
    nx, ny, nz = (int(v) for v in Ngrid)
    Et = po.wave_space(grid.reshape(nz, ny, nx), Ngrid, box, xi, eta).real.reshape(-1)
    amin = float(np.min(a))
    lin_e, rvec_e = po.stencil(x_E, Ngrid, h, P)
    g_e = np.stack([po.kernel_over_d(np.sqrt(np.sum(rvec_e[j] ** 2, axis=1)), amin, xi, eta)
                    for j in range(x_E.shape[0])])
    Eq = np.prod(h) * np.einsum("np,npc->nc", g_e * Et[lin_e], rvec_e)
    # real space: every probe/particle pair within rc, column of (class of min(a), class of the particle)
    col = po.pair_columns(len(a_uniq))
    cmin = cls[int(np.argmin(a))]
    ia, ib = np.meshgrid(np.arange(x_E.shape[0]), np.arange(x_p.shape[0]), indexing="ij")
    ia, ib = ia.reshape(-1), ib.reshape(-1)
    r = x_E[ia] - x_p[ib]
    r = r - box * np.trunc(2 * r / box)
    d = np.sqrt(np.sum(r * r, axis=1))
    keep = d < rc
    ia, ib, r, d = ia[keep], ib[keep], r[keep], d[keep]
    i = np.searchsorted(r_table, d, side="left")
    if np.any(i <= 0) or np.any(i >= r_table.size):
        raise ValueError("separation outside the real-space table")
    cij = col[cmin, cls[ib]]
    t = (d - r_table[i - 1]) / (r_table[i] - r_table[i - 1])
    A = perp[i - 1, cij] * (1 - t) + perp[i, cij] * t
    B = para[i - 1, cij] * (1 - t) + para[i, cij] * t
    rh = r / d[:, None]
    pj = p[ib]
    pr = np.sum(pj * rh, axis=1)
    Er = np.zeros_like(x_E)
    np.add.at(Er, ia, A[:, None] * (pj - pr[:, None] * rh) + (B * pr)[:, None] * rh)
    return -(Eq + Er)
