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


def field_map(x_E, x_p, p, box, xi):
    """E = -(Hk + Hr) at the probes (FieldMap.m:1-59); complex (the reference's pipeline)."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = field_parameters(box, xi)
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
