"""NumPy restatement of the reference's point-dipole pair forces (CPU oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``compute_forces_bruteforce`` of
``CPU - HOOMD simulation test/dipole_forces_ext/_dipole_forces_ext.cpp:119-250``:
minimum image ``d - L rint(d/L)`` in x, y (and z when periodic), pairs with
``1e-24 <= r^2 <= r_cut^2``, pair energy
``U = pref [(mi.mj)/r^3 - 3 (mi.r)(mj.r)/r^5]`` split half per particle, and
``F_i = 3 pref / r^5 [(mi.mj) r + (mj.r) mi + (mi.r) mj - 5 (mi.r)(mj.r) r / r^2]``
with ``r = r_i - r_j``.  All pairs are formed at once (small N only).
"""
from __future__ import annotations

import numpy as np


def compute_forces(pos, dip, box, r_cut, prefactor=1.0, periodic_z=True):
    pos = np.asarray(pos, dtype=np.float64)
    dip = np.asarray(dip, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    if pos.ndim != 2 or pos.shape[1] != 3 or dip.shape != pos.shape:
        raise RuntimeError("Invalid shapes: pos(N,3), dip(N,3), box(3) required.")
    if not np.all(box > 0):
        raise RuntimeError("Box lengths must be positive.")
    if not r_cut > 0:
        raise RuntimeError("r_cut must be > 0.")
    if r_cut >= 0.5 * min(box[0], box[1]) or (periodic_z and r_cut >= 0.5 * box[2]):
        raise RuntimeError("r_cut too large for minimum-image periodicity.")
    d = pos[:, None, :] - pos[None, :, :]
    for k in range(3 if periodic_z else 2):
        d[..., k] -= box[k] * np.rint(d[..., k] / box[k])
    r2 = np.sum(d * d, axis=2)
    keep = (r2 <= r_cut * r_cut) & (r2 >= 1e-24)
    np.fill_diagonal(keep, False)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv_r2 = np.where(keep, 1.0 / r2, 0.0)
    inv_r = np.sqrt(inv_r2)
    inv_r3 = inv_r2 * inv_r
    inv_r5 = inv_r3 * inv_r2
    mi, mj = dip[:, None, :], dip[None, :, :]
    mimj = np.sum(mi * mj, axis=2)
    mir = np.sum(mi * d, axis=2)
    mjr = np.sum(mj * d, axis=2)
    U = prefactor * (mimj * inv_r3 - 3.0 * mir * mjr * inv_r5)
    coef = prefactor * 3.0 * inv_r5
    F = coef[..., None] * (mimj[..., None] * d + mjr[..., None] * mi + mir[..., None] * mj
                           - 5.0 * (mir * mjr * inv_r2)[..., None] * d)
    F = np.where(keep[..., None], F, 0.0)
    U = np.where(keep, U, 0.0)
    return F.sum(axis=1), 0.5 * U.sum(axis=1)
