"""NumPy restatement of the dipole + quadrupole operator (CPU oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates the MATLAB variant ``Capacitance_Quadrupole`` (cited ``CQ/``): 8 unknowns
per sphere, the dipole S (3) and the traceless quadrupole Q stored as
(xx, xy, xz, yy, yz) with zz = -(xx + yy).

* tables ``CQ/RealSpaceTable.m:171-378`` (field/quadrupole and gradient/
  quadrupole couplings, written here as polynomial-coefficient sets like the
  dipole tables of ``ewald_oracle``);
* spread of the 8 moment components with the dipole path's Gaussian
  (``CQ/Spread.m:41-71``);
* wave-space scaling with the four couplings ``9 j1^2``, ``-45/2 i j1 j2``,
  ``45 i j2 j1``, ``225/2 j2^2`` (``CQ/Scale.m:19-72``);
* contraction to the field E (3) and field gradient G (5) (``CQ/Contract.m:49-77``);
* real-space pair sum with nine interpolated couplings (``CQ/RealSpace.m:27-100``);
* the block system ``[M_ES M_EQ; M_GS M_GQ][S; Q] = [E0; 0]`` solved by GMRES
  (``CQ/MatrixVectorSolve.m:35-43``) and the tensor driver
  (``CQ/CapacitanceTensor.m:49-65``).

Table convention: the MATLAB drivers pass a separation table that already
contains r = 0 (``CQ/CapacitanceTensorSpectrum.m:26-28``), which makes the
tables one entry longer than the separations.  This restatement uses the
consistent layout of the dipole path: separations ``[0, r_1, ...]`` and tables
``[self, T(r_1), ...]``.

Parity unpinned: the reference is MATLAB, which cannot run here, and it ships
no golden vectors for this path.  The restatement is checked instead by
(a) its dipole block against the reference Python dipole operator (golden
vectors), (b) the Ewald-split invariance of the full operator (the result must
not depend on xi), and (c) symmetry properties (tests/test_quadrupole_oracle.py).
"""
from __future__ import annotations

import math

import numpy as np

from . import ewald_oracle as ew

PI = math.pi
SP3 = PI ** 1.5

QUAD_TABLES = ("field_quad_1", "field_quad_2", "field_quad_3", "grad_quad_1", "grad_quad_2", "grad_quad_3",
               "grad_quad_4")


def _quad_terms(xi):
    """(cE, pE, E+, E-, E0, cF, pF, F+, F-, F0, reg) per table, same meaning as
    ``ewald_oracle._table_terms``."""
    x2 = xi * xi
    x4, x6, x8, x10 = x2 ** 2, x2 ** 3, x2 ** 4, x2 ** 5
    t = {}
    a = 45 - 120 * x2 + 192 * x4 - 512 * x6
    b = 2 * (45 + 24 * x2 - 64 * x4 + 512 * x6)
    # field/quadrupole, rrr.S
    t["field_quad_1"] = (
        15.0 / (16384 * SP3 * xi ** 7), 4,
        [-24 * x6, 48 * x6, -4 * x4 * (9 - 8 * x2), 8 * x4 * (3 - 8 * x2), 2 * x2 * (21 - 80 * x2 + 64 * x4),
         -4 * x2 * (3 - 8 * x2) ** 2, -a, -b],
        [-24 * x6, -48 * x6, -4 * x4 * (9 - 8 * x2), -8 * x4 * (3 - 8 * x2), 2 * x2 * (21 - 80 * x2 + 64 * x4),
         4 * x2 * (3 - 8 * x2) ** 2, -a, b],
        [48 * x6, 0, 8 * x4 * (9 - 32 * x2), 0, -4 * x2 * (21 - 128 * x2), 0, 2 * (45 - 480 * x2), 0],
        15.0 / (32768 * PI * x8), 4,
        [48 * x8, 0, 32 * x6 * (3 - 8 * x2), 0, -24 * x4 * (3 - 16 * x2), 0, 72 * x2 * (1 - 8 * x2), 0,
         -45 + 480 * x2 + 4096 * x8],
        [48 * x8, 0, 32 * x6 * (3 - 8 * x2), 0, -24 * x4 * (3 - 16 * x2), 0, 72 * x2 * (1 - 8 * x2), 0,
         -45 + 480 * x2 + 4096 * x8],
        [2 * v for v in [-48 * x8, 0, -32 * x6 * (3 - 8 * x2), 0, 24 * x4 * (3 - 16 * x2), 0,
                         -72 * x2 * (1 - 8 * x2), 0, 45 - 480 * x2]],
        lambda r: -15.0 / (4 * PI * r ** 4) + 15 * r ** 2 / (64 * PI) * (1 - 3 * r ** 2 / 16))
    # field/quadrupole, Ir.S + Sr + rS
    t["field_quad_2"] = (
        3.0 / (16384 * SP3 * xi ** 7), 4,
        [-40 * x6, 80 * x6, -20 * x4 * (11 - 24 * x2), 8 * x4 * (45 + 8 * x2), -2 * x2 * (45 - 80 * x2 + 64 * x4),
         -4 * x2 * (15 + 48 * x2 - 64 * x4), a, b],
        [-40 * x6, -80 * x6, -20 * x4 * (11 - 24 * x2), -8 * x4 * (45 + 8 * x2), -2 * x2 * (45 - 80 * x2 + 64 * x4),
         4 * x2 * (15 + 48 * x2 - 64 * x4), a, -b],
        [10 * v for v in [8 * x6, 0, 4 * x4 * (11 - 32 * x2), 0, 2 * x2 * (9 - 64 * x2), 0, -9 + 96 * x2, 0]],
        3.0 / (32768 * PI * x8), 4,
        [80 * x8, 0, 160 * x6 * (3 - 8 * x2), -2048 * x8, 120 * x4 * (3 - 16 * x2), 0, -120 * x2 * (1 - 8 * x2), 0,
         45 - 480 * x2 - 4096 * x8],
        [80 * x8, 0, 160 * x6 * (3 - 8 * x2), 2048 * x8, 120 * x4 * (3 - 16 * x2), 0, -120 * x2 * (1 - 8 * x2), 0,
         45 - 480 * x2 - 4096 * x8],
        [10 * v for v in [-16 * x8, 0, -32 * x6 * (3 - 8 * x2), 0, -24 * x4 * (3 - 16 * x2), 0,
                          24 * x2 * (1 - 8 * x2), 0, -9 + 96 * x2]],
        lambda r: 3.0 / (4 * PI * r ** 4) - 3 * r / (8 * PI) * (1 - 5 * r / 8 + 5 * r ** 3 / 128))
    # field/quadrupole, Ir.S
    t["field_quad_3"] = (
        5.0 / (1024 * SP3 * xi ** 5), 2,
        [4 * x4, -8 * x4, 16 * x2 * (1 - 2 * x2), -24 * x2, 3, 6],
        [4 * x4, 8 * x4, 16 * x2 * (1 - 2 * x2), 24 * x2, 3, -6],
        [-8 * x4, 0, -32 * x2 * (1 - 3 * x2), 0, 2 * (-3 + 24 * x2), 0],
        5.0 / (2048 * PI * x6), 2,
        [-8 * x6, 0, -12 * x4 * (3 - 8 * x2), 128 * x6, -6 * x2 * (3 - 16 * x2), 0, 3 - 24 * x2],
        [-8 * x6, 0, -12 * x4 * (3 - 8 * x2), -128 * x6, -6 * x2 * (3 - 16 * x2), 0, 3 - 24 * x2],
        [16 * x6, 0, 24 * x4 * (3 - 8 * x2), 0, 12 * x2 * (3 - 16 * x2), 0, 2 * (-3 + 24 * x2)],
        lambda r: 5 * r / (8 * PI) * (1 - 3 * r / 4 + r ** 3 / 16))
    # gradient/quadrupole, Irr:Q
    p1 = [16 * x8, 0, 96 * x6 - 128 * x8, 0, 72 * x4 - 192 * x6 + 256 * x8, 0, -(24 * x2 - 96 * x4 + 256 * x6), 0,
          9 - 48 * x2 + 192 * x4]
    t["grad_quad_1"] = (
        75.0 / (16384 * SP3 * xi ** 7), 3,
        [8 * x6, -16 * x6, 44 * x4 - 32 * x6, -(72 * x4 - 64 * x6), 18 * x2 + 32 * x4, 12 * x2 - 64 * x4,
         -(9 + 24 * x2), -(18 - 48 * x2)],
        [8 * x6, 16 * x6, 44 * x4 - 32 * x6, 72 * x4 - 64 * x6, 18 * x2 + 32 * x4, -(12 * x2 - 64 * x4),
         -(9 + 24 * x2), 18 - 48 * x2],
        [-2 * v for v in [8 * x6, 0, 44 * x4 - 64 * x6, 0, 18 * x2 - 64 * x4 + 128 * x6, 0,
                          -9 + 48 * x2 - 192 * x4, 0]],
        75.0 / (32768 * PI * x8), 3,
        [-v for v in p1], [-v for v in p1], [2 * v for v in p1],
        lambda r: 75 * r * (4 - r ** 2) ** 2 / (1024 * PI))
    # gradient/quadrupole, Q
    q0 = [288 * x10, 0, 3600 * x8 - 4800 * x10, 0, 10800 * x6 - 28800 * x8 + 38400 * x10, 0,
          5400 * x4 - 21600 * x6 + 57600 * x8, 0, -(1350 * x2 - 7200 * x4 + 28800 * x6), 0,
          405 - 2700 * x2 + 14400 * x4]
    qp = list(q0)
    qp[5] = 49152 * x10
    qp[10] = q0[10] + 49152 * x10
    qm = list(qp)
    qm[5] = -49152 * x10
    e1 = 135 + 180 * x2 + 480 * x4 - 768 * x6 + 2048 * x8
    e0 = 270 - 1080 * x2 - 192 * x4 + 512 * x6 - 4096 * x8
    t["grad_quad_2"] = (
        3.0 / (32768 * SP3 * xi ** 9), 5,
        [-48 * x8, 96 * x8, -(576 * x6 - 608 * x8), 1056 * x6 - 1216 * x8, -(1536 * x4 - 2576 * x6 + 3968 * x8),
         2160 * x4 - 4320 * x6 - 256 * x8, -(360 * x2 + 360 * x4 + 640 * x6 - 512 * x8),
         -(360 * x2 - 1680 * x4 - 768 * x6 + 1024 * x8), e1, e0],
        [-48 * x8, -96 * x8, -(576 * x6 - 608 * x8), -(1056 * x6 - 1216 * x8), -(1536 * x4 - 2576 * x6 + 3968 * x8),
         -(2160 * x4 - 4320 * x6 - 256 * x8), -(360 * x2 + 360 * x4 + 640 * x6 - 512 * x8),
         360 * x2 - 1680 * x4 - 768 * x6 + 1024 * x8, e1, -e0],
        [2.0 / 3.0 * v for v in [144 * x8, 0, 1728 * x6 - 2400 * x8, 0, 4608 * x4 - 13200 * x6 + 19200 * x8, 0,
                                 1080 * x2 - 5400 * x4 + 19200 * x6, 0, -405 + 2700 * x2 - 14400 * x4, 0]],
        1.0 / (65536 * PI * x10), 5,
        qp, qm, [-2 * v for v in q0],
        lambda r: -3.0 / (2 * PI) * (1 / r ** 5 - 1 + 25 * r / 32 - 25 * r ** 3 / 256 + 3 * r ** 5 / 512))
    # gradient/quadrupole, Irr:Q + 2Q.rr + 2rr.Q
    g1 = 135 + 180 * x2 + 480 * x4 - 768 * x6 + 2048 * x8
    g0 = -270 + 1080 * x2 + 192 * x4 - 512 * x6 + 4096 * x8
    rr = [-96 * x10, 0, -720 * x8 + 960 * x10, 0, -(720 * x6 - 1920 * x8 + 2560 * x10), 0,
          360 * x4 - 1440 * x6 + 3840 * x8, 0, -(270 * x2 - 1440 * x4 + 5760 * x6), 0,
          135 - 900 * x2 + 4800 * x4 + 16384 * x10]
    ss = [96 * x10, 0, 720 * x8 - 960 * x10, 0, 720 * x6 - 1920 * x8 + 2560 * x10, 0,
          -(360 * x4 - 1440 * x6 + 3840 * x8), 0, 270 * x2 - 1440 * x4 + 5760 * x6, 0, -135 + 900 * x2 - 4800 * x4]
    t["grad_quad_3"] = (
        -15.0 / (65536 * SP3 * xi ** 9), 5,
        [48 * x8, -96 * x8, 336 * x6 - 288 * x8, -576 * (x6 - x8), 216 * x4 + 144 * x6 + 128 * x8,
         -(480 * x6 + 256 * x8), -(180 * x2 - 120 * x4 + 640 * x6 - 512 * x8), 720 * x4 + 768 * x6 - 1024 * x8, g1,
         -g0],
        [48 * x8, 96 * x8, 336 * x6 - 288 * x8, 576 * (x6 - x8), 216 * x4 + 144 * x6 + 128 * x8,
         480 * x6 + 256 * x8, -(180 * x2 - 120 * x4 + 640 * x6 - 512 * x8), -(720 * x4 + 768 * x6 - 1024 * x8), g1,
         g0],
        [-2 * v for v in [48 * x8, 0, 336 * x6 - 480 * x8, 0, 216 * x4 - 720 * x6 + 1280 * x8, 0,
                          -(180 * x2 - 840 * x4 + 2560 * x6), 0, 135 - 900 * x2 + 4800 * x4, 0]],
        -15.0 / (131072 * PI * x10), 5,
        rr, rr, [2 * v for v in ss],
        lambda r: -15 * (r ** 2 - 4) ** 3 * (3 * r ** 4 + 6 * r ** 2 + 8) / (2048 * PI * r ** 5))
    # gradient/quadrupole, rrrr:Q
    h1 = 945 + 1260 * x2 + 3360 * x4 - 5376 * x6 + 14336 * x8
    h0 = 1890 - 7560 * x2 - 1344 * x4 + 3584 * x6 - 28672 * x8
    tt = [288 * x10, 0, 720 * x8 - 960 * x10, 0, -(720 * x6 - 1920 * x8 + 2560 * x10), 0,
          1080 * x4 - 4320 * x6 + 11520 * x8, 0, -(1350 * x2 - 7200 * x4 + 28800 * x6), 0,
          945 - 6300 * x2 + 33600 * x4 + 114688 * x10]
    uu = list(tt)
    uu[10] = 945 - 6300 * x2 + 33600 * x4
    t["grad_quad_4"] = (
        -15.0 / (65536 * SP3 * xi ** 9), 5,
        [144 * x8, -288 * x8, 288 * x6 + 96 * x8, -(288 * x6 + 192 * x8), -(432 * x4 - 912 * x6 + 896 * x8),
         720 * x4 - 480 * x6 + 1792 * x8, 720 * x2 - 2280 * x4 + 4480 * x6 - 3584 * x8,
         -(1080 * x2 + 2160 * x4 + 5376 * x6 - 7168 * x8), -h1, -h0],
        [144 * x8, 288 * x8, 288 * x6 + 96 * x8, 288 * x6 + 192 * x8, -(432 * x4 - 912 * x6 + 896 * x8),
         -(720 * x4 - 480 * x6 + 1792 * x8), 720 * x2 - 2280 * x4 + 4480 * x6 - 3584 * x8,
         1080 * x2 + 2160 * x4 + 5376 * x6 - 7168 * x8, -h1, h0],
        [-2 * v for v in [144 * x8, 0, 288 * x6 - 480 * x8, 0, -(432 * x4 - 1200 * x6 + 1280 * x8), 0,
                          720 * x2 - 3000 * x4 + 6400 * x6, 0, -945 + 6300 * x2 - 33600 * x4, 0]],
        15.0 / (131072 * PI * x10), 5,
        tt, tt, [-2 * v for v in uu],
        lambda r: -15 * (3584 - 80 * r ** 6 - 30 * r ** 8 + 9 * r ** 10) / (2048 * PI * r ** 5))
    return t


def quad_self(xi):
    """Gradient/quadrupole self value prepended to grad_quad_2 (CQ/RealSpaceTable.m:373-375)."""
    e4 = math.exp(-4 * xi * xi)
    return 1.0 / (2 * PI) * (3 * (3 - 10 * xi ** 2 + 20 * xi ** 4) / (8 * math.sqrt(PI) * xi ** 5)
                             - 3 * (3 + 2 * xi ** 2 + 4 * xi ** 4) * e4 / (8 * math.sqrt(PI) * xi ** 5)
                             + 3 * float(ew.erfc(2 * xi)))


def quadrupole_tables(r, xi):
    """The 9 couplings used by the solve, each with its r = 0 value prepended:
    field_dip_1, field_dip_2 (self = the dipole self term), field_quad_1..3 (0),
    grad_quad_1 (0), grad_quad_2 (self), grad_quad_3, grad_quad_4 (0)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    _, _, f1, f2, _, _ = ew.real_space_table(r, xi)
    t = _quad_terms(float(xi))
    out = {"field_dip_1": f1, "field_dip_2": f2}
    for k in QUAD_TABLES:
        v = ew._eval_table(r, float(xi), t[k])
        head = quad_self(float(xi)) if k == "grad_quad_2" else 0.0
        out[k] = np.concatenate(([head], v))
    return out


def default_quad_tables(xi, rmin=0.001, dr=0.001, rmax=10.0):
    r = np.arange(rmin, rmax + 1e-12, dr, dtype=np.float64)
    return quadrupole_tables(r, xi), np.concatenate(([0.0], r))


TABLE_ORDER = ("field_dip_1", "field_dip_2", "field_quad_1", "field_quad_2", "field_quad_3", "grad_quad_1",
               "grad_quad_2", "grad_quad_3", "grad_quad_4")


# ---------------------------------------------------------------------------
# Wave space (CQ/Scale.m:19-72)
# ---------------------------------------------------------------------------
def _sph_j1_j2(k):
    with np.errstate(divide="ignore", invalid="ignore"):
        s, c = np.sin(k), np.cos(k)
        j1 = s / k ** 2 - c / k
        j2 = (3.0 / k ** 2 - 1.0) * s / k - 3.0 * c / k ** 2
    return np.nan_to_num(j1), np.nan_to_num(j2)


def quad_factors(khat):
    """(Qfactor, Qfactor_dot) 5-vectors of the unit wave vector (CQ/Scale.m:32-43)."""
    kx, ky, kz = khat[..., 0], khat[..., 1], khat[..., 2]
    qf = np.stack((kx * kx - 1 / 3, kx * ky, kx * kz, ky * ky - 1 / 3, ky * kz), axis=-1)
    qd = np.stack((kx * kx - kz * kz, 2 * kx * ky, 2 * kx * kz, ky * ky - kz * kz, 2 * ky * kz), axis=-1)
    return qf, qd


def wave_space_quad(grids, Ngrid, box, xi, eta):
    """FFT -> scale -> IFFT of the 8 spread grids (Nx,Ny,Nz,8), complex output."""
    k, _ = ew.kspace_unshifted(Ngrid, box, xi, eta)
    k2 = np.sum(k * k, axis=3)
    kk = np.sqrt(k2)
    den = np.where(kk == 0, 1.0, kk)
    khat = k / den[..., None]
    eta = np.asarray(eta, dtype=np.float64).reshape(3)
    etak2 = np.sum((1.0 - eta) * k * k, axis=3)
    j1, j2 = _sph_j1_j2(kk)
    with np.errstate(divide="ignore", invalid="ignore"):
        g = np.exp(-etak2 / (4 * xi * xi)) / k2
    g[k2 == 0] = 0.0
    g = np.nan_to_num(g)
    hes = 9 * j1 * j1 * g
    heq = -22.5j * j1 * j2 * g
    hgs = 45j * j2 * j1 * g
    hgq = 112.5 * j2 * j2 * g
    qf, qd = quad_factors(khat)
    f = np.fft.fftn(grids, axes=(0, 1, 2))
    dS = np.sum(khat * f[..., :3], axis=3)
    dQ = np.sum(qd * f[..., 3:], axis=3)
    out = np.empty_like(f)
    out[..., :3] = ((hes * dS + heq * dQ)[..., None]) * khat
    out[..., 3:] = ((hgs * dS + hgq * dQ)[..., None]) * qf
    return np.fft.ifftn(out, axes=(0, 1, 2))


# ---------------------------------------------------------------------------
# Real space (CQ/RealSpace.m:27-100)
# ---------------------------------------------------------------------------
def _lerp_all(tables, rvals, d):
    i = np.searchsorted(rvals, d, side="left")
    if np.any(i <= 0) or np.any(i >= len(rvals)):
        raise ValueError("separation outside the real-space table")
    t = (d - rvals[i - 1]) / (rvals[i] - rvals[i - 1])
    return [tables[name][i - 1] * (1 - t) + tables[name][i] * t for name in TABLE_ORDER]


def real_space_quad(x, S, Q, lam, box, pairs, rc, tables, rvals):
    """Dielectric + self + pair terms, returns (E (N,3), G (N,5))."""
    lam = np.asarray(lam, dtype=np.float64).reshape(-1)
    E = (3.0 / (4 * PI * (lam - 1)))[:, None] * S + S * tables["field_dip_1"][0]
    G = (15.0 / (8 * PI * (lam - 1)))[:, None] * Q + 0.5 * Q * tables["grad_quad_2"][0]
    p1, p2 = pairs
    if len(p1) == 0:
        return E, G
    r = ew.min_image(x[p1] - x[p2], box)
    d = np.sqrt(np.sum(r * r, axis=1))
    keep = d < rc
    p1, p2, r, d = p1[keep], p2[keep], r[keep], d[keep]
    dE, dG = quad_pair_terms(r / d[:, None], d, S[p2], Q[p2], tables, rvals)
    np.add.at(E, p1, dE)
    np.add.at(G, p1, dG)
    return E, G


def quad_pair_terms(r, d, Sj, Qj, tables, rvals):
    """Field and gradient contributions of sources (Sj, Qj) at unit vectors r (target minus
    source) and separations d (CQ/RealSpace.m:56-99, Compute_Field_Quadrupole/RealSpace.m:53-73)."""
    A, B, C, D, Ec, F, Gc, H, I = _lerp_all(tables, rvals, d)
    rx, ry, rz = r[:, 0], r[:, 1], r[:, 2]
    sr = np.sum(Sj * r, axis=1)
    q5 = np.stack((rx * rx, rx * ry, rx * rz, ry * ry, ry * rz), axis=1)   # rr in 5-component form
    i5 = np.array([1.0, 0, 0, 1.0, 0])
    Qr = np.stack((Qj[:, 0] * rx + Qj[:, 1] * ry + Qj[:, 2] * rz,
                   Qj[:, 1] * rx + Qj[:, 3] * ry + Qj[:, 4] * rz,
                   Qj[:, 2] * rx + Qj[:, 4] * ry - (Qj[:, 0] + Qj[:, 3]) * rz), axis=1)
    qd = np.stack((rx * rx - rz * rz, 2 * rx * ry, 2 * rx * rz, ry * ry - rz * rz, 2 * ry * rz), axis=1)
    rQr = np.sum(qd * Qj, axis=1)
    Sr = np.stack((Sj[:, 0] * rx, Sj[:, 0] * ry, Sj[:, 0] * rz, Sj[:, 1] * ry, Sj[:, 1] * rz), axis=1)
    rS = np.stack((rx * Sj[:, 0], rx * Sj[:, 1], rx * Sj[:, 2], ry * Sj[:, 1], ry * Sj[:, 2]), axis=1)
    Qrr = np.stack((Qr[:, 0] * rx, Qr[:, 0] * ry, Qr[:, 0] * rz, Qr[:, 1] * ry, Qr[:, 1] * rz), axis=1)
    rrQ = np.stack((rx * Qr[:, 0], rx * Qr[:, 1], rx * Qr[:, 2], ry * Qr[:, 1], ry * Qr[:, 2]), axis=1)
    IrrQ = rQr[:, None] * i5
    dE = A[:, None] * (Sj - sr[:, None] * r) + (B * sr)[:, None] * r \
        - 0.5 * ((C * rQr)[:, None] * r + 2 * D[:, None] * Qr)
    dG = (C * sr)[:, None] * q5 + D[:, None] * (Sr + rS) + ((D + Ec) * sr)[:, None] * i5 \
        + 0.5 * (F[:, None] * IrrQ + Gc[:, None] * Qj + H[:, None] * (IrrQ + 2 * Qrr + 2 * rrQ)
                 + (I * rQr)[:, None] * q5)
    return dE, dG


class QuadGeometry:
    """Geometry of one configuration for the 8-unknown operator."""

    def __init__(self, x, lam, box, xi, rc, Ngrid, P, tables, rvals):
        self.x = np.asarray(x, dtype=np.float64)
        self.box = np.asarray(box, dtype=np.float64).reshape(3)
        self.lam = np.asarray(lam, dtype=np.float64).reshape(-1)
        self.xi, self.rc = float(xi), float(rc)
        self.Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
        self.h = self.box / self.Ngrid
        self.P = int(P)
        self.eta = self.P * (self.h * self.xi) ** 2 / PI
        self.tables, self.rvals = tables, rvals
        cell, nc = ew.cell_list(self.x, self.box, self.rc)
        self.pairs = ew.neighbor_list(cell, nc)
        self.lin, self.w, self.wc = ew.prepare_grid_kernel(self.x, self.Ngrid, self.h, self.xi, self.eta, self.P)

    def apply(self, S, Q, real=True):
        """(E, G) from (S, Q): the operator of CQ/MatrixVectorMultiply.m:31-77.
        real=True returns the real part (the GPU operator for real moments)."""
        S = np.asarray(S)
        Q = np.asarray(Q)
        n = self.x.shape[0]
        G = int(np.prod(self.Ngrid))
        nx, ny, nz = (int(v) for v in self.Ngrid)
        mom = np.concatenate((S, Q), axis=1).astype(np.complex128)
        grids = np.empty((G, 8), dtype=np.complex128)
        lin = self.lin.reshape(-1)
        for c in range(8):
            v = (self.w * mom[:, c:c + 1]).reshape(-1)
            grids[:, c] = np.bincount(lin, v.real, minlength=G) + 1j * np.bincount(lin, v.imag, minlength=G)
        grids = grids.reshape(nz, ny, nx, 8).transpose(2, 1, 0, 3)
        Ht = wave_space_quad(grids, self.Ngrid, self.box, self.xi, self.eta)
        flat = Ht.transpose(2, 1, 0, 3).reshape(G, 8)
        K = np.einsum("np,npc->nc", self.wc, flat[self.lin])
        Er, Gr = real_space_quad(self.x, S, Q, self.lam, self.box, self.pairs, self.rc, self.tables, self.rvals)
        E = K[:, :3] + Er
        Gg = K[:, 3:] + Gr
        if real:
            return np.real(E), np.real(Gg)
        return E, Gg

    def matvec(self, v, real=True):
        """On the MATLAB vector layout [S (3N, xyz per particle); Q (5N)]."""
        n = self.x.shape[0]
        v = np.asarray(v)
        S = v[:3 * n].reshape(n, 3)
        Q = v[3 * n:].reshape(n, 5)
        E, G = self.apply(S, Q, real=real)
        return np.concatenate((E.reshape(-1), G.reshape(-1)))


def solve_quad(geom, E0, S_guess, Q_guess, tol, restart=10, maxit=100):
    """GMRES on [E0; 0] (CQ/MatrixVectorSolve.m:35-43); returns (S, Q, info)."""
    from .capacitance_oracle import gmres
    n = geom.x.shape[0]
    b = np.concatenate((np.tile(np.asarray(E0, dtype=np.float64).reshape(3), n), np.zeros(5 * n)))
    x0 = np.concatenate((np.asarray(S_guess, dtype=np.float64).reshape(-1),
                         np.asarray(Q_guess, dtype=np.float64).reshape(-1)))
    sol, flag, relres, nmv = gmres(lambda v: geom.matvec(v), b, x0, tol, restart, maxit)
    return sol[:3 * n].reshape(n, 3), sol[3 * n:].reshape(n, 5), {"flag": flag, "relres": relres, "matvecs": nmv}


def quad_tensor(geom, S_guess, Q_guess, tol, restart=10, maxit=100):
    """CQ/CapacitanceTensor.m:49-65: column i of C is the mean dipole for the unit
    field along i; warm start S[:, [z, x, y]] and Q -> (-xx-yy, yz, xy, xx, xz)."""
    n = geom.x.shape[0]
    C = np.zeros((3, 3))
    S = np.zeros((n, 3, 3))
    Q = np.zeros((n, 5, 3))
    sg, qg = np.asarray(S_guess, float), np.asarray(Q_guess, float)
    infos = []
    for i in range(3):
        Si, Qi, info = solve_quad(geom, np.eye(3)[i], sg, qg, tol, restart, maxit)
        S[:, :, i], Q[:, :, i] = Si, Qi
        C[:, i] = Si.mean(axis=0)
        sg = Si[:, [2, 0, 1]]
        qg = np.stack((-Qi[:, 0] - Qi[:, 3], Qi[:, 4], Qi[:, 1], Qi[:, 0], Qi[:, 2]), axis=1)
        infos.append(info)
    return C, S, Q, infos
