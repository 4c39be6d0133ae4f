"""NumPy restatement of the polydisperse dipole operator (CPU oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates the MATLAB variant ``Capacitance_Sizes`` (cited ``CS/``): spheres of
different radii a_i, 3 unknowns (the dipole p) per sphere.

* couplings ``CS/RealSpaceTable.m:27-149`` per radius pair (I - rr and rr parts,
  eight exp/erfc terms with polynomial prefactors, overlap regularisation, and
  the r -> 0 self value), tabulated per pair of distinct radii;
* real space ``CS/RealSpace.m:18-76``: dielectric ``3 p / (4 pi a^3 (eps - 1))``,
  self term ``Ep_perp(0, col(a_i, a_i)) p``, pair sum with the table column of
  the pair's radii and linear interpolation;
* wave space ``CS/ComputeField.m:23-57``: the dipoles are spread as charges with
  the kernel of ``CS/Spread.m:39-72`` onto ONE scalar grid, scaled by
  ``exp(-(1 - eta) q^2 / 4 xi^2) / q^2`` (``CS/Scale.m:16-21``) and contracted
  with the same kernel times r-hat (``CS/Contract.m:39-73``); eta is a scalar
  ``P (mean(h) xi)^2 / pi`` with ``P = ceil(2 / mean(h) - 2 ln(tol) / pi)``;
* solve ``CS/ComputeDipole.m:32-34`` (GMRES, restart min(3N,10), maxit
  min(3N,100)) and tensor ``CS/CapacitanceTensor.m:39-54``.

The small-d form of the spread kernel (``CS/Spread.m:60-61``) is kept as the
reference writes it, including its ``exp(-2 a xi^2 / eta)`` factor.

Parity unpinned: the reference is MATLAB, which cannot run here, and it ships
no golden vectors for this path.  The restatement is checked instead by
(a) the monodisperse limit against the dipole operator of ``ewald_oracle``,
itself pinned to the reference Python's golden vectors, (b) Ewald-split
invariance, (c) symmetry of the operator (tests/test_polydisperse_oracle.py).
"""
from __future__ import annotations

import math

import numpy as np

from . import ewald_oracle as ew

PI = math.pi
SP3 = PI ** 1.5

try:
    from scipy.special import erf, erfc
except ImportError:  # pragma: no cover
    erf = np.vectorize(math.erf)
    erfc = np.vectorize(math.erfc)


# ---------------------------------------------------------------------------
# Radius classes (MATLAB uniquetol with its default tolerance for doubles)
# ---------------------------------------------------------------------------
def unique_radii(a, tol=1e-12):
    """(a_uniq, class index per particle).  Sorted values closer than
    tol * max|a| to the first member of a group join that group."""
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    order = np.argsort(a, kind="stable")
    thr = tol * np.max(np.abs(a))
    uniq = []
    cls = np.empty(a.size, dtype=np.int64)
    for i in order:
        if not uniq or a[i] - uniq[-1] > thr:
            uniq.append(a[i])
        cls[i] = len(uniq) - 1
    return np.array(uniq), cls


def pair_columns(M):
    """col[i, j] = column of radii pair (i, j) in the tables, upper triangle in
    row order (CS/RealSpace.m:25-36)."""
    col = np.zeros((M, M), dtype=np.int64)
    lin = 0
    for i in range(M):
        for j in range(i, M):
            col[i, j] = col[j, i] = lin
            lin += 1
    return col


# ---------------------------------------------------------------------------
# Couplings (CS/RealSpaceTable.m:34-146)
# ---------------------------------------------------------------------------
def couplings(r, ai, aj, xi):
    """(perp, para) closed forms at separations r > 0 (no self value)."""
    r = np.asarray(r, dtype=np.float64)
    x2, x4, x6 = xi ** 2, xi ** 4, xi ** 6
    s, d = ai + aj, ai - aj
    A3 = ai ** 3 * aj ** 3
    c1 = 4 * ai ** 3 - 3 * ai ** 2 * aj - 3 * ai * aj ** 2 + 4 * aj ** 3
    c2 = 4 * ai ** 3 + 3 * ai ** 2 * aj - 3 * ai * aj ** 2 - 4 * aj ** 3
    q1 = ai ** 2 - 4 * ai * aj + aj ** 2
    q2 = ai ** 2 + 4 * ai * aj + aj ** 2
    # I - rr part
    k5 = 1.0 / (1024 * SP3 * A3 * r ** 3 * xi ** 5)
    base_s = r * (3 - 12 * (ai ** 2 - ai * aj + aj ** 2) * x2 - 4 * s ** 2 * q1 * x4)
    tail_s = 3 * s + 4 * c1 * x2 + 4 * s ** 3 * q1 * x4
    mid_s = r ** 3 * (16 * x2 + 8 * (-4 * ai ** 2 + ai * aj - 4 * aj ** 2) * x4)
    f1 = k5 * (4 * r ** 5 * x4 - 4 * s * r ** 4 * x4 + mid_s + r ** 2 * (-12 * s * x2 - 8 * c1 * x4) + base_s + tail_s)
    f2 = k5 * (4 * r ** 5 * x4 + 4 * s * r ** 4 * x4 + mid_s + r ** 2 * (12 * s * x2 + 8 * c1 * x4) + base_s - tail_s)
    base_d = r * (-3 + 12 * (ai ** 2 + ai * aj + aj ** 2) * x2 + 4 * d ** 2 * q2 * x4)
    mid_d = r ** 3 * (-16 * x2 + 8 * (4 * ai ** 2 + ai * aj + 4 * aj ** 2) * x4)
    tail_d = 3 * d + 4 * c2 * x2 + 4 * d ** 3 * q2 * x4
    f3 = k5 * (-4 * r ** 5 * x4 - 4 * d * r ** 4 * x4 + mid_d + r ** 2 * (-12 * d * x2 - 8 * c2 * x4) + base_d + tail_d)
    f4 = k5 * (-4 * r ** 5 * x4 + 4 * d * r ** 4 * x4 + mid_d + r ** 2 * (12 * d * x2 + 8 * c2 * x4) + base_d - tail_d)
    k6 = 1.0 / (2048 * PI * A3 * r ** 3 * xi ** 6)
    sq = ai ** 2 + aj ** 2
    dq = (ai ** 2 - aj ** 2) ** 2
    g_s = r ** 2 * (-18 * x2 + 72 * sq * x4 + 72 * dq * x6) + 3 - 18 * sq * x2 - 36 * dq * x4
    f5 = k6 * (-8 * r ** 6 * x6 + 36 * r ** 4 * x4 * (-1 + 2 * sq * x2) + 128 * (ai ** 3 + aj ** 3) * r ** 3 * x6
               + g_s - 8 * s ** 4 * q1 * x6)
    f6 = k6 * (-8 * r ** 6 * x6 + 36 * r ** 4 * x4 * (-1 + 2 * sq * x2) - 128 * (ai ** 3 + aj ** 3) * r ** 3 * x6
               + g_s - 8 * s ** 4 * q1 * x6)
    f7 = k6 * (8 * r ** 6 * x6 + 36 * r ** 4 * x4 * (1 - 2 * sq * x2) + 128 * (ai ** 3 - aj ** 3) * r ** 3 * x6
               - g_s + 8 * d ** 4 * q2 * x6)
    f8 = k6 * (8 * r ** 6 * x6 + 36 * r ** 4 * x4 * (1 - 2 * sq * x2) - 128 * (ai ** 3 - aj ** 3) * r ** 3 * x6
               - g_s + 8 * d ** 4 * q2 * x6)
    reg = np.zeros_like(r)
    m = (r < s) & (r >= d) & (r >= -d)
    rm = r[m]
    reg[m] = (s - rm) ** 3 / (128 * PI * A3 * rm ** 3) * (-rm ** 3 - 3 * s * rm ** 2 + 3 * q1 * rm
                                                          + ai ** 3 - 3 * ai ** 2 * aj - 3 * ai * aj ** 2 + aj ** 3)
    m = (r < -d) & (r > d)
    reg[m] = (r[m] ** 3 - aj ** 3) / (4 * PI * aj ** 3 * r[m] ** 3)
    m = (r < d) & (r > -d)
    reg[m] = (r[m] ** 3 - ai ** 3) / (4 * PI * ai ** 3 * r[m] ** 3)
    perp = _combine(r, ai, aj, xi, (f1, f2, f3, f4, f5, f6, f7, f8)) + reg
    # rr part
    k5 = 1.0 / (512 * SP3 * A3 * r ** 3 * xi ** 5)
    mid_s = r ** 3 * (14 * x2 - 4 * (7 * ai ** 2 - 4 * ai * aj + 7 * aj ** 2) * x4)
    c3 = ai ** 3 - 3 * ai ** 2 * aj - 3 * ai * aj ** 2 + aj ** 3
    c4 = ai ** 3 + 3 * ai ** 2 * aj - 3 * ai * aj ** 2 - aj ** 3
    f1 = k5 * (8 * r ** 5 * x4 - 8 * s * r ** 4 * x4 + mid_s + r ** 2 * (-6 * s * x2 - 4 * c3 * x4) - base_s - tail_s)
    f2 = k5 * (8 * r ** 5 * x4 + 8 * s * r ** 4 * x4 + mid_s + r ** 2 * (6 * s * x2 + 4 * c3 * x4) - base_s + tail_s)
    mid_d = r ** 3 * (-14 * x2 + 4 * (7 * ai ** 2 + 4 * ai * aj + 7 * aj ** 2) * x4)
    f3 = k5 * (-8 * r ** 5 * x4 - 8 * d * r ** 4 * x4 + mid_d + r ** 2 * (-6 * d * x2 - 4 * c4 * x4) - base_d
               - tail_d)
    f4 = k5 * (-8 * r ** 5 * x4 + 8 * d * r ** 4 * x4 + mid_d + r ** 2 * (6 * d * x2 + 4 * c4 * x4) - base_d + tail_d)
    k6 = 1.0 / (1024 * PI * A3 * r ** 3 * xi ** 6)
    h_s = -3 + 18 * sq * x2 + 36 * dq * x4
    f5 = k6 * (-16 * r ** 6 * x6 + 36 * r ** 4 * x4 * (-1 + 2 * sq * x2) + 64 * (ai ** 3 + aj ** 3) * r ** 3 * x6
               + h_s + 8 * s ** 4 * q1 * x6)
    f6 = k6 * (-16 * r ** 6 * x6 + 36 * r ** 4 * x4 * (-1 + 2 * sq * x2) - 64 * (ai ** 3 + aj ** 3) * r ** 3 * x6
               + h_s + 8 * s ** 4 * q1 * x6)
    f7 = k6 * (16 * r ** 6 * x6 + 36 * r ** 4 * x4 * (1 - 2 * sq * x2) + 64 * (ai ** 3 - aj ** 3) * r ** 3 * x6
               - h_s - 8 * d ** 4 * q2 * x6)
    f8 = k6 * (16 * r ** 6 * x6 + 36 * r ** 4 * x4 * (1 - 2 * sq * x2) - 64 * (ai ** 3 - aj ** 3) * r ** 3 * x6
               - h_s - 8 * d ** 4 * q2 * x6)
    reg = np.zeros_like(r)
    m = (r < s) & (r >= d) & (r >= -d)
    rm = r[m]
    reg[m] = -1.0 / (64 * PI * A3 * rm ** 3) * (s ** 4 * q1 - 8 * (ai ** 3 + aj ** 3) * rm ** 3 + 9 * sq * rm ** 4
                                                - 2 * rm ** 6)
    m = (r < -d) & (r > d)
    reg[m] = (r[m] ** 3 + 2 * aj ** 3) / (4 * PI * aj ** 3 * r[m] ** 3)
    m = (r < d) & (r > -d)
    reg[m] = (r[m] ** 3 + 2 * ai ** 3) / (4 * PI * ai ** 3 * r[m] ** 3)
    para = _combine(r, ai, aj, xi, (f1, f2, f3, f4, f5, f6, f7, f8)) + reg
    return perp, para


def _combine(r, ai, aj, xi, f):
    f1, f2, f3, f4, f5, f6, f7, f8 = f
    return (f1 * np.exp(-(r + ai + aj) ** 2 * xi ** 2) + f2 * np.exp(-(r - ai - aj) ** 2 * xi ** 2)
            + f3 * np.exp(-(r - ai + aj) ** 2 * xi ** 2) + f4 * np.exp(-(r + ai - aj) ** 2 * xi ** 2)
            + f5 * erfc((r + ai + aj) * xi) + f6 * erfc((r - ai - aj) * xi) + f7 * erfc((r - ai + aj) * xi)
            + f8 * erfc((r + ai - aj) * xi))


def self_value(ai, aj, xi):
    """r -> 0 value of both parts (CS/RealSpaceTable.m:87-89, 146)."""
    x2 = xi * xi
    return (1.0 / (16 * SP3 * ai ** 3 * aj ** 3 * xi ** 3)
            * ((1 - 2 * ai ** 2 * x2 + 2 * ai * aj * x2 - 2 * aj ** 2 * x2) * math.exp(-(ai + aj) ** 2 * x2)
               + (-1 + 2 * ai ** 2 * x2 + 2 * ai * aj * x2 + 2 * aj ** 2 * x2) * math.exp(-(ai - aj) ** 2 * x2))
            + 1.0 / (8 * PI * ai ** 3 * aj ** 3) * ((ai ** 3 - aj ** 3) * float(erf((ai - aj) * xi))
                                                    - (ai ** 3 + aj ** 3) * float(erf((ai + aj) * xi)))
            + min(ai ** 3, aj ** 3) / (4 * PI * ai ** 3 * aj ** 3))


def real_space_table(r, a_uniq, xi):
    """(perp, para), each (n, m) for the m = M(M+1)/2 radius pairs; r[0] must be 0
    and row 0 holds the self value (CS/RealSpaceTable.m:1-149)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    if r[0] != 0.0:
        raise ValueError("first entry of the separation table must be r = 0")
    a_uniq = np.asarray(a_uniq, dtype=np.float64).reshape(-1)
    M = a_uniq.size
    m = M * (M + 1) // 2
    perp = np.zeros((r.size, m))
    para = np.zeros((r.size, m))
    lin = 0
    for i in range(M):
        for j in range(i, M):
            pp, pa = couplings(r[1:], a_uniq[i], a_uniq[j], xi)
            sv = self_value(a_uniq[i], a_uniq[j], xi)
            perp[0, lin] = para[0, lin] = sv
            perp[1:, lin], para[1:, lin] = pp, pa
            lin += 1
    return perp, para


def default_r_table(tol=1e-3):
    """[0, 1:tol:10] (CS/CapacitanceTensorSpectrum.m:26)."""
    return np.concatenate(([0.0], np.arange(1.0, 10.0 + 1e-12, tol)))


# ---------------------------------------------------------------------------
# Spectral parameters and wave space (CS/ComputeField.m:23-57)
# ---------------------------------------------------------------------------
def spectral_parameters(box, xi, tol):
    box = np.asarray(box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(tol))
    rc = lt / xi
    qc = 2 * xi * lt
    Ngrid = np.ceil(1 + box * qc / PI).astype(np.int64)
    h = box / Ngrid
    hm = float(np.mean(h))
    P = int(math.ceil(2 / hm - 2 * math.log(tol) / PI))
    eta = P * (hm * xi) ** 2 / PI
    return rc, Ngrid, h, P, eta


def kernel_over_d(d, a, xi, eta):
    """K(d) / d with the spread weight K(d) (r-hat . p) of CS/Spread.m:56-61;
    for d < 1e-6 the reference's small-d form c0 (r . p) gives K/d = c0."""
    d = np.asarray(d, dtype=np.float64)
    small = d < 1e-6
    ds = np.where(small, 1.0, d)
    K = 3.0 / (8 * math.sqrt(2) * SP3 * a ** 3 * math.sqrt(eta) * xi * ds ** 2) * (
        (eta + 4 * a * xi ** 2 * ds) * np.exp(-2 * (ds + a) ** 2 * xi ** 2 / eta)
        - (eta - 4 * a * xi ** 2 * ds) * np.exp(-2 * (ds - a) ** 2 * xi ** 2 / eta))
    c0 = 8 * math.sqrt(2) * xi ** 5 * math.exp(-2 * a * xi ** 2 / eta) / (SP3 * eta ** 2.5)
    return np.where(small, c0, K / ds)


def stencil(x, Ngrid, h, P):
    """Per particle: linear node indices (N, P^3) and node - particle vectors
    (N, P^3, 3), offsets ordered x fastest (CS/Spread.m:28-52)."""
    x = np.asarray(x, dtype=np.float64)
    lo = (P - 1) // 2
    lin = np.arange(P ** 3)
    off = np.stack((lin % P - lo, (lin // P) % P - lo, lin // (P * P) - lo), axis=1)
    node0 = ew.matlab_round(x / h)
    nodes_xyz = node0[:, None, :] * h + (off * h)[None]
    r = nodes_xyz - x[:, None, :]
    node = np.mod(node0[:, None, :].astype(np.int64) + off[None] - 1, Ngrid)
    linnode = node[..., 0] + Ngrid[0] * (node[..., 1] + Ngrid[1] * node[..., 2])
    return linnode, r


def wave_space(grid, Ngrid, box, xi, eta):
    """FFT, scale exp(-(1-eta) q^2/4 xi^2)/q^2 (q = 0 -> 0), inverse FFT of a
    (Nz, Ny, Nx) scalar grid (CS/Scale.m:16-21)."""
    k, _ = ew.kspace_unshifted(Ngrid, box, xi, [eta, eta, eta])
    q2 = np.sum(k * k, axis=3).transpose(2, 1, 0)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.exp(-(1 - eta) * q2 / (4 * xi * xi)) / q2
    s[q2 == 0] = 0.0
    return np.fft.ifftn(np.fft.fftn(grid) * s)


class PolyGeometry:
    """Geometry of one configuration for the polydisperse operator.

    ``tables=None`` evaluates each pair's couplings in closed form at its exact
    separation; otherwise ``(r_table, perp, para, a_uniq)`` interpolates like
    CS/RealSpace.m."""

    def __init__(self, x, a, eps_p, box, xi, tol, tables=None, rc=None, Ngrid=None, P=None):
        self.x = np.asarray(x, dtype=np.float64)
        self.a = np.asarray(a, dtype=np.float64).reshape(-1)
        self.eps = np.asarray(eps_p, dtype=np.float64).reshape(-1)
        self.box = np.asarray(box, dtype=np.float64).reshape(3)
        self.xi = float(xi)
        rc0, ng0, _, P0, _ = spectral_parameters(self.box, self.xi, tol)
        self.rc = rc0 if rc is None else float(rc)
        self.Ngrid = ng0 if Ngrid is None else np.asarray(Ngrid, dtype=np.int64).reshape(3)
        self.h = self.box / self.Ngrid
        self.P = P0 if P is None else int(P)
        self.eta = self.P * (float(np.mean(self.h)) * self.xi) ** 2 / PI
        n = self.x.shape[0]
        cell, nc = ew.cell_list(self.x, self.box, self.rc)
        p1, p2 = ew.neighbor_list(cell, nc)
        r = ew.min_image(self.x[p1] - self.x[p2], self.box)
        d = np.sqrt(np.sum(r * r, axis=1))
        keep = d < self.rc
        self.p1, self.p2, d, r = p1[keep], p2[keep], d[keep], r[keep]
        self.rhat = r / d[:, None]
        if tables is None:
            A = np.empty(d.size)
            B = np.empty(d.size)
            for k in range(d.size):
                pp, pa = couplings(np.array([d[k]]), self.a[self.p1[k]], self.a[self.p2[k]], self.xi)
                A[k], B[k] = pp[0], pa[0]
            self.A, self.B = A, B
            self.self_term = np.array([self_value(ai, ai, self.xi) for ai in self.a])
        else:
            rt, perp, para, a_uniq = tables
            _, cls = unique_radii(self.a)
            col = pair_columns(len(a_uniq))
            cij = col[cls[self.p1], cls[self.p2]]
            i = np.searchsorted(rt, d, side="left")
            if np.any(i <= 0) or np.any(i >= len(rt)):
                raise ValueError("separation outside the real-space table")
            t = (d - rt[i - 1]) / (rt[i] - rt[i - 1])
            self.A = perp[i - 1, cij] * (1 - t) + perp[i, cij] * t
            self.B = para[i - 1, cij] * (1 - t) + para[i, cij] * t
            self.self_term = perp[0, col[cls, cls]]
        self.linnode, self.rvec = stencil(self.x, self.Ngrid, self.h, self.P)
        self.g = np.stack([kernel_over_d(np.sqrt(np.sum(self.rvec[j] ** 2, axis=1)), self.a[j], self.xi, self.eta)
                           for j in range(n)])

    def field(self, p):
        """E (N,3) from dipoles p (N,3): CS/ComputeField.m:23-57 (real)."""
        p = np.asarray(p, dtype=np.float64)
        n = self.x.shape[0]
        G = int(np.prod(self.Ngrid))
        vals = self.g * np.einsum("npc,nc->np", self.rvec, p)
        grid = np.bincount(self.linnode.reshape(-1), vals.reshape(-1), minlength=G)
        nx, ny, nz = (int(v) for v in self.Ngrid)
        Et = wave_space(grid.reshape(nz, ny, nx), self.Ngrid, self.box, self.xi, self.eta).real.reshape(-1)
        Eq = np.prod(self.h) * np.einsum("np,npc->nc", self.g * Et[self.linnode], self.rvec)
        Er = 3 * p / (4 * PI * self.a[:, None] ** 3 * (self.eps[:, None] - 1)) + p * self.self_term[:, None]
        pj = p[self.p2]
        pr = np.sum(pj * self.rhat, axis=1)
        dE = self.A[:, None] * (pj - pr[:, None] * self.rhat) + (self.B * pr)[:, None] * self.rhat
        np.add.at(Er, self.p1, dE)
        return Eq + Er


def solve(geom, E0, p_guess, tol, restart=None, maxit=None):
    """CS/ComputeDipole.m:25-36."""
    from .capacitance_oracle import gmres
    n = geom.x.shape[0]
    b = np.tile(np.asarray(E0, dtype=np.float64).reshape(3), n)
    restart = min(3 * n, 10) if restart is None else restart
    maxit = min(3 * n, 100) if maxit is None else maxit
    sol, flag, relres, nmv = gmres(lambda v: geom.field(v.reshape(n, 3)).reshape(-1), b,
                                   np.asarray(p_guess, dtype=np.float64).reshape(-1), tol, restart, maxit)
    return sol.reshape(n, 3), {"flag": flag, "relres": relres, "matvecs": nmv}


def capacitance_tensor(geom, p_guess, tol):
    """CS/CapacitanceTensor.m:39-54: C (1,9) with C[3i:3i+3] the mean dipole for
    the field along i, p (N,9); warm start p_i[:, [z, x, y]]."""
    n = geom.x.shape[0]
    C = np.zeros(9)
    p = np.zeros((n, 9))
    guess = np.asarray(p_guess, dtype=np.float64)
    for i in range(3):
        pi, _ = solve(geom, np.eye(3)[i], guess, tol)
        p[:, 3 * i:3 * i + 3] = pi
        C[3 * i:3 * i + 3] = pi.mean(axis=0)
        guess = pi[:, [2, 0, 1]]
    return C, p
