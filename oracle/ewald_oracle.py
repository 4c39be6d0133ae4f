"""NumPy restatement of the dipole-only spectral-Ewald kernels (the CPU oracle).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py`` as the checker.  The GPU package never
imports it.

Every function restates one function of the reference module
``CPU - Ewald test/ewald.py`` (cited per function as ``EW/ewald.py:<lines>``) in
this project's own formulation:

* the neighbour list is generated block-wise with index arithmetic instead of a
  Python loop over cells;
* the Gaussian grid weights are evaluated as a product of three separable 1-D
  factors (the same Gaussian, ``exp(a+b+c) = exp(a)exp(b)exp(c)``);
* the k-space scaling is applied in unshifted FFT order with the fftshift folded
  into the frequency index map (a permutation: no arithmetic changes);
* the real-space tables are written as polynomial-coefficient tables evaluated
  with Horner's rule.

Parity status: pinned against vectors produced by importing the reference module
itself (``tests/golden/make_golden.py``) -- integer lists bit-exact, floating
point within the tolerances written in ``tests/test_oracle_golden.py``.
"""
from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor
from typing import Tuple

import numpy as np
import scipy.fft as _sfft
from scipy.special import erfc as _erfc

PI = math.pi
SQRT_PI3 = PI ** 1.5


# -----------------------------------------------------------------------------
# Small helpers (EW/ewald.py:40-78)
# -----------------------------------------------------------------------------
def erfc(x):
    """Complementary error function (EW/ewald.py:40-48 uses scipy's)."""
    return _erfc(np.asarray(x, dtype=np.float64))


def besselj_3_over_2(x):
    """J_{3/2}(x) = sqrt(2/(pi x)) (sin x / x - cos x), J(0) = 0 (EW/ewald.py:51-65)."""
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    nz = x != 0
    v = x[nz]
    out[nz] = np.sqrt(2.0 / (PI * v)) * (np.sin(v) / v - np.cos(v))
    return out


def matlab_round(x):
    """Round half away from zero (EW/ewald.py:71-78)."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


# -----------------------------------------------------------------------------
# Cell list + candidate neighbour list (EW/ewald.py:84-199)
# -----------------------------------------------------------------------------
def cell_list(x, box, rmax):
    """Cell coordinates of every particle (EW/ewald.py:84-111).

    Positions are wrapped with numpy's floating ``mod``; the cell count per axis
    is ``floor(L / rmax)`` clamped to at least 3; the cell coordinate is
    ``floor((x_wrapped / L) * Ncell)``.
    """
    x = np.asarray(x, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    xw = np.mod(x, box)
    ncell = np.maximum(np.floor(box / rmax).astype(np.int64), 3)
    cell = np.floor((xw / box) * ncell).astype(np.int64)
    return cell, ncell


# Neighbour-cell offsets in emission order: x offset outermost, z innermost
# (the triple loop of EW/ewald.py:171-173).
_OFFS = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)],
                 dtype=np.int64)


def _cell_sort(cell, ncell):
    n = cell.shape[0]
    nx, ny, nz = (int(v) for v in ncell)
    lin = cell[:, 0] + nx * cell[:, 1] + nx * ny * cell[:, 2]
    order = np.lexsort((np.arange(n), lin))          # by cell, then particle id
    counts = np.bincount(lin, minlength=nx * ny * nz)
    starts = np.cumsum(counts) - counts
    return lin, order, counts, starts


def neighbor_list(cell, ncell):
    """Directed candidate pairs from the 27 surrounding cells (EW/ewald.py:114-199).

    Order of the output (what makes it bit-exact with the reference): occupied
    cells in increasing linear index; for each, the 27 neighbour cells with the x
    offset outermost; for each such cell pair, every particle ``a`` of the home
    cell (increasing id) paired with every particle ``b`` of the neighbour cell
    (increasing id); finally self pairs are removed.
    """
    cell = np.asarray(cell, dtype=np.int64)
    ncell = np.asarray(ncell, dtype=np.int64).reshape(3)
    nx, ny, nz = (int(v) for v in ncell)
    lin, order, counts, starts = _cell_sort(cell, ncell)
    occupied = np.nonzero(counts)[0]
    if occupied.size == 0:
        e = np.array([], dtype=np.int64)
        return e, e.copy()
    # cell coordinates of each occupied cell
    cz = occupied // (nx * ny)
    cy = (occupied // nx) % ny
    cx = occupied % nx
    home = np.repeat(occupied, 27)
    nbx = (np.repeat(cx, 27) + np.tile(_OFFS[:, 0], occupied.size)) % nx
    nby = (np.repeat(cy, 27) + np.tile(_OFFS[:, 1], occupied.size)) % ny
    nbz = (np.repeat(cz, 27) + np.tile(_OFFS[:, 2], occupied.size)) % nz
    nb = nbx + nx * nby + nx * ny * nbz
    na = counts[home]
    nbn = counts[nb]
    size = na * nbn
    total = int(size.sum())
    blk = np.repeat(np.arange(home.size), size)
    q = np.arange(total) - np.repeat(np.cumsum(size) - size, size)
    ra = q // nbn[blk]
    rb = q % nbn[blk]
    p1 = order[starts[home[blk]] + ra]
    p2 = order[starts[nb[blk]] + rb]
    keep = p1 != p2
    return p1[keep].astype(np.int64), p2[keep].astype(np.int64)


# -----------------------------------------------------------------------------
# Stencil (EW/ewald.py:205-223)
# -----------------------------------------------------------------------------
def pre_calculations(P, h):
    """P^3 stencil offsets, x fastest, starting at -floor((P-1)/2) (EW/ewald.py:205-223)."""
    P = int(P)
    h = np.asarray(h, dtype=np.float64).reshape(3)
    lo = (P - 1) // 2
    j = np.arange(P ** 3)
    offset = np.stack((j % P - lo, (j // P) % P - lo, j // (P * P) - lo), axis=1).astype(np.int64)
    return offset, offset.astype(np.float64) * h.reshape(1, 3)


# -----------------------------------------------------------------------------
# Gaussian grid weights, spread, contract (EW/ewald.py:233-467)
# -----------------------------------------------------------------------------
def gaussian_const(xi, eta):
    eta = np.asarray(eta, dtype=np.float64).reshape(3)
    return (2.0 * xi * xi / PI) ** 1.5 * math.sqrt(1.0 / float(np.prod(eta)))


def separable_weights(x, Ngrid, h, xi, eta, P):
    """Per-particle 1-D Gaussian factors and the first stencil node.

    Returns ``start`` (N,3) int64 = wrapped grid index of stencil column 0 and
    ``wd`` (N,3,P) with ``prod_d wd[n,d,j_d] * const`` equal to the spreading
    weight of node ``(j_x,j_y,j_z)`` (EW/ewald.py:275-293: nearest node by
    half-away rounding of ``x/h``, node index ``(node0 + off - 1) mod Ngrid``,
    weight evaluated at ``(node0 + off) h - x``).
    """
    x = np.asarray(x, dtype=np.float64)
    Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
    h = np.asarray(h, dtype=np.float64).reshape(3)
    eta = np.asarray(eta, dtype=np.float64).reshape(3)
    lo = (int(P) - 1) // 2
    node0 = matlab_round(x / h).astype(np.int64)
    off = np.arange(int(P)) - lo
    start = np.mod(node0 - lo - 1, Ngrid)
    base = node0.astype(np.float64) * h - x                         # (N,3)
    r = base[:, :, None] + (off.astype(np.float64)[None, None, :] * h[None, :, None])
    wd = np.exp(-2.0 * xi * xi * (r * r) / eta[None, :, None])
    return start, wd


def prepare_grid_kernel(x, Ngrid, h, xi, eta, P, offset=None, offsetxyz=None):
    """Dense (N,P^3) node indices and weights (EW/ewald.py:233-296)."""
    Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
    h = np.asarray(h, dtype=np.float64).reshape(3)
    P = int(P)
    start, wd = separable_weights(x, Ngrid, h, xi, eta, P)
    c = gaussian_const(xi, eta)
    j = np.arange(P)
    ix = np.mod(start[:, 0, None] + j, Ngrid[0])          # (N,P)
    iy = np.mod(start[:, 1, None] + j, Ngrid[1])
    iz = np.mod(start[:, 2, None] + j, Ngrid[2])
    # stencil order: x fastest, then y, then z
    lin = (ix[:, None, None, :] + Ngrid[0] * iy[:, None, :, None]
           + Ngrid[0] * Ngrid[1] * iz[:, :, None, None]).reshape(x.shape[0], -1)
    w = (c * wd[:, 2, :, None, None] * wd[:, 1, None, :, None] * wd[:, 0, None, None, :]).reshape(x.shape[0], -1)
    return lin.astype(np.int64), w, w * float(np.prod(h))


def spread_fast(m, Ngrid, linnode, w_spread):
    """Grid[c] += w * m_c (EW/ewald.py:299-331); returns (Nx,Ny,Nz,3) complex."""
    m = np.asarray(m, dtype=np.complex128)
    Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
    G = int(np.prod(Ngrid))
    lin = np.asarray(linnode).reshape(-1)
    out = np.empty((G, 3), dtype=np.complex128)
    for c in range(3):
        v = (np.asarray(w_spread)[:, :] * m[:, c:c + 1]).reshape(-1)
        out[:, c] = np.bincount(lin, v.real, minlength=G) + 1j * np.bincount(lin, v.imag, minlength=G)
    return out.reshape(int(Ngrid[2]), int(Ngrid[1]), int(Ngrid[0]), 3).transpose(2, 1, 0, 3)


def contract_fast(Htilde, Ngrid, linnode, w_contract):
    """H_k[n,c] = sum_nodes w_c * grid_c (EW/ewald.py:334-368)."""
    Htilde = np.asarray(Htilde, dtype=np.complex128)
    out = np.empty((linnode.shape[0], 3), dtype=np.complex128)
    for c in range(3):
        flat = Htilde[..., c].transpose(2, 1, 0).reshape(-1)
        out[:, c] = np.sum(w_contract * flat[linnode], axis=1)
    return out


def spread(x, m, Ngrid, h, xi, eta, P, offset=None, offsetxyz=None):
    """On-the-fly spread (EW/ewald.py:370-418); returns (Hx, Hy, Hz)."""
    lin, w, _ = prepare_grid_kernel(x, Ngrid, h, xi, eta, P)
    H = spread_fast(m, Ngrid, lin, w)
    return H[..., 0], H[..., 1], H[..., 2]


def contract(x, Ngrid, h, xi, eta, P, Htilde, offset=None, offsetxyz=None):
    """On-the-fly contract (EW/ewald.py:421-467)."""
    lin, _, wc = prepare_grid_kernel(x, Ngrid, h, xi, eta, P)
    return contract_fast(Htilde, Ngrid, lin, wc)


# -----------------------------------------------------------------------------
# Reciprocal space (EW/ewald.py:473-599)
# -----------------------------------------------------------------------------
def fft_freq(n):
    """Integer frequency of each unshifted FFT index, with the reference's
    fftshift convention ``k in [-ceil((n-1)/2), floor((n-1)/2)]`` (EW/ewald.py:550-552):
    an even-length axis carries its Nyquist bin as the negative frequency."""
    c = n // 2
    i = np.arange(n)
    return ((i + c) % n) - c


def _kcoef(k2, etak2, xi):
    kk = np.sqrt(k2)
    J = besselj_3_over_2(kk)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        H = (9.0 * PI) / (2.0 * kk) * (J * J) * np.exp(-etak2 / (4.0 * xi * xi)) / k2
    H[k2 == 0] = 0.0
    return np.nan_to_num(H)


def kspace_unshifted(Ngrid, box, xi, eta):
    """k vectors (Nx,Ny,Nz,3) and the scalar Green's coefficient in unshifted order.

    Coefficient (EW/ewald.py:573-580):
    ``9 pi / (2|k|) J_{3/2}(|k|)^2 exp(-sum_d (1-eta_d) k_d^2 / (4 xi^2)) / |k|^2``,
    zero at k = 0.
    """
    Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    eta = np.asarray(eta, dtype=np.float64).reshape(3)
    ks = [fft_freq(int(Ngrid[d])) * (2.0 * PI / box[d]) for d in range(3)]
    KX, KY, KZ = np.meshgrid(*ks, indexing="ij")
    k = np.stack((KX, KY, KZ), axis=3)
    k2 = np.sum(k * k, axis=3)
    etak2 = (1.0 - eta[0]) * KX ** 2 + (1.0 - eta[1]) * KY ** 2 + (1.0 - eta[2]) * KZ ** 2
    return k, _kcoef(k2, etak2, xi)


def precompute_kspace(Ngrid, box, xi, eta):
    """khat (complex) and coefficient in the reference's fftshift order (EW/ewald.py:523-582)."""
    k, H = kspace_unshifted(Ngrid, box, xi, eta)
    kk = np.sqrt(np.sum(k * k, axis=3))
    kk[kk == 0] = 1.0
    khat = k / kk[..., None]
    khat = np.fft.fftshift(khat, axes=(0, 1, 2)).astype(np.complex128)
    return khat, np.fft.fftshift(H, axes=(0, 1, 2))


def scale_fast(fH, khat, Htildecoeff):
    """f~ = H(k) (khat . f) khat (EW/ewald.py:585-599)."""
    d = np.sum(khat * fH, axis=3)
    return (Htildecoeff * d)[..., None] * khat


def _khat_unshifted(Ngrid, box, xi, eta):
    k, H = kspace_unshifted(Ngrid, box, xi, eta)
    kk = np.sqrt(np.sum(k * k, axis=3))
    kk[kk == 0] = 1.0
    return k / kk[..., None], H


def wave_space_complex(Hgrid, Ngrid, box, xi, eta):
    """FFT -> scale -> IFFT exactly as the reference's complex pipeline (EW/ewald.py:1199-1217)."""
    khat, H = _khat_unshifted(Ngrid, box, xi, eta)
    f = np.fft.fftn(Hgrid, axes=(0, 1, 2))
    g = (H * np.sum(khat * f, axis=3))[..., None] * khat
    return np.fft.ifftn(g, axes=(0, 1, 2))


def nyquist_mask(Ngrid):
    """Boolean per axis index: True on the unpaired Nyquist bin of an even axis."""
    out = []
    for n in np.asarray(Ngrid, dtype=np.int64).reshape(3):
        m = np.zeros(int(n), dtype=bool)
        if n % 2 == 0:
            m[n // 2] = True
        out.append(m)
    return out


def wave_space_real(Hgrid_real, Ngrid, box, xi, eta):
    """Real part of the reference wave-space operator applied to a REAL grid.

    For real input the reference's complex pipeline returns ``A_r g + i A_i g``
    where ``A_i`` is non-zero only through the unpaired Nyquist bins of even
    axes.  Its real part equals a Hermitian operator whose scaling tensor is
    ``H k^ k^T`` with every entry coupling a Nyquist axis to a non-Nyquist axis
    set to zero (average of the tensor at k and at its conjugate partner).
    """
    khat, H = _khat_unshifted(Ngrid, box, xi, eta)
    nyq = nyquist_mask(Ngrid)
    NX, NY, NZ = np.meshgrid(*nyq, indexing="ij")
    nq = np.stack((NX, NY, NZ), axis=3)
    f = np.fft.fftn(Hgrid_real, axes=(0, 1, 2))
    g = np.zeros_like(f)
    for a in range(3):
        acc = 0.0
        for b in range(3):
            same = (nq[..., a] == nq[..., b])
            acc = acc + np.where(same, khat[..., a] * khat[..., b], 0.0) * f[..., b]
        g[..., a] = H * acc
    return np.real(np.fft.ifftn(g, axes=(0, 1, 2)))


# -----------------------------------------------------------------------------
# Real-space tables (EW/ewald.py:604-931) written as polynomial coefficient sets
# -----------------------------------------------------------------------------
def _table_terms(xi):
    """For each of the 6 tables: (cE, rpowE, E+, E-, E0, cF, rpowF, F+, F-, F0, reg).

    A table value at separation r is
      cE r^-rpowE [E+(r) e^{-xi^2 (r+2)^2} + E-(r) e^{-xi^2 (r-2)^2} + E0(r) e^{-xi^2 r^2}]
    + cF r^-rpowF [F+(r) erfc(xi (r+2)) + F-(r) erfc(xi (r-2)) + F0(r) erfc(xi r)]
    + [r < 2] reg(r)
    with E*, F* polynomials in r (coefficients highest power first).
    """
    x2 = xi * xi
    x4 = x2 * x2
    x6 = x4 * x2
    q = 3.0 - 12.0 * x2 + 32.0 * x4
    s = 2.0 * (3.0 + 4.0 * x2 - 32.0 * x4)
    t = {}
    # potential / charge
    t["pot_charge"] = (
        1.0 / (32.0 * SQRT_PI3 * xi), 1, [-1.0, -2.0], [-1.0, 2.0], [2.0, 0.0],
        1.0 / (64.0 * PI * x2), 1, [2 * x2, 8 * x2, 8 * x2 + 1.0], [2 * x2, -8 * x2, 8 * x2 + 1.0], [-4 * x2, 0.0, -2.0],
        lambda r: -1.0 / (4.0 * PI * r) + (4.0 - r) / (16.0 * PI))
    # potential / dipole
    t["pot_dip"] = (
        1.0 / (256.0 * SQRT_PI3 * xi ** 3), 2,
        [-6 * x2, -4 * x2, 8 * x2 - 3.0, 2.0 - 16 * x2], [-6 * x2, 4 * x2, 8 * x2 - 3.0, 16 * x2 - 2.0],
        [12 * x2, 0.0, 6.0, 0.0],
        1.0 / (512.0 * PI * x4), 2,
        [12 * x4, 32 * x4, 12 * x2, 0.0, 64 * x4 - 3.0], [12 * x4, -32 * x4, 12 * x2, 0.0, 64 * x4 - 3.0],
        [-24 * x4, 0.0, -24 * x2, 0.0, 6.0],
        lambda r: -1.0 / (4.0 * PI * r ** 2) + r / (8.0 * PI) * (1.0 - 3.0 / 8.0 * r))
    # field / dipole, (I - rr) part
    t["field_dip_1"] = (
        1.0 / (1024.0 * SQRT_PI3 * xi ** 5), 3,
        [4 * x4, -8 * x4, 8 * x2 * (2 - 7 * x2), -8 * x2 * (3 + 2 * x2), q, s],
        [4 * x4, 8 * x4, 8 * x2 * (2 - 7 * x2), 8 * x2 * (3 + 2 * x2), q, -s],
        [-8 * x4, 0.0, -16 * x2 * (2 - 9 * x2), 0.0, 2 * (36 * x2 - 3), 0.0],
        1.0 / (2048.0 * PI * x6), 3,
        [-8 * x6, 0.0, -36 * x4 * (1 - 4 * x2), 256 * x6, -18 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6],
        [-8 * x6, 0.0, -36 * x4 * (1 - 4 * x2), -256 * x6, -18 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6],
        [16 * x6, 0.0, 72 * x4 * (1 - 4 * x2), 0.0, 36 * x2 * (1 - 8 * x2), 0.0, 2 * (36 * x2 - 3)],
        lambda r: -1.0 / (4.0 * PI * r ** 3) + (1.0 - 9.0 * r / 16.0 + r ** 3 / 32.0) / (4.0 * PI))
    # field / dipole, rr part
    t["field_dip_2"] = (
        1.0 / (512.0 * SQRT_PI3 * xi ** 5), 3,
        [8 * x4, -16 * x4, 2 * x2 * (7 - 20 * x2), -4 * x2 * (3 - 4 * x2), -q, -s],
        [8 * x4, 16 * x4, 2 * x2 * (7 - 20 * x2), 4 * x2 * (3 - 4 * x2), -q, s],
        [-16 * x4, 0.0, -4 * x2 * (7 - 36 * x2), 0.0, 2 * (3 - 36 * x2), 0.0],
        1.0 / (1024.0 * PI * x6), 3,
        [-16 * x6, 0.0, -36 * x4 * (1 - 4 * x2), 128 * x6, 0.0, 0.0, -3 + 36 * x2 - 256 * x6],
        [-16 * x6, 0.0, -36 * x4 * (1 - 4 * x2), -128 * x6, 0.0, 0.0, -3 + 36 * x2 - 256 * x6],
        [32 * x6, 0.0, 72 * x4 * (1 - 4 * x2), 0.0, 0.0, 0.0, 2 * (3 - 36 * x2)],
        lambda r: 1.0 / (2.0 * PI * r ** 3) + (1.0 - 9.0 * r / 8.0 + r ** 3 / 8.0) / (4.0 * PI))
    # force: coefficient of -(mi.mj) r and related terms
    t["field_dip_force_1"] = (
        3.0 / (1024.0 * SQRT_PI3 * xi ** 5), 4,
        [4 * x4, -8 * x4, 4 * x2 * (1 - 2 * x2), 16 * x4, -q, -s],
        [4 * x4, 8 * x4, 4 * x2 * (1 - 2 * x2), -16 * x4, -q, s],
        [-8 * x4, 0.0, -8 * x2 * (1 - 6 * x2), 0.0, 2 * (3 - 36 * x2), 0.0],
        3.0 / (2048.0 * PI * x6), 4,
        [-8 * x6, 0.0, -12 * x4 * (1 - 4 * x2), 0.0, 6 * x2 * (1 - 8 * x2), 0.0, -3 + 36 * x2 - 256 * x6],
        [-8 * x6, 0.0, -12 * x4 * (1 - 4 * x2), 0.0, 6 * x2 * (1 - 8 * x2), 0.0, -3 + 36 * x2 - 256 * x6],
        [16 * x6, 0.0, 24 * x4 * (1 - 4 * x2), 0.0, -12 * x2 * (1 - 8 * x2), 0.0, 2 * (3 - 36 * x2)],
        lambda r: 3.0 / (4.0 * PI * r ** 4) - 3.0 / (64.0 * PI) * (3.0 - r ** 2 / 2.0))
    # force: coefficient of -(mi.r)(mj.r) r
    t["field_dip_force_2"] = (
        9.0 / (1024.0 * SQRT_PI3 * xi ** 5), 4,
        [4 * x4, -8 * x4, 8 * x4, 8 * x2 * (1 - 2 * x2), q, s],
        [4 * x4, 8 * x4, 8 * x4, -8 * x2 * (1 - 2 * x2), q, -s],
        [-8 * x4, 0.0, 16 * x4, 0.0, 2 * (36 * x2 - 3), 0.0],
        9.0 / (2048.0 * PI * x6), 4,
        [-8 * x6, 0.0, -4 * x4 * (1 - 4 * x2), 0.0, -2 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6],
        [-8 * x6, 0.0, -4 * x4 * (1 - 4 * x2), 0.0, -2 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6],
        [16 * x6, 0.0, 8 * x4 * (1 - 4 * x2), 0.0, 4 * x2 * (1 - 8 * x2), 0.0, 2 * (36 * x2 - 3)],
        lambda r: -9.0 / (4.0 * PI * r ** 4) - 9.0 / (64.0 * PI) * (1.0 - r ** 2 / 2.0))
    return t


TABLE_NAMES = ("pot_charge", "pot_dip", "field_dip_1", "field_dip_2", "field_dip_force_1", "field_dip_force_2")


def table_coefficients(xi):
    """The coefficient sets of ``_table_terms`` (shared with the GPU table kernel's tests)."""
    return _table_terms(xi)


def _eval_table(r, xi, spec):
    cE, pE, Ep, Em, E0, cF, pF, Fp, Fm, F0, reg = spec
    ep = np.exp(-(r + 2.0) ** 2 * xi * xi)
    em = np.exp(-(r - 2.0) ** 2 * xi * xi)
    e0 = np.exp(-r * r * xi * xi)
    fp = erfc((r + 2.0) * xi)
    fm = erfc((r - 2.0) * xi)
    f0 = erfc(r * xi)
    val = cE / r ** pE * (np.polyval(Ep, r) * ep + np.polyval(Em, r) * em + np.polyval(E0, r) * e0)
    val = val + cF / r ** pF * (np.polyval(Fp, r) * fp + np.polyval(Fm, r) * fm + np.polyval(F0, r) * f0)
    return val + np.where(r < 2.0, reg(r), 0.0)


def self_terms(xi):
    """Values prepended at r = 0 (EW/ewald.py:918-931): (charge, field/dipole)."""
    e4 = math.exp(-4.0 * xi * xi)
    ec = float(erfc(2.0 * xi))
    s_pc = (1.0 - e4) / (8.0 * SQRT_PI3 * xi) + ec / (4.0 * PI)
    s_fd = (-1.0 + 6.0 * xi * xi + (1.0 - 2.0 * xi * xi) * e4) / (16.0 * SQRT_PI3 * xi ** 3) + ec / (4.0 * PI)
    return s_pc, s_fd


def real_space_table(r, xi):
    """Six tables at separations r (no zero), each with the r = 0 self value
    prepended (EW/ewald.py:604-931)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    t = _table_terms(float(xi))
    vals = {k: _eval_table(r, float(xi), t[k]) for k in TABLE_NAMES}
    s_pc, s_fd = self_terms(float(xi))
    heads = {"pot_charge": s_pc, "pot_dip": 0.0, "field_dip_1": s_fd, "field_dip_2": s_fd,
             "field_dip_force_1": 0.0, "field_dip_force_2": 0.0}
    return tuple(np.concatenate(([heads[k]], vals[k])) for k in TABLE_NAMES)


def default_table(xi):
    """The fixed table of ``run_capacitance`` (EW/capacitance.py:471-477):
    r = 0.001..10 step 0.001 with 0 prepended; returns (perp, para, rvals)."""
    r = np.arange(0.001, 10.0 + 1e-12, 0.001, dtype=np.float64)
    _, _, f1, f2, _, _ = real_space_table(r, xi)
    return f1, f2, np.concatenate(([0.0], r))


# -----------------------------------------------------------------------------
# Real-space pairs and pair sum (EW/ewald.py:939-1139)
# -----------------------------------------------------------------------------
def min_image(r, box):
    """r - L trunc(2 r / L) (EW/ewald.py:980)."""
    box = np.asarray(box, dtype=np.float64).reshape(1, 3)
    return r - box * np.trunc(2.0 * r / box)


def prepare_real_space_pairs(x, box, p1, p2, rc, perp, para, rvals):
    """Keep pairs with d < rc; unit vectors; table interpolation (EW/ewald.py:939-1016).

    The interpolation index is the first table entry >= d (``searchsorted``
    left); an index of 0 or past the end raises ``ValueError`` like the reference.
    """
    x = np.asarray(x, dtype=np.float64)
    p1 = np.asarray(p1, dtype=np.int64).reshape(-1)
    p2 = np.asarray(p2, dtype=np.int64).reshape(-1)
    ei = np.array([], dtype=np.int64)
    ef = np.array([], dtype=np.float64)
    if p1.size == 0:
        return ei, ei.copy(), ef.reshape(0, 3), ef, ef.copy()
    r = min_image(x[p1] - x[p2], box)
    d = np.sqrt(np.sum(r * r, axis=1))
    keep = d < float(rc)
    p1, p2, r, d = p1[keep], p2[keep], r[keep], d[keep]
    if d.size == 0:
        return p1, p2, ef.reshape(0, 3), ef, ef.copy()
    rhat = r / d[:, None]
    i = np.searchsorted(rvals, d, side="left")
    if np.any(i <= 0) or np.any(i >= len(rvals)):
        raise ValueError("RealSpace interpolation: pair separations fall outside rvals table.")
    t = (d - rvals[i - 1]) / (rvals[i] - rvals[i - 1])
    A = perp[i - 1] * (1.0 - t) + perp[i] * t
    B = para[i - 1] * (1.0 - t) + para[i] * t
    return p1, p2, rhat, A, B


def dielectric_diag(lambdap):
    """-3 / (4 pi (1 - lambda)) per particle (EW/ewald.py:1058)."""
    lam = np.asarray(lambdap, dtype=np.float64).reshape(-1)
    return -3.0 / (4.0 * PI * (1.0 - lam))


def real_space_fast(m, lambdap, p1, p2, rhat, A, B, self_perp):
    """Hr = (diag + self) m + sum_pairs [A m_j + (B-A)(m_j.rhat) rhat] (EW/ewald.py:1019-1072)."""
    m = np.asarray(m)
    Hr = dielectric_diag(lambdap)[:, None] * m + m * float(self_perp)
    if len(p1) == 0:
        return Hr
    mj = m[p2]
    proj = np.sum(mj * rhat, axis=1)
    contrib = A[:, None] * mj + ((B - A) * proj)[:, None] * rhat
    np.add.at(Hr, p1, contrib)
    return Hr


def real_space(x, m, lambdap, box, p1, p2, rc, perp, para, rvals, real_precomp=None):
    """Pair-loop form (EW/ewald.py:1076-1139), restated through the pair preparation."""
    pr = prepare_real_space_pairs(x, box, p1, p2, rc, perp, para, rvals)
    return real_space_fast(m, lambdap, *pr, self_perp=perp[0])


# -----------------------------------------------------------------------------
# Full matvec (EW/ewald.py:1146-1327)
# -----------------------------------------------------------------------------
def slab_term(m, box, slab_factor):
    """+ slab_factor * sum(m_z) / V along z, added to every particle (EW/ewald.py:1233-1236)."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    out = np.zeros_like(np.asarray(m))
    out[:, 2] = float(slab_factor) * np.sum(np.asarray(m)[:, 2]) / float(np.prod(box))
    return out


class Geometry:
    """Everything that depends on positions only, built once per solve
    (the role of real_precomp / grid_precomp / k_precomp, EW/capacitance.py:370-385)."""

    def __init__(self, x, lambdap, box, xi, rc, Ngrid, P, perp, para, rvals, slab_factor=1.0):
        self.x = np.asarray(x, dtype=np.float64)
        self.box = np.asarray(box, dtype=np.float64).reshape(3)
        self.lambdap = np.asarray(lambdap, dtype=np.float64).reshape(-1)
        self.xi = float(xi)
        self.rc = float(rc)
        self.Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
        self.h = self.box / self.Ngrid
        self.P = int(P)
        self.eta = self.P * (self.h * self.xi) ** 2 / PI
        self.perp, self.para, self.rvals = perp, para, rvals
        self.slab_factor = float(slab_factor)
        cell, ncell = cell_list(self.x, self.box, self.rc)
        p1, p2 = neighbor_list(cell, ncell)
        self.pairs = prepare_real_space_pairs(self.x, self.box, p1, p2, self.rc, perp, para, rvals)
        self.lin, self.w, self.wc = prepare_grid_kernel(self.x, self.Ngrid, self.h, self.xi, self.eta, self.P)

    def field_complex(self, m):
        """The reference matvec with its complex FFT pipeline (EW/ewald.py:1146-1236)."""
        H = spread_fast(m, self.Ngrid, self.lin, self.w)
        Ht = wave_space_complex(H, self.Ngrid, self.box, self.xi, self.eta)
        Hk = contract_fast(Ht, self.Ngrid, self.lin, self.wc)
        Hr = real_space_fast(np.asarray(m, dtype=np.complex128), self.lambdap, *self.pairs, self.perp[0])
        return Hk + Hr + slab_term(np.asarray(m, dtype=np.complex128), self.box, self.slab_factor)

    def field_real(self, m):
        """Real part of the reference matvec for real moments (the GPU operator)."""
        m = np.asarray(m, dtype=np.float64)
        H = np.real(spread_fast(m, self.Ngrid, self.lin, self.w))
        Ht = wave_space_real(H, self.Ngrid, self.box, self.xi, self.eta)
        Hk = np.real(contract_fast(Ht, self.Ngrid, self.lin, self.wc))
        Hr = real_space_fast(m, self.lambdap, *self.pairs, self.perp[0])
        return Hk + Hr + slab_term(m, self.box, self.slab_factor)

    def field_real_many(self, M, threads=None):
        """``field_real`` for R vectors (R, N, 3) using ``threads`` host threads
        (all cores by default): the same operator, with sums regrouped over
        particle chunks (agrees with ``field_real`` to rounding)."""
        return _field_real_many(self, M, threads)


# -----------------------------------------------------------------------------
# The real operator on several vectors, spread over host threads
# -----------------------------------------------------------------------------
def host_threads(threads=None):
    """Threads the multi-threaded forms below use (all host cores by default)."""
    return max(1, int(threads or os.cpu_count() or 1))


def _bounds(n, k):
    k = max(1, min(int(k), int(n)))
    b = np.linspace(0, n, k + 1).astype(np.int64)
    return [(int(b[i]), int(b[i + 1])) for i in range(k)]


def wave_space_real_many(grids, Ngrid, box, xi, eta, threads=None):
    """``wave_space_real`` for R real grids (R, Nx, Ny, Nz, 3) at once: the same
    masked scaling tensor and operation order per element, FFTs by scipy's
    pocketfft with ``workers`` and the scaling split over x-slabs in threads."""
    t = host_threads(threads)
    khat, H = _khat_unshifted(Ngrid, box, xi, eta)
    nyq = nyquist_mask(Ngrid)
    NX, NY, NZ = np.meshgrid(*nyq, indexing="ij")
    nq = np.stack((NX, NY, NZ), axis=3)
    f = _sfft.fftn(grids, axes=(1, 2, 3), workers=t)
    g = np.empty_like(f)

    def part(lo, hi):
        kh, nql, Hs = khat[lo:hi], nq[lo:hi], H[lo:hi]
        for a in range(3):
            acc = 0.0
            for b in range(3):
                same = (nql[..., a] == nql[..., b])
                acc = acc + np.where(same, kh[..., a] * kh[..., b], 0.0)[None] * f[:, lo:hi, :, :, b]
            g[:, lo:hi, :, :, a] = Hs[None] * acc

    with ThreadPoolExecutor(t) as ex:
        list(ex.map(lambda b: part(*b), _bounds(grids.shape[1], t)))
    return np.real(_sfft.ifftn(g, axes=(1, 2, 3), workers=t))


def _field_real_many(geom, M, threads=None):
    """Real operator on R vectors M (R, N, 3); see ``Geometry.field_real_many``."""
    t = host_threads(threads)
    M = np.asarray(M, dtype=np.float64).reshape(-1, geom.x.shape[0], 3)
    R, N = M.shape[0], M.shape[1]
    Ng = geom.Ngrid
    G = int(np.prod(Ng))
    comps = [(r, c) for r in range(R) for c in range(3)]
    chunks = _bounds(N, max(1, -(-t // len(comps))))
    # spread: one bincount per (vector, component, particle chunk); partial grids summed in chunk order
    def spread_task(task):
        r, c, lo, hi = task
        return np.bincount(geom.lin[lo:hi].reshape(-1), (geom.w[lo:hi] * M[r, lo:hi, c:c + 1]).reshape(-1),
                           minlength=G)

    tasks = [(r, c, lo, hi) for (r, c) in comps for (lo, hi) in chunks]
    flat = np.zeros((R, 3, G))
    with ThreadPoolExecutor(t) as ex:
        for (r, c, _, _), part in zip(tasks, ex.map(spread_task, tasks)):
            flat[r, c] += part
    grids = flat.reshape(R, 3, int(Ng[2]), int(Ng[1]), int(Ng[0])).transpose(0, 4, 3, 2, 1)
    Ht = wave_space_real_many(grids, Ng, geom.box, geom.xi, geom.eta, t)
    hflat = np.ascontiguousarray(Ht.transpose(0, 4, 3, 2, 1)).reshape(R, 3, G)
    out = np.empty((R, N, 3))

    def contract_task(task):
        r, c, lo, hi = task
        out[r, lo:hi, c] = np.sum(geom.wc[lo:hi] * hflat[r, c][geom.lin[lo:hi]], axis=1)

    def real_task(r):
        return real_space_fast(M[r], geom.lambdap, *geom.pairs, geom.perp[0]) + slab_term(M[r], geom.box,
                                                                                        geom.slab_factor)

    with ThreadPoolExecutor(t) as ex:
        list(ex.map(contract_task, tasks))
        hr = list(ex.map(real_task, range(R)))
    return out + np.stack(hr)


def magnetic_field(x, m, lambdap, box, p1, p2, Ngrid, h, P, xi, eta, rc, offset, offsetxyz,
                   Hperp, Hpara, rvals, real_precomp=None, grid_precomp=None, k_precomp=None,
                   slab_factor=1.0):
    """Field at the particles from their dipoles (EW/ewald.py:1146-1236), complex pipeline."""
    x = np.asarray(x, dtype=np.float64)
    m = np.asarray(m, dtype=np.complex128)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    if grid_precomp is None:
        grid_precomp = prepare_grid_kernel(x, Ngrid, h, xi, eta, P)
    lin, w, wc = grid_precomp
    Hg = spread_fast(m, Ngrid, lin, w)
    Ht = wave_space_complex(Hg, Ngrid, box, xi, eta)
    Hk = contract_fast(Ht, Ngrid, lin, wc)
    if real_precomp is None:
        real_precomp = prepare_real_space_pairs(x, box, p1, p2, rc, Hperp, Hpara, rvals)
    Hr = real_space_fast(m, lambdap, *real_precomp, Hperp[0])
    return Hk + Hr + slab_term(m, box, slab_factor)
