"""Drop-in for the reference module ``CPU - Ewald test/ewald.py``.

Same function names, argument order and meaning; every computation runs on the
GPU through ``libmps_gb300.so``.  Arguments may be numpy arrays (results come
back as numpy arrays, like the reference) or CUDA tensors (results stay on the
device).  Complex moment arrays are handled as their real and imaginary parts
(every operator here is real-linear).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .system import SpectralEwaldSystem, as_device

__all__ = [
    "erfc", "besselj_3_over_2", "matlab_round", "cell_list", "neighbor_list", "pre_calculations",
    "prepare_grid_kernel", "spread_fast", "contract_fast", "spread", "contract", "scale", "precompute_kspace",
    "scale_fast", "real_space_table", "prepare_real_space_pairs", "real_space_fast", "real_space",
    "magnetic_field", "magnetic_field_components",
]


def _is_np(*args):
    return not any(isinstance(a, torch.Tensor) for a in args)


def _ret(t, as_numpy):
    if not as_numpy:
        return t
    return t.cpu().numpy()


def _ri(m):
    """(2, N, 3) float64 device stack of the real and imaginary parts."""
    if isinstance(m, torch.Tensor):
        mc = m.to("cuda")
        if mc.is_complex():
            return torch.stack((mc.real, mc.imag)).to(torch.float64).contiguous(), True
        return mc.to(torch.float64).reshape(1, -1, 3).contiguous(), False
    a = np.asarray(m)
    if np.iscomplexobj(a):
        return torch.as_tensor(np.stack((a.real, a.imag)), dtype=torch.float64, device="cuda").contiguous(), True
    return torch.as_tensor(a, dtype=torch.float64, device="cuda").reshape(1, -1, 3).contiguous(), False


def _cplx(t_ri, was_complex):
    if was_complex:
        return torch.complex(t_ri[0], t_ri[1])
    return torch.complex(t_ri[0], torch.zeros_like(t_ri[0]))


# -----------------------------------------------------------------------------
# Helpers (ewald.py:40-78)
# -----------------------------------------------------------------------------
def erfc(x):
    """Complementary error function (ewald.py:40-48), evaluated on the GPU."""
    t = as_device(x)
    return _ret(torch.special.erfc(t), _is_np(x))


def besselj_3_over_2(x):
    """J_{3/2}(x) with J(0) = 0 (ewald.py:51-65), evaluated on the GPU."""
    t = as_device(x)
    safe = torch.where(t != 0, t, torch.ones_like(t))
    v = torch.sqrt(2.0 / (np.pi * safe)) * (torch.sin(safe) / safe - torch.cos(safe))
    return _ret(torch.where(t != 0, v, torch.zeros_like(t)), _is_np(x))


def matlab_round(x):
    """Round half away from zero (ewald.py:71-78)."""
    t = as_device(x)
    return _ret(torch.sign(t) * torch.floor(torch.abs(t) + 0.5), _is_np(x))


# -----------------------------------------------------------------------------
# Cell list / neighbour list (ewald.py:84-199)
# -----------------------------------------------------------------------------
def cell_list(x, box, rmax):
    """Cell coordinates (N,3) int64 and cell counts (3,) (ewald.py:84-111)."""
    lib = L.lib()
    xd = as_device(x).reshape(-1, 3)
    n = xd.shape[0]
    cell = torch.empty((n, 3), dtype=torch.int64, device="cuda")
    nc = (C.c_int64 * 3)()
    L.check(lib.mps_cell_list(L.dptr(xd), n, L.host_f64(np.asarray(box).reshape(3)), float(rmax), L.dptr(cell), nc,
                              L.stream_handle()), "cell_list")
    ncell = np.array(list(nc), dtype=np.int64)
    return _ret(cell, _is_np(x)), ncell


def neighbor_list(cell, Ncell):
    """Directed candidate pairs (p1, p2) in the reference's order (ewald.py:114-199)."""
    lib = L.lib()
    cd = as_device(cell, torch.int64).reshape(-1, 3)
    n = cd.shape[0]
    nc = L.host_i64(np.asarray(Ncell).reshape(3))
    wsb = lib.mps_neighbor_list_workspace(n, nc)
    ws = torch.empty(int(wsb), dtype=torch.uint8, device="cuda")
    total = C.c_int64(0)
    s = L.stream_handle()
    L.check(lib.mps_neighbor_list_count(L.dptr(cd), n, nc, L.dptr(ws), wsb, C.byref(total), s), "neighbor_list")
    p1 = torch.empty(total.value, dtype=torch.int64, device="cuda")
    p2 = torch.empty(total.value, dtype=torch.int64, device="cuda")
    if total.value:
        L.check(lib.mps_neighbor_list_fill(L.dptr(cd), n, nc, L.dptr(ws), wsb, L.dptr(p1), L.dptr(p2), s),
                "neighbor_list")
    asnp = _is_np(cell)
    return _ret(p1, asnp), _ret(p2, asnp)


# -----------------------------------------------------------------------------
# Stencil and grid kernel (ewald.py:205-296)
# -----------------------------------------------------------------------------
def pre_calculations(P, h):
    """P^3 stencil offsets and their coordinates (ewald.py:205-223)."""
    lib = L.lib()
    P = int(P)
    off = torch.empty((P ** 3, 3), dtype=torch.int64, device="cuda")
    offxyz = torch.empty((P ** 3, 3), dtype=torch.float64, device="cuda")
    hv = np.asarray(h.cpu() if isinstance(h, torch.Tensor) else h, dtype=np.float64).reshape(3)
    L.check(lib.mps_pre_calculations(P, L.host_f64(hv), L.dptr(off), L.dptr(offxyz), L.stream_handle()),
            "pre_calculations")
    asnp = not isinstance(h, torch.Tensor)
    return _ret(off, asnp), _ret(offxyz, asnp)


def _host3(v, dtype=np.float64):
    if isinstance(v, torch.Tensor):
        v = v.cpu().numpy()
    return np.asarray(v, dtype=dtype).reshape(3)


def prepare_grid_kernel(x, Ngrid, h, xi, eta, P, offset=None, offsetxyz=None):
    """Dense (N,P^3) node indices and spread / contract weights (ewald.py:233-296)."""
    lib = L.lib()
    P = int(P)
    if offset is not None and np.asarray(offset.shape if isinstance(offset, torch.Tensor) else np.shape(offset))[0] != P ** 3:
        raise ValueError("offset/offsetxyz shapes do not match P^3. Recompute PreCalculations.")
    xd = as_device(x).reshape(-1, 3)
    n = xd.shape[0]
    P3 = P ** 3
    lin = torch.empty((n, P3), dtype=torch.int64, device="cuda")
    ws = torch.empty((n, P3), dtype=torch.float64, device="cuda")
    wc = torch.empty((n, P3), dtype=torch.float64, device="cuda")
    L.check(lib.mps_grid_kernel(L.dptr(xd), n, L.host_i64(_host3(Ngrid, np.int64)), L.host_f64(_host3(h)), float(xi),
                                L.host_f64(_host3(eta)), P, L.dptr(lin), L.dptr(ws), L.dptr(wc), L.stream_handle()),
            "prepare_grid_kernel")
    asnp = _is_np(x)
    return _ret(lin, asnp), _ret(ws, asnp), _ret(wc, asnp)


def _grid_to_ref(grid_ri, Ngrid, was_complex):
    """(V,3,Nz,Ny,Nx) planar grids -> (Nx,Ny,Nz,3) complex in the reference's axis order."""
    nx, ny, nz = (int(v) for v in Ngrid)
    g = grid_ri.reshape(grid_ri.shape[0], 3, nz, ny, nx).permute(0, 4, 3, 2, 1)
    re = g[0]
    im = g[1] if was_complex else torch.zeros_like(re)
    return torch.complex(re, im)


def _ref_to_grid(H):
    """(Nx,Ny,Nz,3) complex/real array -> (2,3,G) planar real/imag grids on the device."""
    if isinstance(H, torch.Tensor):
        t = H.to("cuda")
    else:
        t = torch.as_tensor(np.asarray(H), device="cuda")
    if not t.is_complex():
        t = t.to(torch.float64).to(torch.complex128)
    t = t.to(torch.complex128).permute(3, 2, 1, 0)  # (3, Nz, Ny, Nx)
    return torch.stack((t.real, t.imag)).reshape(2, 3, -1).contiguous()


def spread_fast(m, Ngrid, linnode, w_spread):
    """Spread with precomputed indices and weights (ewald.py:299-331); (Nx,Ny,Nz,3) complex."""
    lib = L.lib()
    mri, cplx = _ri(m)
    lin = as_device(linnode, torch.int64)
    w = as_device(w_spread)
    n, P3 = lin.shape
    Ng = _host3(Ngrid, np.int64)
    G = int(np.prod(Ng))
    grid = torch.empty((mri.shape[0], 3, G), dtype=torch.float64, device="cuda")
    L.check(lib.mps_spread_fast(L.dptr(mri), n, mri.shape[0], L.host_i64(Ng), L.dptr(lin), L.dptr(w), P3,
                                L.dptr(grid), L.stream_handle()), "spread_fast")
    return _ret(_grid_to_ref(grid, Ng, cplx), _is_np(m, linnode))


def contract_fast(Htilde, Ngrid, linnode, w_contract):
    """Interpolate grid values back to the particles (ewald.py:334-368); (N,3) complex."""
    lib = L.lib()
    g = _ref_to_grid(Htilde)
    lin = as_device(linnode, torch.int64)
    w = as_device(w_contract)
    n, P3 = lin.shape
    out = torch.empty((2, n, 3), dtype=torch.float64, device="cuda")
    L.check(lib.mps_contract_fast(L.dptr(g), n, 2, L.host_i64(_host3(Ngrid, np.int64)), L.dptr(lin), L.dptr(w), P3,
                                  L.dptr(out), L.stream_handle()), "contract_fast")
    return _ret(torch.complex(out[0], out[1]), _is_np(Htilde, linnode))


def spread(x, m, Ngrid, h, xi, eta, P, offset=None, offsetxyz=None):
    """On-the-fly spread (ewald.py:370-418); returns (Hx, Hy, Hz)."""
    lin, w, _ = prepare_grid_kernel(as_device(x), Ngrid, h, xi, eta, P)
    H = spread_fast(m if isinstance(m, torch.Tensor) else torch.as_tensor(np.asarray(m), device="cuda"), Ngrid, lin, w)
    asnp = _is_np(x, m)
    return tuple(_ret(H[..., c], asnp) for c in range(3))


def contract(x, Ngrid, h, xi, eta, P, Htilde, offset=None, offsetxyz=None):
    """On-the-fly contract including the trapezoid factor (ewald.py:421-467)."""
    lin, _, wc = prepare_grid_kernel(as_device(x), Ngrid, h, xi, eta, P)
    Ht = Htilde if isinstance(Htilde, torch.Tensor) else torch.as_tensor(np.asarray(Htilde), device="cuda")
    return _ret(contract_fast(Ht, Ngrid, lin, wc), _is_np(x, Htilde))


# -----------------------------------------------------------------------------
# Reciprocal space (ewald.py:473-599)
# -----------------------------------------------------------------------------
def precompute_kspace(Ngrid, box, xi, eta):
    """khat (complex, zero imaginary part) and the Green's coefficient, fftshift order (ewald.py:523-582)."""
    lib = L.lib()
    Ng = _host3(Ngrid, np.int64)
    nx, ny, nz = (int(v) for v in Ng)
    khat = torch.empty((nx, ny, nz, 3), dtype=torch.float64, device="cuda")
    Hc = torch.empty((nx, ny, nz), dtype=torch.float64, device="cuda")
    L.check(lib.mps_precompute_kspace(L.host_i64(Ng), L.host_f64(_host3(box)), float(xi), L.host_f64(_host3(eta)),
                                      L.dptr(khat), L.dptr(Hc), L.stream_handle()), "precompute_kspace")
    asnp = _is_np(box, eta)
    return _ret(khat.to(torch.complex128), asnp), _ret(Hc, asnp)


def scale_fast(fH, khat, Htildecoeff):
    """f~ = H (khat . f) khat (ewald.py:585-599) on (Nx,Ny,Nz,3) complex arrays."""
    lib = L.lib()
    f = as_device(fH, torch.complex128)
    kh = as_device(khat, torch.complex128).real.contiguous() if (isinstance(khat, torch.Tensor) and khat.is_complex()) \
        or np.iscomplexobj(khat) else as_device(khat)
    Hc = as_device(Htildecoeff)
    out = torch.empty_like(f)
    G = int(Hc.numel())
    L.check(lib.mps_scale_fast(L.dptr(torch.view_as_real(f)), L.dptr(kh), L.dptr(Hc), G,
                               L.dptr(torch.view_as_real(out)), L.stream_handle()), "scale_fast")
    return _ret(out, _is_np(fH, khat, Htildecoeff))


def scale(fH, k, Ngrid, xi, eta):
    """Scale with an explicit k grid (ewald.py:473-516): khat and coefficient from k, then scale_fast."""
    kt = as_device(k)
    k2 = (kt * kt).sum(dim=3)
    nx, ny, nz = (int(v) for v in _host3(Ngrid, np.int64))
    c0 = ((nx - 1) + 1) // 2, ((ny - 1) + 1) // 2, ((nz - 1) + 1) // 2
    den = torch.sqrt(k2)
    den = torch.where(den == 0, torch.ones_like(den), den)
    khat = kt / den[..., None]
    khat[c0[0], c0[1], c0[2], :] = 0.0
    e = torch.as_tensor(_host3(eta), device="cuda")
    etak2 = ((1.0 - e) * kt * kt).sum(dim=3)
    kk = torch.sqrt(k2)
    J = besselj_3_over_2(kk)
    Hc = (9.0 * np.pi) / (2.0 * kk) * (J * J) * torch.exp(-etak2 / (4.0 * float(xi) ** 2)) / k2
    Hc[c0[0], c0[1], c0[2]] = 0.0
    Hc = torch.nan_to_num(Hc, nan=0.0, posinf=0.0, neginf=0.0)
    out = scale_fast(as_device(fH, torch.complex128), khat, Hc)
    out[c0[0], c0[1], c0[2], :] = 0.0
    return _ret(torch.nan_to_num(out), _is_np(fH, k))


# -----------------------------------------------------------------------------
# Real space (ewald.py:604-1139)
# -----------------------------------------------------------------------------
def real_space_table(r, xi):
    """Six coupling tables with the r = 0 self value prepended (ewald.py:604-931)."""
    lib = L.lib()
    rd = as_device(r).reshape(-1)
    n = rd.numel()
    out = torch.empty((6, n + 1), dtype=torch.float64, device="cuda")
    L.check(lib.mps_real_space_table(L.dptr(rd), n, float(xi), L.dptr(out), L.stream_handle()), "real_space_table")
    asnp = _is_np(r)
    return tuple(_ret(out[i].clone(), asnp) for i in range(6))


def prepare_real_space_pairs(x, box, p1, p2, rc, perp, para, rvals):
    """Cutoff-filtered pairs, unit vectors and interpolated couplings (ewald.py:939-1016)."""
    lib = L.lib()
    xd = as_device(x).reshape(-1, 3)
    a = as_device(p1, torch.int64).reshape(-1)
    b = as_device(p2, torch.int64).reshape(-1)
    nc = a.numel()
    asnp = _is_np(x, p1, p2)
    bx = L.host_f64(_host3(box))
    s = L.stream_handle()
    wsb = lib.mps_real_space_pairs_workspace(nc)
    ws = torch.empty(int(wsb), dtype=torch.uint8, device="cuda")
    kept = C.c_int64(0)
    L.check(lib.mps_real_space_pairs_count(L.dptr(xd), xd.shape[0], bx, L.dptr(a), L.dptr(b), nc, float(rc),
                                           L.dptr(ws), wsb, C.byref(kept), s), "prepare_real_space_pairs")
    k = kept.value
    p1f = torch.empty(k, dtype=torch.int64, device="cuda")
    p2f = torch.empty(k, dtype=torch.int64, device="cuda")
    rhat = torch.empty((k, 3), dtype=torch.float64, device="cuda")
    A = torch.empty(k, dtype=torch.float64, device="cuda")
    B = torch.empty(k, dtype=torch.float64, device="cuda")
    if k:
        pe, pa, rv = as_device(perp), as_device(para), as_device(rvals)
        st = lib.mps_real_space_pairs_fill(L.dptr(xd), xd.shape[0], bx, L.dptr(a), L.dptr(b), nc, float(rc),
                                           L.dptr(pe), L.dptr(pa), L.dptr(rv), rv.numel(), L.dptr(ws), wsb,
                                           L.dptr(p1f), L.dptr(p2f), L.dptr(rhat), L.dptr(A), L.dptr(B), s)
        if st == L.MPS_TABLE_RANGE:
            raise ValueError("RealSpace interpolation: pair separations fall outside rvals table. "
                             "Increase r_table max (in RunCapacitance) or adjust xi/errortol.")
        L.check(st, "prepare_real_space_pairs")
    return tuple(_ret(t, asnp) for t in (p1f, p2f, rhat, A, B))


def real_space_fast(m, lambdap, p1, p2, rhat, A, B, self_perp):
    """(diag + self) m + sum over pairs (ewald.py:1019-1072); (N,3) complex."""
    lib = L.lib()
    mri, cplx = _ri(m)
    nv, n = mri.shape[0], mri.shape[1]
    lam = as_device(lambdap).reshape(-1)
    a, b = as_device(p1, torch.int64), as_device(p2, torch.int64)
    rh, Ad, Bd = as_device(rhat), as_device(A), as_device(B)
    out = torch.empty_like(mri)
    L.check(lib.mps_real_space_fast(L.dptr(mri), n, nv, L.dptr(lam), L.dptr(a), L.dptr(b), L.dptr(rh), L.dptr(Ad),
                                    L.dptr(Bd), a.numel(), float(self_perp), L.dptr(out), L.stream_handle()),
            "real_space_fast")
    return _ret(_cplx(out, cplx), _is_np(m, p1))


def real_space(x, m, lambdap, box, p1, p2, rc, perp, para, rvals, real_precomp=None):
    """Pair-loop real-space field (ewald.py:1076-1139): pairs prepared on the GPU, then summed."""
    pre = real_precomp if real_precomp is not None else prepare_real_space_pairs(x, box, p1, p2, rc, perp, para,
                                                                                  rvals)
    sp = float(perp[0])
    out = real_space_fast(m, lambdap, *pre, self_perp=sp)
    return out


# -----------------------------------------------------------------------------
# Matvec (ewald.py:1146-1327)
# -----------------------------------------------------------------------------
_SYS_CACHE: dict = {}


def _fingerprint(a):
    if isinstance(a, torch.Tensor):
        return ("t", a.data_ptr(), tuple(a.shape), float(a.double().sum()))
    a = np.asarray(a)
    return ("n", a.__array_interface__["data"][0], a.shape, float(np.sum(a)) if a.size else 0.0)


def system_for(x, lambdap, box, Ngrid, P, xi, eta, rc, Hperp, Hpara, rvals, slab_factor, max_rhs=2):
    """A cached SpectralEwaldSystem for repeated matvecs on one configuration (on the current device)."""
    key = (_fingerprint(x), _fingerprint(lambdap), tuple(_host3(box)), tuple(_host3(Ngrid, np.int64)), int(P),
           float(xi), tuple(_host3(eta)), float(rc), _fingerprint(Hperp), _fingerprint(rvals), float(slab_factor),
           int(max_rhs), torch.cuda.current_device())
    s = _SYS_CACHE.get(key)
    if s is None:
        _SYS_CACHE.clear()
        s = SpectralEwaldSystem(x, lambdap, box, xi, rc, Ngrid, P, Hperp, Hpara, rvals, slab_factor=slab_factor,
                                eta=_host3(eta), max_rhs=max_rhs)
        _SYS_CACHE[key] = s
    return s


def magnetic_field(x, m, lambdap, box, p1, p2, Ngrid, h, P, xi, eta, rc, offset, offsetxyz, Hperp, Hpara, rvals,
                   real_precomp=None, grid_precomp=None, k_precomp=None, slab_factor=1.0):
    """Field at the particles due to their dipoles (ewald.py:1146-1236).

    Runs the reference's complex pipeline (complex-to-complex FFTs) on the GPU.
    The pair set is the cell-list candidate set of (x, box, rc) filtered at rc,
    i.e. what ``neighbor_list(cell_list(x, box, rc))`` gives the reference; the
    precomputed tuples are accepted for signature compatibility and not needed.
    """
    sysm = system_for(x, lambdap, box, Ngrid, P, xi, eta, rc, Hperp, Hpara, rvals, slab_factor)
    out = sysm.matvec_complex(m)
    return _ret(out, _is_np(x, m))


def magnetic_field_components(x, m, lambdap, box, p1, p2, Ngrid, h, P, xi, eta, rc, offset, offsetxyz, Hperp,
                              Hpara, rvals, real_precomp=None, grid_precomp=None, k_precomp=None, slab_factor=1.0):
    """(Hk, Hr, H_slab) separately (ewald.py:1239-1327)."""
    asnp = _is_np(x, m)
    total = magnetic_field(x, m, lambdap, box, p1, p2, Ngrid, h, P, xi, eta, rc, offset, offsetxyz, Hperp, Hpara,
                           rvals, slab_factor=0.0)
    total = as_device(total, torch.complex128)
    pre = real_precomp if real_precomp is not None else prepare_real_space_pairs(x, box, p1, p2, rc, Hperp, Hpara,
                                                                                  rvals)
    Hr = as_device(real_space_fast(m, lambdap, *[as_device(t, torch.int64 if i < 2 else torch.float64)
                                                 for i, t in enumerate(pre)], float(Hperp[0])), torch.complex128)
    mc = as_device(m, torch.complex128).reshape(-1, 3)
    V = float(np.prod(_host3(box)))
    Hs = torch.zeros_like(mc)
    Hs[:, 2] = -float(slab_factor) * mc[:, 2].sum() / V
    return _ret(total - Hr, asnp), _ret(Hr, asnp), _ret(Hs, asnp)
