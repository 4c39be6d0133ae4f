"""Device-resident spectral-Ewald system: the GPU form of the reference's
``real_precomp`` / ``grid_precomp`` / ``k_precomp`` tuples
(``CPU - Ewald test/capacitance.py:369-385``) plus FFT plans and grids.

One object per particle configuration.  It owns device memory through the C ABI
(``mps_system_create``) and frees it on ``close()`` / garbage collection.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L

PRECISIONS = {"fp64": L.MPS_FP64, "fp32": L.MPS_FP32, "mixed": L.MPS_FP32, "df": L.MPS_DF,
              "fp32grad": L.MPS_FP32_GRAD}


_NP_TYPES = {torch.float64: np.dtype(np.float64), torch.float32: np.dtype(np.float32),
             torch.complex128: np.dtype(np.complex128), torch.int32: np.dtype(np.int32),
             torch.int64: np.dtype(np.int64)}


def as_device(a, dtype=torch.float64, non_blocking=False) -> torch.Tensor:
    """Contiguous CUDA tensor view/copy of a numpy array or tensor.  With
    ``non_blocking`` a contiguous numpy array of the target type in page-locked
    memory is copied without blocking the host, in the order of the current
    stream: only for callers that synchronise that stream before they return
    (system creation, solves), so the caller's array cannot change under the copy."""
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=dtype).contiguous()
    arr = np.asarray(a)
    if non_blocking and arr.flags.c_contiguous and arr.flags.writeable and arr.dtype == _NP_TYPES.get(dtype):
        t = torch.from_numpy(arr)
        if t.is_pinned():
            return t.to(device="cuda", non_blocking=True)
    return torch.as_tensor(np.ascontiguousarray(arr), dtype=dtype, device="cuda")


def to_host(t: torch.Tensor) -> np.ndarray:
    """NumPy copy of a device tensor in page-locked host memory (torch's caching
    host allocator: the block returns to its cache when the array is dropped), so
    the device-to-host copy runs at the link's DMA rate instead of through a
    pageable staging buffer."""
    if t.is_cuda:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        return h.numpy()
    return t.numpy()


def clear_kspace_cache():
    """Drop the process's cached Green's coefficients and scale tensors (shared by
    systems built on the same device, grid, box, xi and eta), so the next system
    recomputes its k-space data as the reference does on every ``capacitance()``
    call (``CPU - Ewald test/capacitance.py:385``).  Existing systems keep theirs."""
    L.check(L.lib().mps_kspace_cache_clear())


@dataclass
class SolveInfo:
    converged: bool
    relres: float
    matvecs_fp64: int
    matvecs_fp32: int
    cycles: int


def spectral_parameters(box, xi, errortol):
    """rc, Ngrid, h, P, eta derived from one tolerance (``capacitance.py:357-362``)."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(errortol))
    rc = lt / xi
    kcut = 2.0 * xi * lt
    Ngrid = np.ceil(1.0 + box * kcut / math.pi).astype(np.int64)
    h = box / Ngrid
    P = int(math.ceil(-2.0 * math.log(errortol) / math.pi))
    eta = P * (h * xi) ** 2 / math.pi
    return rc, Ngrid, h, P, eta


# cuFFT runs sizes 2^a 3^b 5^c fastest; the inner grid takes the smallest of these with b + c <= 2 (128, 144,
# 160, 192, 200, ...) at or above the tolerance rule's size
def _fast_size(n: int) -> int:
    m = max(int(n), 1)
    while True:
        k = m
        b = c = 0
        while k % 2 == 0:
            k //= 2
        while k % 3 == 0:
            k //= 3
            b += 1
        while k % 5 == 0:
            k //= 5
            c += 1
        if k == 1 and b + c <= 2:
            return m
        m += 1


def inner_grid(box, xi, Ngrid, P, tol=2.5e-4):
    """Coarser grid for the float32 gradient-form inner operator of the mixed
    solve: the tolerance rule's grid at ``tol`` rounded up to a fast FFT size,
    with the system's own support ``P`` (the gradient form's error grows fast as
    P shrinks); None for grids below 128^3 (the FFTs are then a small share of a
    matvec) or when the inner grid would not be clearly smaller than ``Ngrid``.
    Measured at N = 1e5 (192^3 -> 144^3) and N = 2e5 (240^3 -> 192^3): 3e-5..6e-5
    from the reference operator, the same refinement steps and matvec counts, and
    10-12 % less time per solve.  A grid at 1e-3 (about 1e-4 from the reference)
    made the refinement take a second float64-accurate residual and lost time."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
    if np.prod(Ngrid) < 128 ** 3:
        return None
    lt = math.sqrt(-math.log(tol))
    ng = np.array([_fast_size(math.ceil(1.0 + L * 2.0 * xi * lt / math.pi)) for L in box], dtype=np.int64)
    ng = np.maximum(ng, max(16, int(P)))
    if np.prod(ng) >= 0.8 * np.prod(Ngrid) or np.any(ng > Ngrid):
        return None
    return ng, int(P)


def fft_size(n: int) -> int:
    """Smallest m >= n whose prime factors are 2, 3 and 5 (radices cuFFT runs
    fast; few such sizes, so many configurations share their plans)."""
    m = max(int(n), 1)
    while True:
        k = m
        for p in (2, 3, 5):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


class SpectralEwaldSystem:
    """Precomputed geometry of one configuration and its batched operator.

    Parameters mirror ``magnetic_field`` (``ewald.py:1146-1168``): positions
    ``x (N,3)``, permittivities ``lambdap`` (``(N,)`` or ``(n_sets, N)`` for a
    contrast spectrum), ``box``, ``xi``, cutoff ``rc``, grid ``Ngrid``, support
    ``P``, tables ``perp``/``para`` on separations ``rvals`` (``rvals[0] = 0``,
    self value in ``perp[0]``), ``slab_factor``.

    With ``quad_tables`` (a (7, n_tab) array: field_quad_1..3, grad_quad_1..4 on
    ``rvals``) the object is the dipole + quadrupole operator of
    ``Capacitance_Quadrupole/MatrixVectorMultiply.m``: 8 unknowns per sphere,
    stored per particle as (Sx, Sy, Sz, Qxx, Qxy, Qxz, Qyy, Qyz); it has no slab term.

    ``inner`` sets the discretisation of the float32 gradient-form operator
    (the mixed solve's inner operator, dipole systems): None uses the system's
    grid, ``(Ngrid_in, P_in)`` a grid of its own, ``"auto"`` the coarser grid of
    ``inner_grid`` when there is one.

    With ``radius`` (N radii) it is the polydisperse operator of
    ``Capacitance_Sizes/ComputeField.m`` (scalar eta, no slab term; ``perp``,
    ``para`` unused).  ``sizes_tables`` ((2, M(M+1)/2, n_tab) on ``rvals``) with
    ``radius_class`` (class of each particle among ``n_class`` distinct radii)
    interpolates the couplings like ``CS/RealSpace.m``; without them every pair's
    couplings are evaluated in closed form at its separation.

    ``create=False`` checks the arguments and prepares the device arrays and the
    C descriptor (``desc``) without building the system: the many-configuration
    solve (``mps_solve_batched``) builds and releases it itself.
    """

    def __init__(self, x, lambdap, box, xi, rc, Ngrid, P, perp, para, rvals, slab_factor=1.0, eta=None,
                 max_rhs=3, quad_tables=None, radius=None, radius_class=None, n_class=0, sizes_tables=None,
                 inner=None, *, create=True):
        lib = L.lib()
        self._lib = lib
        self._h = C.c_void_p(0)
        self.x = as_device(x, non_blocking=True).reshape(-1, 3)
        # complex permittivities (frequency-dependent eps, as the MATLAB spectrum drivers allow): vectors become
        # complex; the device stores them as (Re m, Im m) per particle
        self.cplx = bool(torch.is_complex(lambdap)) if isinstance(lambdap, torch.Tensor) else \
            bool(np.iscomplexobj(lambdap))
        if self.cplx:
            lc = lambdap.to(device="cuda", dtype=torch.complex128) if isinstance(lambdap, torch.Tensor) else \
                torch.as_tensor(np.asarray(lambdap, dtype=np.complex128), device="cuda")
            if lc.dim() == 1:
                lc = lc.reshape(1, -1)
            lam = lc.real.contiguous()
            self.lambdap_imag = lc.imag.contiguous()
        else:
            lam = as_device(lambdap, non_blocking=True)
            if lam.dim() == 1:
                lam = lam.reshape(1, -1)
            self.lambdap_imag = None
        self.lambdap = lam.contiguous()
        self.n = int(self.x.shape[0])
        if self.lambdap.shape[1] != self.n:
            raise ValueError("lambdap must have N entries per permittivity set")
        self.box = np.asarray(box, dtype=np.float64).reshape(3)
        self.xi = float(xi)
        self.rc = float(rc)
        self.Ngrid = np.asarray(Ngrid, dtype=np.int64).reshape(3)
        self.P = int(P)
        self.slab_factor = float(slab_factor)
        self.max_rhs = int(max_rhs)
        self.perp = None if perp is None else as_device(perp)
        self.para = None if para is None else as_device(para)
        self.rvals = None if rvals is None else as_device(rvals)
        self.kind = L.MPS_DIPOLE if quad_tables is None else L.MPS_DIPOLE_QUADRUPOLE
        if radius is not None:
            if quad_tables is not None:
                raise ValueError("radius and quad_tables select different operators")
            self.kind = L.MPS_POLYDISPERSE
        self.ndof = 3 if quad_tables is None else 8
        self.radius = None if radius is None else as_device(radius).reshape(-1).contiguous()
        self.radius_class = None if radius_class is None else as_device(radius_class, torch.int32).reshape(-1)
        self.sizes_tables = None if sizes_tables is None else as_device(sizes_tables).contiguous()
        if self.kind == L.MPS_POLYDISPERSE:
            if self.radius.numel() != self.x.shape[0]:
                raise ValueError("radius must have N entries")
            if self.slab_factor != 0.0:
                raise ValueError("the polydisperse operator has no slab term (slab_factor must be 0)")
            if (self.radius_class is None) != (self.sizes_tables is None):
                raise ValueError("radius_class and sizes_tables go together")
            if self.sizes_tables is not None and self.sizes_tables.shape[-1] != self.rvals.numel():
                raise ValueError("sizes_tables must have n_tab entries per column")
        self.quad_tables = None
        if quad_tables is not None:
            self.quad_tables = as_device(quad_tables).reshape(7, -1).contiguous()
            if self.quad_tables.shape[1] != self.rvals.numel():
                raise ValueError("quad_tables must have one row of n_tab entries per coupling")
            if self.slab_factor != 0.0:
                raise ValueError("the dipole + quadrupole operator has no slab term (slab_factor must be 0)")
        if np.any(self.rc > self.box / 2.0):
            raise ValueError("Real-space cutoff exceeds half the box size; tolerance unmet.")
        d = L.SystemDesc()
        d.n = self.n
        d.x = self.x.data_ptr()
        d.lambdap = self.lambdap.data_ptr()
        d.n_diag = int(self.lambdap.shape[0])
        d.box = (C.c_double * 3)(*self.box)
        d.xi = self.xi
        d.rc = self.rc
        d.Ngrid = (C.c_int64 * 3)(*self.Ngrid)
        d.P = self.P
        eta = np.zeros(3) if eta is None else np.asarray(eta, dtype=np.float64).reshape(3)
        d.eta = (C.c_double * 3)(*eta)
        d.perp = self.perp.data_ptr() if self.perp is not None else None
        d.para = self.para.data_ptr() if self.para is not None else None
        d.rvals = self.rvals.data_ptr() if self.rvals is not None else None
        d.n_tab = int(self.rvals.numel()) if self.rvals is not None else 0
        d.slab_factor = self.slab_factor
        d.max_rhs = self.max_rhs
        d.kind = self.kind
        d.quad_tables = self.quad_tables.data_ptr() if self.quad_tables is not None else None
        d.radius = self.radius.data_ptr() if self.radius is not None else None
        d.radius_class = self.radius_class.data_ptr() if self.radius_class is not None else None
        d.n_class = int(n_class)
        d.sizes_tables = self.sizes_tables.data_ptr() if self.sizes_tables is not None else None
        d.lambdap_imag = self.lambdap_imag.data_ptr() if self.lambdap_imag is not None else None
        if isinstance(inner, str) and inner == "auto":
            inner = inner_grid(self.box, self.xi, self.Ngrid, self.P) if self.kind == L.MPS_DIPOLE else None
        self.inner = None
        if inner is not None:
            if self.kind != L.MPS_DIPOLE:
                raise ValueError("an inner grid is available for the dipole operator")
            ng_in, p_in = inner
            self.inner = (np.asarray(ng_in, dtype=np.int64).reshape(3), int(p_in))
            d.inner_Ngrid = (C.c_int64 * 3)(*self.inner[0])
            d.inner_P = self.inner[1]
        if self.cplx and self.kind != L.MPS_DIPOLE:
            raise ValueError("complex permittivities are supported for the dipole operator")
        self.desc = d
        if not create:
            # the validated descriptor and the device arrays it points to, for mps_solve_batched, which builds
            # and releases the system itself
            self.n_pairs, self.ncell = None, None
            return
        L.check(lib.mps_system_create(C.byref(d), C.byref(self._h), L.stream_handle()), "mps_system_create")
        np_ = C.c_int64(0)
        nc = (C.c_int64 * 3)()
        L.check(lib.mps_system_info(self._h, C.byref(np_), nc))
        self.n_pairs = int(np_.value)
        self.ncell = np.array(list(nc), dtype=np.int64)

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if self._h and self._h.value:
            self._lib.mps_system_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- diagnostics --------------------------------------------------------
    STAGES = ("slab", "spread", "fft_fwd", "scale", "fft_inv", "contract", "real_space")

    def profile(self, enable=True):
        """Record CUDA events around every matvec stage from now on."""
        L.check(self._lib.mps_system_profile(self._h, 1 if enable else 0))

    def stage_times(self):
        """{precision: (matvec count, {stage: total ms})} since the last call."""
        ms = (C.c_double * 21)()
        cnt = (C.c_int64 * 3)()
        L.check(self._lib.mps_system_stage_times(self._h, ms, cnt))
        out = {}
        for p, name in ((0, "fp64"), (1, "fp32"), (2, "df")):
            out[name] = (int(cnt[p]), {s: float(ms[p * 7 + k]) for k, s in enumerate(self.STAGES)})
        return out

    def tuning(self):
        """Autotuned tile depth per precision and the timings it was chosen from (ms)."""
        tz = (C.c_int32 * 2)()
        ms = (C.c_float * 4)()
        L.check(self._lib.mps_system_tuning(self._h, tz, ms))
        return {"fp64": {"tile": [16, 16, int(tz[0])], "ms_depth4": ms[0], "ms_depth8": ms[1]},
                "fp32": {"tile": [16, 16, int(tz[1])], "ms_depth4": ms[2], "ms_depth8": ms[3]}}

    def graphs(self):
        """GMRES step graphs of this system: (instantiated, refused by the runtime).
        The solves run each cycle's Arnoldi steps as one CUDA graph launch once a
        matvec of that precision and batch width has run; MPS_GMRES_GRAPH=0 in the
        environment keeps the host-driven steps."""
        built, failed = C.c_int32(0), C.c_int32(0)
        L.check(self._lib.mps_system_graphs(self._h, C.byref(built), C.byref(failed)))
        return int(built.value), int(failed.value)

    # -- operator ---------------------------------------------------------
    def _diag_arg(self, nrhs, diag_index):
        if diag_index is None:
            return None
        arr = (C.c_int32 * nrhs)(*[int(v) for v in diag_index])
        return arr

    # complex vectors (complex permittivities) <-> the device's (Re m, Im m) per particle
    def _pack(self, v):
        vc = v.to(device="cuda", dtype=torch.complex128) if isinstance(v, torch.Tensor) else \
            torch.as_tensor(np.asarray(v, dtype=np.complex128), device="cuda")
        return torch.cat((vc.real, vc.imag), dim=-1).contiguous()

    @staticmethod
    def _unpack(v6):
        return torch.complex(v6[..., :3].contiguous(), v6[..., 3:].contiguous())

    def matvec(self, m, precision="fp64", diag_index=None, out=None) -> torch.Tensor:
        """Field at the particles from real moments ``m`` of shape (N,ndof) or (R,N,ndof)
        (ndof = 3, or 8 for the dipole + quadrupole operator).  With complex
        permittivities ``m`` and the result are complex (N,3) / (R,N,3)."""
        if self.cplx:
            m6 = self._pack(m)
            single = m6.dim() == 2
            m6 = m6.reshape(-1, self.n, 6).contiguous()
            o6 = torch.empty_like(m6)
            L.check(self._lib.mps_matvec(self._h, L.dptr(m6), L.dptr(o6), m6.shape[0],
                                         self._diag_arg(m6.shape[0], diag_index), PRECISIONS[precision],
                                         L.stream_handle()), "mps_matvec")
            r = self._unpack(o6)
            return r[0] if single else r
        m = as_device(m)
        single = m.dim() == 2
        m = m.reshape(-1, self.n, self.ndof).contiguous()
        nrhs = m.shape[0]
        if out is None:
            out = torch.empty_like(m)
        L.check(self._lib.mps_matvec(self._h, L.dptr(m), L.dptr(out), nrhs, self._diag_arg(nrhs, diag_index),
                                     PRECISIONS[precision], L.stream_handle()), "mps_matvec")
        return out[0] if single else out

    def matvec_complex(self, m, diag_index=0) -> torch.Tensor:
        """The reference's complex pipeline on one complex (N,3) vector; returns complex128."""
        if isinstance(m, torch.Tensor):
            mc = m.to(device="cuda", dtype=torch.complex128)
        else:
            mc = torch.as_tensor(np.asarray(m, dtype=np.complex128), device="cuda")
        ri = torch.stack((mc.real, mc.imag)).contiguous()
        out = torch.empty_like(ri)
        L.check(self._lib.mps_matvec_complex(self._h, L.dptr(ri), L.dptr(out), int(diag_index), L.stream_handle()),
                "mps_matvec_complex")
        return torch.complex(out[0], out[1])

    def solve(self, b, x0=None, tol=1e-8, restart=30, maxit=100, precision="fp64", inner_tol=1e-4,
              inner_maxit=4, diag_index=None, raise_on_fail=False, residual_policy=0, verify=False,
              residual_precision="df", inner_operator="grad"):
        """GMRES (``precision='fp64'``, or ``'df'`` for the float64 operator with
        double-float FFTs) or float64 iterative refinement around a float32-operator
        GMRES (``'mixed'``) for R right-hand sides at once.  The refinement
        residuals use ``residual_precision`` ('df': double-float FFTs, the default;
        'fp64': cuFFT float64); operators without a double-float path use float64.
        ``inner_operator='grad'`` runs the inner GMRES on the gradient form of the
        float32 operator (one FFT pair per vector; it differs from the reference
        operator by ~1e-5, which the refinement removes).

        ``b``, ``x0``: (N,ndof) or (R,N,ndof); complex (N,3) / (R,N,3) with complex
        permittivities.  Returns (x, [SolveInfo] * R)."""
        nd = 6 if self.cplx else self.ndof
        b = self._pack(b) if self.cplx else as_device(b, non_blocking=True)
        single = b.dim() == 2
        b = b.reshape(-1, self.n, nd).contiguous()
        nrhs = b.shape[0]
        x = torch.empty_like(b)
        if x0 is None:
            x0d = None
        else:
            x0d = (self._pack(x0) if self.cplx else as_device(x0, non_blocking=True)).reshape(nrhs, self.n,
                                                                                             nd).contiguous()
        opts = L.SolveOpts(tol=float(tol), restart=int(restart), maxit=int(maxit),
                           precision=PRECISIONS[precision], inner_tol=float(inner_tol), inner_maxit=int(inner_maxit),
                           residual_policy=int(residual_policy), verify=1 if verify else 0,
                           residual_precision=PRECISIONS[residual_precision],
                           inner_operator={"reference": 0, "grad": 1}[inner_operator])
        info = (L.SolveInfo * nrhs)()
        st = self._lib.mps_gmres(self._h, L.dptr(b), L.dptr(x0d) if x0d is not None else C.c_void_p(0), L.dptr(x),
                                 nrhs, self._diag_arg(nrhs, diag_index), C.byref(opts), info, L.stream_handle())
        if st != L.MPS_NOT_CONVERGED or raise_on_fail:
            L.check(st, "mps_gmres")
        infos = [SolveInfo(bool(i.converged), float(i.relres), int(i.matvecs_fp64), int(i.matvecs_fp32),
                           int(i.cycles)) for i in info]
        if self.cplx:
            x = self._unpack(x)
        return (x[0] if single else x), infos
