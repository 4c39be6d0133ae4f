"""ctypes binding of ``libmps_gb300.so`` (the C ABI declared in ``include/mps_gb300.h``).

There is no CPU fallback: every entry point needs the CUDA library and a CUDA
device, and fails loudly (``RuntimeError``) when either is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmps_gb300.so")

MPS_OK, MPS_BAD_ARG, MPS_RC_GT_HALF_BOX, MPS_TABLE_RANGE, MPS_NOT_CONVERGED, MPS_CUDA_ERR, MPS_CUFFT_ERR, \
    MPS_NO_MEMORY, MPS_SCRATCH_LIMIT = range(9)
NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024
MPS_FP64, MPS_FP32, MPS_DF, MPS_FP32_GRAD = 0, 1, 2, 3
MPS_DIPOLE, MPS_DIPOLE_QUADRUPOLE, MPS_POLYDISPERSE = 0, 1, 2

EXPORTS = (
    "mps_status_string", "mps_abi_version", "mps_real_space_table", "mps_cell_list",
    "mps_neighbor_list_workspace", "mps_neighbor_list_count", "mps_neighbor_list_fill",
    "mps_real_space_pairs_workspace", "mps_real_space_pairs_count", "mps_real_space_pairs_fill",
    "mps_real_space_fast", "mps_pre_calculations", "mps_grid_kernel", "mps_spread_fast", "mps_contract_fast",
    "mps_precompute_kspace", "mps_scale_fast", "mps_system_create", "mps_system_destroy", "mps_system_info",
    "mps_matvec", "mps_matvec_complex", "mps_gmres", "mps_kernel_launches", "mps_system_profile",
    "mps_system_stage_times", "mps_neighbor_list_noalloc", "mps_system_tuning", "mps_system_graphs",
    "mps_dipole_forces", "mps_quad_table", "mps_sizes_table", "mps_adjoint_forces",
    "mps_real_space_table_probe", "mps_field_map", "mps_quad_table_probe", "mps_field_map_quad",
    "mps_field_map_sizes", "mps_kspace_cache_clear", "mps_solve_batched",
)

p = C.c_void_p
i64 = C.c_int64
i32 = C.c_int32
f64 = C.c_double
sz = C.c_size_t
P64 = C.POINTER(C.c_int64)
PD = C.POINTER(C.c_double)


class SystemDesc(C.Structure):
    _fields_ = [
        ("n", i64), ("x", p), ("lambdap", p), ("n_diag", i64), ("box", f64 * 3), ("xi", f64), ("rc", f64),
        ("Ngrid", i64 * 3), ("P", i32), ("eta", f64 * 3), ("perp", p), ("para", p), ("rvals", p),
        ("n_tab", i64), ("slab_factor", f64), ("max_rhs", i32), ("kind", i32), ("quad_tables", p),
        ("radius", p), ("radius_class", p), ("n_class", i32), ("sizes_tables", p), ("lambdap_imag", p),
        ("inner_Ngrid", i64 * 3), ("inner_P", i32),
    ]


class SolveOpts(C.Structure):
    _fields_ = [("tol", f64), ("restart", i32), ("maxit", i32), ("precision", i32), ("inner_tol", f64),
                ("inner_maxit", i32), ("residual_policy", i32), ("verify", i32), ("residual_precision", i32),
                ("inner_operator", i32)]


class SolveInfo(C.Structure):
    _fields_ = [("converged", i32), ("matvecs_fp64", i32), ("matvecs_fp32", i32), ("cycles", i32),
                ("relres", f64)]


class BatchItem(C.Structure):
    _fields_ = [("desc", SystemDesc), ("b", p), ("x0", p), ("x", p), ("nrhs", i32), ("diag_index", C.POINTER(i32)),
                ("info", C.POINTER(SolveInfo)), ("status", i32)]


_SIGS = {
    "mps_status_string": (C.c_char_p, [C.c_int]),
    "mps_abi_version": (C.c_int, []),
    "mps_real_space_table": (C.c_int, [p, i64, f64, p, p]),
    "mps_cell_list": (C.c_int, [p, i64, PD, f64, p, P64, p]),
    "mps_neighbor_list_workspace": (sz, [i64, P64]),
    "mps_neighbor_list_count": (C.c_int, [p, i64, P64, p, sz, P64, p]),
    "mps_neighbor_list_fill": (C.c_int, [p, i64, P64, p, sz, p, p, p]),
    "mps_real_space_pairs_workspace": (sz, [i64]),
    "mps_real_space_pairs_count": (C.c_int, [p, i64, PD, p, p, i64, f64, p, sz, P64, p]),
    "mps_real_space_pairs_fill": (C.c_int, [p, i64, PD, p, p, i64, f64, p, p, p, i64, p, sz, p, p, p, p, p, p]),
    "mps_real_space_fast": (C.c_int, [p, i64, i64, p, p, p, p, p, p, i64, f64, p, p]),
    "mps_pre_calculations": (C.c_int, [C.c_int, PD, p, p, p]),
    "mps_grid_kernel": (C.c_int, [p, i64, P64, PD, f64, PD, C.c_int, p, p, p, p]),
    "mps_spread_fast": (C.c_int, [p, i64, i64, P64, p, p, i64, p, p]),
    "mps_contract_fast": (C.c_int, [p, i64, i64, P64, p, p, i64, p, p]),
    "mps_precompute_kspace": (C.c_int, [P64, PD, f64, PD, p, p, p]),
    "mps_scale_fast": (C.c_int, [p, p, p, i64, p, p]),
    "mps_system_create": (C.c_int, [C.POINTER(SystemDesc), C.POINTER(p), p]),
    "mps_system_destroy": (None, [p]),
    "mps_system_info": (C.c_int, [p, P64, P64]),
    "mps_matvec": (C.c_int, [p, p, p, i32, C.POINTER(i32), i32, p]),
    "mps_matvec_complex": (C.c_int, [p, p, p, i32, p]),
    "mps_gmres": (C.c_int, [p, p, p, p, i32, C.POINTER(i32), C.POINTER(SolveOpts), C.POINTER(SolveInfo), p]),
    "mps_solve_batched": (C.c_int, [C.POINTER(BatchItem), i32, C.POINTER(SolveOpts), i32, p]),
    "mps_kernel_launches": (C.c_uint64, []),
    "mps_system_profile": (C.c_int, [p, i32]),
    "mps_system_stage_times": (C.c_int, [p, PD, P64]),
    "mps_neighbor_list_noalloc": (C.c_int, [p, i64, P64, p, p, i64, P64, p]),
    "mps_system_tuning": (C.c_int, [p, C.POINTER(i32), C.POINTER(C.c_float)]),
    "mps_system_graphs": (C.c_int, [p, C.POINTER(i32), C.POINTER(i32)]),
    "mps_kspace_cache_clear": (C.c_int, []),
    "mps_dipole_forces": (C.c_int, [p, p, i64, PD, f64, f64, i32, p, p, p]),
    "mps_quad_table": (C.c_int, [p, i64, f64, p, p]),
    "mps_sizes_table": (C.c_int, [p, i64, p, i64, f64, p, p, p]),
    "mps_adjoint_forces": (C.c_int, [p, p, p, p, p, i64, i32, p, p, p]),
    "mps_real_space_table_probe": (C.c_int, [p, i64, f64, p, p]),
    "mps_field_map": (C.c_int, [p, i64, p, p, i64, PD, f64, f64, P64, i32, PD, p, p, p, i64, i32, p, p]),
    "mps_quad_table_probe": (C.c_int, [p, i64, f64, p, p]),
    "mps_field_map_quad": (C.c_int, [p, i64, p, p, i64, PD, f64, f64, P64, i32, PD, p, p, i64, i32, p, p]),
    "mps_field_map_sizes": (C.c_int, [p, i64, p, p, p, i32, p, i64, PD, f64, f64, P64, i32, f64, p, p, p, i64, i32,
                                      p, p]),
}

_lib = None
_lock = threading.Lock()


class MpsError(RuntimeError):
    """A CUDA-side failure reported through the C ABI."""


class NotConvergedError(RuntimeError):
    """GMRES reached its iteration cap (status MPS_NOT_CONVERGED)."""


def load_library(path: str = LIB_PATH):
    """Load the shared library (no device needed): used by the CPU-side ABI tests."""
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def lib():
    """The loaded library; builds it first if it is missing, requires CUDA."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            import torch
            if not torch.cuda.is_available():
                raise RuntimeError("mutual_polarization_slab_gb300 needs a CUDA device (no CPU fallback)")
            if not os.path.exists(LIB_PATH):
                from . import _build
                _build.build()
            torch.cuda.init()
            _lib = load_library(LIB_PATH)
    return _lib


def check(status: int, what: str = "") -> None:
    if status == MPS_OK:
        return
    msg = _lib.mps_status_string(status).decode() if _lib is not None else str(status)
    if what:
        msg = f"{what}: {msg}"
    if status in (MPS_BAD_ARG, MPS_RC_GT_HALF_BOX, MPS_TABLE_RANGE):
        raise ValueError(msg)
    if status == MPS_NOT_CONVERGED:
        raise NotConvergedError(msg)
    raise MpsError(msg)


def stream_handle():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def dptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else C.c_void_p(0)


def host_f64(vals):
    arr = (C.c_double * len(vals))(*[float(v) for v in vals])
    return arr


def host_i64(vals):
    return (C.c_int64 * len(vals))(*[int(v) for v in vals])
