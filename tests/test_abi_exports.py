"""The C-ABI library builds, loads without a GPU, and exports every entry point
declared in include/mps_gb300.h (no compute calls here)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "mps_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mps_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from mutual_polarization_slab_gb300 import _build, _lib
    if _build.is_stale():
        try:
            _build.build()
        except RuntimeError as e:  # no nvcc in this environment
            pytest.skip(str(e))
    lib = _lib.load_library()
    missing = [name for name in _declared() if not hasattr(lib, name)]
    assert not missing, f"not exported: {missing}"
    assert set(_declared()) == set(_lib.EXPORTS) | set(n for n in _declared() if n in _lib.EXPORTS)
    assert lib.mps_abi_version() == 4
    assert lib.mps_status_string(3).decode().startswith("pair separation")


def test_workspace_queries_are_host_only():
    from mutual_polarization_slab_gb300 import _build, _lib
    if _build.is_stale():
        pytest.skip("library not built")
    import ctypes as C
    lib = _lib.load_library()
    nc = (C.c_int64 * 3)(3, 3, 3)
    assert lib.mps_neighbor_list_workspace(1000, nc) > 27 * 1000 * 8
    assert lib.mps_real_space_pairs_workspace(10) > 10 * 12


def test_neighbor_list_sizes_that_overflow_are_rejected_on_the_host():
    """Cell counts whose product wraps int64 (or exceeds the kernels' int32 cell
    index) make the workspace query return SIZE_MAX and the allocation-free entry
    point return MPS_BAD_ARG before any CUDA call (null device pointers are safe)."""
    from mutual_polarization_slab_gb300 import _build, _lib
    if _build.is_stale():
        pytest.skip("library not built")
    import ctypes as C
    lib = _lib.load_library()
    size_max = (1 << (8 * C.sizeof(C.c_size_t))) - 1
    for nc in [(1 << 22, 1 << 22, 1 << 22), (1 << 40, 1 << 40, 4), (1 << 31, 1, 1), (70000, 70000, 1)]:
        ncell = (C.c_int64 * 3)(*nc)
        assert lib.mps_neighbor_list_workspace(100, ncell) == size_max
        npairs = C.c_int64(-1)
        st = lib.mps_neighbor_list_noalloc(C.c_void_p(0), 100, ncell, C.c_void_p(0), C.c_void_p(0), 0,
                                           C.byref(npairs), C.c_void_p(0))
        assert st == _lib.MPS_BAD_ARG and npairs.value == 0
    ok = (C.c_int64 * 3)(19, 19, 19)
    assert lib.mps_neighbor_list_workspace(1000, ok) < size_max
