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
    assert lib.mps_abi_version() == 5
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


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the ABI's structs have the C compiler's sizes and
    field offsets (compiled from include/mps_gb300.h on this host)."""
    import ctypes as C
    import shutil
    import subprocess

    from mutual_polarization_slab_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"mps_system_desc": _lib.SystemDesc, "mps_solve_opts": _lib.SolveOpts,
               "mps_solve_info": _lib.SolveInfo, "mps_batch_item": _lib.BatchItem}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mps_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    want = []
    for cname, py in structs.items():
        want.append(f"{cname} size {C.sizeof(py)}")
        want += [f"{cname} {fname} {getattr(py, fname).offset}" for fname, _ in py._fields_]
    assert [g for g in got if g] == want


def test_solve_batched_rejects_bad_arguments_on_the_host():
    """Argument errors, invalid solver options included, return MPS_BAD_ARG
    before any CUDA call (no device here), and an empty batch is MPS_OK."""
    from mutual_polarization_slab_gb300 import _build, _lib
    if _build.is_stale():
        pytest.skip("library not built")
    import ctypes as C
    lib = _lib.load_library()
    opts = _lib.SolveOpts(tol=1e-8, restart=30, maxit=10)
    items = (_lib.BatchItem * 1)()
    null = C.c_void_p(0)
    assert lib.mps_solve_batched(items, -1, C.byref(opts), 1, null) == _lib.MPS_BAD_ARG
    assert lib.mps_solve_batched(items, 1, None, 1, null) == _lib.MPS_BAD_ARG
    assert lib.mps_solve_batched(items, 1, C.byref(opts), 0, null) == _lib.MPS_BAD_ARG
    assert lib.mps_solve_batched(None, 1, C.byref(opts), 1, null) == _lib.MPS_BAD_ARG
    assert lib.mps_solve_batched(items, 0, C.byref(opts), 4, null) == _lib.MPS_OK
    for bad in (dict(restart=0), dict(maxit=0), dict(tol=0.0), dict(precision=7), dict(residual_precision=1),
                dict(inner_operator=2)):
        o = _lib.SolveOpts(tol=1e-8, restart=30, maxit=10)
        for k, v in bad.items():
            setattr(o, k, v)
        assert lib.mps_solve_batched(items, 1, C.byref(o), 1, null) == _lib.MPS_BAD_ARG, bad


def _c_kind(param):
    """('ptr', 8) / ('float', size) / ('int', size) of one C parameter of the header."""
    import ctypes as C
    if "*" in param or "mps_stream_t" in param:
        return ("ptr", C.sizeof(C.c_void_p))
    words = param.replace("const", " ").split()
    t = words[0]
    if t in ("double", "float"):
        return ("float", 8 if t == "double" else 4)
    return ("int", {"int64_t": 8, "uint64_t": 8, "size_t": C.sizeof(C.c_size_t), "int32_t": 4, "int": 4}[t])


def _py_kind(t):
    import ctypes as C
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return ("ptr", C.sizeof(C.c_void_p))
    if t in (C.c_double, C.c_float):
        return ("float", C.sizeof(t))
    return ("int", C.sizeof(t))


def test_ctypes_signatures_match_the_header():
    """Every prototype of include/mps_gb300.h has a ctypes signature of the same
    arity, argument kinds and widths, and return type (no library needed)."""
    import ctypes as C

    from mutual_polarization_slab_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "mps_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    decls = re.findall(r"\b(int|void|size_t|uint64_t|const char \*)\s*(mps_[a-z0-9_]+)\s*\(([^;]*?)\)\s*;", src,
                       flags=re.S)
    assert sorted(name for _, name, _ in decls) == sorted(_lib._SIGS)
    ret = {"int": C.c_int, "void": None, "size_t": C.c_size_t, "uint64_t": C.c_uint64, "const char *": C.c_char_p}
    for rt, name, args in decls:
        restype, argtypes = _lib._SIGS[name]
        assert restype is ret[rt], name
        params = [] if args.strip() in ("", "void") else [a.strip() for a in args.split(",")]
        assert [_c_kind(a) for a in params] == [_py_kind(t) for t in argtypes], name
