"""The allocation-free neighbour-list entry point (mps_neighbor_list_noalloc).

It exists for callers that may not allocate device memory while they run (a
simulation engine that owns all device memory and calls plugins every step;
cudaMalloc would synchronise the device and can fail mid-run).  Its scratch is a
fixed 16 MiB device array inside the library, shared by every call.  These tests
call it through the C ABI twice in a row, on two different configurations, and
compare each result with the workspace-based entry points
(mps_neighbor_list_count / _fill): the pair lists are integers, so they must be
identical.  The file is named to run last so that a failure here does not stop
the other GPU tests of an ``-x`` run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import _lib as L  # noqa: E402
from mutual_polarization_slab_gb300 import ewald as gew  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402


def _noalloc(cell, ncell, max_pairs):
    lib = L.lib()
    n = cell.shape[0]
    p1 = torch.empty(max(max_pairs, 1), dtype=torch.int64, device="cuda")
    p2 = torch.empty(max(max_pairs, 1), dtype=torch.int64, device="cuda")
    npairs = C.c_int64(-1)
    st = lib.mps_neighbor_list_noalloc(L.dptr(cell), n, L.host_i64(ncell), L.dptr(p1), L.dptr(p2), max_pairs,
                                       C.byref(npairs), L.stream_handle())
    return st, npairs.value, p1, p2


def _case(n, phi, seed, rc):
    x, box, _ = rsa(n, phi, seed=seed)
    xd = torch.as_tensor(x, device="cuda")
    cell, ncell = gew.cell_list(xd, box, rc)          # device tensor in, device tensor out
    ref1, ref2 = gew.neighbor_list(cell, ncell)       # workspace-based entry points
    return cell.contiguous(), ncell, ref1, ref2


def test_noalloc_matches_workspace_entry_points_twice():
    cases = [_case(3000, 0.25, 21, 4.5), _case(1200, 0.1, 22, 6.0)]
    for cell, ncell, ref1, ref2 in cases:          # two calls in a row, different sizes
        st, npairs, p1, p2 = _noalloc(cell, ncell, ref1.numel())
        assert st == L.MPS_OK, L.lib().mps_status_string(st).decode()
        assert npairs == ref1.numel()
        assert torch.equal(p1[:npairs], ref1) and torch.equal(p2[:npairs], ref2)
    # and once more on the first case: the leftover scratch of the second call must not leak in
    cell, ncell, ref1, ref2 = cases[0]
    st, npairs, p1, p2 = _noalloc(cell, ncell, ref1.numel())
    assert st == L.MPS_OK and npairs == ref1.numel()
    assert torch.equal(p1[:npairs], ref1) and torch.equal(p2[:npairs], ref2)


def test_noalloc_rejects_oversize_inputs_and_small_outputs():
    cell, ncell, ref1, _ = _case(500, 0.2, 23, 4.0)
    lib = L.lib()
    # more particles than the fixed scratch can bin: rejected before any GPU access
    big = C.c_int64(-1)
    st = lib.mps_neighbor_list_noalloc(L.dptr(cell), 10_000_000, L.host_i64(ncell), C.c_void_p(0), C.c_void_p(0),
                                       0, C.byref(big), L.stream_handle())
    assert st == L.MPS_SCRATCH_LIMIT
    assert "scratch" in lib.mps_status_string(st).decode()
    assert lib.mps_neighbor_list_workspace(10_000_000, L.host_i64(ncell)) > L.NOALLOC_SCRATCH_BYTES
    # outputs too small: reports the needed pair count
    st, npairs, _, _ = _noalloc(cell, ncell, 10)
    assert st == L.MPS_SCRATCH_LIMIT and npairs == ref1.numel()
