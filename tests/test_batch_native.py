"""The many-configuration entry point mps_solve_batched (batch.solve_batched).

It replaces the spectrum drivers' parfor over configurations
(Capacitance_Hetero/CapacitanceTensorSpectrum.m:45,
Capacitance_Sizes/CapacitanceTensorSpectrum.m:44): the library builds, solves
and releases every configuration itself, several at a time on host threads and
streams of its own.  Checked against the same configurations solved one at a
time through the Python system objects (batch.solve_configuration): capacitance
spectra within 1e-5 of their scale for the mixed solve at tol 1e-6 (as the
threaded Python batch is checked), within 1e-9 for float64 GMRES at tol 1e-10;
and a configuration that cannot be built gets its own status while the others
are solved."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import _lib as L  # noqa: E402
from mutual_polarization_slab_gb300 import batch  # noqa: E402


@pytest.fixture(scope="module")
def configs():
    return batch.make_configurations(count=5, seed=17, n_range=(300, 1500))


SCAL = np.linspace(0.25, 1.0, 3)


@pytest.mark.parametrize("precision,tol,bound", [("mixed", 1e-6, 1e-5), ("fp64", 1e-10, 1e-9)])
def test_native_batch_matches_one_at_a_time(configs, precision, tol, bound):
    native = batch.solve_batched(configs, SCAL, tol=tol, precision=precision, streams=3)
    assert sorted(native) == [c.index for c in configs]
    for cfg in configs:
        Cs, conv_s = batch.solve_configuration(cfg, SCAL, tol=tol, precision=precision)
        Cn, conv_n = native[cfg.index]
        assert conv_s and conv_n
        assert Cn.shape == (SCAL.size, 3, 3)
        assert np.abs(Cn - Cs).max() <= bound * np.abs(Cs).max()


def test_native_batch_twice_and_one_stream(configs):
    """Two calls in a row, with one and with four workers, give the same spectra."""
    one = batch.solve_batched(configs[:3], SCAL, tol=1e-10, precision="fp64", streams=1)
    four = batch.solve_batched(configs[:3], SCAL, tol=1e-10, precision="fp64", streams=4)
    for k in one:
        assert np.abs(one[k][0] - four[k][0]).max() <= 1e-9 * np.abs(one[k][0]).max()


def test_native_batch_item_status(configs):
    """A configuration whose cutoff exceeds half its box is refused on its own
    (MPS_RC_GT_HALF_BOX); the call returns that status, and the other items are
    solved."""
    from mutual_polarization_slab_gb300.sizes import PolydisperseSystem
    from mutual_polarization_slab_gb300.system import PRECISIONS

    items = (L.BatchItem * 2)()
    keep = []
    for j, cfg in enumerate(configs[:2]):
        xi, ng, P, eps_sets, b, x0, dix = batch._configuration_inputs(cfg, SCAL, 1e-6, None, True)
        spec = PolydisperseSystem(cfg.x, cfg.radii, eps_sets, cfg.box, xi, 1e-6, Ngrid=ng, P=P,
                                  max_rhs=3 * SCAL.size, create=False)
        x = torch.full_like(b, float("nan"))
        items[j].desc = spec.desc
        items[j].b, items[j].x0, items[j].x = b.data_ptr(), x0.data_ptr(), x.data_ptr()
        items[j].nrhs = 3 * SCAL.size
        dia = (C.c_int32 * (3 * SCAL.size))(*dix)
        items[j].diag_index = C.cast(dia, C.POINTER(C.c_int32))
        keep += [spec, b, x0, x, dia]
    items[1].desc.rc = 0.6 * float(np.min(configs[1].box))
    opts = L.SolveOpts(tol=1e-8, restart=30, maxit=100, precision=PRECISIONS["fp64"], inner_tol=1e-4,
                       inner_maxit=4, residual_policy=0, verify=0, residual_precision=PRECISIONS["df"],
                       inner_operator=1)
    st = L.lib().mps_solve_batched(items, 2, C.byref(opts), 2, L.stream_handle())
    assert st == L.MPS_RC_GT_HALF_BOX
    assert items[0].status == L.MPS_OK and items[1].status == L.MPS_RC_GT_HALF_BOX
    assert torch.isfinite(keep[3]).all()          # the first item's solutions were written
    assert torch.isnan(keep[8]).all()             # the refused item's were not touched
