"""Hand-written FFT paths: precision 'df' (the float64-accurate matvec whose FFTs
and Green's scale run in float-pair arithmetic) and the float32 operator (same
transforms in float32).  Checked against the float64
(cuFFT) operator and the oracle on grids that exercise every radix (2, 3, 4, 5),
odd Ny / Nz (unpaired x rows), and the fallback for unsupported grids.
Tolerance: 1e-12 relative (max-norm), the float64 operators' bar."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402
from oracle import ewald_oracle as ew  # noqa: E402


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def config():
    x, box, _ = rsa(400, 0.2, seed=5)
    eps = np.full(400, 12.0)
    return x, box, eps


@pytest.mark.parametrize("Ngrid", [(64, 64, 64), (60, 45, 50), (96, 81, 40), (30, 32, 25)])
def test_df_matvec_matches_fp64_and_oracle(config, Ngrid):
    x, box, eps = config
    xi, rc, P = 0.7, 5.5, 8
    perp, para, rv = gcap.default_table(xi)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, Ngrid, P, perp, para, rv, slab_factor=1.0, max_rhs=3)
    m = np.random.default_rng(1).standard_normal((3, 400, 3))
    o64 = s.matvec(m, precision="fp64").cpu().numpy()
    odf = s.matvec(m, precision="df").cpu().numpy()
    assert _rel(odf, o64) < 1e-12
    os.environ["MPS_DF_CONTRACT"] = "tiled"                # tiled double-float contraction (default: warp gather)
    try:
        odf_tiled = s.matvec(m, precision="df").cpu().numpy()
    finally:
        del os.environ["MPS_DF_CONTRACT"]
    assert _rel(odf_tiled, o64) < 1e-12
    for k in (1, 2):                                       # 1 and 2 vectors per launch
        assert _rel(s.matvec(m[:k], precision="df").cpu().numpy(), o64[:k]) < 1e-12
    o32 = s.matvec(m, precision="fp32").cpu().numpy()     # float32 operator, cuFFT
    assert _rel(o32, o64) < 2e-5
    os.environ["MPS_FFT32"] = "own"                        # float32 operator on the hand-written FFT
    try:
        o32own = s.matvec(m, precision="fp32").cpu().numpy()
    finally:
        del os.environ["MPS_FFT32"]
    assert _rel(o32own, o64) < 2e-5
    pn, pa, rvn = ew.default_table(xi)
    g = ew.Geometry(x, eps, box, xi, rc, Ngrid, P, pn, pa, rvn, slab_factor=1.0)
    assert _rel(odf[1], g.field_real(m[1])) < 1e-12
    s.close()


def test_df_unsupported_grid_falls_back_to_fp64(config):
    x, box, eps = config
    xi, rc, P = 0.7, 5.5, 8
    perp, para, rv = gcap.default_table(xi)
    for Ngrid in ((63, 64, 64), (56, 64, 64)):        # odd Nx; factor 7
        s = SpectralEwaldSystem(x, eps, box, xi, rc, Ngrid, P, perp, para, rv, slab_factor=0.0, max_rhs=1)
        m = np.random.default_rng(2).standard_normal((400, 3))
        np.testing.assert_array_equal(s.matvec(m, precision="df").cpu().numpy(),
                                      s.matvec(m, precision="fp64").cpu().numpy())
        s.close()


def test_df_residual_in_mixed_solve_and_df_gmres(config):
    x, box, eps = config
    xi, rc, P = 0.7, 5.5, 8
    perp, para, rv = gcap.default_table(xi)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, (64, 64, 64), P, perp, para, rv, slab_factor=0.0, max_rhs=3)
    s.profile(True)
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[:, None, :].expand(3, 400, 3).contiguous()
    ref, _ = s.solve(b, None, tol=1e-12, restart=30, maxit=50, precision="fp64")
    sol, info = s.solve(b, None, tol=1e-9, restart=30, maxit=8, precision="mixed", residual_precision="df",
                        verify=True)
    assert all(i.converged for i in info)
    for r in range(3):
        assert float(torch.linalg.vector_norm(sol[r] - ref[r]) / torch.linalg.vector_norm(ref[r])) < 1e-7
    sdf, idf = s.solve(b, None, tol=1e-10, restart=30, maxit=50, precision="df")
    assert all(i.converged for i in idf)
    for r in range(3):
        assert float(torch.linalg.vector_norm(sdf[r] - ref[r]) / torch.linalg.vector_norm(ref[r])) < 1e-8
    st = s.stage_times()
    assert st["df"][0] > 0 and st["fp32"][0] > 0
    s.close()
