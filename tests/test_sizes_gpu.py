"""GPU parity of the polydisperse operator (Capacitance_Sizes) against the oracle.
Tolerances: tables 1e-11 of each column's scale; float64 operator 1e-11
relative (max-norm; float64 atomics reorder sums); float32 operator 2e-5;
solutions within the solver tolerance times a conditioning margin."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import sizes as gs  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from oracle import ewald_oracle as ew  # noqa: E402
from oracle import polydisperse_oracle as po  # noqa: E402


def spheres(n, box, seed):
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < n:
        p = rng.random(3) * box
        if all(np.linalg.norm(ew.min_image((p - q)[None], box)) > 2.05 for q in pts):
            pts.append(p)
    return np.array(pts)


BOX = np.array([20.0, 20.0, 20.0])
X = spheres(60, BOX, 3)
N = X.shape[0]
EPS = np.linspace(4.0, 30.0, N)
RADII = np.random.default_rng(4).uniform(0.6, 1.0, N)
CLASSES = np.where(np.arange(N) % 3 == 0, 0.7, np.where(np.arange(N) % 3 == 1, 1.0, 0.85))


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


def test_sizes_tables_match_oracle():
    rt = po.default_r_table()
    uniq = np.array([0.6, 0.8, 1.0])
    for xi in (0.4, 0.6, 0.9):
        gp, ga = (t.cpu().numpy() for t in gs.real_space_table(rt, uniq, xi))
        op, oa = po.real_space_table(rt, uniq, xi)
        assert gp.shape == op.shape == (rt.size, 6)
        for c in range(6):
            for g, o in ((gp, op), (ga, oa)):
                np.testing.assert_allclose(g[:, c], o[:, c], rtol=1e-11, atol=1e-11 * np.abs(o[:, c]).max())


@pytest.mark.parametrize("Ngrid", [None, (37, 39, 41)])
def test_matvec_closed_form_vs_oracle(Ngrid):
    xi, tol = 0.6, 1e-10
    og = po.PolyGeometry(X, RADII, EPS, BOX, xi, tol, Ngrid=Ngrid)
    rng = np.random.default_rng(7)
    p = rng.standard_normal((N, 3))
    Eo = og.field(p)
    sysm = gs.PolydisperseSystem(X, RADII, EPS, BOX, xi, tol, Ngrid=Ngrid, max_rhs=3)
    assert sysm.n_pairs == og.p1.size and sysm.P == og.P
    E = gs.compute_field(X, RADII, p, EPS, BOX, None, None, xi, None, None, None, tol, system=sysm)
    assert _rel(E, Eo) < 1e-11
    E32 = gs.compute_field(X, RADII, p, EPS, BOX, None, None, xi, None, None, None, tol, system=sysm,
                           precision="fp32")
    assert _rel(E32, Eo) < 2e-5
    out3 = sysm.matvec(np.stack((p, 2 * p, -p))).cpu().numpy()
    for i, c in enumerate((1, 2, -1)):
        assert _rel(out3[i], c * Eo) < 1e-11
    sysm.close()


def test_matvec_table_mode_vs_oracle():
    xi, tol = 0.6, 1e-8
    rt = po.default_r_table()
    uniq, cls = po.unique_radii(CLASSES)
    op, oa = po.real_space_table(rt, uniq, xi)
    og = po.PolyGeometry(X, CLASSES, EPS, BOX, xi, tol, tables=(rt, op, oa, uniq))
    p = np.random.default_rng(8).standard_normal((N, 3))
    gp, ga = gs.real_space_table(rt, gs.unique_radii(CLASSES)[0], xi)
    E = gs.compute_field(X, CLASSES, p, EPS, BOX, None, None, xi, rt, gp, ga, tol)
    assert _rel(E, og.field(p)) < 1e-11


def test_permittivity_sets():
    xi, tol = 0.6, 1e-8
    eps2 = np.stack((EPS, EPS[::-1] + 2.0))
    sysm = gs.PolydisperseSystem(X, RADII, eps2, BOX, xi, tol, max_rhs=2)
    m = np.random.default_rng(9).standard_normal((2, N, 3))
    out = sysm.matvec(m, diag_index=[1, 0]).cpu().numpy()
    for r, e in ((0, eps2[1]), (1, eps2[0])):
        og = po.PolyGeometry(X, RADII, e, BOX, xi, tol)
        assert _rel(out[r], og.field(m[r])) < 1e-11
    sysm.close()


def test_tensor_vs_oracle_batched_mixed():
    xi, tol = 0.6, 1e-6
    og = po.PolyGeometry(X, RADII, EPS, BOX, xi, tol)
    guess = np.zeros((N, 3))
    guess[:, 0] = 1.0
    Co, po_ = po.capacitance_tensor(og, guess, tol)
    Cs, ps, inf = gs.capacitance_tensor(X, RADII, EPS, BOX, guess, xi, tol, batched=False, return_info=True)
    assert all(i.converged for i in inf)
    assert np.abs(Cs - Co).max() < 20 * tol * np.abs(Co).max()
    assert _rel(ps, po_) < 50 * tol
    Cb, _, infb = gs.capacitance_tensor(X, RADII, EPS, BOX, guess, xi, tol, batched=True, return_info=True)
    assert all(i.converged for i in infb)
    assert np.abs(Cb - Co).max() < 20 * tol * np.abs(Co).max()
    Cm, _, infm = gs.capacitance_tensor(X, RADII, EPS, BOX, guess, xi, 1e-9, precision="mixed", return_info=True)
    assert all(i.converged for i in infm)
    assert np.abs(Cm - Co).max() < 20 * tol * np.abs(Co).max()


def test_spectrum_drivers():
    xi = 0.6
    eps = np.stack((EPS, np.full(N, 9.0)), axis=1)
    C, p = gs.capacitance_tensor_spectrum(X, BOX, CLASSES, eps, xi, tol=1e-8)
    assert C.shape == (2, 9) and p.shape == (N, 9, 2, 1)
    rt = gs.default_r_table()
    perp, para = gs.real_space_table(rt, gs.unique_radii(CLASSES)[0], xi)
    for k in range(2):
        Ck, pk = gs.capacitance_tensor(X, CLASSES, eps[:, k], BOX, np.zeros((N, 3)), xi, 1e-8, rt, perp, para)
        assert np.abs(C[k] - Ck).max() < 1e-6 * np.abs(Ck).max()
    pav, pd = gs.dipole_spectrum(X, BOX, CLASSES, eps, [0.0, 0.0, 1.0], xi, tol=1e-8)
    assert pav.shape == (2, 3) and pd.shape == (N, 3, 2, 1)
    np.testing.assert_allclose(pav[0], C[0, 6:9], rtol=1e-6, atol=1e-9)
    p_ave, p1 = gs.dipole(X, CLASSES, eps[:, 1], BOX, [0.0, 0.0, 1.0], np.zeros((N, 3)), xi, 1e-8, rt, perp, para)
    np.testing.assert_allclose(p_ave, pav[1], rtol=1e-6, atol=1e-9)


def test_sizes_errors():
    with pytest.raises(ValueError):
        gs.PolydisperseSystem(X, RADII, EPS, np.array([8.0, 8.0, 8.0]), 0.6, 1e-8)   # rc > L/2
    with pytest.raises(ValueError):
        SpectralEwaldSystem(X, EPS, BOX, 0.6, 7.0, (38, 38, 38), 15, None, None, None, slab_factor=1.0,
                            radius=RADII)
    with pytest.raises(ValueError):
        gs.real_space_table(np.arange(1.0, 2.0, 0.1), [1.0], 0.6)      # r[0] != 0
    rt = np.array([0.0, 1.0, 2.0])                                       # too short for rc
    perp, para = gs.real_space_table(rt, gs.unique_radii(CLASSES)[0], 0.6)
    with pytest.raises(ValueError):
        gs.PolydisperseSystem(X, CLASSES, EPS, BOX, 0.6, 1e-8, rt, perp, para)


def test_batch_concurrent_workers_match_serial():
    """Configurations solved three at a time (host threads, one CUDA stream each)
    give the same capacitance spectra as one at a time, to the solve tolerance."""
    from mutual_polarization_slab_gb300 import batch

    cfgs = batch.make_configurations(count=5, seed=11, n_range=(300, 1200))
    scal = np.linspace(0.2, 1.0, 4)
    serial = batch.solve_configurations(cfgs, scal, tol=1e-6, workers=1)
    threaded = batch.solve_configurations(cfgs, scal, tol=1e-6, workers=3)
    assert sorted(serial) == sorted(threaded) == [c.index for c in cfgs]
    for k in serial:
        (Cs, conv_s), (Ct, conv_t) = serial[k], threaded[k]
        assert conv_s and conv_t
        assert np.abs(Cs - Ct).max() <= 1e-5 * np.abs(Cs).max()
