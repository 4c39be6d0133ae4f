"""The dipole + quadrupole oracle (CPU).  No MATLAB run is possible here, so the
restatement of CQ/ is pinned by properties that any correct form must have:

* its dipole block with Q = 0 is the dipole operator, which is itself pinned to
  the reference Python's golden vectors (1e-12);
* Ewald-split invariance: the operator does not depend on xi (1e-6, the table
  interpolation and the 1e-10 spectral tolerance set the floor);
* symmetry under the metric diag(I_3, W/2), W the Gram matrix of the
  5-component traceless quadrupole: S1.E(S2) = S2.E(S1), Q1.W.G(Q2) symmetric,
  and S.E(Q) = (1/2) Q.W.G(S) (1e-10);
* planted mistakes in the oracle (a perturbed table, a flipped wave-space
  coupling) break these properties, so the checks have teeth.
"""
import numpy as np
import pytest

from oracle import ewald_oracle as ew
from oracle import quadrupole_oracle as qo

W5 = np.array([[2, 0, 0, 1, 0], [0, 2, 0, 0, 0], [0, 0, 2, 0, 0], [1, 0, 0, 2, 0], [0, 0, 0, 0, 2]], float)


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
LAM = np.linspace(4.0, 30.0, N)


def geom(xi, tol=1e-10, tables=None):
    lt = np.sqrt(-np.log(tol))
    rc = lt / xi
    ng = np.ceil(1 + BOX * 2 * xi * lt / np.pi).astype(int)
    P = int(np.ceil(-2 * np.log(tol) / np.pi))
    tabs, rv = qo.default_quad_tables(xi)
    if tables is not None:
        tabs = tables(tabs)
    return qo.QuadGeometry(X, LAM, BOX, xi, rc, ng, P, tabs, rv)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def moments():
    rng = np.random.default_rng(11)
    return rng.standard_normal((N, 3)), rng.standard_normal((N, 5))


def test_dipole_block_is_the_dipole_operator(moments):
    S, _ = moments
    g = geom(0.6)
    E, _ = g.apply(S, np.zeros((N, 5)))
    perp, para, rv = ew.default_table(0.6)
    gd = ew.Geometry(X, LAM, BOX, 0.6, g.rc, g.Ngrid, g.P, perp, para, rv, slab_factor=0.0)
    assert _rel(E, gd.field_real(S)) < 1e-12


def test_tables_self_values_and_dipole_tables():
    tabs, rv = qo.default_quad_tables(0.7)
    perp, para, _ = ew.default_table(0.7)
    np.testing.assert_array_equal(tabs["field_dip_1"], perp)
    np.testing.assert_array_equal(tabs["field_dip_2"], para)
    assert tabs["grad_quad_2"][0] == qo.quad_self(0.7)
    for k in ("field_quad_1", "field_quad_2", "field_quad_3", "grad_quad_1", "grad_quad_3", "grad_quad_4"):
        assert tabs[k][0] == 0.0
    assert rv[0] == 0.0 and rv.size == tabs["grad_quad_4"].size


def test_xi_invariance(moments):
    S, Q = moments
    E1, G1 = geom(0.6).apply(S, Q)
    E2, G2 = geom(0.85).apply(S, Q)
    assert _rel(E1, E2) < 1e-6
    assert _rel(G1, G2) < 1e-6


def _symmetry_errors(g, seed=5):
    rng = np.random.default_rng(seed)
    S1, S2 = rng.standard_normal((N, 3)), rng.standard_normal((N, 3))
    Q1, Q2 = rng.standard_normal((N, 5)), rng.standard_normal((N, 5))
    z3, z5 = np.zeros((N, 3)), np.zeros((N, 5))
    E_s1, G_s1 = g.apply(S1, z5)
    E_s2, _ = g.apply(S2, z5)
    E_q2, G_q2 = g.apply(z3, Q2)
    _, G_q1 = g.apply(z3, Q1)
    a, b = np.sum(S1 * E_s2), np.sum(S2 * E_s1)
    c, d = np.sum(Q2 @ W5 * G_q1), np.sum(Q1 @ W5 * G_q2)
    e, f = np.sum(S1 * E_q2), 0.5 * np.sum(Q2 @ W5 * G_s1)
    return abs(a - b) / abs(a), abs(c - d) / abs(c), abs(e - f) / abs(e)


def test_metric_symmetry():
    for err in _symmetry_errors(geom(0.6)):
        assert err < 1e-10


def test_planted_table_error_breaks_invariance(moments):
    S, Q = moments

    def bad(t):
        t = dict(t)
        t["field_quad_2"] = t["field_quad_2"] * 1.001
        return t

    E1, G1 = geom(0.6, tables=bad).apply(S, Q)
    E2, G2 = geom(0.85, tables=bad).apply(S, Q)
    assert max(_rel(E1, E2), _rel(G1, G2)) > 1e-5


def test_planted_wave_space_error_breaks_symmetry(monkeypatch):
    orig = qo.wave_space_quad

    def flipped(grids, Ngrid, box, xi, eta):
        # a wrong sign on the S -> G coupling (45 i j2 j1 -> -45 i j2 j1)
        out_s = orig(np.concatenate((grids[..., :3], 0 * grids[..., 3:]), axis=3), Ngrid, box, xi, eta)
        out_q = orig(np.concatenate((0 * grids[..., :3], grids[..., 3:]), axis=3), Ngrid, box, xi, eta)
        out = out_s + out_q
        out[..., 3:] = -out_s[..., 3:] + out_q[..., 3:]
        return out

    monkeypatch.setattr(qo, "wave_space_quad", flipped)
    assert _symmetry_errors(geom(0.6))[2] > 1e-4


def test_tensor_solve_converges():
    g = geom(0.6, tol=1e-6)
    sg = np.zeros((N, 3))
    sg[:, 0] = 1.0
    C, S, Q, infos = qo.quad_tensor(g, sg, np.zeros((N, 5)), 1e-8, restart=10, maxit=100)
    assert all(i["flag"] == 0 and i["relres"] <= 1e-8 for i in infos)
    # column i is the mean dipole for the field along i
    np.testing.assert_allclose(C[:, 1], S[:, :, 1].mean(axis=0))
    assert np.all(np.diag(C) > 0)


def test_fft_friendly_grid_rule():
    """``fft_friendly`` rounds each axis of the tolerance rule's grid up to a
    5-smooth size and keeps the rule's cutoff and support (host logic only)."""
    torch = pytest.importorskip("torch")  # noqa: F841  (the package imports torch)
    from mutual_polarization_slab_gb300 import quadrupole as gq
    from mutual_polarization_slab_gb300.system import fft_size, spectral_parameters

    box = np.array([69.2820323, 69.2820323, 74.0])
    xi, tol = 0.6506, 1e-4
    rc0, ng0, _, P0, _ = spectral_parameters(box, xi, tol)
    rc, ng, P, eta = gq._params(box, xi, tol, None, None, None, fft_friendly=True)
    assert list(ng0) == [89, 89, 95] and list(ng) == [90, 90, 96]
    assert rc == rc0 and P == P0
    assert all(fft_size(int(v)) == int(v) for v in ng)
    np.testing.assert_allclose(eta, P * (box / ng * xi) ** 2 / np.pi)
    rc, ng_rule, _, _ = gq._params(box, xi, tol, None, None, None)
    assert list(ng_rule) == [89, 89, 95]
