"""The polydisperse oracle (CPU).  No MATLAB run is possible here, so the
restatement of CS/ is pinned by:

* the monodisperse limit: couplings at a_i = a_j = 1 equal the dipole tables
  (1e-14) and the whole operator equals the dipole operator, itself pinned to
  the reference Python's golden vectors, to the spectral tolerance;
* Ewald-split invariance with unequal radii (exercises every a_i != a_j term);
* symmetry p.E(q) = q.E(p) and continuity of the overlap branches;
* a planted mistake in the oracle's couplings breaks the invariance.
"""
import numpy as np
import pytest

from oracle import ewald_oracle as ew
from oracle import polydisperse_oracle as po

BOX = np.array([20.0, 20.0, 20.0])


def spheres(n, box, seed):
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < n:
        p = rng.random(3) * box
        if all(np.linalg.norm(ew.min_image((p - q)[None], box)) > 2.05 for q in pts):
            pts.append(p)
    return np.array(pts)


X = spheres(60, BOX, 3)
N = X.shape[0]
EPS = np.linspace(4.0, 30.0, N)
RADII = np.random.default_rng(4).uniform(0.6, 1.0, N)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def dip():
    return np.random.default_rng(1).standard_normal((N, 3))


def test_monodisperse_couplings_are_the_dipole_tables():
    r = np.linspace(0.5, 9.0, 400)
    for xi in (0.4, 0.6, 0.9):
        perp, para = po.couplings(r, 1.0, 1.0, xi)
        f = ew.real_space_table(r, xi)
        np.testing.assert_allclose(perp, f[2][1:], rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(para, f[3][1:], rtol=1e-9, atol=1e-14)
        assert abs(po.self_value(1.0, 1.0, xi) - f[2][0]) < 1e-15


def test_monodisperse_operator_is_the_dipole_operator(dip):
    g = po.PolyGeometry(X, np.ones(N), EPS, BOX, 0.6, 1e-10)
    perp, para, rv = ew.default_table(0.6)
    gd = ew.Geometry(X, EPS, BOX, 0.6, g.rc, g.Ngrid, 15, perp, para, rv, slab_factor=0.0)
    assert _rel(g.field(dip), gd.field_real(dip)) < 1e-7


def test_xi_invariance_unequal_radii(dip):
    E1 = po.PolyGeometry(X, RADII, EPS, BOX, 0.6, 1e-10).field(dip)
    E2 = po.PolyGeometry(X, RADII, EPS, BOX, 0.85, 1e-10).field(dip)
    assert _rel(E1, E2) < 1e-7


def test_symmetry(dip):
    g = po.PolyGeometry(X, RADII, EPS, BOX, 0.6, 1e-6)
    q = np.random.default_rng(2).standard_normal((N, 3))
    a, b = np.sum(q * g.field(dip)), np.sum(dip * g.field(q))
    assert abs(a - b) < 1e-12 * abs(a)


def test_overlap_branches_continuous():
    for ai, aj in ((0.7, 1.0), (1.0, 0.55), (0.8, 0.8)):
        for r0 in (ai + aj, abs(ai - aj)):
            if r0 == 0.0:
                continue
            lo, hi = po.couplings(np.array([r0 * (1 - 1e-9), r0 * (1 + 1e-9)]), ai, aj, 0.6)
            assert abs(lo[0] - lo[1]) < 1e-6 * abs(lo[0]) + 1e-9
            assert abs(hi[0] - hi[1]) < 1e-6 * abs(hi[0]) + 1e-9


def test_table_mode_matches_closed_form(dip):
    a2 = np.where(np.arange(N) % 3 == 0, 0.7, 1.0)
    uniq, cls = po.unique_radii(a2)
    assert np.allclose(uniq, [0.7, 1.0]) and np.array_equal(cls, (a2 == 1.0).astype(int))
    col = po.pair_columns(2)
    assert col.tolist() == [[0, 1], [1, 2]]
    rt = po.default_r_table()
    perp, para = po.real_space_table(rt, uniq, 0.6)
    assert perp.shape == (rt.size, 3) and perp[0, 2] == para[0, 2] == po.self_value(1.0, 1.0, 0.6)
    gt = po.PolyGeometry(X, a2, EPS, BOX, 0.6, 1e-8, tables=(rt, perp, para, uniq))
    gc = po.PolyGeometry(X, a2, EPS, BOX, 0.6, 1e-8)
    assert _rel(gt.field(dip), gc.field(dip)) < 1e-6   # linear interpolation on dr = 1e-3


def test_planted_coupling_error_breaks_invariance(dip, monkeypatch):
    orig = po.couplings

    def bad(r, ai, aj, xi):
        pp, pa = orig(r, ai, aj, xi)
        return (pp * 1.001, pa) if ai != aj else (pp, pa)

    monkeypatch.setattr(po, "couplings", bad)
    E1 = po.PolyGeometry(X, RADII, EPS, BOX, 0.6, 1e-10).field(dip)
    E2 = po.PolyGeometry(X, RADII, EPS, BOX, 0.85, 1e-10).field(dip)
    assert _rel(E1, E2) > 1e-6          # vs < 1e-7 (measured 2e-9) without the mistake


def test_tensor_solve_converges():
    g = po.PolyGeometry(X, RADII, EPS, BOX, 0.6, 1e-6)
    guess = np.zeros((N, 3))
    C, p = po.capacitance_tensor(g, guess, 1e-8)
    assert C.shape == (9,) and p.shape == (N, 9)
    np.testing.assert_allclose(C[3:6], p[:, 3:6].mean(axis=0))
    assert C[0] > 0 and C[4] > 0 and C[8] > 0
