"""Slab / surface-energy workflow (CPU - Ewald test/surface_energy.py,
test_driver_BCT110.py).

CPU: the BCT(110) slab builder against a direct loop over basis and cells in
the reference's emission order, the axis permutation, and the surface-energy
arithmetic on stand-in capacitances.  GPU: the whole workflow against the same
arithmetic on the oracle's float64 capacitances (CPU GMRES) for a 108-sphere
slab; both solve to the reference's errortol = 1e-8, compared at 1e-6."""
import numpy as np
import pytest

from mutual_polarization_slab_gb300 import surface_energy as se


def _slab_loops(nc):
    a1, a2, a3 = np.array([np.sqrt(12.0), 0, 0]), np.array([0, np.sqrt(12.0), 0]), np.array([0, 0, 2.0])
    J = [(0, 0, 0), (0, 0.5, 0.5), (0.5, 0, 0.5), (0.5, 0.5, 0)]
    rows = [(a + j[0]) * a1 + (b + j[1]) * a2 + (c + j[2]) * a3
            for j in J for a in range(nc) for b in range(nc) for c in range(nc)]
    return np.array(rows)


@pytest.mark.parametrize("nc", [1, 3, 8])
def test_bct_110_slab_builder(nc):
    x, L0, A = se.build_bct_110_slab(nc, permute_for_solver=False)
    ref = _slab_loops(nc)
    assert x.shape == (4 * nc ** 3, 3)
    np.testing.assert_allclose(x, ref, rtol=0, atol=1e-12)
    np.testing.assert_allclose(L0, nc * np.array([np.sqrt(12.0), np.sqrt(12.0), 2.0]), rtol=1e-15)
    assert A == pytest.approx(L0[1] * L0[2], rel=1e-15)
    xs, Ls, As = se.build_bct_110_slab(nc, permute_for_solver=True)
    np.testing.assert_array_equal(xs, x[:, [2, 1, 0]])
    np.testing.assert_array_equal(Ls, L0[[2, 1, 0]])
    assert As == A and As == pytest.approx(Ls[0] * Ls[1], rel=1e-15)


def test_surface_energy_arithmetic(monkeypatch):
    calls = []

    def fake_run(x, L, eps, xi, H, slab_factor=1.0, verbose=0, **kw):
        calls.append((float(L[2]), float(eps[0]), slab_factor))
        C = 0.1 + 0.01 * float(L[2]) + 0.001 * float(eps[0])
        return np.array([C + 0j]), None

    monkeypatch.setattr(se, "run_capacitance", fake_run)
    x = np.zeros((10, 3))
    L = np.array([4.0, 5.0, 6.0])
    g = se.surface_energy_from_two_separations(x, L, 3.0, 0.5, [0, 0, 1], [0.0, 2.0], slab_factor=0.5)
    C = np.array([0.1 + 0.06 + 0.003, 0.1 + 0.18 + 0.003])
    U = -0.5 * C * 10
    expect = (U[1] - U[0]) / (2 * 20.0) / (C[0] / np.sqrt(4 * np.pi)) ** 2
    assert g == pytest.approx(expect, rel=1e-14)
    assert calls == [(6.0, 3.0, 0.5), (18.0, 3.0, 0.5)]
    with pytest.raises(ValueError):
        se.surface_energy_from_two_separations(x, L, 3.0, 0.5, [0, 0, 1], [0.0, 1.0, 2.0])
    calls.clear()
    s = se.surface_energy_scan(x, L, 20.0, [-0.01, 0.5], [0.0, 1.0, 3.0], 0.5, [1, 0, 0])
    assert s.shape == (2, 3) and np.all(s[:, 0] == 0.0)
    eps = (1 + 2 * 0.5) / (1 - 0.5)
    Cb = 0.1 + 0.01 * np.array([6.0, 12.0, 24.0]) + 0.001 * eps
    Ub = -0.5 * Cb * 10
    np.testing.assert_allclose(s[1], (Ub - Ub[0]) / 40.0 / (Cb[0] / np.sqrt(4 * np.pi)) ** 2, rtol=1e-13)


@pytest.mark.gpu
def test_surface_energy_vs_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("CUDA device required")
    from oracle import capacitance_oracle as co
    from oracle import ewald_oracle as ew

    x, L0, A = se.build_bct_110_slab(3, permute_for_solver=True)
    n = x.shape[0]
    xi, tol, beta = 1.5, 1e-8, 0.5
    eps = (1 + 2 * beta) / (1 - beta)
    H = np.array([1.0, 0.0, 0.0])
    solver = dict(restart=30, maxit=50)
    g = se.surface_energy_from_two_separations(x, L0, eps, xi, H, [0.0, 2.0], errortol=tol, **solver)
    perp, para, rv = ew.default_table(xi)
    C = []
    for hj in (0.0, 2.0):
        L = L0.copy()
        L[2] *= 1 + hj
        phi = 4 * np.pi * n / (3 * np.prod(L))
        guess = co.dilute_guess(np.full(n, eps), phi, H)
        c, _, _ = co.capacitance(x, np.full(n, eps), L, guess, xi, tol, perp, para, rv, H, slab_factor=1.0,
                                 restart=30, maxit=50)
        C.append(c)
    C = np.array(C)
    U = -0.5 * C * n
    ref = (U[1] - U[0]) / (2 * A) / (C[0] / np.sqrt(4 * np.pi)) ** 2
    assert abs(g - ref) <= 1e-6 * abs(ref)
