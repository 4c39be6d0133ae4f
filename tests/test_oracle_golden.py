"""The CPU oracle against vectors produced by the reference module itself
(tests/golden/make_golden.py).  Integer lists must be bit-exact."""
import hashlib

import numpy as np
import pytest

from oracle import capacitance_oracle as co
from oracle import ewald_oracle as ew


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype=np.int64)).tobytes()).hexdigest()


def test_cell_and_neighbor_lists_bit_exact(golden_small):
    g = golden_small
    cell, nc = ew.cell_list(g["x"], g["box"], float(g["rc"]))
    assert np.array_equal(cell, g["cell"]) and np.array_equal(nc, g["Ncell"])
    p1, p2 = ew.neighbor_list(cell, nc)
    assert np.array_equal(p1, g["p1"]) and np.array_equal(p2, g["p2"])


def test_c1_lists_bit_exact(golden_c1):
    g = golden_c1
    cell, nc = ew.cell_list(g["x"], g["box"], float(g["rc"]))
    assert np.array_equal(nc, g["Ncell"])
    p1, p2 = ew.neighbor_list(cell, nc)
    assert p1.size == int(g["n_cand"])
    assert _sha(p1) == str(g["cand_p1_sha"]) and _sha(p2) == str(g["cand_p2_sha"])
    perp, para, rv = ew.default_table(float(g["xi"]))
    pr = ew.prepare_real_space_pairs(g["x"], g["box"], p1, p2, float(g["rc"]), perp, para, rv)
    assert pr[0].size == int(g["n_pairs"])
    assert _sha(pr[0]) == str(g["p1f_sha"]) and _sha(pr[1]) == str(g["p2f_sha"])
    np.testing.assert_allclose(pr[3][::97], g["pair_A_sel"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(pr[4][::97], g["pair_B_sel"], rtol=1e-13, atol=1e-15)


def test_tables(golden_small):
    g = golden_small
    r = np.arange(0.001, 10.0 + 1e-12, 0.001)
    T = np.stack(ew.real_space_table(r, float(g["xi"])))[:, g["table_idx"]]
    rs = g["rvals_sel"]
    ref = g["tables"]
    # r >= 1: relative 1e-12 of the value plus 1e-15 absolute (values decay to 1e-24 in the erfc tail)
    far = rs >= 1.0
    assert np.all(np.abs(T - ref)[:, far] <= 1e-12 * np.abs(ref[:, far]) + 1e-15)
    # r < 1: the closed forms cancel terms of size r^-4; compare against that scale
    near = ~far & (rs > 0)
    scale = rs[near] ** -4.0
    assert np.all(np.abs(T - ref)[:, near] <= 1e-12 * scale)
    np.testing.assert_allclose(T[:, 0], ref[:, 0], rtol=1e-14)


def test_pairs_grid_kspace(golden_small):
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    pr = ew.prepare_real_space_pairs(g["x"], g["box"], g["p1"], g["p2"], float(g["rc"]), perp, para, rv)
    assert np.array_equal(pr[0], g["p1f"]) and np.array_equal(pr[1], g["p2f"])
    np.testing.assert_array_equal(pr[2], g["rhat"])
    np.testing.assert_allclose(pr[3], g["A"], rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose(pr[4], g["B"], rtol=1e-13, atol=1e-16)
    off, offxyz = ew.pre_calculations(int(g["P"]), g["h"])
    assert np.array_equal(off, g["offset"])
    lin, w, wc = ew.prepare_grid_kernel(g["x"], g["Ngrid"], g["h"], float(g["xi"]), g["eta"], int(g["P"]))
    assert np.array_equal(lin, g["linnode"])
    np.testing.assert_allclose(w, g["w_spread"], rtol=1e-13)
    np.testing.assert_allclose(wc, g["w_contract"], rtol=1e-13)
    kh, Hc = ew.precompute_kspace(g["Ngrid"], g["box"], float(g["xi"]), g["eta"])
    np.testing.assert_allclose(kh.real, g["khat"], atol=1e-15)
    np.testing.assert_allclose(Hc, g["Htildecoeff"], rtol=1e-13, atol=1e-300)


def test_operator_pieces(golden_small):
    g = golden_small
    H = ew.spread_fast(g["m_real"], g["Ngrid"], g["linnode"], g["w_spread"])
    np.testing.assert_allclose(H.real, g["grid_spread"], rtol=1e-12, atol=1e-14)
    Hk = ew.contract_fast(H, g["Ngrid"], g["linnode"], g["w_contract"])
    np.testing.assert_allclose(Hk, g["contract_of_spread"], rtol=1e-12, atol=1e-14)
    fH = np.fft.fftshift(np.fft.fftn(H, axes=(0, 1, 2)), axes=(0, 1, 2))
    sc = ew.scale_fast(fH, g["khat"].astype(np.complex128), g["Htildecoeff"])
    np.testing.assert_allclose(sc, g["scaled"], rtol=1e-12, atol=1e-12 * np.abs(g["scaled"]).max())
    perp, para, rv = ew.default_table(float(g["xi"]))
    Hr = ew.real_space_fast(g["m_real"], g["eps"], g["p1f"], g["p2f"], g["rhat"], g["A"], g["B"], perp[0])
    np.testing.assert_allclose(Hr, g["Hr_fast"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("which", ["H_real", "H_cplx"])
def test_matvec_complex_pipeline(golden_small, which):
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    geo = ew.Geometry(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]),
                      perp, para, rv, 1.0)
    m = g["m_real"] if which == "H_real" else g["m_cplx"]
    out = geo.field_complex(m)
    ref = g[which]
    assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()


def test_real_operator_is_real_part(golden_small, golden_c1):
    for g, slab in ((golden_small, 1.0), (golden_c1, 0.0)):
        perp, para, rv = ew.default_table(float(g["xi"]))
        geo = ew.Geometry(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]),
                          perp, para, rv, slab)
        out = geo.field_real(g["m_real"])
        ref = g["H_real"].real
        assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()


def test_solve_matches_reference(golden_small):
    """Oracle GMRES on the real operator vs the reference's SciPy GMRES run."""
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    N = g["x"].shape[0]
    phi = 4 * np.pi * N / (3 * np.prod(g["box"]))
    guess = co.dilute_guess(g["eps"], phi, [0, 0, 1.0])
    C, S, info = co.capacitance(g["x"], g["eps"], g["box"], guess, float(g["xi"]), 1e-5, perp, para, rv,
                                [0, 0, 1.0], tol=1e-12, restart=30, maxit=50)
    ref = g["p"][:, :, 0]
    # the reference stopped at relres 1e-5; its solution error is bounded by cond(A) * 1e-5
    assert np.linalg.norm(S - ref.real) / np.linalg.norm(ref.real) < 1e-4
    assert abs(C - g["C"][0].real) / abs(g["C"][0].real) < 1e-4


def test_c1_tensor(golden_c1):
    """Config 1 (N=1000, 64^3, P=8, GMRES(30) to 1e-8): oracle tensor vs reference tensor."""
    g = golden_c1
    perp, para, rv = ew.default_table(float(g["xi"]))
    geo = ew.Geometry(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]),
                      perp, para, rv, 0.0)
    N = g["x"].shape[0]
    phi = 4 * np.pi * N / (3 * np.prod(g["box"]))
    guess = co.dilute_guess(g["eps"], phi, [1.0, 0, 0])
    C, S, infos = co.capacitance_tensor(geo, guess, 1e-10, 30, 20)
    assert all(i["flag"] == 0 for i in infos)
    np.testing.assert_allclose(C, g["C"].real, rtol=0, atol=1e-7 * np.abs(g["C"]).max())
    assert np.linalg.norm(S - g["S"].real) / np.linalg.norm(g["S"].real) < 1e-7
    # the tensor is symmetric
    assert np.abs(C - C.T).max() < 1e-8 * np.abs(C).max()


def test_threaded_real_operator_matches_single_thread():
    """Geometry.field_real_many (threads over grid components and particle chunks,
    scipy FFTs with workers) is the same operator as field_real, to rounding."""
    from mutual_polarization_slab_gb300.workloads import rsa
    x, box, _ = rsa(2500, 0.3, seed=12)
    xi, rc = 0.7, 5.5
    perp, para, rv = ew.default_table(xi)
    g = ew.Geometry(x, np.full(x.shape[0], 9.0), box, xi, rc, [40, 40, 40], 8, perp, para, rv, 0.7)
    M = np.random.default_rng(3).standard_normal((3, x.shape[0], 3))
    ref = np.stack([g.field_real(M[i]) for i in range(3)])
    for threads in (1, 5):
        got = g.field_real_many(M, threads=threads)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_single_sphere_polarisability_is_clausius_mossotti():
    """One sphere per cubic cell: m = 4 pi beta / (1 - beta phi) H0, beta = (eps - 1)/(eps + 2),
    for real and complex eps (the cubic lattice sum vanishes; the conducting boundary adds
    phi m / (4 pi)): the oracle's operator with the dielectric term of a complex eps."""
    import math
    L = 20.0
    box = np.full(3, L)
    x = np.array([[L / 2, L / 2, L / 2]])
    xi = 0.5
    rc, Ng, _, P, _ = co.spectral_parameters(box, xi, 1e-10)
    perp, para, rv = ew.default_table(xi)
    g = ew.Geometry(x, np.array([2.0]), box, xi, rc, Ng, P, perp, para, rv, 0.0)
    A2 = np.stack([g.field_real(np.eye(3)[c][None])[0] for c in range(3)], axis=1)
    phi = 4.0 * math.pi / (3.0 * L ** 3)
    d = lambda e: -3.0 / (4.0 * math.pi * (1.0 - e))
    for eps in (5.0, 28.0, 5.0 + 2.0j, 3.0 - 0.5j):
        A = A2 + (d(eps) - d(2.0)) * np.eye(3)
        m = np.linalg.solve(A, np.array([0.0, 0.0, 1.0]))
        beta = (eps - 1.0) / (eps + 2.0)
        pred = 4.0 * math.pi * beta / (1.0 - beta * phi)
        assert abs(m[2] - pred) <= 1e-7 * abs(pred), (eps, m[2], pred)
