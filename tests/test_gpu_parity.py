"""GPU parity: every drop-in function and the system operator / solver against the
oracle and the reference's golden vectors.  Tolerances: integer lists bit-exact;
float64 operators 1e-12 relative (max-norm); float32 operator 2e-5; solutions
within the solver tolerance times a conditioning margin."""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402
from mutual_polarization_slab_gb300 import ewald as gew  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402
from oracle import capacitance_oracle as co  # noqa: E402
from oracle import ewald_oracle as ew  # noqa: E402


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype=np.int64)).tobytes()).hexdigest()


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


# ---------------------------------------------------------------- integer lists
def test_cell_neighbor_pairs_bit_exact(golden_small):
    g = golden_small
    cell, nc = gew.cell_list(g["x"], g["box"], float(g["rc"]))
    assert np.array_equal(cell, g["cell"]) and np.array_equal(nc, g["Ncell"])
    p1, p2 = gew.neighbor_list(cell, nc)
    assert np.array_equal(p1, g["p1"]) and np.array_equal(p2, g["p2"])
    perp, para, rv = ew.default_table(float(g["xi"]))
    p1f, p2f, rhat, A, B = gew.prepare_real_space_pairs(g["x"], g["box"], p1, p2, float(g["rc"]), perp, para, rv)
    assert np.array_equal(p1f, g["p1f"]) and np.array_equal(p2f, g["p2f"])
    np.testing.assert_array_equal(rhat, g["rhat"])   # same rounded operations as numpy
    # same tables in -> bit-identical interpolation (no FMA contraction on either side)
    o = ew.prepare_real_space_pairs(g["x"], g["box"], p1, p2, float(g["rc"]), perp, para, rv)
    np.testing.assert_array_equal(A, o[3])
    np.testing.assert_array_equal(B, o[4])
    # the reference's own tables differ from the restated ones by ~1e-14 relative
    np.testing.assert_allclose(A, g["A"], rtol=1e-12, atol=1e-17)
    np.testing.assert_allclose(B, g["B"], rtol=1e-12, atol=1e-17)


def test_c1_lists_bit_exact(golden_c1):
    g = golden_c1
    cell, nc = gew.cell_list(g["x"], g["box"], float(g["rc"]))
    p1, p2 = gew.neighbor_list(cell, nc)
    assert p1.size == int(g["n_cand"])
    assert _sha(p1) == str(g["cand_p1_sha"]) and _sha(p2) == str(g["cand_p2_sha"])
    perp, para, rv = ew.default_table(float(g["xi"]))
    pr = gew.prepare_real_space_pairs(g["x"], g["box"], p1, p2, float(g["rc"]), perp, para, rv)
    assert pr[0].size == int(g["n_pairs"])
    assert _sha(pr[0]) == str(g["p1f_sha"]) and _sha(pr[1]) == str(g["p2f_sha"])


def test_lists_deterministic_and_ragged():
    """Run-to-run identical integer outputs; uneven cell occupancy; a particle outside [0, L)."""
    rng = np.random.default_rng(9)
    x = rng.random((300, 3)) * 20.0
    x[:40] *= 0.1                      # crowd one corner (ragged cells)
    x[5] = [-3.2, 21.5, 7.0]           # outside the box: wrapped by the cell list
    box = np.array([20.0, 20.0, 20.0])
    cell, nc = gew.cell_list(x, box, 4.0)
    ocell, onc = ew.cell_list(x, box, 4.0)
    assert np.array_equal(cell, ocell) and np.array_equal(nc, onc)
    a = gew.neighbor_list(cell, nc)
    b = gew.neighbor_list(cell, nc)
    o = ew.neighbor_list(ocell, onc)
    for u, v, w in zip(a, b, o):
        assert np.array_equal(u, v) and np.array_equal(u, w)


def test_empty_inputs():
    x = np.zeros((0, 3))
    box = np.array([10.0, 10.0, 10.0])
    cell, nc = gew.cell_list(x, box, 3.0)
    assert cell.shape == (0, 3)
    p1, p2 = gew.neighbor_list(cell, nc)
    assert p1.size == 0 and p2.size == 0
    perp, para, rv = ew.default_table(0.5)
    out = gew.prepare_real_space_pairs(np.zeros((2, 3)), box, np.array([], dtype=np.int64),
                                       np.array([], dtype=np.int64), 3.0, perp, para, rv)
    assert all(o.shape[0] == 0 for o in out)


def test_table_range_error():
    x = np.array([[0.0, 0.0, 0.0], [0.0005, 0.0, 0.0]])
    box = np.array([10.0, 10.0, 10.0])
    perp, para, rv = ew.default_table(0.5)
    with pytest.raises(ValueError):
        gew.prepare_real_space_pairs(x, box, np.array([0, 1]), np.array([1, 0]), 3.0, perp[1:], para[1:], rv[1:])


def test_system_table_range_reported_by_first_use():
    """A dipole system whose pair list holds a separation below the table's
    first entry builds (its table-range check completes on the stream after
    mps_system_create returns) and every call that uses it raises: a matvec, a
    solve (after it ran) and the calls after them."""
    x = np.array([[1.0, 1.0, 1.0], [1.0005, 1.0, 1.0], [5.0, 5.0, 5.0]])
    box = np.array([10.0, 10.0, 10.0])
    perp, para, rv = ew.default_table(0.5)
    s = SpectralEwaldSystem(x, np.full(3, 4.0), box, 0.5, 3.0, [16, 16, 16], 6, perp[1:], para[1:], rv[1:],
                            max_rhs=1)
    m = np.ones((3, 3))
    with pytest.raises(ValueError):
        s.matvec(m, precision="fp64")
    with pytest.raises(ValueError):
        s.solve(m, None, tol=1e-6, restart=5, maxit=2, precision="fp64")
    s.close()
    s = SpectralEwaldSystem(x, np.full(3, 4.0), box, 0.5, 3.0, [16, 16, 16], 6, perp[1:], para[1:], rv[1:],
                            max_rhs=1)
    with pytest.raises(ValueError):
        s.solve(m, None, tol=1e-6, restart=5, maxit=2, precision="fp64")
    s.close()


def test_rc_greater_than_half_box_raises():
    x, box, _ = rsa(20, 0.1, seed=2)
    perp, para, rv = ew.default_table(0.5)
    with pytest.raises(ValueError):
        SpectralEwaldSystem(x, np.full(20, 4.0), box, 0.5, box[0] * 0.6, [16, 16, 16], 6, perp, para, rv)


# ---------------------------------------------------------------- tables, grids, k-space
def test_tables(golden_small):
    g = golden_small
    r = np.arange(0.001, 10.0 + 1e-12, 0.001)
    T = np.stack(gew.real_space_table(r, float(g["xi"])))[:, g["table_idx"]]
    O = np.stack(ew.real_space_table(r, float(g["xi"])))[:, g["table_idx"]]
    rs = g["rvals_sel"]
    far = rs >= 1.0
    assert np.all(np.abs(T - g["tables"])[:, far] <= 1e-12 * np.abs(g["tables"][:, far]) + 1e-15)
    near = ~far & (rs > 0)
    assert np.all(np.abs(T - O)[:, near] <= 1e-12 * rs[near] ** -4.0)


def test_grid_kernel_and_wave_pieces(golden_small):
    g = golden_small
    off, offxyz = gew.pre_calculations(int(g["P"]), g["h"])
    assert np.array_equal(off, g["offset"])
    np.testing.assert_array_equal(offxyz, g["offsetxyz"])
    lin, w, wc = gew.prepare_grid_kernel(g["x"], g["Ngrid"], g["h"], float(g["xi"]), g["eta"], int(g["P"]))
    assert np.array_equal(lin, g["linnode"])
    np.testing.assert_allclose(w, g["w_spread"], rtol=1e-13)
    np.testing.assert_allclose(wc, g["w_contract"], rtol=1e-13)
    H = gew.spread_fast(g["m_real"], g["Ngrid"], lin, w)
    assert _rel(H.real, g["grid_spread"]) < 1e-13
    Hk = gew.contract_fast(H, g["Ngrid"], lin, wc)
    assert _rel(Hk, g["contract_of_spread"]) < 1e-13
    kh, Hc = gew.precompute_kspace(g["Ngrid"], g["box"], float(g["xi"]), g["eta"])
    np.testing.assert_allclose(kh.real, g["khat"], atol=1e-15)
    assert _rel(Hc, g["Htildecoeff"]) < 1e-13
    fH = np.fft.fftshift(np.fft.fftn(H, axes=(0, 1, 2)), axes=(0, 1, 2))
    sc = gew.scale_fast(fH, kh, Hc)
    assert _rel(sc, g["scaled"]) < 1e-12
    Hs = gew.spread(g["x"], g["m_cplx"], g["Ngrid"], g["h"], float(g["xi"]), g["eta"], int(g["P"]))
    Ho = ew.spread(g["x"], g["m_cplx"], g["Ngrid"], g["h"], float(g["xi"]), g["eta"], int(g["P"]))
    for a, b in zip(Hs, Ho):
        assert _rel(a, b) < 1e-13


def test_real_space_fast(golden_small):
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    Hr = gew.real_space_fast(g["m_real"], g["eps"], g["p1f"], g["p2f"], g["rhat"], g["A"], g["B"], perp[0])
    assert _rel(Hr, g["Hr_fast"]) < 1e-14
    Hc = gew.real_space_fast(g["m_cplx"], g["eps"], g["p1f"], g["p2f"], g["rhat"], g["A"], g["B"], perp[0])
    Ho = ew.real_space_fast(g["m_cplx"], g["eps"], g["p1f"], g["p2f"], g["rhat"], g["A"], g["B"], perp[0])
    assert _rel(Hc, Ho) < 1e-14


# ---------------------------------------------------------------- matvec
@pytest.mark.parametrize("which", ["H_real", "H_cplx"])
def test_magnetic_field_complex_pipeline(golden_small, which):
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    m = g["m_real"] if which == "H_real" else g["m_cplx"]
    out = gew.magnetic_field(g["x"], m, g["eps"], g["box"], g["p1"], g["p2"], g["Ngrid"], g["h"], int(g["P"]),
                             float(g["xi"]), g["eta"], float(g["rc"]), g["offset"], g["offsetxyz"], perp, para, rv,
                             slab_factor=1.0)
    assert _rel(out, g[which]) < 1e-12


def test_magnetic_field_components(golden_small):
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    Hk, Hr, Hs = gew.magnetic_field_components(g["x"], g["m_real"], g["eps"], g["box"], g["p1"], g["p2"], g["Ngrid"],
                                               g["h"], int(g["P"]), float(g["xi"]), g["eta"], float(g["rc"]),
                                               g["offset"], g["offsetxyz"], perp, para, rv, slab_factor=1.0)
    assert _rel(Hk, g["Hk"]) < 1e-11
    assert _rel(Hr, g["Hr"]) < 1e-13
    assert _rel(Hs, g["Hslab"]) < 1e-13


@pytest.mark.parametrize("case", ["small", "c1"])
def test_system_matvec_fp64_fp32(golden_small, golden_c1, case):
    g = golden_small if case == "small" else golden_c1
    slab = 1.0 if case == "small" else 0.0
    perp, para, rv = ew.default_table(float(g["xi"]))
    geo = ew.Geometry(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]),
                      perp, para, rv, slab)
    rng = np.random.default_rng(3)
    m = rng.normal(size=(3,) + g["x"].shape)
    ref = np.stack([geo.field_real(mi) for mi in m])
    with SpectralEwaldSystem(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]),
                             perp, para, rv, slab_factor=slab, max_rhs=3) as s:
        out64 = s.matvec(m).cpu().numpy()
        out32 = s.matvec(m, precision="fp32").cpu().numpy()
        one = s.matvec(m[1]).cpu().numpy()
    assert _rel(out64, ref) < 1e-12
    assert _rel(one, ref[1]) < 1e-12
    assert _rel(out32, ref) < 2e-5
    # against the reference's own complex matvec (real part) for the golden vector
    if case == "c1":
        with SpectralEwaldSystem(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"],
                                 int(g["P"]), perp, para, rv, slab_factor=0.0, max_rhs=1) as s:
            assert _rel(s.matvec(g["m_real"]).cpu().numpy(), g["H_real"].real) < 1e-12


def test_tiled_kernels_odd_noncubic_grid():
    """Partial tiles in every axis, odd axes (no Nyquist bin) and one even axis, P < tile depth mix."""
    x, box, _ = rsa(400, 0.15, seed=8)
    xi, rc, P = 0.7, 5.0, 8
    Ng = np.array([25, 17, 12])
    eps = np.where(np.arange(400) % 3 == 0, 28.0, 3.0)
    perp, para, rv = ew.default_table(xi)
    geo = ew.Geometry(x, eps, box, xi, rc, Ng, P, perp, para, rv, 0.5)
    m = np.random.default_rng(4).normal(size=(3, 400, 3))
    ref = np.stack([geo.field_real(mi) for mi in m])
    with SpectralEwaldSystem(x, eps, box, xi, rc, Ng, P, perp, para, rv, slab_factor=0.5, max_rhs=3) as s:
        for r in (1, 2, 3):
            assert _rel(s.matvec(m[:r]).cpu().numpy(), ref[:r]) < 1e-12
            assert _rel(s.matvec(m[:r], precision="fp32").cpu().numpy(), ref[:r]) < 2e-5
        again = s.matvec(m).cpu().numpy()
        assert np.array_equal(again, s.matvec(m).cpu().numpy())   # deterministic summation order


# ---------------------------------------------------------------- solves
def test_run_capacitance_matches_reference(golden_small):
    g = golden_small
    C, p = gcap.run_capacitance(g["x"], g["box"], g["eps"], float(g["xi"]), np.array([0.0, 0.0, 1.0]),
                                errortol=float(g["tol"]))
    assert p.dtype == np.complex128 and p.shape == g["p"].shape
    # both stop at relres <= 1e-5 from the same guess: solutions agree to cond(A) x tol
    assert np.linalg.norm(p - g["p"].real) / np.linalg.norm(g["p"]) < 1e-4
    assert abs(C[0] - g["C"][0]) / abs(g["C"][0]) < 1e-4
    # tight solve agrees with the oracle's tight solve
    C2, p2 = gcap.run_capacitance(g["x"], g["box"], g["eps"], float(g["xi"]), np.array([1.0, 1.0, 0.0]),
                                  errortol=1e-6, restart=30, maxit=50)
    perp, para, rv = ew.default_table(float(g["xi"]))
    N = g["x"].shape[0]
    phi = 4 * np.pi * N / (3 * np.prod(g["box"]))
    hh = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    Co, So, _ = co.capacitance(g["x"], g["eps"], g["box"], co.dilute_guess(g["eps"], phi, hh), float(g["xi"]), 1e-6,
                               perp, para, rv, hh, tol=1e-12, restart=30, maxit=50)
    assert np.linalg.norm(p2[:, :, 0].real - So) / np.linalg.norm(So) < 1e-5
    assert np.linalg.norm(p2[:, :, 0].real - g["p2sol"][:, :, 0].real) / np.linalg.norm(So) < 1e-4


def test_c1_capacitance_tensor(golden_c1):
    """Config 1: N=1000, 64^3, P=8, rc=8, GMRES(30) to 1e-8, fully periodic; vs the reference tensor."""
    g = golden_c1
    N = g["x"].shape[0]
    phi = 4 * np.pi * N / (3 * np.prod(g["box"]))
    guess = co.dilute_guess(g["eps"], phi, [1.0, 0.0, 0.0])
    for batched in (True, False):
        C, S, infos = gcap.capacitance_tensor(g["x"], g["eps"], g["box"], guess, float(g["xi"]), 1e-8,
                                              rc=float(g["rc"]), Ngrid=g["Ngrid"], P=int(g["P"]), restart=30,
                                              maxit=100, batched=batched)
        assert all(i.converged for i in infos)
        assert _rel(C, g["C"].real) < 1e-7
        assert np.linalg.norm(S - g["S"].real) / np.linalg.norm(g["S"].real) < 1e-7
        assert np.abs(C - C.T).max() < 1e-7 * np.abs(C).max()


def test_mixed_precision_accuracy(golden_c1):
    """FP32 operator inside FP64 refinement reaches <= 1e-6 relative moment error vs the FP64 solve."""
    g = golden_c1
    perp, para, rv = ew.default_table(float(g["xi"]))
    N = g["x"].shape[0]
    b = np.zeros((3, N, 3))
    for i in range(3):
        b[i, :, i] = 1.0
    with SpectralEwaldSystem(g["x"], g["eps"], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]),
                             perp, para, rv, slab_factor=0.0, max_rhs=3) as s:
        x64, i64 = s.solve(b, tol=1e-11, restart=30, maxit=50)
        runs = [s.solve(b, tol=1e-8, restart=30, maxit=10, precision="mixed", inner_tol=1e-4, residual_policy=pol,
                        verify=True, inner_operator=inner)
                for pol, inner in ((0, "reference"), (1, "reference"), (0, "grad"))]
    x64 = x64.cpu().numpy()
    assert all(i.converged for i in i64)
    for xm, im in runs:
        xm = xm.cpu().numpy()
        assert all(i.converged for i in im)            # verified with a float64 true residual
        for r in range(3):
            err = np.linalg.norm(xm[r] - x64[r]) / np.linalg.norm(x64[r])
            assert err < 1e-6, err
        assert im[0].matvecs_fp32 > im[0].matvecs_fp64
    # policy 0 with the reference-discretisation inner operator: one float64 residual + the verification;
    # with the gradient form at most one more true residual (the drift check)
    assert runs[0][1][0].matvecs_fp64 == 2
    assert runs[2][1][0].matvecs_fp64 <= 3


def test_contrast_batch_diag_index(golden_small):
    """Several permittivity sets in one batch (the spectrum axis) vs separate solves."""
    g = golden_small
    perp, para, rv = ew.default_table(float(g["xi"]))
    N = g["x"].shape[0]
    lam = np.stack([np.full(N, 4.0), np.full(N, 1.5), np.where(np.arange(N) % 2 == 0, 3.0, 28.0)])
    b = np.tile([0.0, 0.0, 1.0], (3, N, 1))
    with SpectralEwaldSystem(g["x"], lam, g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]), perp,
                             para, rv, slab_factor=1.0, max_rhs=3) as s:
        xb, _ = s.solve(b, tol=1e-11, restart=30, maxit=30, diag_index=[0, 1, 2])
        xb = xb.cpu().numpy()
    for k in range(3):
        geo = ew.Geometry(g["x"], lam[k], g["box"], float(g["xi"]), float(g["rc"]), g["Ngrid"], int(g["P"]), perp,
                          para, rv, 1.0)
        res = geo.field_real(xb[k]) - b[k]
        assert np.abs(res).max() < 1e-9


def test_gmres_restarted_matches_the_reference_solver():
    """The drop-in gmres_restarted against the reference's own gmres_restarted
    (tests/golden/golden_gmres.npz, recorded by make_golden.py): a converging
    solve, one stopped by maxit, whose x is each cycle's best iterate, and a
    stagnating cyclic shift (no column improves on a cycle's start)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_gmres.npz"))
    A = g["A"]
    for tag in ("conv", "stop"):
        tol, restart, maxit = g[f"ctl_{tag}"]
        x, flag, relres = gcap.gmres_restarted(lambda v: A @ v, g["b"], g["x0"], float(tol), int(restart),
                                               int(maxit))
        assert flag == int(g[f"flag_{tag}"])
        ref = g[f"x_{tag}"]
        assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max(), tag
        if tag == "stop":
            assert abs(relres - float(g["relres_stop"])) <= 1e-8 * float(g["relres_stop"])
        else:
            assert relres <= float(tol)
    S = g["S"]
    x, flag, relres = gcap.gmres_restarted(lambda v: S @ v, g["bs"], np.zeros(S.shape[0], dtype=complex), 1e-8, 5, 3)
    assert flag == int(g["flag_stag"]) == 1
    np.testing.assert_allclose(x, g["x_stag"], atol=1e-14)
    assert abs(relres - float(g["relres_stag"])) <= 1e-12


def test_gmres_restarted_solves_complex_systems():
    """Complex (non-real) systems converge to the direct solution: the drop-in's
    Givens rotation is unitary for complex entries."""
    rng = np.random.default_rng(29)
    n = 50
    A = 4.0 * np.eye(n) + 0.3 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    b = rng.normal(size=n) + 1j * rng.normal(size=n)
    x, flag, relres = gcap.gmres_restarted(lambda v: A @ v, b, np.zeros(n, dtype=complex), 1e-12, 10, 50)
    assert flag == 0 and relres <= 1e-12
    ref = np.linalg.solve(A, b)
    assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()
