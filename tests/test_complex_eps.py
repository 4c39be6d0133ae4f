"""Complex permittivities (the spectra of Capacitance_Hetero/CapacitanceSpectrum.m
and CapacitanceTensorSpectrum.m with frequency-dependent eps).

The operator is D m + M m with D = -3/(4 pi (1 - eps)) + self term complex and
M the real interaction operator; the oracle builds it from its real operator
(``Geometry.field_real`` on Re m and Im m, dielectric term swapped for the
complex one) and solves with its complex GMRES.  Matvec 1e-12 (float64,
double-float) and 2e-5 (float32); solves to 1e-7 relative (mixed) and 1e-9
(float64) in the moments."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402
from oracle import capacitance_oracle as co  # noqa: E402
from oracle import ewald_oracle as ew  # noqa: E402


def _d(lam):
    return -3.0 / (4.0 * np.pi * (1.0 - lam))


@pytest.fixture(scope="module")
def case():
    x, box, _ = rsa(300, 0.2, seed=8)
    rng = np.random.default_rng(8)
    eps = rng.uniform(2.0, 6.0, 300) + 1j * rng.uniform(0.3, 3.0, 300)
    xi, rc, P, Ng = 0.7, 5.5, 8, (48, 48, 48)
    perp, para, rv = gcap.default_table(xi)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, Ng, P, perp, para, rv, slab_factor=1.0, max_rhs=3)
    pn, pa, rvn = ew.default_table(xi)
    g = ew.Geometry(x, np.full(300, 2.0), box, xi, rc, Ng, P, pn, pa, rvn, slab_factor=1.0)

    def op(m):
        m = np.asarray(m).reshape(300, 3)
        out = g.field_real(m.real) + 1j * g.field_real(m.imag)
        return out + ((_d(eps) - _d(2.0))[:, None]) * m

    yield s, op, eps
    s.close()


def test_complex_matvec(case):
    s, op, _ = case
    rng = np.random.default_rng(1)
    m = rng.standard_normal((2, 300, 3)) + 1j * rng.standard_normal((2, 300, 3))
    ref = np.stack([op(m[k]) for k in range(2)])
    scale = np.abs(ref).max()
    for prec, tol in (("fp64", 1e-12), ("df", 1e-12), ("fp32", 2e-5)):
        out = s.matvec(m, precision=prec).cpu().numpy()
        assert out.dtype == np.complex128
        assert np.abs(out - ref).max() <= tol * scale, prec


def test_complex_solve_vs_oracle(case):
    s, op, eps = case
    b = np.zeros((300, 3), dtype=np.complex128)
    b[:, 2] = 1.0
    ref, flag, relres, _ = co.gmres(lambda v: op(v).reshape(-1), b.reshape(-1), np.zeros(900, complex), 1e-12, 30,
                                    200)
    ref = ref.reshape(300, 3)
    assert flag == 0
    x64, info = s.solve(b, None, tol=1e-11, restart=30, maxit=100, precision="fp64")
    assert info[0].converged
    x64 = x64.cpu().numpy()
    assert np.linalg.norm(x64 - ref) / np.linalg.norm(ref) < 1e-9
    xm, info = s.solve(b, None, tol=1e-8, restart=30, maxit=10, precision="mixed")
    assert info[0].converged
    xm = xm.cpu().numpy()
    assert np.linalg.norm(xm - ref) / np.linalg.norm(ref) < 1e-7


def test_complex_spectrum_api():
    x, box, _ = rsa(200, 0.15, seed=9)
    eps = np.stack([np.full(200, 4.0 + 1.0j), np.full(200, 9.0 + 4.0j)], axis=1)
    C, p = gcap.capacitance_tensor_spectrum(x, box, eps, 0.7, 1e-6, rc=5.5, Ngrid=(40, 40, 40), P=8,
                                            restart=30, maxit=50)
    assert C.shape == (3, 3, 2) and np.iscomplexobj(C)
    # the real-eps limit: Im eps -> 0 gives the real tensor
    C0, _ = gcap.capacitance_tensor_spectrum(x, box, eps.real, 0.7, 1e-6, rc=5.5, Ngrid=(40, 40, 40), P=8,
                                             restart=30, maxit=50)
    Cs, _ = gcap.capacitance_tensor_spectrum(x, box, eps.real + 1e-9j, 0.7, 1e-6, rc=5.5, Ngrid=(40, 40, 40), P=8,
                                             restart=30, maxit=50)
    assert np.abs(Cs.real - C0).max() <= 1e-6 * np.abs(C0).max()
    assert np.abs(Cs.imag).max() <= 1e-6 * np.abs(C0).max()
    assert np.abs(C.imag).max() > 1e-3 * np.abs(C.real).max()


def test_single_sphere_complex_polarisability_is_clausius_mossotti():
    """One sphere per cubic cell: the lattice sum of a cubic lattice vanishes and the
    conducting boundary adds phi m / (4 pi), so m = 4 pi beta / (1 - beta phi) H0
    with beta = (eps - 1) / (eps + 2) exactly (the real-eps case agrees to the Ewald
    tolerance, 4e-9).  With a complex eps this is the complex polarisability: an
    analytic pin of the complex semantics independent of the restatement."""
    L = 20.0
    box = np.full(3, L)
    x = np.array([[L / 2, L / 2, L / 2]])
    xi, tol = 0.5, 1e-10
    rc, Ng, _, P, _ = co.spectral_parameters(box, xi, tol)
    perp, para, rv = gcap.default_table(xi)
    phi = 4.0 * np.pi / (3.0 * L ** 3)
    for eps in (5.0 + 2.0j, 28.0 + 9.0j, 3.0 - 0.5j):
        s = SpectralEwaldSystem(x, np.array([eps]), box, xi, rc, Ng, P, perp, para, rv, slab_factor=0.0, max_rhs=1)
        m, info = s.solve(np.array([[0.0, 0.0, 1.0]], dtype=complex), None, tol=1e-12, restart=10, maxit=20,
                          precision="fp64")
        s.close()
        beta = (eps - 1.0) / (eps + 2.0)
        pred = 4.0 * np.pi * beta / (1.0 - beta * phi)
        m = m.cpu().numpy()[0]
        assert abs(m[2] - pred) <= 1e-7 * abs(pred), (eps, m[2], pred)
        assert abs(m[0]) + abs(m[1]) <= 1e-12 * abs(pred)
