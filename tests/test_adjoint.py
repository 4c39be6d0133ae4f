"""Adjoint forces and dE/d beta (GPU) against finite differences.

* operator derivative: F = -1/2 d(m^T A(x) m)/dx with m fixed, against a central
  difference of the oracle's m^T A m (h = 1e-7): 1e-6 of the largest force;
* full energy: F against central differences of E = -1/2 m.H0 re-solved at
  x +- h (h = 1e-4, tight float64 solves, tables at dr = 1e-5 so the slopes of
  the interpolated couplings match the smooth ones): 1e-5 relative;
* dE/d beta against central differences in beta (h = 1e-5): 1e-5 relative;
* two well-separated spheres: the adjoint force equals the reference's
  point-dipole kernel with prefactor 1/(4 pi) on the same moments to 2e-3
  (periodic images and the kernel's cutoff make the difference);
* the torch.autograd.Function and the Brownian-dynamics driver run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402
from mutual_polarization_slab_gb300 import ewald as gew  # noqa: E402
from mutual_polarization_slab_gb300 import forces as gf  # noqa: E402
from mutual_polarization_slab_gb300.dipole_forces import compute_forces  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402
from oracle import ewald_oracle as ew  # noqa: E402

XI, RC, NG, P = 0.6, 6.6, (48, 48, 48), 12


def dense_tables(xi, rmax, dr=1e-5):
    r = torch.arange(1, int(rmax / dr) + 2, dtype=torch.float64, device="cuda") * dr
    t = gew.real_space_table(r, xi)
    rv = torch.cat((torch.zeros(1, dtype=torch.float64, device="cuda"), r))
    return t[2], t[3], rv


@pytest.fixture(scope="module")
def config():
    x, box, _ = rsa(300, 0.15, seed=11)
    beta = np.where(np.arange(300) % 2 == 0, 0.9, 0.4)
    return x, box, beta


def test_operator_derivative_vs_oracle(config):
    x, box, beta = config
    eps = gf.eps_from_beta(beta)
    perp, para, rv = gcap.default_table(XI)
    s = SpectralEwaldSystem(x, eps, box, XI, RC, NG, P, perp, para, rv, slab_factor=0.0, max_rhs=1)
    m = np.random.default_rng(3).standard_normal((300, 3))
    F, _ = gf.adjoint_forces(s, m)
    F = F.cpu().numpy()
    s.close()
    pn, pa, rvn = ew.default_table(XI)

    def phi(xx):
        g = ew.Geometry(xx, eps, box, XI, RC, NG, P, pn, pa, rvn, slab_factor=0.0)
        return float(np.sum(m * g.field_real(m)))

    h = 1e-7      # well inside one table segment (dr = 1e-3) for almost every pair
    scale = np.abs(F).max()
    for k in (0, 7, 150):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[k, d] += h
            xm[k, d] -= h
            fd = -0.5 * (phi(xp) - phi(xm)) / (2 * h)
            assert abs(F[k, d] - fd) < 1e-6 * scale, (k, d, F[k, d], fd)


def _energy_var(x, beta, box, H0, tables, guess=None):
    """Variational form 1/2 m.A m - m.H0 of E = -1/2 m.H0: its error is quadratic
    in the solve's error, so the finite differences see the exact energy."""
    eps = gf.eps_from_beta(np.asarray(beta))
    s = SpectralEwaldSystem(x, eps, box, XI, RC, NG, P, *tables, slab_factor=0.0, max_rhs=1)
    h0 = torch.as_tensor(np.asarray(H0, dtype=np.float64), device="cuda")
    m, _ = s.solve(h0.repeat(x.shape[0], 1), guess, tol=1e-12, restart=30, maxit=200, precision="fp64")
    Am = s.matvec(m, precision="fp64")
    s.close()
    return float(0.5 * (m * Am).sum() - (m @ h0).sum())


def test_energy_forces_vs_finite_differences(config):
    x, box, beta = config
    tables = dense_tables(XI, RC + 0.5)
    H0 = [0.0, 0.0, 1.0]
    r0 = gf.polarization_energy(x, beta, box, H0, XI, RC, NG, P, tol=1e-13, tables=tables)
    assert abs(_energy_var(x, beta, box, H0, tables) - r0.energy) < 1e-10 * abs(r0.energy)
    F = r0.forces.cpu().numpy()
    h = 1e-4
    for k in (3, 100):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[k, d] += h
            xm[k, d] -= h
            fd = -(_energy_var(xp, beta, box, H0, tables, r0.moments)
                   - _energy_var(xm, beta, box, H0, tables, r0.moments)) / (2 * h)
            assert abs(F[k, d] - fd) <= 1e-5 * np.abs(F[k]).max(), (k, d, F[k, d], fd)
    dEdb = r0.dE_dbeta.cpu().numpy()
    hb = 1e-5
    for k in (5, 42):
        bp, bm = beta.copy(), beta.copy()
        bp[k] += hb
        bm[k] -= hb
        fd = (_energy_var(x, bp, box, H0, tables, r0.moments) - _energy_var(x, bm, box, H0, tables, r0.moments)) \
            / (2 * hb)
        assert abs(dEdb[k] - fd) <= 1e-5 * abs(fd), (k, dEdb[k], fd)


def test_two_spheres_match_point_dipole_kernel():
    box = np.array([40.0, 40.0, 40.0])
    x = np.array([[20.0, 20.0, 17.0], [20.0, 20.0, 23.0]])
    r = gf.polarization_energy(x, [0.75, 0.75], box, [0.0, 0.0, 1.0], 0.5, 9.0, (64, 64, 64), 12, tol=1e-13)
    F = r.forces.cpu().numpy()
    Fpd, _ = compute_forces(x, r.moments.cpu().numpy(), box, 15.0, 1.0 / (4 * np.pi), True)
    assert F[0, 2] > 0 and F[1, 2] < 0        # head-to-tail spheres attract
    np.testing.assert_allclose(F[:, 2], Fpd[:, 2], rtol=2e-3)


def test_autograd_function_and_bd(config):
    x, box, beta = config
    xt = torch.as_tensor(x, device="cuda").requires_grad_(True)
    bt = torch.as_tensor(beta, device="cuda").requires_grad_(True)
    params = dict(box=box, H0=[0.0, 0.0, 1.0], xi=XI, rc=RC, Ngrid=NG, P=P, tol=1e-12)
    E = gf.PolarizationEnergy.apply(xt, bt, params)
    E.backward()
    r = gf.polarization_energy(x, beta, box, [0.0, 0.0, 1.0], XI, RC, NG, P, tol=1e-12)
    assert abs(E.item() - r.energy) < 1e-12 * abs(r.energy)
    np.testing.assert_allclose(xt.grad.cpu().numpy(), -r.forces.cpu().numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(bt.grad.cpu().numpy(), r.dE_dbeta.cpu().numpy(), rtol=0, atol=1e-12)
    bd = gf.BrownianDynamics(x, beta, box, [0.0, 0.0, 1.0], XI, RC, NG, P, dt=1e-4, pol_every=2, seed=1)
    bd.run(4)
    assert bd.solves == 2 and bd.step_count == 4
    assert np.all(np.isfinite(bd.x.cpu().numpy())) and np.isfinite(bd.energy)


def test_cached_hoomd_style_force(config):
    x, box, beta = config
    drv = gf.MutualPolarizationDipoleForceCached(eps_p=10.0, xi=0.6, errtol=1e-6, slab_factor=0.0,
                                                 Hhat=[0.0, 0.0, 1.0], r_cut=6.0, prefactor=1.0,
                                                 field_strength=2.0, pol_every_steps=3)
    tags = np.arange(x.shape[0])
    for t in range(5):
        f, e = drv.set_forces(t, x, tags, box)
    assert drv.calls == 5 and drv.pol_solves == 2
    f2, e2 = compute_forces(x, drv.last_dipoles, box, 6.0, 1.0, True)
    np.testing.assert_allclose(f, f2)
    np.testing.assert_allclose(e, e2)
