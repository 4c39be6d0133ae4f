"""Gradient form of the float32 operator (precision 'fp32grad', the optional inner
operator of the mixed solve).

* against a NumPy statement of the same formulation (rho = sum m.grad w on one
  grid, scale H/|k|^2, contraction with grad w): 2e-5, the float32 bar;
* against the reference operator (float64): the formulation's own
  discretisation difference, below 1e-4 here;
* the mixed solve with inner_operator='grad' converges to the float64 solution
  of the reference operator (the refinement residual is the reference operator).
"""
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


def grad_form_numpy(g, m):
    """Wave part of the gradient formulation on an oracle Geometry, plus its real part."""
    n = g.x.shape[0]
    P = g.P
    lo = (P - 1) // 2
    offs = np.arange(P ** 3)
    off = np.stack((offs % P - lo, (offs // P) % P - lo, offs // (P * P) - lo), axis=1)
    node0 = ew.matlab_round(g.x / g.h)
    r = (node0[:, None, :] + off[None]) * g.h - g.x[:, None, :]
    gr = -(4 * g.xi ** 2 / g.eta)[None, None, :] * r * g.w[:, :, None]
    G = int(np.prod(g.Ngrid))
    rho = np.bincount(g.lin.reshape(-1), np.einsum("npc,nc->np", gr, m).reshape(-1), minlength=G)
    nx, ny, nz = (int(v) for v in g.Ngrid)
    k, Hc = ew.kspace_unshifted(g.Ngrid, g.box, g.xi, g.eta)
    k2 = np.sum(k * k, axis=3).transpose(2, 1, 0)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(k2 > 0, Hc.transpose(2, 1, 0) / k2, 0.0)
    phi = np.fft.ifftn(np.fft.fftn(rho.reshape(nz, ny, nx)) * s).real.reshape(-1)
    E = np.prod(g.h) * np.einsum("npc,np->nc", gr, phi[g.lin])
    Hr = ew.real_space_fast(m.astype(complex), g.lambdap, *g.pairs, g.perp[0]).real
    return E + Hr


@pytest.mark.parametrize("Ngrid", [(48, 48, 48), (50, 45, 40)])
def test_grad_matvec(Ngrid):
    x, box, _ = rsa(600, 0.25, seed=4)
    eps = np.full(600, 19.0)
    xi, rc, P = 0.7, 5.5, 10
    perp, para, rv = gcap.default_table(xi)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, Ngrid, P, perp, para, rv, slab_factor=0.0, max_rhs=3)
    m = np.random.default_rng(2).standard_normal((3, 600, 3))
    og = s.matvec(m, precision="fp32grad").cpu().numpy()
    o64 = s.matvec(m, precision="fp64").cpu().numpy()
    pn, pa, rvn = ew.default_table(xi)
    g = ew.Geometry(x, eps, box, xi, rc, Ngrid, P, pn, pa, rvn, slab_factor=0.0)
    ref = grad_form_numpy(g, m[1])
    assert np.abs(og[1] - ref).max() / np.abs(ref).max() < 2e-5
    assert np.linalg.norm(og - o64) / np.linalg.norm(o64) < 1e-4
    s.close()


def test_mixed_solve_with_grad_inner_operator():
    x, box, _ = rsa(600, 0.25, seed=4)
    eps = np.full(600, 19.0)
    xi, rc, P = 0.7, 5.5, 10
    perp, para, rv = gcap.default_table(xi)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, (48, 48, 48), P, perp, para, rv, slab_factor=0.0, max_rhs=3)
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[:, None, :].expand(3, 600, 3).contiguous()
    ref, _ = s.solve(b, None, tol=1e-12, restart=30, maxit=50, precision="fp64")
    sol, info = s.solve(b, None, tol=1e-8, restart=30, maxit=10, precision="mixed", inner_operator="grad",
                        verify=True)
    assert all(i.converged for i in info)
    for r in range(3):
        assert float(torch.linalg.vector_norm(sol[r] - ref[r]) / torch.linalg.vector_norm(ref[r])) < 1e-6
    s.close()


@pytest.mark.parametrize("nrhs,Ngrid", [(1, (51, 47, 45)), (2, (51, 47, 45)), (3, (51, 47, 45)), (3, (16, 17, 16))])
def test_grad_kernel_forms_agree(monkeypatch, nrhs, Ngrid):
    """The staged home-block contraction (default) and the warp gather from L2
    give bit-identical operators (the same sums in the same order); the tiled
    contraction agrees to float32 rounding.  For 1-3 vectors, a grid with odd
    sizes (partial home blocks) and a grid barely above the support, where a
    block's staged region is longer than the grid's axis (nodes staged twice);
    the operator is deterministic."""
    x, box, _ = rsa(900, 0.25, seed=7)
    eps = np.full(900, 19.0)
    xi, rc, P = 0.7, 5.5, 10
    perp, para, rv = gcap.default_table(xi)
    # the tiled contraction runs on depth-8 tiles (the default spread depth, 12, has none)
    monkeypatch.setenv("MPS_TILE_DEPTH", "8")
    s = SpectralEwaldSystem(x, eps, box, xi, rc, Ngrid, P, perp, para, rv, slab_factor=0.0, max_rhs=3)
    m = np.random.default_rng(5).standard_normal((nrhs, 900, 3))
    home = s.matvec(m, precision="fp32grad").cpu().numpy()
    assert s.tuning()["fp32"]["tile"][2] == 8
    monkeypatch.setenv("MPS_GRAD_CONTRACT", "warp")
    warp = s.matvec(m, precision="fp32grad").cpu().numpy()
    assert np.array_equal(home, warp)
    monkeypatch.setenv("MPS_GRAD_CONTRACT", "tiled")
    tiled = s.matvec(m, precision="fp32grad").cpu().numpy()
    assert np.linalg.norm(home - tiled) / np.linalg.norm(tiled) < 2e-6
    monkeypatch.delenv("MPS_GRAD_CONTRACT")
    again = s.matvec(m, precision="fp32grad").cpu().numpy()
    assert np.array_equal(again, home)          # deterministic
    s.close()


def test_inner_grid_operator_and_mixed_solve():
    """The gradient-form operator on a system's own coarser inner grid is the
    gradient form of that grid (NumPy statement on an oracle geometry at the
    inner grid and support, 2e-5); the mixed solve whose inner solves run on it
    converges to the float64 solution of the system's own operator (1e-6)."""
    n = 600
    x, box, _ = rsa(n, 0.25, seed=4)
    eps = np.full(n, 19.0)
    xi, rc, P = 0.7, 5.5, 10
    perp, para, rv = gcap.default_table(xi)
    inner = (np.array([32, 30, 36]), 10)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, (48, 48, 48), P, perp, para, rv, slab_factor=0.0, max_rhs=3,
                            inner=inner)
    m = np.random.default_rng(2).standard_normal((3, n, 3))
    og = s.matvec(m, precision="fp32grad").cpu().numpy()
    pn, pa, rvn = ew.default_table(xi)
    g_in = ew.Geometry(x, eps, box, xi, rc, inner[0], inner[1], pn, pa, rvn, slab_factor=0.0)
    ref = grad_form_numpy(g_in, m[2])
    assert np.abs(og[2] - ref).max() / np.abs(ref).max() < 2e-5
    o64 = s.matvec(m, precision="fp64").cpu().numpy()
    assert np.linalg.norm(og - o64) / np.linalg.norm(o64) < 2e-3
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[:, None, :].expand(3, n, 3).contiguous()
    ref_sol, _ = s.solve(b, None, tol=1e-12, restart=30, maxit=50, precision="fp64")
    sol, info = s.solve(b, None, tol=1e-8, restart=30, maxit=10, precision="mixed", inner_operator="grad")
    assert all(i.converged for i in info)
    for r in range(3):
        assert float(torch.linalg.vector_norm(sol[r] - ref_sol[r]) / torch.linalg.vector_norm(ref_sol[r])) < 1e-6
    s.close()
