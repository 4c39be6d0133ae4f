"""GMRES step graphs against host-driven steps.

mps_gmres runs the Arnoldi steps of a cycle as one CUDA graph launch (a
while-conditional node; the step index, the frozen flags and the loop exit live
on the device).  The graph holds the same kernels in the same order as the
host-driven steps (MPS_GMRES_GRAPH=0), so solutions, residual estimates and
matvec counts must agree bit for bit, for every operator and precision: the
dipole operator in float64, double-float and mixed precision (reference-form
and gradient-form inner operators, with and without a coarser inner grid),
complex permittivities.  The quadrupole and polydisperse operators accumulate
with float64 atomics, which reorder sums from run to run: there the two forms
agree to rounding (1e-11) with the same matvec counts."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402
from mutual_polarization_slab_gb300 import quadrupole as gq  # noqa: E402
from mutual_polarization_slab_gb300 import sizes as gs  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402


def _run(make, b, graph, **kw):
    old = os.environ.get("MPS_GMRES_GRAPH")
    os.environ["MPS_GMRES_GRAPH"] = "1" if graph else "0"
    try:
        s = make()
        x, info = s.solve(b, None, **kw)
        torch.cuda.synchronize()
        out = (x.cpu().numpy(), [(i.converged, i.relres, i.matvecs_fp32, i.matvecs_fp64, i.cycles) for i in info],
               s.graphs())
        s.close()
    finally:
        if old is None:
            os.environ.pop("MPS_GMRES_GRAPH", None)
        else:
            os.environ["MPS_GMRES_GRAPH"] = old
    return out


def _same(make, b, exact=True, **kw):
    xg, ig, (built, failed) = _run(make, b, True, **kw)
    xh, ih, (built_h, _) = _run(make, b, False, **kw)
    assert failed == 0 and built >= 1
    assert built_h == 0
    assert all(c for c, *_ in ig)
    if exact:
        np.testing.assert_array_equal(xg, xh)
        assert ig == ih
    else:
        # float64 atomics in the operator reorder sums from run to run: agreement to rounding, same counts
        assert np.abs(xg - xh).max() <= 1e-11 * np.abs(xh).max()
        assert [i[2:] for i in ig] == [i[2:] for i in ih]


@pytest.fixture(scope="module")
def dipole():
    x, box, _ = rsa(2000, 0.25, seed=11)
    xi = 0.7
    perp, para, rv = gcap.default_table(xi)
    eps = np.full(2000, 12.0)

    def make(inner=None, e=eps):
        return SpectralEwaldSystem(x, e, box, xi, 5.0, (48, 48, 48), 8, perp, para, rv, slab_factor=1.0,
                                   max_rhs=3, inner=inner)

    b = np.zeros((3, 2000, 3))
    for k in range(3):
        b[k, :, k] = 1.0
    return make, b


@pytest.mark.parametrize("precision,inner_operator,inner", [
    ("fp64", "grad", None), ("df", "grad", None), ("mixed", "reference", None), ("mixed", "grad", None),
    ("mixed", "grad", ((40, 40, 40), 8))])
def test_dipole_graph_matches_host_steps(dipole, precision, inner_operator, inner):
    make, b = dipole
    tol = 1e-7 if precision == "mixed" else 1e-10
    _same(lambda: make(inner), b, tol=tol, restart=30, maxit=20, precision=precision, inner_operator=inner_operator)


def test_complex_permittivity_graph_matches_host_steps(dipole):
    make, b = dipole
    eps = np.full(2000, 12.0 + 3.0j)
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-7)):
        _same(lambda: make(None, eps), b.astype(complex), tol=tol, restart=30, maxit=20, precision=precision)


def _spheres(n, box, seed):
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < n:
        p = rng.random(3) * box
        d = p - np.array(pts).reshape(-1, 3)
        d -= box * np.round(d / box)
        if len(pts) == 0 or np.sqrt((d ** 2).sum(1)).min() > 2.05:
            pts.append(p)
    return np.array(pts)


def test_quadrupole_and_polydisperse_graph_match_host_steps():
    box = np.array([20.0, 20.0, 20.0])
    x = _spheres(60, box, 3)
    n = x.shape[0]
    lam = np.linspace(4.0, 30.0, n)
    bq = np.zeros((3, n, 8))
    for k in range(3):
        bq[k, :, k] = 1.0
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        _same(lambda: gq.QuadrupoleSystem(x, lam, box, 0.6, 1e-8, max_rhs=3), bq, exact=False, tol=tol, restart=30,
              maxit=20, precision=precision)
    radii = np.random.default_rng(4).uniform(0.6, 1.0, n)
    bp = np.zeros((3, n, 3))
    for k in range(3):
        bp[k, :, k] = 1.0
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        _same(lambda: gs.PolydisperseSystem(x, radii, lam, box, 0.6, 1e-8, max_rhs=3), bp, exact=False, tol=tol,
              restart=30, maxit=20, precision=precision)
