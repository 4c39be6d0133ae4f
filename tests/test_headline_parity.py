"""Parity at the headline configuration itself: N = 100,000 unit spheres by
seeded random sequential addition at volume fraction 0.3 (seed 2), contrast
beta = 0.9 (eps = 28), 192^3 grid, P = 10, rc = (60 / 0.3)^(1/3) = 5.848,
xi = 4 / rc, fully periodic -- the workload bench.py times.

* one batch of three seeded random moment vectors through every GPU operator
  against the oracle's float64 operator (``Geometry.field_real``, the real part
  of ``EW/ewald.py:1146-1236``): float64 and double-float 1e-12, float32 of the
  reference discretisation 2e-5 (max-norm relative); the gradient form of the
  float32 operator differs from the reference discretisation by the sampling
  error of the Gaussian's derivative, 3e-5 relative in the 2-norm;
* the mixed-precision tensor solve (the headline solve, tol 1e-7, inner solves
  on the coarser inner grid) and a float64 GPU solve (tol 1e-11): their true
  residuals under the ORACLE operator,
  ||b - A_oracle m|| / ||b|| per field direction, and the mixed moments against
  the float64 ones (<= 1e-6, the mixed-precision bound)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402  (dilute_guess)
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402
from oracle import ewald_oracle as ew  # noqa: E402

N, PHI, SEED, BETA, GRID, P = 100_000, 0.3, 2, 0.9, 192, 10


@pytest.fixture(scope="module")
def headline():
    x, box, _ = rsa(N, PHI, seed=SEED)
    rc = (60.0 / PHI) ** (1.0 / 3.0)
    xi = 4.0 / rc
    eps = np.full(N, (1.0 + 2.0 * BETA) / (1.0 - BETA))
    perp, para, rv = ew.default_table(xi)
    geo = ew.Geometry(x, eps, box, xi, rc, [GRID] * 3, P, perp, para, rv, 0.0)
    # the oracle's own tables on both sides: the comparison is of the operators, not of two table builds
    # (the GPU's tables agree with the reference's to 1e-12 relative, tests/test_gpu_parity.py)
    s = SpectralEwaldSystem(x, eps, box, xi, rc, [GRID] * 3, P, perp, para, rv, slab_factor=0.0, max_rhs=3)
    # the headline solve's system: its mixed solve runs the inner operator on the coarser inner grid
    s_in = SpectralEwaldSystem(x, eps, box, xi, rc, [GRID] * 3, P, perp, para, rv, slab_factor=0.0, max_rhs=3,
                               inner="auto")
    yield dict(x=x, box=box, xi=xi, rc=rc, eps=eps, geo=geo, sys=s, sys_inner=s_in)
    s.close()
    s_in.close()


def _maxrel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_operators_against_oracle_at_headline_size(headline):
    s, geo = headline["sys"], headline["geo"]
    M = np.random.default_rng(101).standard_normal((3, N, 3))
    ref = geo.field_real_many(M)
    Md = torch.as_tensor(M, device="cuda")
    got = {p: s.matvec(Md, precision=p).cpu().numpy() for p in ("fp64", "df", "fp32", "fp32grad")}
    assert _maxrel(got["fp64"], ref) <= 1e-12
    assert _maxrel(got["df"], ref) <= 1e-12
    assert _maxrel(got["fp32"], ref) <= 2e-5
    grad_rel = float(np.linalg.norm(got["fp32grad"] - ref) / np.linalg.norm(ref))
    assert grad_rel <= 3e-5, grad_rel


def test_tensor_solves_true_residual_under_oracle(headline):
    s, geo = headline["sys"], headline["geo"]
    box = headline["box"]
    phi = 4.0 * math.pi * N / (3.0 * float(np.prod(box)))
    amp = torch.as_tensor(gcap.dilute_guess(headline["eps"], phi, [1.0, 0.0, 0.0])[:, 0], device="cuda")
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[:, None, :].expand(3, N, 3).contiguous()
    x0 = torch.stack([amp[:, None] * eye[i] for i in range(3)]).contiguous()
    assert headline["sys_inner"].inner is not None
    m_mix, info_mix = headline["sys_inner"].solve(b, x0, tol=1e-7, restart=30, maxit=8, precision="mixed",
                                                  inner_tol=1e-4, inner_maxit=3)
    m_64, info_64 = s.solve(b, x0, tol=1e-11, restart=30, maxit=100, precision="fp64")
    assert all(i.converged for i in info_mix) and all(i.converged for i in info_64)
    bh = b.cpu().numpy()
    for m, bound in ((m_mix.cpu().numpy(), 2e-7), (m_64.cpu().numpy(), 1e-10)):
        r = bh - geo.field_real_many(m)
        relres = [float(np.linalg.norm(r[i]) / np.linalg.norm(bh[i])) for i in range(3)]
        assert max(relres) <= bound, relres
    err = [float(torch.linalg.vector_norm(m_mix[i] - m_64[i]) / torch.linalg.vector_norm(m_64[i]))
           for i in range(3)]
    assert max(err) <= 1e-6, err
