"""Host-side parameter rules (CPU): the tolerance rule that turns one error
tolerance into cutoff, grid, support and Gaussian widths (capacitance.py:357-362
in the reference's Python path), and the coarser grid the mixed solve gives its
float32 inner operator."""
import math

import numpy as np
import pytest

pytest.importorskip("torch")

from mutual_polarization_slab_gb300 import system as S  # noqa: E402


def test_spectral_parameters_match_the_golden_case(golden_small):
    g = golden_small
    rc, Ngrid, h, P, eta = S.spectral_parameters(g["box"], float(g["xi"]), float(g["tol"]))
    assert rc == pytest.approx(float(g["rc"]), rel=1e-15)
    assert np.array_equal(Ngrid, g["Ngrid"]) and P == int(g["P"])
    np.testing.assert_allclose(h, g["h"], rtol=1e-15)
    np.testing.assert_allclose(eta, g["eta"], rtol=1e-14)


def _smooth_with_few_odd_factors(m):
    b = c = 0
    while m % 2 == 0:
        m //= 2
    while m % 3 == 0:
        m //= 3
        b += 1
    while m % 5 == 0:
        m //= 5
        c += 1
    return m == 1 and b + c <= 2


def test_fast_sizes():
    for n in range(1, 400):
        m = S._fast_size(n)
        assert m >= n and _smooth_with_few_odd_factors(m)
        assert not any(_smooth_with_few_odd_factors(k) for k in range(n, m))   # the smallest such size


def test_inner_grid_of_the_measured_workloads():
    """N = 1e5 at phi = 0.3 on 192^3 gets 144^3; N = 2e5 at phi = 0.35 on 240^3
    gets 192^3 (both with the system's support P = 10); small grids keep their own."""
    for n, phi, ng, want in ((100_000, 0.3, 192, 144), (200_000, 0.35, 240, 192)):
        L = (4 * math.pi * n / (3 * phi)) ** (1 / 3)
        xi = 4 / (60 / phi) ** (1 / 3)
        got = S.inner_grid([L] * 3, xi, [ng] * 3, 10)
        assert got is not None
        assert list(got[0]) == [want] * 3 and got[1] == 10
    assert S.inner_grid([30.0] * 3, 0.6, [64] * 3, 8) is None           # below 128^3
    L = (4 * math.pi * 1e5 / (3 * 0.3)) ** (1 / 3)
    assert S.inner_grid([L] * 3, 4 / 5.848, [150] * 3, 10) is None      # not clearly smaller than the grid
