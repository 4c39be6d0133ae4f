"""The oracle's pure-Python random sequential addition (used by the CPU
reference arm of bench.py, which loads no compiled library of the package)
places the same spheres as the package's C generator, bit for bit."""
import numpy as np

from mutual_polarization_slab_gb300.workloads import rsa as c_rsa
from oracle.rsa_oracle import rsa as py_rsa


def test_python_rsa_matches_c_generator_bit_for_bit():
    for n, phi, seed in [(1500, 0.3, 2), (400, 0.35, 5)]:
        xp, bp, rp = py_rsa(n, phi, seed)
        xc, bc, rc = c_rsa(n, phi, seed)
        assert np.array_equal(xp, xc) and np.array_equal(bp, bc) and np.array_equal(rp, rc)
    radii = np.random.default_rng(4).uniform(0.7, 1.3, 600)
    xp, bp, _ = py_rsa(600, 0.25, 4, radii=radii)
    xc, bc, _ = c_rsa(600, 0.25, 4, radii=radii)
    assert np.array_equal(xp, xc) and np.array_equal(bp, bc)
