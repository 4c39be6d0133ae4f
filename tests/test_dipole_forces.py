"""Point-dipole pair forces (the HOOMD plugin kernel, _dipole_forces_ext.cpp):
the oracle against the reference's own compiled extension (golden vectors), and
the GPU kernel against both, plus the reference's diagnostic checks T1-T5
(force_energy_diagnostics.py:830-867) re-expressed without HOOMD."""
import os

import numpy as np
import pytest

from oracle import dipole_forces_oracle as dfo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def golden_forces():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_forces.npz")))


def test_oracle_matches_reference_extension(golden_forces):
    g = golden_forces
    for pz in (1, 0):
        F, e = dfo.compute_forces(g["pos"], g["dip"], g["box"], float(g["r_cut"]), float(g["pref"]), bool(pz))
        for cl in (1, 0):
            np.testing.assert_allclose(F, g[f"F_pz{pz}_cl{cl}"], rtol=0, atol=1e-13 * np.abs(F).max())
            np.testing.assert_allclose(e, g[f"pe_pz{pz}_cl{cl}"], rtol=0, atol=1e-13 * np.abs(e).max())


def test_oracle_rejects_large_cutoff():
    with pytest.raises(RuntimeError):
        dfo.compute_forces(np.zeros((2, 3)), np.ones((2, 3)), [10.0, 10.0, 10.0], 5.0)


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("CUDA device required")
    from mutual_polarization_slab_gb300 import dipole_forces
    return dipole_forces


@pytest.mark.gpu
def test_gpu_matches_reference(golden_forces):
    gf = _gpu()
    g = golden_forces
    for pz in (1, 0):
        F, e = gf.compute_forces(g["pos"], g["dip"], g["box"], float(g["r_cut"]), float(g["pref"]), bool(pz))
        np.testing.assert_allclose(F, g[f"F_pz{pz}_cl1"], rtol=0, atol=1e-12 * np.abs(F).max())
        np.testing.assert_allclose(e, g[f"pe_pz{pz}_cl1"], rtol=0, atol=1e-12 * np.abs(e).max())
        # momentum: forces sum to zero
        assert np.abs(F.sum(axis=0)).max() < 1e-10 * np.abs(F).max()


@pytest.mark.gpu
def test_gpu_diagnostics_t1_t5():
    gf = _gpu()
    box = np.array([20.0, 20.0, 20.0])

    def pair(r, mode, mu, pref):
        if mode == "head":   # dipoles along z, separated along z; "top" particle is index 1
            pos = np.array([[0, 0, -r / 2], [0, 0, r / 2]])
            comp = 2
        else:                # side by side along x, dipoles along z
            pos = np.array([[-r / 2, 0, 0], [r / 2, 0, 0]])
            comp = 0
        dip = np.array([[0, 0, mu], [0, 0, mu]], dtype=float)
        F, e = gf.compute_forces(pos, dip, box, 8.0, pref)
        return F[1, comp], e.sum()

    Fh, _ = pair(2.0, "head", 1.0, 1.0)
    assert Fh < 0                                               # T1 head-to-tail attracts
    Fs, _ = pair(2.0, "side", 1.0, 1.0)
    assert Fs > 0                                               # T2 side-by-side repels
    assert abs(pair(2.0, "head", 1.0, 3.0)[0] / Fh - 3.0) < 1e-12   # T3 prefactor linearity
    assert abs(pair(2.0, "head", 2.0, 1.0)[0] / Fh - 4.0) < 1e-12   # T4 mu^2 scaling
    dr = 1e-4                                                   # T5 F = -dU/dr
    Up = pair(2.0 + dr, "head", 1.0, 1.0)[1]
    Um = pair(2.0 - dr, "head", 1.0, 1.0)[1]
    ref = -(Up - Um) / (2 * dr)
    assert abs((Fh - ref) / ref) < 2e-3
    # point-dipole analytics: U = -2 m^2/r^3, F = -6 m^2/r^4 (head), pe split in half
    assert abs(Fh - (-6.0 / 16.0)) < 1e-14


@pytest.mark.gpu
def test_gpu_errors_and_empty():
    gf = _gpu()
    with pytest.raises(RuntimeError):
        gf.compute_forces(np.zeros((2, 3)), np.ones((2, 3)), [10.0, 10.0, 10.0], 5.0)
    F, e = gf.compute_forces(np.zeros((0, 3)), np.zeros((0, 3)), [10.0, 10.0, 10.0], 3.0)
    assert F.shape == (0, 3) and e.shape == (0,)
