"""Surface energy of a slab from capacitances at two box heights.

Drop-in for ``CPU - Ewald test/surface_energy.py`` (``surface_energy_from_two_separations``,
lines 20-68) and the post-processing of the BCT(110) slab driver
(``CPU - Ewald test/test_driver_BCT110.py``: ``build_bct_110_slab`` :39-116 and the
height scan of ``main`` :119-170).  The capacitances come from this package's
``run_capacitance`` (the GPU solve); everything else is host arithmetic on a
handful of numbers.

The slab normal is the solver's z axis: the slab term (``slab_factor``) of the
operator acts along z, and vacuum is added by stretching ``L[2]`` to
``L0[2] * (1 + h)``.  ``build_bct_110_slab(permute_for_solver=True)`` maps the
physical slab normal (x) to solver z.
"""
from __future__ import annotations

import numpy as np

from .capacitance import run_capacitance

__all__ = ["surface_energy_from_two_separations", "build_bct_110_slab", "surface_energy_scan"]


def _capacitance(x, L, eps_p, xi, Hhat, slab_factor, verbose, solver):
    n = x.shape[0]
    C, _ = run_capacitance(x, L, eps_p * np.ones((n,), dtype=np.float64), xi, Hhat, slab_factor=slab_factor,
                           verbose=verbose, **solver)
    return float(np.real(np.asarray(C).reshape(-1)[0]))


def surface_energy_from_two_separations(xyz, Lbox, epsp, xi, Hhat, hsep, slab_factor=1.0, verbose=0, **solver):
    """Nondimensional surface energy u_S / p_B^2 from two capacitance solves
    (``surface_energy.py:20-68``).

    The box height is ``Lbox[2] * (1 + hsep[j])`` for the two entries of ``hsep``;
    U_j = -C_j N / 2, u_S = (U_1 - U_0) / (2 A) with A = Lbox[0] Lbox[1], and
    p_B = C_0 / sqrt(4 pi).  ``solver`` keywords go to ``run_capacitance``
    (``precision='mixed'``, ``rc=``, ``Ngrid=``, ...).  Raises ``ValueError``
    unless ``hsep`` has exactly two entries, as the reference does."""
    xyz = np.asarray(xyz, dtype=np.float64)
    Lbox = np.asarray(Lbox, dtype=np.float64).reshape(3)
    Hhat = np.asarray(Hhat, dtype=np.float64).reshape(3)
    hsep = np.asarray(hsep, dtype=np.float64).reshape(-1)
    if hsep.size != 2:
        raise ValueError("hsep must have exactly two entries (e.g., [0, 2]).")
    n = xyz.shape[0]
    area = float(Lbox[0] * Lbox[1])
    C = np.zeros(2, dtype=np.float64)
    for j in range(2):
        L = Lbox.copy()
        L[2] = L[2] + hsep[j] * Lbox[2]
        C[j] = _capacitance(xyz, L, epsp, xi, Hhat, slab_factor, verbose, solver)
    U = -0.5 * C * float(n)
    uS = (U[1] - U[0]) / (2.0 * area)
    pB = C[0] / np.sqrt(4.0 * np.pi)
    return float(uS / pB ** 2)


def build_bct_110_slab(numCells=8, permute_for_solver=True):
    """BCT lattice with lattice vectors (sqrt 12, 0, 0), (0, sqrt 12, 0), (0, 0, 2)
    and the 4-site face-centred basis, numCells^3 cells (``test_driver_BCT110.py:39-116``).

    Returns positions (N, 3), box lengths (3,) and the slab face area A (the
    physical yz area).  With ``permute_for_solver`` the axes are permuted
    (x, y, z)_solver = (z, y, x)_physical so that the slab normal is solver z;
    A is then the solver's Lx * Ly."""
    lat = np.array([np.sqrt(12.0), np.sqrt(12.0), 2.0])
    basis = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
    k = np.arange(numCells, dtype=np.float64)
    # basis-major, then cell indices a (x), b (y), c (z) with c fastest: the reference's emission order
    cells = np.stack(np.meshgrid(k, k, k, indexing="ij"), axis=-1).reshape(-1, 3)
    x = ((basis[:, None, :] + cells[None, :, :]) * lat).reshape(-1, 3)
    L0 = numCells * lat
    area = float(L0[1] * L0[2])
    if not permute_for_solver:
        return x, L0, area
    return x[:, [2, 1, 0]].copy(), L0[[2, 1, 0]].copy(), area


def surface_energy_scan(x, L0, area, betas, h, xi, H0, slab_factor=1.0, verbose=0, **solver):
    """u_S(h) / p_B^2 for every contrast beta and stretch h (``test_driver_BCT110.py:119-170``):
    C at each height L0[2] (1 + h_j), U = -C N / 2, u_S(h) = (U - U(h_0)) / (2 A),
    divided by p_B^2 = (C(h_0) / sqrt(4 pi))^2.  Returns (len(betas), len(h))."""
    x = np.asarray(x, dtype=np.float64)
    L0 = np.asarray(L0, dtype=np.float64).reshape(3)
    betas = np.asarray(betas, dtype=np.float64).reshape(-1)
    h = np.asarray(h, dtype=np.float64).reshape(-1)
    n = x.shape[0]
    surfs = np.zeros((betas.size, h.size), dtype=np.float64)
    for i, beta in enumerate(betas):
        eps_p = (1.0 + 2.0 * beta) / (1.0 - beta)
        C = np.zeros(h.size, dtype=np.float64)
        for j, hj in enumerate(h):
            L = L0.copy()
            L[2] = L0[2] + hj * L0[2]
            C[j] = _capacitance(x, L, eps_p, xi, H0, slab_factor, verbose, solver)
        U = -0.5 * C * float(n)
        pB = C[0] / np.sqrt(4.0 * np.pi)
        surfs[i] = (U - U[0]) / (2.0 * area) / pB ** 2
    return surfs
