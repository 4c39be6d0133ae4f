"""Seeded synthetic particle configurations (host-side input generation).

These stand in for the reference's lattice builders and hand-made
configurations (``CPU - Ewald test/test_driver_BCT110.py:39-116``,
``CPU - Ewald test/test_driver_scerrorrep2.py:22-45``): non-overlapping
random sequential addition (RSA) of spheres in a periodic cube, polydisperse
RSA, and a body-centred-tetragonal chain lattice with jitter and vacancies.
"""
from __future__ import annotations

import math

import numpy as np

_OFFS = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])


def box_for_fraction(n_particles: int, phi: float, radius: float = 1.0) -> float:
    """Cube edge giving volume fraction ``phi`` for ``n`` spheres of ``radius``."""
    return (4.0 * math.pi * n_particles * radius ** 3 / (3.0 * phi)) ** (1.0 / 3.0)


def rsa(n: int, phi: float, seed: int, radii=None, batch: int = 64, max_rounds: int = 2000):
    """Random sequential addition of spheres in a periodic cube.

    Particle ``i`` is placed at the first of ``batch`` uniformly drawn candidate
    positions that overlaps no earlier sphere (contact at ``a_i + a_j``); the
    check goes through a cell grid whose cell edge is at least the largest
    contact distance.  Returns ``(x, box, radii)`` with ``x`` in ``[0, L)``.
    """
    rng = np.random.default_rng(seed)
    radii = np.ones(n) if radii is None else np.asarray(radii, dtype=np.float64).reshape(n)
    L = (4.0 * math.pi * float(np.sum(radii ** 3)) / (3.0 * phi)) ** (1.0 / 3.0)
    nc = max(3, int(L // (2.0 * radii.max())))
    cw = L / nc
    cap = 24
    grid = np.full((nc, nc, nc, cap), -1, dtype=np.int64)
    fill = np.zeros((nc, nc, nc), dtype=np.int64)
    x = np.zeros((n, 3))
    for i in range(n):
        for _ in range(max_rounds):
            cand = rng.random((batch, 3)) * L
            ci = np.minimum((cand // cw).astype(np.int64), nc - 1)
            nb = (ci[:, None, :] + _OFFS[None]) % nc
            ids = grid[nb[..., 0], nb[..., 1], nb[..., 2]].reshape(batch, -1)
            valid = ids >= 0
            if not valid.any():
                c = 0
            else:
                safe = np.where(valid, ids, 0)
                d = cand[:, None, :] - x[safe]
                d -= L * np.round(d / L)
                bad = valid & (np.sum(d * d, axis=2) < (radii[safe] + radii[i]) ** 2)
                okc = np.nonzero(~bad.any(axis=1))[0]
                if okc.size == 0:
                    continue
                c = int(okc[0])
            x[i] = cand[c]
            cc = ci[c]
            s = fill[cc[0], cc[1], cc[2]]
            if s >= cap:
                raise RuntimeError("RSA cell capacity exceeded")
            grid[cc[0], cc[1], cc[2], s] = i
            fill[cc[0], cc[1], cc[2]] = s + 1
            break
        else:
            raise RuntimeError(f"RSA stalled at particle {i}/{n} (phi={phi})")
    return x, np.array([L, L, L]), radii


def bct_chain_lattice(ncx: int, ncy: int, ncz: int, vacancy: float, jitter: float, seed: int):
    """Body-centred-tetragonal chain lattice of touching unit spheres (c = 2,
    a = sqrt(6)), written in its face-centred setting: a sqrt(12) x sqrt(12) x 2
    cell with a 4-site basis, seeded Gaussian jitter and random vacancies."""
    rng = np.random.default_rng(seed)
    a = math.sqrt(12.0)
    basis = np.array([[0.0, 0.0, 0.0], [a / 2, a / 2, 0.0], [a / 2, 0.0, 1.0], [0.0, a / 2, 1.0]])
    cells = np.stack(np.meshgrid(np.arange(ncx), np.arange(ncy), np.arange(ncz), indexing="ij"), -1).reshape(-1, 3)
    x = (cells[:, None, :] * np.array([a, a, 2.0]) + basis[None]).reshape(-1, 3)
    keep = rng.random(x.shape[0]) >= vacancy
    x = x[keep] + rng.normal(0.0, jitter, size=(int(keep.sum()), 3))
    box = np.array([ncx * a, ncy * a, ncz * 2.0])
    return np.mod(x, box), box
