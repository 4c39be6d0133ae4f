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


def _rsa_lib():
    import ctypes as C
    import os
    from . import _build
    if not os.path.exists(_build.RSA_LIB) or os.path.getmtime(_build.RSA_LIB) < os.path.getmtime(
            os.path.join(_build.CSRC, "rsa_host.c")):
        _build.build_host()
    lib = C.CDLL(_build.RSA_LIB)
    lib.mps_rsa.restype = C.c_int
    lib.mps_rsa.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int64, C.c_void_p]
    return lib


def rsa(n: int, phi: float, seed: int, radii=None, max_tries: int = 10_000_000):
    """Random sequential addition of ``n`` spheres in a periodic cube at volume
    fraction ``phi`` (host C routine ``mps_rsa`` in ``csrc/rsa_host.c``).

    Sphere i takes ``radii[i]`` (default 1) and is placed at the first uniformly
    drawn position overlapping no earlier sphere.  Returns ``(x, box, radii)``
    with ``x`` in ``[0, L)``.
    """
    import ctypes as C
    rad = np.ones(n) if radii is None else np.ascontiguousarray(np.asarray(radii, dtype=np.float64).reshape(n))
    L = (4.0 * math.pi * float(np.sum(rad ** 3)) / (3.0 * phi)) ** (1.0 / 3.0)
    box = np.array([L, L, L])
    x = np.zeros((n, 3))
    rc = _rsa_lib().mps_rsa(n, rad.ctypes.data_as(C.c_void_p), box.ctypes.data_as(C.c_void_p), int(seed),
                            int(max_tries), x.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise RuntimeError(f"RSA failed (code {rc}) for n={n}, phi={phi}")
    return x, box, rad


def bct_chain_lattice(ncx: int, ncy: int, ncz: int, vacancy: float, jitter: float, seed: int):
    """Body-centred-tetragonal chain lattice of touching unit spheres (c = 2,
    a = sqrt(6)), written in its face-centred setting: a sqrt(12) x sqrt(12) x 2
    cell with the 4-site basis (0,0,0), (0,1/2,1/2), (1/2,0,1/2), (1/2,1/2,0) in
    cell units, sites listed basis-major then by cell (x outer, z inner) as
    ``CPU - Ewald test/test_driver_BCT110.py:74-95`` does, then seeded random
    vacancies and Gaussian jitter.  Returns (positions wrapped into the box, box)."""
    rng = np.random.default_rng(seed)
    a = math.sqrt(12.0)
    cell = np.array([a, a, 2.0])
    basis = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
    cells = np.stack(np.meshgrid(np.arange(ncx), np.arange(ncy), np.arange(ncz), indexing="ij"), -1).reshape(-1, 3)
    x = ((cells[None, :, :] + basis[:, None, :]) * cell).reshape(-1, 3)
    keep = rng.random(x.shape[0]) >= vacancy
    x = x[keep] + rng.normal(0.0, jitter, size=(int(keep.sum()), 3))
    box = np.array([ncx * a, ncy * a, ncz * 2.0])
    return np.mod(x, box), box
