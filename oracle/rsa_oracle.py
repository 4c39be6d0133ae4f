"""Pure-Python restatement of the seeded random-sequential-addition generator.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the CPU reference arm of
``bench.py`` places its particles with this, so that arm loads none of the
package's compiled libraries.  It restates the package's host generator
``mutual_polarization_slab_gb300/csrc/rsa_host.c`` (``mps_rsa``) step for step
-- xoshiro256** seeded through splitmix64, three uniform draws per trial
position, overlap test against the spheres of the 27 surrounding cells of a
grid whose edge is at least the largest contact distance -- so the same seed
gives the same positions (``tests/test_oracle_rsa.py`` checks this bit for bit).
"""
from __future__ import annotations

import math

import numpy as np

_M64 = (1 << 64) - 1


class _Xoshiro256ss:
    """xoshiro256** (Blackman and Vigna), state seeded by four splitmix64 outputs."""

    def __init__(self, seed: int):
        z = seed & _M64
        s = []
        for _ in range(4):
            z = (z + 0x9E3779B97F4A7C15) & _M64
            r = z
            r = ((r ^ (r >> 30)) * 0xBF58476D1CE4E5B9) & _M64
            r = ((r ^ (r >> 27)) * 0x94D049BB133111EB) & _M64
            s.append(r ^ (r >> 31))
        self.s = s

    def next(self) -> int:
        s0, s1, s2, s3 = self.s
        x = (s1 * 5) & _M64
        result = ((((x << 7) | (x >> 57)) & _M64) * 9) & _M64
        t = (s1 << 17) & _M64
        s2 ^= s0
        s3 ^= s1
        s1 ^= s2
        s0 ^= s3
        s2 ^= t
        s3 = ((s3 << 45) | (s3 >> 19)) & _M64
        self.s = [s0, s1, s2, s3]
        return result

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)


def rsa(n: int, phi: float, seed: int, radii=None, max_tries: int = 10_000_000):
    """Same arguments and result as ``mutual_polarization_slab_gb300.workloads.rsa``:
    ``(x (n,3), box (3,), radii (n,))`` for ``n`` spheres in a periodic cube at
    volume fraction ``phi``.  The order in which earlier spheres are tested does
    not change whether a trial position is accepted, so the cells' contents are
    tested through per-cell lists of (x, y, z, radius)."""
    rad = [1.0] * n if radii is None else [float(v) for v in np.asarray(radii, dtype=np.float64).reshape(n)]
    L = (4.0 * math.pi * float(np.sum(np.asarray(rad) ** 3)) / (3.0 * phi)) ** (1.0 / 3.0)
    Lx = Ly = Lz = L
    rmax = max(rad) if n else 1.0
    nx, ny, nz = (max(int(math.floor(v / (2.0 * rmax))), 3) for v in (Lx, Ly, Lz))
    cwx, cwy, cwz = Lx / nx, Ly / ny, Lz / nz
    hx, hy, hz = 0.5 * Lx, 0.5 * Ly, 0.5 * Lz
    cells = [[] for _ in range(nx * ny * nz)]
    nb27 = []
    for cz in range(nz):
        for cy in range(ny):
            for cx in range(nx):
                nb27.append([(((cz + e) % nz) * ny + (cy + b) % ny) * nx + (cx + a) % nx
                             for a in (-1, 0, 1) for b in (-1, 0, 1) for e in (-1, 0, 1)])
    st = _Xoshiro256ss(int(seed)).s
    s0, s1, s2, s3 = st
    M = _M64
    scale = 1.0 / 9007199254740992.0
    out = np.zeros((n, 3))
    for i in range(n):
        ri = rad[i]
        placed = False
        for _ in range(int(max_tries)):
            u = []
            for _k in range(3):     # three xoshiro256** draws, inlined
                x = (s1 * 5) & M
                u.append(((((((x << 7) | (x >> 57)) & M) * 9) & M) >> 11) * scale)
                t = (s1 << 17) & M
                s2 ^= s0
                s3 ^= s1
                s1 ^= s2
                s0 ^= s3
                s2 ^= t
                s3 = ((s3 << 45) | (s3 >> 19)) & M
            px, py, pz = u[0] * Lx, u[1] * Ly, u[2] * Lz
            cx, cy, cz = min(int(px / cwx), nx - 1), min(int(py / cwy), ny - 1), min(int(pz / cwz), nz - 1)
            home = (cz * ny + cy) * nx + cx
            ok = True
            for cc in nb27[home]:
                for qx, qy, qz, qr in cells[cc]:
                    dx = px - qx
                    if dx > hx:
                        dx -= Lx
                    elif dx < -hx:
                        dx += Lx
                    dy = py - qy
                    if dy > hy:
                        dy -= Ly
                    elif dy < -hy:
                        dy += Ly
                    dz = pz - qz
                    if dz > hz:
                        dz -= Lz
                    elif dz < -hz:
                        dz += Lz
                    cd = ri + qr
                    if dx * dx + dy * dy + dz * dz < cd * cd:
                        ok = False
                        break
                if not ok:
                    break
            if ok:
                cells[home].append((px, py, pz, ri))
                out[i] = (px, py, pz)
                placed = True
                break
        if not placed:
            raise RuntimeError(f"RSA failed: sphere {i} found no place in {max_tries} draws")
    return out, np.array([Lx, Ly, Lz]), np.asarray(rad)
