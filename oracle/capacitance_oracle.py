"""NumPy restatement of the dipole solve and the capacitance drivers (CPU oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``CPU - Ewald test/capacitance.py`` (cited ``EW/capacitance.py``) and the
MATLAB tensor / spectrum drivers of ``Capacitance_Hetero`` (cited ``CH/``).
"""
from __future__ import annotations

import math

import numpy as np

from . import ewald_oracle as ew

PI = math.pi


def spectral_parameters(box, xi, errortol):
    """rc, Ngrid, h, P, eta derived from one tolerance (EW/capacitance.py:357-362)."""
    box = np.asarray(box, dtype=np.float64).reshape(3)
    lt = math.sqrt(-math.log(errortol))
    rc = lt / xi
    kcut = 2.0 * xi * lt
    Ngrid = np.ceil(1.0 + box * kcut / PI).astype(np.int64)
    h = box / Ngrid
    P = int(math.ceil(-2.0 * math.log(errortol) / PI))
    eta = P * (h * xi) ** 2 / PI
    return rc, Ngrid, h, P, eta


def gmres(matvec, b, x0, tol, restart, maxit):
    """Restarted GMRES with modified Gram-Schmidt and Givens rotations.

    Same controls as the reference's ``gmres_restarted`` (EW/capacitance.py:60-199):
    ``maxit`` restart cycles of at most ``restart`` inner steps, stop when the
    (estimated) relative residual is <= tol; the iterate is updated at the end of
    each cycle from the least-squares solution.  Returns (x, flag, relres, nmatvec).
    """
    b = np.asarray(b)
    x = np.array(x0, dtype=np.result_type(b, x0), copy=True).reshape(-1)
    nb = float(np.linalg.norm(b))
    if nb == 0.0:
        return x, 0, 0.0, 0
    nmv = 0
    relres = math.inf
    for _ in range(int(maxit)):
        r = b - matvec(x)
        nmv += 1
        beta = float(np.linalg.norm(r))
        relres = beta / nb
        if relres <= tol:
            return x, 0, relres, nmv
        V = np.zeros((restart + 1, b.size), dtype=x.dtype)
        Hm = np.zeros((restart + 1, restart), dtype=x.dtype)
        cs = np.zeros(restart, dtype=x.dtype)
        sn = np.zeros(restart, dtype=x.dtype)
        g = np.zeros(restart + 1, dtype=x.dtype)
        g[0] = beta
        V[0] = r / beta
        k = 0
        for j in range(restart):
            w = matvec(V[j])
            nmv += 1
            for i in range(j + 1):
                Hm[i, j] = np.vdot(V[i], w)
                w = w - Hm[i, j] * V[i]
            Hm[j + 1, j] = np.linalg.norm(w)
            if Hm[j + 1, j] != 0:
                V[j + 1] = w / Hm[j + 1, j]
            for i in range(j):
                a0 = cs[i] * Hm[i, j] + sn[i] * Hm[i + 1, j]
                Hm[i + 1, j] = -np.conj(sn[i]) * Hm[i, j] + cs[i] * Hm[i + 1, j]
                Hm[i, j] = a0
            den = math.hypot(abs(Hm[j, j]), abs(Hm[j + 1, j]))
            cs[j], sn[j] = (1.0, 0.0) if den == 0 else (Hm[j, j] / den, Hm[j + 1, j] / den)
            Hm[j, j] = cs[j] * Hm[j, j] + sn[j] * Hm[j + 1, j]
            Hm[j + 1, j] = 0
            g[j + 1] = -np.conj(sn[j]) * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            if abs(g[j + 1]) / nb <= tol:
                break
        y = np.linalg.solve(np.triu(Hm[:k, :k]), g[:k])
        x = x + V[:k].T @ y
    r = b - matvec(x)
    nmv += 1
    relres = float(np.linalg.norm(r)) / nb
    return x, int(relres > tol), relres, nmv


def dilute_guess(eps_p, phi, Hhat):
    """Initial moments 4 pi beta / (1 - beta phi) Hhat with beta = (eps-1)/(eps+2),
    beta(eps = inf) = 1 (EW/capacitance.py:497-501)."""
    eps_p = np.asarray(eps_p, dtype=np.float64).reshape(-1)
    with np.errstate(invalid="ignore"):
        beta = (eps_p - 1.0) / (eps_p + 2.0)
    beta[np.isinf(eps_p)] = 1.0
    amp = 4.0 * PI * beta / (1.0 - beta * phi)
    return amp[:, None] * np.asarray(Hhat, dtype=np.float64).reshape(1, 3)


def solve_dipoles(geom, Hhat, guess, tol, restart, maxit, complex_pipeline=False):
    """A m = tile(Hhat, N) (EW/capacitance.py:205-321); returns ((N,3) moments, info dict)."""
    N = geom.x.shape[0]
    b = np.tile(np.asarray(Hhat, dtype=np.float64).reshape(3), N)
    if complex_pipeline:
        mv = lambda v: geom.field_complex(v.reshape(N, 3)).reshape(-1)
        b = b.astype(np.complex128)
        x0 = np.asarray(guess, dtype=np.complex128).reshape(-1)
    else:
        mv = lambda v: geom.field_real(v.reshape(N, 3)).reshape(-1)
        x0 = np.asarray(guess, dtype=np.float64).reshape(-1)
    x, flag, relres, nmv = gmres(mv, b, x0, tol, restart, maxit)
    return x.reshape(N, 3), {"flag": flag, "relres": relres, "matvecs": nmv}


def capacitance(x, lambdap, box, Sguess, xi, errortol, perp, para, rvals, Hhat,
                slab_factor=1.0, rc=None, Ngrid=None, P=None, restart=None, maxit=None, tol=None):
    """C = mean(S . Hhat) for one field direction (EW/capacitance.py:327-418).

    ``rc, Ngrid, P`` default to the tolerance-derived values; ``restart`` and
    ``maxit`` default to ``min(3N, 10)`` and ``min(3N, 100)`` (EW/capacitance.py:259-260).
    """
    x = np.asarray(x, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    N = x.shape[0]
    rc0, Ng0, _, P0, _ = spectral_parameters(box, xi, errortol)
    rc = rc0 if rc is None else float(rc)
    Ngrid = Ng0 if Ngrid is None else np.asarray(Ngrid, dtype=np.int64).reshape(3)
    P = P0 if P is None else int(P)
    if np.any(rc > box / 2.0):
        raise ValueError("Real-space cutoff exceeds half the box size; tolerance unmet.")
    geom = ew.Geometry(x, lambdap, box, xi, rc, Ngrid, P, perp, para, rvals, slab_factor)
    restart = min(3 * N, 10) if restart is None else int(restart)
    maxit = min(3 * N, 100) if maxit is None else int(maxit)
    S, info = solve_dipoles(geom, Hhat, Sguess, errortol if tol is None else tol, restart, maxit)
    return float(np.mean(S @ np.asarray(Hhat, dtype=np.float64))), S, info


def capacitance_tensor(geom, Sguess, tol, restart, maxit):
    """3x3 tensor from the unit fields along x, y, z; each solve warm-starts from
    the previous solution with its columns permuted [z, x, y]
    (CH/Capacitance_Tensor.m:23-59).  Row i of C is the mean moment for field i."""
    C = np.zeros((3, 3))
    S = np.zeros((geom.x.shape[0], 3, 3))
    guess = np.asarray(Sguess, dtype=np.float64)
    infos = []
    for i in range(3):
        Hhat = np.eye(3)[i]
        Si, info = solve_dipoles(geom, Hhat, guess, tol, restart, maxit)
        S[:, :, i] = Si
        C[i] = Si.mean(axis=0)
        guess = Si[:, [2, 0, 1]]
        infos.append(info)
    return C, S, infos
