"""Drop-in for the reference module ``CPU - Ewald test/capacitance.py`` plus the
capacitance-tensor and spectrum drivers of the MATLAB variant
(``Capacitance_Hetero/Capacitance_Tensor.m``, ``CapacitanceTensorSpectrum.m``).

The solve runs on the GPU: ``SpectralEwaldSystem`` builds the geometry once per
configuration and ``mps_gmres`` runs restarted GMRES with batched matvecs.
Keyword-only extras (not in the reference): ``rc, Ngrid, P`` overrides of the
tolerance-derived parameters, ``restart, maxit`` overrides of the GMRES
controls, and ``precision='fp64' | 'mixed'``.

The GPU operator is real: it equals the real part of the reference's complex
FFT pipeline applied to real moments (the reference's imaginary parts come only
from the unpaired Nyquist bins of even grids and stay at round-off level).
Moments are returned as complex128 arrays with zero imaginary part, like the
reference's dtype.
"""
from __future__ import annotations

import math
import time
from typing import Callable, Tuple

import numpy as np
import torch

from . import ewald
from .system import SpectralEwaldSystem, as_device, spectral_parameters, to_host

__all__ = ["gmres_restarted", "magnetic_dipole", "capacitance", "run_capacitance", "capacitance_tensor",
           "capacitance_tensor_spectrum", "dilute_guess", "default_table"]

_REALSPACE_TABLE_CACHE: dict = {}


def default_table(xi):
    """r = 0.001..10 step 0.001 with 0 prepended and its two field/dipole tables,
    cached per xi (capacitance.py:471-477) and per device (a system reads them on
    its own device).  Returns device tensors (perp, para, rvals) on the current device."""
    key = (float(xi), torch.cuda.current_device())
    if key not in _REALSPACE_TABLE_CACHE:
        r = np.arange(0.001, 10.0 + 1e-12, 0.001, dtype=np.float64)
        tabs = ewald.real_space_table(torch.as_tensor(r, device="cuda"), float(xi))
        rv = torch.cat((torch.zeros(1, dtype=torch.float64, device="cuda"), torch.as_tensor(r, device="cuda")))
        _REALSPACE_TABLE_CACHE[key] = (tabs[2], tabs[3], rv)
    return _REALSPACE_TABLE_CACHE[key]


def dilute_guess(eps_p, phi, Hhat):
    """4 pi beta / (1 - beta phi) Hhat, beta = (eps-1)/(eps+2), beta(inf) = 1 (capacitance.py:497-501)."""
    eps = np.asarray(eps_p)
    eps = eps.astype(np.complex128 if np.iscomplexobj(eps) else np.float64).reshape(-1)
    with np.errstate(invalid="ignore"):
        beta = (eps - 1.0) / (eps + 2.0)
    beta[np.isinf(eps)] = 1.0
    amp = 4.0 * np.pi * beta / (1.0 - beta * phi)
    return amp[:, None] * np.asarray(Hhat, dtype=np.float64).reshape(1, 3)


def gmres_restarted(matvec: Callable, b, x0, tol: float, restart: int, maxit: int, verbose: int = 0):
    """Restarted GMRES for a caller's matvec (the reference's ``gmres_restarted``,
    ``CPU - Ewald test/capacitance.py:60-199``): same arguments, same return value
    ``(x, flag, relres)`` (flag 0 when ``||b - A x|| / ||b|| <= tol``).

    Each cycle builds a Krylov basis on the GPU (modified Gram-Schmidt, complex
    Givens rotations for the small least-squares problem) and ends with the
    cycle's best iterate: the least-squares solution over the columns up to the
    last strict drop of the residual estimate; when no column improved on the
    cycle's start, over all of them.  numpy in, numpy out; CUDA tensors stay on
    the device."""
    on_host = not isinstance(b, torch.Tensor)
    rhs = as_device(b, torch.complex128).reshape(-1)
    sol = as_device(x0, torch.complex128).reshape(-1).clone()
    bnorm = torch.linalg.vector_norm(rhs).item()

    def result(flag, rr):
        return (sol.cpu().numpy() if on_host else sol), flag, rr

    if bnorm == 0.0:
        return result(0, 0.0)

    def apply(v):
        return as_device(matvec(v.cpu().numpy() if on_host else v), torch.complex128).reshape(-1)

    started = time.perf_counter()
    n_apply = 0
    for cycle in range(int(maxit)):
        resid = rhs - apply(sol)
        n_apply += 1
        rnorm = torch.linalg.vector_norm(resid).item()
        if verbose >= 2:
            print(f"    [gmres] cycle {cycle + 1} of {maxit}: relative residual {rnorm / bnorm:.3e}", flush=True)
        if rnorm / bnorm <= tol:
            if verbose >= 1:
                print(f"    [gmres] converged: relative residual {rnorm / bnorm:.3e}, {cycle + 1} cycles, "
                      f"{n_apply} matvecs, {time.perf_counter() - started:.2f} s", flush=True)
            return result(0, rnorm / bnorm)
        basis = [resid / rnorm]
        hess = np.zeros((restart + 1, restart), dtype=np.complex128)   # rotated in place: upper triangle
        rot = []                                                          # (c, s) of each Givens rotation
        proj = np.zeros(restart + 1, dtype=np.complex128)                 # rotated projection of the residual
        proj[0] = rnorm
        best_est, best_cols, done_cols, hit = rnorm / bnorm, 0, 0, False
        for col in range(restart):
            w = apply(basis[col])
            n_apply += 1
            for i, v in enumerate(basis):                                 # modified Gram-Schmidt
                hess[i, col] = torch.vdot(v, w).item()
                w = w - hess[i, col] * v
            wn = torch.linalg.vector_norm(w).item()
            hess[col + 1, col] = wn
            basis.append(w / wn if wn != 0.0 else torch.zeros_like(w))
            for i, (c, sg) in enumerate(rot):                             # earlier rotations on the new column
                top, bot = hess[i, col], hess[i + 1, col]
                hess[i, col] = c * top + sg * bot
                hess[i + 1, col] = -np.conj(sg) * top + c * bot
            # complex Givens rotation with a real cosine, c = |top| / rho, s = (top / |top|) conj(bot) / rho: unitary
            # for complex entries too (for real data it agrees with the reference's c = top / rho up to a common
            # sign, which leaves the least-squares solution unchanged)
            top, bot = hess[col, col], hess[col + 1, col]
            scale = math.hypot(abs(top), abs(bot))
            if scale == 0.0:
                c, sg = 1.0, 0.0
            elif top == 0:
                c, sg = 0.0, np.conj(bot) / abs(bot)
            else:
                c, sg = abs(top) / scale, (top / abs(top)) * np.conj(bot) / scale
            rot.append((c, sg))
            hess[col, col] = c * top + sg * bot
            hess[col + 1, col] = 0.0
            proj[col], proj[col + 1] = c * proj[col], -np.conj(sg) * proj[col]
            done_cols = col + 1
            est = abs(proj[col + 1]) / bnorm
            if verbose >= 3:
                print(f"      [gmres] step {col + 1}: estimated residual {est:.3e}", flush=True)
            if est < best_est:
                best_est, best_cols = est, col + 1
            if est <= tol:
                hit = True
                break
        k = done_cols if hit else (best_cols or done_cols)
        coef = np.linalg.lstsq(hess[:k, :k], proj[:k], rcond=None)[0]
        sol = sol + (torch.as_tensor(coef, device=sol.device)[:, None] * torch.stack(basis[:k])).sum(dim=0)
    resid = rhs - apply(sol)
    n_apply += 1
    rr = torch.linalg.vector_norm(resid).item() / bnorm
    if verbose >= 1:
        print(f"    [gmres] not converged: relative residual {rr:.3e} after {maxit} cycles, {n_apply} matvecs, "
              f"{time.perf_counter() - started:.2f} s", flush=True)
    return result(1, rr)


def _np_or_t(t, asnp):
    return to_host(t) if asnp else t


def _inner(precision, inner_operator, inner_grid):
    """The system's inner discretisation: ``inner_grid`` ("auto", None or (Ngrid, P)) matters only for the
    mixed solve with the gradient-form inner operator."""
    return inner_grid if precision == "mixed" and inner_operator == "grad" else None


def magnetic_dipole(x, lambdap, H, box, p1, p2, Ngrid, h, P, xi, eta, rc, mold, offset, offsetxyz, Hperp, Hpara,
                    rvals, errortol, real_precomp=None, grid_precomp=None, k_precomp=None, slab_factor=1.0,
                    use_scipy_gmres=True, verbose=0, *, restart=None, maxit=None, precision="fp64",
                    inner_tol=1e-4, inner_maxit=4, system=None, return_info=False, inner_grid="auto"):
    """Solve A m = tile(H, N) for the moments (capacitance.py:205-321) on the GPU.

    ``restart`` / ``maxit`` default to the reference's ``min(3N, 10)`` /
    ``min(3N, 100)``; ``precision='mixed'`` runs float64 iterative refinement
    with float32-operator GMRES corrections (``maxit`` then counts refinement
    steps).  ``use_scipy_gmres`` chooses, in the reference, between SciPy's
    ``gmres`` and its own ``gmres_restarted``; both are restarted GMRES with the
    same relative-residual stopping rule, and here both choices run the device
    GMRES (``mps_gmres``), which keeps each cycle's best iterate like
    ``gmres_restarted``.  Returns (N,3) complex128 (numpy in, numpy out)."""
    asnp = not isinstance(x, torch.Tensor)
    xd = as_device(x).reshape(-1, 3)
    N = xd.shape[0]
    sysm = system or SpectralEwaldSystem(xd, lambdap, box, xi, rc, Ngrid, P, Hperp, Hpara, rvals,
                                         slab_factor=slab_factor, eta=eta, max_rhs=1,
                                         inner=_inner(precision, "grad", inner_grid))
    Hv = torch.as_tensor(np.real(np.asarray(H.cpu() if isinstance(H, torch.Tensor) else H)).astype(np.float64).reshape(3),
                         device="cuda")
    b = Hv.repeat(N, 1)
    mold_t = as_device(np.real(mold) if not isinstance(mold, torch.Tensor) else mold.real).reshape(N, 3)
    restart = min(3 * N, 10) if restart is None else int(restart)
    maxit = min(3 * N, 100) if maxit is None else int(maxit)
    sol, info = sysm.solve(b, mold_t, tol=float(errortol), restart=restart, maxit=maxit, precision=precision,
                           inner_tol=inner_tol, inner_maxit=inner_maxit)
    if verbose >= 1:
        print(f"  MagneticDipole(GPU {precision}): converged={info[0].converged} relres={info[0].relres:.3e} "
              f"matvecs fp64={info[0].matvecs_fp64} fp32={info[0].matvecs_fp32}", flush=True)
    out = torch.complex(sol, torch.zeros_like(sol))
    res = _np_or_t(out, asnp)
    return (res, info[0]) if return_info else res


def _resolve_params(box, xi, errortol, rc, Ngrid, P):
    rc0, Ng0, _, P0, _ = spectral_parameters(box, xi, errortol)
    rc = rc0 if rc is None else float(rc)
    Ngrid = Ng0 if Ngrid is None else np.asarray(Ngrid, dtype=np.int64).reshape(3)
    P = P0 if P is None else int(P)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    h = box / Ngrid
    eta = P * (h * xi) ** 2 / math.pi
    return rc, Ngrid, h, P, eta


def capacitance(x, lambdap, box, Sguess, xi, errortol, dipoletable1, dipoletable2, rtable, offset, offsetxyz, Hhat,
                slab_factor=1.0, use_scipy_gmres=True, verbose=0, *, rc=None, Ngrid=None, P=None, restart=None,
                maxit=None, precision="fp64", inner_tol=1e-4, inner_maxit=4, inner_grid="auto"):
    """Induced dipoles and C = mean(S . Hhat) for one field direction (capacitance.py:327-418)."""
    asnp = not isinstance(x, torch.Tensor)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = _resolve_params(box, xi, errortol, rc, Ngrid, P)
    if np.any(rc > box / 2.0):
        raise ValueError("Real-space cutoff exceeds half the box size; tolerance unmet.")
    t0 = time.perf_counter()
    sysm = SpectralEwaldSystem(x, lambdap, box, xi, rc, Ngrid, P, dipoletable1, dipoletable2, rtable,
                               slab_factor=slab_factor, eta=eta, max_rhs=1, inner=_inner(precision, "grad", inner_grid))
    if verbose >= 1:
        print(f"Capacitance: N={sysm.n} rc={rc:.3f} Ngrid={tuple(Ngrid.tolist())} P={P} "
              f"Ncell={tuple(sysm.ncell.tolist())} pairs(kept)={sysm.n_pairs}", flush=True)
    S = magnetic_dipole(x, lambdap, Hhat, box, None, None, Ngrid, h, P, xi, eta, rc, Sguess, offset, offsetxyz,
                        dipoletable1, dipoletable2, rtable, errortol, slab_factor=slab_factor, verbose=verbose,
                        restart=restart, maxit=maxit, precision=precision, inner_tol=inner_tol,
                        inner_maxit=inner_maxit, system=sysm)
    St = as_device(S, torch.complex128)
    Hh = torch.as_tensor(np.asarray(Hhat, dtype=np.float64).reshape(3), device="cuda").to(torch.complex128)
    C = (St @ Hh).mean()
    sysm.close()
    if verbose >= 1:
        print(f"Capacitance: done C={C.real.item():.6g} total_time={time.perf_counter() - t0:.2f}s", flush=True)
    return (complex(C.item()) if asnp else C), S


def run_capacitance(x, box, eps_p, xi, H0, errortol=1e-5, slab_factor=1.0, use_scipy_gmres=True, verbose=0, *,
                    rc=None, Ngrid=None, P=None, restart=None, maxit=None, precision="fp64", inner_tol=1e-4,
                    inner_maxit=4):
    """C per frame and moments p (N,3,Nframes) for a configuration or trajectory (capacitance.py:424-515)."""
    asnp = not isinstance(x, torch.Tensor)
    xn = x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x, dtype=np.float64)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    eps = np.asarray(eps_p.cpu() if isinstance(eps_p, torch.Tensor) else eps_p, dtype=np.float64).reshape(-1)
    if xn.ndim == 2:
        xn = xn[:, :, None]
    N, nframes = xn.shape[0], xn.shape[2]
    phi = 4.0 * np.pi * N / (3.0 * np.prod(box))
    perp, para, rv = default_table(xi)
    H0 = np.asarray(H0, dtype=np.float64).reshape(3)
    Hhat = H0 / np.linalg.norm(H0)
    C = np.zeros(nframes, dtype=np.complex128)
    p = np.zeros((N, 3, nframes), dtype=np.complex128)
    for f in range(nframes):
        guess = dilute_guess(eps, phi, Hhat)
        C[f], S = capacitance(xn[:, :, f], eps, box, guess, xi, errortol, perp, para, rv, None, None, Hhat,
                              slab_factor=slab_factor, verbose=verbose, rc=rc, Ngrid=Ngrid, P=P, restart=restart,
                              maxit=maxit, precision=precision, inner_tol=inner_tol, inner_maxit=inner_maxit)
        p[:, :, f] = S
    if not asnp:
        return torch.as_tensor(C, device="cuda"), torch.as_tensor(p, device="cuda")
    return C, p


_UNIT_FIELDS: dict = {}


def _unit_fields(N):
    """(3, N, 3) unit fields along x, y, z on the current device, kept per (N, device): the solves only read
    their right-hand sides, and building them is several launches per call."""
    key = (int(N), torch.cuda.current_device())
    b = _UNIT_FIELDS.get(key)
    if b is None:
        if len(_UNIT_FIELDS) >= 8:
            _UNIT_FIELDS.clear()
        b = torch.zeros((3, int(N), 3), dtype=torch.float64, device="cuda")
        b.diagonal(dim1=0, dim2=2).fill_(1.0)
        _UNIT_FIELDS[key] = b
    return b


def capacitance_tensor(x, lambdap, box, Sguess, xi, errortol, dipoletable1=None, dipoletable2=None, rtable=None,
                       offset=None, offsetxyz=None, *, slab_factor=0.0, rc=None, Ngrid=None, P=None, restart=None,
                       maxit=None, precision="fp64", inner_tol=1e-4, inner_maxit=4, batched=True, system=None,
                       residual_precision="df", inner_operator="grad", inner_grid="auto"):
    """3x3 capacitance tensor for unit fields along x, y, z (Capacitance_Hetero/Capacitance_Tensor.m:23-59).

    ``batched=True`` solves the three directions together (one batched matvec
    per iteration); each starts from ``Sguess`` rotated onto its field axis.
    ``batched=False`` follows the reference: sequential solves, each warm-started
    from the previous solution with columns permuted [z, x, y].
    With ``precision='mixed'`` and the gradient-form inner operator,
    ``inner_grid="auto"`` runs the inner solves on a coarser grid when one is
    cheaper (``system.inner_grid``; None keeps the system's grid); the
    refinement residuals keep the system's grid.
    Returns (C (3,3), S (N,3,3)) with row i of C the mean moment for field i.
    The MATLAB driver has no slab term, hence ``slab_factor=0`` by default."""
    asnp = not isinstance(x, torch.Tensor)
    box = np.asarray(box, dtype=np.float64).reshape(3)
    rc, Ngrid, h, P, eta = _resolve_params(box, xi, errortol, rc, Ngrid, P)
    if dipoletable1 is None:
        dipoletable1, dipoletable2, rtable = default_table(xi)
    xd = as_device(x, non_blocking=system is None).reshape(-1, 3)   # the system's creation synchronises
    N = xd.shape[0]
    sysm = system or SpectralEwaldSystem(xd, lambdap, box, xi, rc, Ngrid, P, dipoletable1, dipoletable2, rtable,
                                         slab_factor=slab_factor, eta=eta, max_rhs=3,
                                         inner=_inner(precision, inner_operator, inner_grid))
    restart = min(3 * N, 10) if restart is None else int(restart)
    maxit = min(3 * N, 100) if maxit is None else int(maxit)
    infos = []
    if batched:
        b = _unit_fields(N)
        # dilute-type guess along each axis: amplitude of the given guess projected on x, rotated (only that
        # column goes to the device); x0[i, :, i] = amplitude
        g0x = Sguess.real.reshape(N, 3)[:, 0] if isinstance(Sguess, torch.Tensor) else \
            np.real(np.asarray(Sguess)).reshape(N, 3)[:, 0]
        x0 = torch.zeros((3, N, 3), dtype=torch.float64, device="cuda")
        x0.diagonal(dim1=0, dim2=2).copy_(as_device(g0x, non_blocking=True).reshape(N, 1))   # the solve syncs
        S3, infos = sysm.solve(b, x0, tol=float(errortol), restart=restart, maxit=maxit, precision=precision,
                               inner_tol=inner_tol, inner_maxit=inner_maxit, residual_precision=residual_precision,
                               inner_operator=inner_operator)
    else:
        eye = torch.eye(3, dtype=torch.float64, device="cuda")
        sols = []
        guess = as_device(np.real(Sguess) if not isinstance(Sguess, torch.Tensor) else Sguess.real).reshape(N, 3)
        for i in range(3):
            b = eye[i].repeat(N, 1)
            Si, inf = sysm.solve(b, guess, tol=float(errortol), restart=restart, maxit=maxit, precision=precision,
                                 inner_tol=inner_tol, inner_maxit=inner_maxit,
                                 residual_precision=residual_precision, inner_operator=inner_operator)
            sols.append(Si)
            infos += inf
            guess = Si[:, [2, 0, 1]].contiguous()
        S3 = torch.stack(sols)
    S = S3.permute(1, 2, 0).contiguous()          # (N, 3 components, 3 fields)
    Cm = S3.mean(dim=1)                            # row i = mean moment for field i
    if system is None:
        sysm.close()
    if asnp:
        return to_host(Cm), to_host(S), infos
    return Cm, S, infos


def capacitance_tensor_spectrum(x, box, eps_p, xi, errortol=1e-3, *, slab_factor=0.0, rc=None, Ngrid=None, P=None,
                                restart=None, maxit=None, precision="fp64", inner_tol=1e-4, inner_maxit=4,
                                inner_grid="auto"):
    """Tensor for every permittivity column of ``eps_p (N, N_k)`` and every frame of
    ``x (N,3[,F])`` (Capacitance_Hetero/CapacitanceTensorSpectrum.m:15-62).
    ``eps_p`` may be complex (frequency-dependent permittivities); C and p are then complex.

    The N_k columns of one frame share one system (the permittivity only enters
    the diagonal), and all 3 N_k systems are solved as one batch.
    Returns C (3,3,N_k) averaged over frames and p (N,3,3,N_k,F)."""
    xn = x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x, dtype=np.float64)
    if xn.ndim == 2:
        xn = xn[:, :, None]
    eps = np.asarray(eps_p.cpu() if isinstance(eps_p, torch.Tensor) else eps_p)
    # complex permittivities (frequency-dependent eps, which the MATLAB driver allows) give complex C and p
    cplx = np.iscomplexobj(eps)
    eps = eps.astype(np.complex128 if cplx else np.float64)
    tdt = torch.complex128 if cplx else torch.float64
    if eps.ndim == 1:
        eps = eps[:, None]
    N, F = xn.shape[0], xn.shape[2]
    K = eps.shape[1]
    box = np.asarray(box, dtype=np.float64).reshape(3)
    phi = 4.0 * np.pi * N / (3.0 * np.prod(box))
    rc, Ngrid, h, P, eta = _resolve_params(box, xi, errortol, rc, Ngrid, P)
    perp, para, rv = default_table(xi)
    restart = min(3 * N, 10) if restart is None else int(restart)
    maxit = min(3 * N, 100) if maxit is None else int(maxit)
    C = np.zeros((3, 3, F, K), dtype=eps.dtype)
    p = np.zeros((N, 3, 3, K, F), dtype=eps.dtype)
    for f in range(F):
        lam = eps.T.copy()                                   # (K, N) permittivity sets
        sysm = SpectralEwaldSystem(xn[:, :, f], lam, box, xi, rc, Ngrid, P, perp, para, rv,
                                   slab_factor=slab_factor, eta=eta, max_rhs=3 * K,
                                   inner=_inner(precision, "grad", inner_grid))
        b = torch.zeros((3 * K, N, 3), dtype=tdt, device="cuda")
        x0 = torch.zeros_like(b)
        diag_index = []
        for k in range(K):
            amp = torch.as_tensor(dilute_guess(eps[:, k], phi, [1.0, 0.0, 0.0])[:, 0], dtype=tdt, device="cuda")
            for i in range(3):
                b[3 * k + i, :, i] = 1.0
                x0[3 * k + i, :, i] = amp
                diag_index.append(k)
        sol, _ = sysm.solve(b, x0, tol=errortol, restart=restart, maxit=maxit, precision=precision,
                            inner_tol=inner_tol, inner_maxit=inner_maxit, diag_index=diag_index)
        sol = sol.reshape(K, 3, N, 3).cpu().numpy()
        for k in range(K):
            for i in range(3):
                C[i, :, f, k] = sol[k, i].mean(axis=0)
                p[:, :, i, k, f] = sol[k, i]
        sysm.close()
    return C.mean(axis=2), p
