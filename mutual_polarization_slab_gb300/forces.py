"""Forces from the polarisation solve.

Two force models sit on top of the GPU solve:

* ``adjoint_forces`` / ``PolarizationEnergy``: the exact gradient of the
  polarisation energy ``E = -1/2 sum_i m_i . H0`` of the solved operator, with
  ``A(x) m = H0``.  The operator is symmetric, so ``dE/dx_k = 1/2 m^T (dA/dx_k) m``
  with the converged moments held fixed (``mps_adjoint_forces``): one pass over
  the pairs and one wave-space pass, no second solve.  ``dE/d beta_k`` follows
  from the diagonal: ``dE/d eps_k = 1/2 |m_k|^2 dD_k/d eps_k``,
  ``eps = (1 + 2 beta) / (1 - beta)``.  ``PolarizationEnergy`` exposes E(x, beta) as a
  ``torch.autograd.Function``.
* ``MutualPolarizationDipoleForceCached``: the reference's HOOMD force
  (``CPU - HOOMD simulation test/dipole_forces_ext/hoomd_force.py:78-243``) without
  HOOMD: induced dipoles from ``run_capacitance`` for the unit field, scaled by
  the field strength, cached by particle tag and re-solved every
  ``pol_every_steps``; forces and energies from the point-dipole kernel
  ``compute_forces``.  Both the solve and the kernel run on the GPU.

``BrownianDynamics`` integrates overdamped dynamics with either model, with the
moments warm-started from the previous solve.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _lib as L
from . import capacitance
from .dipole_forces import compute_forces
from .system import SpectralEwaldSystem, as_device

__all__ = ["eps_from_beta", "beta_from_eps", "adjoint_forces", "polarization_energy", "PolarizationEnergy",
           "BrownianDynamics", "MutualPolarizationDipoleForceCached"]


def eps_from_beta(beta):
    """eps = (1 + 2 beta) / (1 - beta) (the inverse of beta = (eps - 1)/(eps + 2))."""
    return (1.0 + 2.0 * beta) / (1.0 - beta)


def beta_from_eps(eps):
    return (eps - 1.0) / (eps + 2.0)


def adjoint_forces(system: SpectralEwaldSystem, m, diag_index: int = 0):
    """Forces -dE/dx (N,3) and dE/d eps (N,) for converged moments ``m`` (N,3) of
    the field the system was solved for (the system's own tables give the
    coupling slopes)."""
    if system.kind != L.MPS_DIPOLE:
        raise ValueError("adjoint forces are available for the dipole operator")
    md = as_device(m).reshape(system.n, 3).contiguous()
    F = torch.empty((system.n, 3), dtype=torch.float64, device="cuda")
    dE = torch.empty(system.n, dtype=torch.float64, device="cuda")
    L.check(system._lib.mps_adjoint_forces(system._h, L.dptr(md), L.dptr(system.perp), L.dptr(system.para),
                                           L.dptr(system.rvals), int(system.rvals.numel()), int(diag_index),
                                           L.dptr(F), L.dptr(dE), L.stream_handle()), "mps_adjoint_forces")
    return F, dE


@dataclass
class EnergyResult:
    energy: float
    moments: torch.Tensor        # (N,3)
    forces: torch.Tensor         # (N,3) = -dE/dx
    dE_dbeta: torch.Tensor       # (N,)
    relres: float


def polarization_energy(x, beta, box, H0, xi, rc, Ngrid, P, *, tol=1e-10, restart=30, maxit=200, precision="fp64",
                        guess=None, slab_factor=0.0, tables=None, system=None, inner_grid="auto") -> EnergyResult:
    """Solve A(x) m = H0 for spheres of contrast ``beta`` (scalar or (N,)) and
    return E = -1/2 sum m . H0 with its gradients.  ``inner_grid`` as in
    ``capacitance.capacitance_tensor`` (mixed precision only)."""
    xd = as_device(x).reshape(-1, 3)
    n = xd.shape[0]
    b = as_device(np.broadcast_to(np.asarray(beta.cpu() if isinstance(beta, torch.Tensor) else beta,
                                             dtype=np.float64), (n,)).copy())
    eps = eps_from_beta(b)
    if tables is None:
        tables = capacitance.default_table(xi)
    perp, para, rv = tables
    sysm = system or SpectralEwaldSystem(xd, eps, box, xi, rc, Ngrid, P, perp, para, rv, slab_factor=slab_factor,
                                         max_rhs=1, inner=inner_grid if precision == "mixed" else None)
    h0 = torch.as_tensor(np.asarray(H0, dtype=np.float64).reshape(3), device="cuda")
    rhs = h0.repeat(n, 1)
    x0 = None if guess is None else as_device(guess).reshape(n, 3)
    m, info = sysm.solve(rhs, x0, tol=tol, restart=restart, maxit=maxit, precision=precision)
    F, dE_deps = adjoint_forces(sysm, m)
    dE_dbeta = dE_deps * 3.0 / (1.0 - b) ** 2
    E = float(-0.5 * (m @ h0).sum())
    if system is None:
        sysm.close()
    return EnergyResult(E, m, F, dE_dbeta, info[0].relres)


class PolarizationEnergy(torch.autograd.Function):
    """E(x, beta) = -1/2 sum m . H0 with A(x, beta) m = H0, differentiable in the
    positions x (N,3) and the contrasts beta (N,).  ``params`` is a dict with
    box, H0, xi, rc, Ngrid, P and optionally tol, precision, tables, slab_factor."""

    @staticmethod
    def forward(ctx, x, beta, params):
        kw = {k: params[k] for k in ("tol", "precision", "tables", "slab_factor", "guess") if k in params}
        r = polarization_energy(x.detach(), beta.detach(), params["box"], params["H0"], params["xi"], params["rc"],
                                params["Ngrid"], params["P"], **kw)
        ctx.save_for_backward(-r.forces, r.dE_dbeta)
        return torch.tensor(r.energy, dtype=torch.float64, device=x.device)

    @staticmethod
    def backward(ctx, g):
        dEdx, dEdb = ctx.saved_tensors
        return g * dEdx.to(g.device), g * dEdb.to(g.device), None


class BrownianDynamics:
    """Overdamped Brownian dynamics x += mu F dt + sqrt(2 mu kT dt) N(0, 1) with
    the adjoint polarisation forces; moments re-solved every ``pol_every`` steps
    from the previous ones (warm start), positions wrapped into the box."""

    def __init__(self, x0, beta, box, H0, xi, rc, Ngrid, P, *, dt=1e-4, kT=1.0, mobility=1.0, pol_every=1,
                 tol=1e-8, precision="mixed", seed=0, tables=None):
        self.x = as_device(x0).reshape(-1, 3).clone()
        self.n = self.x.shape[0]
        self.beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), (self.n,)).copy()
        self.box = np.asarray(box, dtype=np.float64).reshape(3)
        self.H0 = np.asarray(H0, dtype=np.float64).reshape(3)
        self.xi, self.rc, self.Ngrid, self.P = float(xi), float(rc), Ngrid, int(P)
        self.dt, self.kT, self.mob = float(dt), float(kT), float(mobility)
        self.pol_every = max(1, int(pol_every))
        self.tol, self.precision = float(tol), precision
        self.tables = tables if tables is not None else capacitance.default_table(xi)
        self.gen = torch.Generator(device="cuda").manual_seed(int(seed))
        self.m: Optional[torch.Tensor] = None
        self.forces: Optional[torch.Tensor] = None
        self.energy = float("nan")
        self.step_count = 0
        self.solves = 0
        self.boxd = torch.as_tensor(self.box, device="cuda")

    def _forces(self):
        eps = eps_from_beta(self.beta)
        perp, para, rv = self.tables
        s = SpectralEwaldSystem(self.x, eps, self.box, self.xi, self.rc, self.Ngrid, self.P, perp, para, rv,
                                slab_factor=0.0, max_rhs=1, inner="auto" if self.precision == "mixed" else None)
        try:
            if self.m is None or self.step_count % self.pol_every == 0:
                rhs = torch.as_tensor(self.H0, device="cuda").repeat(self.n, 1)
                self.m, _ = s.solve(rhs, self.m, tol=self.tol, restart=30, maxit=200, precision=self.precision)
                self.solves += 1
            F, _ = adjoint_forces(s, self.m)
        finally:
            s.close()
        self.energy = float(-0.5 * (self.m @ torch.as_tensor(self.H0, device="cuda")).sum())
        return F

    def step(self):
        F = self._forces()
        self.forces = F
        noise = torch.randn((self.n, 3), generator=self.gen, dtype=torch.float64, device="cuda")
        self.x = self.x + self.mob * F * self.dt + math.sqrt(2.0 * self.mob * self.kT * self.dt) * noise
        self.x = torch.remainder(self.x, self.boxd)
        self.step_count += 1

    def run(self, nsteps):
        for _ in range(int(nsteps)):
            self.step()
        return self.x


@dataclass
class _CachedDipoles:
    by_tag: np.ndarray
    last_pol_step: Optional[int] = None


class MutualPolarizationDipoleForceCached:
    """The reference's cached mutual-polarisation force
    (``hoomd_force.py:78-243``) as a plain object: ``set_forces(timestep,
    positions, tags, box)`` returns (forces (N,3), energies (N,)) and keeps the
    same diagnostics (calls, pol_solves, last_dipoles, last_forces, last_energy)."""

    def __init__(self, *, eps_p, xi, errtol, slab_factor, Hhat, r_cut, prefactor, field_strength,
                 pol_every_steps=1, use_scipy_gmres=True, periodic_z=True, use_cell_list=True, precision="fp64"):
        self.eps_p = float(eps_p)
        self.xi = float(xi)
        self.errtol = float(errtol)
        self.slab_factor = float(slab_factor)
        self.Hhat = np.asarray(Hhat, dtype=np.float64).reshape(3)
        self.r_cut = float(r_cut)
        self.prefactor = float(prefactor)
        self.field_strength = float(field_strength)
        self.use_scipy_gmres = bool(use_scipy_gmres)
        self.periodic_z = bool(periodic_z)
        self.use_cell_list = bool(use_cell_list)
        self.pol_every_steps = int(max(1, int(pol_every_steps)))
        self.precision = precision
        self.calls = 0
        self.pol_solves = 0
        self.last_dipoles = None
        self.last_forces = None
        self.last_energy = None
        self._cache: Optional[_CachedDipoles] = None

    def _ensure_cache(self, tags):
        max_tag = int(np.max(tags)) if tags.size else -1
        if self._cache is None:
            self._cache = _CachedDipoles(by_tag=np.zeros((max_tag + 1, 3)))
        elif max_tag >= self._cache.by_tag.shape[0]:
            new = np.zeros((max_tag + 1, 3))
            new[: self._cache.by_tag.shape[0]] = self._cache.by_tag
            self._cache.by_tag = new

    def _solve_dipoles(self, pos, boxL, tags):
        n = pos.shape[0]
        eps = np.full(n, self.eps_p)
        _, p = capacitance.run_capacitance(pos, boxL, eps, self.xi, self.Hhat.copy(), errortol=self.errtol,
                                           slab_factor=self.slab_factor, verbose=0,
                                           use_scipy_gmres=self.use_scipy_gmres, precision=self.precision)
        p0 = np.real(np.asarray(p)[:, :, 0] if np.asarray(p).ndim == 3 else np.asarray(p))
        self._ensure_cache(tags)
        self._cache.by_tag[tags.astype(np.int64)] = p0 * self.field_strength
        self.pol_solves += 1

    def set_forces(self, timestep, positions, tags, box):
        self.calls += 1
        pos = np.asarray(positions, dtype=np.float64)
        tags = np.asarray(tags, dtype=np.int64)
        boxL = np.asarray(box, dtype=np.float64).reshape(3)
        if pos.shape[0] == 0:
            return np.zeros((0, 3)), np.zeros(0)
        self._ensure_cache(tags)
        if self._cache.last_pol_step is None or int(timestep) - self._cache.last_pol_step >= self.pol_every_steps:
            self._solve_dipoles(pos, boxL, tags)
            self._cache.last_pol_step = int(timestep)
        dip = self._cache.by_tag[tags]
        f, e = compute_forces(pos, dip, boxL, self.r_cut, self.prefactor, periodic_z=self.periodic_z,
                              use_cell_list=self.use_cell_list)
        f = np.asarray(f)
        e = np.asarray(e).reshape(-1)
        if not (np.all(np.isfinite(f)) and np.all(np.isfinite(e)) and np.all(np.isfinite(dip))):
            raise RuntimeError("Non-finite values in dipoles/forces/energies")
        self.last_dipoles, self.last_forces, self.last_energy = dip.copy(), f.copy(), e.copy()
        return f, e
