"""Drop-in for the reference's compiled force module ``dipole_forces_ext``
(``CPU - HOOMD simulation test/dipole_forces_ext/_dipole_forces_ext.cpp``).

``compute_forces(pos, dip, box, r_cut, prefactor=1.0, periodic_z=True,
use_cell_list=True) -> (forces (N,3), pe (N,))`` with the reference's meaning;
the pair sum runs on the GPU (``mps_dipole_forces``).  ``use_cell_list`` is
accepted for signature compatibility: the GPU path always bins into cells,
which gives the same pair set as the reference's brute-force loop.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib as L
from .system import as_device

__version__ = "0.5.1"


def compute_forces(pos, dip, box, r_cut, prefactor=1.0, periodic_z=True, use_cell_list=True):
    lib = L.lib()
    asnp = not isinstance(pos, torch.Tensor)
    p = as_device(pos).reshape(-1, 3)
    m = as_device(dip).reshape(-1, 3)
    n = p.shape[0]
    if m.shape[0] != n:
        raise RuntimeError("Invalid shapes: pos(N,3), dip(N,3), box(3) required.")
    b = np.asarray(box.cpu() if isinstance(box, torch.Tensor) else box, dtype=np.float64).reshape(3)
    F = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    pe = torch.empty(n, dtype=torch.float64, device="cuda")
    st = lib.mps_dipole_forces(L.dptr(p), L.dptr(m), n, L.host_f64(b), float(r_cut), float(prefactor),
                               1 if periodic_z else 0, L.dptr(F), L.dptr(pe), L.stream_handle())
    if st in (L.MPS_BAD_ARG, L.MPS_RC_GT_HALF_BOX):
        raise RuntimeError(f"compute_forces: {lib.mps_status_string(st).decode()}")
    L.check(st, "compute_forces")
    if asnp:
        return F.cpu().numpy(), pe.cpu().numpy()
    return F, pe
