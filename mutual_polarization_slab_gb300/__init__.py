"""GB300-native spectral-Ewald mutual-polarisation solve.

Drop-in modules mirroring the reference's Python entry points:

* ``mutual_polarization_slab_gb300.ewald``       <- ``CPU - Ewald test/ewald.py``
* ``mutual_polarization_slab_gb300.capacitance`` <- ``CPU - Ewald test/capacitance.py``
  (+ the capacitance tensor / spectrum drivers of ``Capacitance_Hetero``)

``SpectralEwaldSystem`` is the device-resident operator behind both.  All
compute runs in ``libmps_gb300.so`` (hand-written sm_103a CUDA + cuFFT) through
the C ABI in ``include/mps_gb300.h``.
"""
from __future__ import annotations

__version__ = "0.1.0"


def __getattr__(name):
    if name in ("ewald", "capacitance", "system", "workloads"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    if name == "SpectralEwaldSystem":
        from .system import SpectralEwaldSystem
        return SpectralEwaldSystem
    raise AttributeError(name)
