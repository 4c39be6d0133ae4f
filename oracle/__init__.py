"""CPU oracle for the spectral-Ewald mutual-polarisation solve.

TEST INFRASTRUCTURE ONLY.  Nothing in ``mutual_polarization_slab_gb300`` imports
this package: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use it, and only as the checker (or the timed CPU
baseline), never as the thing measured on the GPU.

Modules
-------
ewald_oracle        NumPy restatement of the dipole-only spectral-Ewald kernels
                    (``CPU - Ewald test/ewald.py``).
capacitance_oracle  Restarted GMRES, the dipole solve, capacitance, the 3x3
                    capacitance tensor and contrast spectra
                    (``CPU - Ewald test/capacitance.py``,
                    ``Capacitance_Hetero/Capacitance_Tensor.m``,
                    ``Capacitance_Hetero/CapacitanceTensorSpectrum.m``).

Parity is pinned against vectors produced by running the reference Python
module itself (``tests/golden/make_golden.py``); the reference ships no golden
vectors of its own.
"""
