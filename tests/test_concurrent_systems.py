"""Systems built and solved at the same time from several host threads, each on
its own CUDA stream, on one grid and box: they share the process's cached cuFFT
plans and Green's coefficients (including the lazily built gradient-form
coefficient and double-float scale tensor, which the first system to need them
fills on its own stream).  Every solver stage is deterministic, so each
concurrent result must equal the serial one bit for bit."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("CUDA device required", allow_module_level=True)

from mutual_polarization_slab_gb300 import capacitance as gcap  # noqa: E402
from mutual_polarization_slab_gb300.system import SpectralEwaldSystem, clear_kspace_cache  # noqa: E402
from mutual_polarization_slab_gb300.workloads import rsa  # noqa: E402


def _setup():
    n, phi = 3000, 0.25
    x, box, _ = rsa(n, phi, seed=31)
    xi = 0.8
    rc = 5.0
    perp, para, rv = gcap.default_table(xi)
    eps_sets = [np.full(n, 8.0), np.full(n, 20.0), np.full(n, 3.0)]
    return x, box, xi, rc, perp, para, rv, eps_sets


def _solve(x, box, xi, rc, perp, para, rv, eps, precision):
    n = x.shape[0]
    eye = torch.eye(3, dtype=torch.float64, device="cuda")
    b = eye[:, None, :].expand(3, n, 3).contiguous()
    s = SpectralEwaldSystem(x, eps, box, xi, rc, [48, 48, 48], 8, perp, para, rv, slab_factor=0.0, max_rhs=3)
    try:
        sol, info = s.solve(b, None, tol=1e-8, restart=30, maxit=8 if precision == "mixed" else 100,
                            precision=precision)
    finally:
        s.close()
    return sol.clone(), [i.converged for i in info]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_concurrent_systems_match_serial_bit_for_bit(precision):
    x, box, xi, rc, perp, para, rv, eps_sets = _setup()
    # serial pass (also fixes the autotuned tile depths, which are timed once per process)
    serial = []
    for eps in eps_sets:
        clear_kspace_cache()
        serial.append(_solve(x, box, xi, rc, perp, para, rv, eps, precision))
        torch.cuda.synchronize()
    assert all(all(c) for _, c in serial)
    # concurrent pass: the cache is empty, so the threads race to build and share the k-space data
    clear_kspace_cache()
    dev = torch.cuda.current_device()
    start = threading.Barrier(len(eps_sets))
    out = [None] * len(eps_sets)
    errors = []

    def work(k):
        try:
            torch.cuda.set_device(dev)
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                start.wait()
                out[k] = _solve(x, box, xi, rc, perp, para, rv, eps_sets[k], precision)
            st.synchronize()
        except BaseException as exc:  # re-raised below
            errors.append(exc)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(eps_sets))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    torch.cuda.synchronize()
    for (ref, _), (got, conv) in zip(serial, out):
        assert all(conv)
        assert torch.equal(ref, got)
