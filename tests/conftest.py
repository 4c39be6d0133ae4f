import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libmps_gb300.so")


@pytest.fixture(scope="session")
def golden_small():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_small.npz")))


@pytest.fixture(scope="session")
def golden_c1():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_c1.npz")))
