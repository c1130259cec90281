import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the sm_103a library."""
    from astr_gb300 import build_ext, capi
    build_ext.build()
    return capi.load()


def relerr(a, b):
    """Max-norm relative difference, the parity measure of the tests."""
    import numpy as np
    a = np.asarray(a)
    b = np.asarray(b)
    den = float(np.max(np.abs(b)))
    if den == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / den)
