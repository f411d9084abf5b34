import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the libdftgpu kernels")
    config.addinivalue_line("markers", "slow: long-running (large grids)")


@pytest.fixture(scope="session")
def port():
    """The oracle restatement (CPU, FP64), built on demand."""
    from oracle import Oracle
    return Oracle("port")


@pytest.fixture(scope="session")
def gpu():
    """The GB300 library; initialised on device 0."""
    import libdft_gb300 as G
    L = G.lib()
    rc = L.dftgpu_init(0)
    if rc:
        raise RuntimeError("dftgpu_init failed: %s" % L.dftgpu_last_error_message())
    return G


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def relerr(a, b):
    """max |a - b| / max |b|"""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
