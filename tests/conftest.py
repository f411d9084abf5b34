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


def coords(shape, step):
    ax = [(np.arange(n) - n // 2) * step for n in shape]
    return np.meshgrid(*ax, indexing="ij")


def liquid_psi(shape, step, seed, amp=0.1):
    rng = np.random.default_rng(seed)
    rho0 = 0.0218360 * 0.529177210903 ** 3
    X, Y, Z = coords(shape, step)
    L = [n * step for n in shape]
    rho = rho0 * (1 + amp * np.cos(2 * np.pi * X / L[0]) * np.cos(2 * np.pi * Y / L[1])
                  + 0.5 * amp * np.sin(4 * np.pi * Z / L[2]))
    phase = 0.4 * np.sin(2 * np.pi * X / L[0]) + 0.3 * np.cos(2 * np.pi * (Y / L[1] + Z / L[2]))
    return (np.sqrt(rho) * np.exp(1j * phase) * (1 + 1e-3 * rng.standard_normal(shape))).astype(np.complex128)


def line_psi(o, n, step, seed=5):
    """a liquid column along z with a density wave and a phase (1-D grid, nx = ny = 1)"""
    rng = np.random.default_rng(seed)
    rho0 = 0.0218360 * o.AUTOANG ** 3
    z = (np.arange(n) - n // 2) * step
    rho = rho0 * (1 + 0.3 * np.cos(2 * np.pi * z / (n * step)) + 0.05 * rng.random(n))
    return (np.sqrt(rho) * np.exp(0.4j * np.sin(2 * np.pi * z / (n * step)))).reshape(1, 1, n)


def thermal_psi(o, shape, step, seed=5):
    """a droplet of radius 5 bohr over a 1e-4 rho0 vapour: the ideal Bose gas
    term takes both of its branches (rho lambda^3 above and below g_{3/2}(1))"""
    rng = np.random.default_rng(seed)
    rho0 = 0.0218360 * o.AUTOANG ** 3
    X = [(np.arange(n) - n // 2) * step for n in shape]
    r = np.sqrt(X[0][:, None, None] ** 2 + X[1][None, :, None] ** 2 + X[2][None, None, :] ** 2)
    rho = rho0 * (0.5 * (1 - np.tanh((r - 5.0) / 1.0)) + 1e-4) * (1 + 0.05 * rng.random(shape))
    return np.sqrt(rho) * np.exp(0.2j * rng.random(shape))
