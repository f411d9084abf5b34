"""The phase factors exp(z) - 1 and psi exp(z) of the propagation passes
(common.cuh: cexpm1, cexpm1_small, mul_cexp) against numpy in FP64, on the
device, through a small CUDA probe built against the header.

* accuracy: |error| <= 4 FP32 ulps of max(|e^z - 1|, 2^-126) on
  |Re z| + |Im z| < 0.25 (Taylor polynomials); 8 ulps of max(|e^z|, 1)
  beyond (library expm1 / sincos, cos y - 1 up to -2); psi exp(z) to 6 ulps
  of |psi e^z|;
* no norm bias for real-time factors: over 2^18 pure phases exp(i theta),
  |psi exp(i theta)|^2 - |psi|^2 averages to zero within 3e-10 (rounding a
  factor as a whole gave a mean of +theta^2 ~ 7e-8 per step).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CSRC = os.path.join(ROOT, "libdft_gb300", "csrc")


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    d = tmp_path_factory.mktemp("phase")
    exe = d / "phase_probe"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                    os.path.join(ROOT, "tests", "cuda", "phase_probe.cu"), "-o", str(exe)], check=True)

    def run(z):
        zi = np.ascontiguousarray(np.stack([z.real, z.imag], -1).astype(np.float32))
        zi.tofile(d / "in.bin")
        subprocess.run([str(exe), str(d / "in.bin"), str(d / "out.bin")], check=True, timeout=120)
        out = np.fromfile(d / "out.bin", dtype=np.float32).reshape(2, -1, 2)
        return out[0, :, 0] + 1j * out[0, :, 1], out[1, :, 0] + 1j * out[1, :, 1], zi[:, 0] + 1j * zi[:, 1]
    return run


def test_expm1_accuracy(probe):
    rng = np.random.default_rng(3)
    small = (rng.uniform(-1, 1, 1 << 20) + 1j * rng.uniform(-1, 1, 1 << 20)) * 0.125
    small = small[np.abs(small.real) + np.abs(small.imag) < 0.25]
    tiny = small * 1e-4
    large = rng.uniform(-3, 1, 1 << 16) + 1j * rng.uniform(-20, 20, 1 << 16)
    for name, z, floor_is_exp, ulps in (("small", small, False, 4), ("tiny", tiny, False, 4), ("large", large, True, 8)):
        got, mul, zf = probe(z)
        zf = zf.astype(np.complex128)           # the exponents as the device saw them
        ref = np.expm1(zf.real) * np.cos(zf.imag) + (np.cos(zf.imag) - 1) + 1j * np.exp(zf.real) * np.sin(zf.imag)
        # beyond the polynomial interval e^z - 1 is formed from e^x - 1 and the
        # half-angle sine: its error is relative to max(|e^z|, 1)
        scale = np.maximum(np.abs(np.exp(zf)), 1.0) if floor_is_exp else np.maximum(np.abs(ref), 2.0 ** -126)
        err = np.abs(got - ref) / scale
        assert err.max() < ulps * 2.0 ** -24, (name, err.max())
        a = 0.6 - 0.8j
        mref = a * np.exp(zf)
        merr = np.abs(mul - mref) / np.abs(mref)
        assert merr.max() < 6 * 2.0 ** -24, (name, merr.max())


def test_pure_phase_has_no_norm_bias(probe):
    rng = np.random.default_rng(4)
    theta = rng.uniform(-0.2, 0.2, 1 << 18)
    _, mul, zf = probe(1j * theta)
    a2 = float(np.float32(0.6)) ** 2 + float(np.float32(-0.8)) ** 2   # |psi|^2 of the probe's psi
    dn = np.abs(mul.astype(np.complex128)) ** 2 - a2
    assert abs(dn.mean()) < 3e-10, dn.mean()
    assert np.abs(dn).max() < 4e-7
