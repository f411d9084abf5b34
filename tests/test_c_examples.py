"""The libdft-style C drivers (libdft_gb300/examples) built against
include/dftgpu.h and run on the GPU: the imaginary-time relaxation of
examples/imag_time/imag_time.c and the moving-background bubble of
examples/gas-bubble/bubble.c (warm-up in imaginary time, then real time with
a small imaginary part of the step).  Both must exit 0 and report a finite
particle number and energy; the bubble's particle number is conserved by the
real-time steps to the damping of the imaginary part of the step."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

LIBDIR = os.path.join(ROOT, "libdft_gb300")


def build(tmp_path, name):
    exe = tmp_path / name
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(LIBDIR, "examples", name + ".c"), "-o", str(exe), "-L", LIBDIR, "-ldftgpu", "-lm",
                    "-Wl,-rpath," + LIBDIR], check=True)
    return exe


def run(exe, *args):
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-1000:] + r.stderr[-1000:]
    nums = dict((k, float(v)) for k, v in re.findall(r"(?:^|\s)(N|E) = ([-+0-9.eE]+)", r.stdout, re.M))
    return r.stdout, nums


@pytest.mark.parametrize("model", ["plain", "hd"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_imag_time_driver_runs(gpu, tmp_path, prec, model):
    """"hd": the functional libdft's imag_time example allocates,
    DFT_OT_PLAIN | DFT_OT_KC | DFT_OT_HD (examples/imag_time/imag_time.c:204)."""
    out, nums = run(build(tmp_path, "imag_time"), 20, prec, model)
    assert nums["N"] > 0 and abs(nums["E"]) < 1e12, out


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_moving_bubble_driver_runs(gpu, tmp_path, prec):
    exe = build(tmp_path, "moving_bubble")
    out0, n0 = run(exe, 20, 0, prec)
    out1, n1 = run(exe, 20, 20, prec)
    assert "background velocity" in out1
    assert n1["N"] > 0 and abs(n1["E"]) < 1e12, out1
    # 20 real-time steps of 5 fs with 0.5 % imaginary time: the particle
    # number changes only by that damping (a few 1e-4 at most)
    assert abs(n1["N"] / n0["N"] - 1) < 1e-2, (n0, n1)
