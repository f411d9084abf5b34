"""Switches that change how the work is scheduled but not what is computed:
DFTGPU_PREFETCH_AHEAD=0 (no one-wave-ahead L2 prefetch in the line passes),
DFTGPU_STREAMS=1 (no parallel graph branches) and DFTGPU_TMA=0 (the z passes'
transposed side staged by load / store loops instead of TMA boxes).  The selections are read
once per process, so the switched side runs in a child process; potentials
and predict-correct steps must be bitwise equal to the default run's."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, liquid_psi

pytestmark = pytest.mark.gpu

CASES = [((64, 64, 64), 0.8, 9, 1), ((32, 24, 40), 0.9, 9, 0), ((32, 64, 256), 0.7, 9, 1)]   # shape, step, model, precision

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
import libdft_gb300 as G
from conftest import liquid_psi
G.check(G.lib().dftgpu_init(0), "init")
for shape, step, model, prec in json.loads(sys.argv[2]):
    shape = tuple(shape)
    G.set_precision(prec)
    w, wp = G.Wf(shape, step), G.Wf(shape, step)
    ot = G.OT(model, w)
    w.set(liquid_psi(shape, step, 5))
    P = G.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    p = P.get()
    ot.run(w, wp, P, None, ot.bulk_chempot(0.0), 41.3 + 0j, 3, False)
    np.save(sys.argv[3] + "/pot_%d_%d.npy" % (shape[0], prec), p)
    np.save(sys.argv[3] + "/psi_%d_%d.npy" % (shape[0], prec), w.get())
    for o in (P, ot, wp, w):
        o.free()
print("ok")
"""


def run_here(gpu, shape, step, model, prec):
    gpu.set_precision(prec)
    w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    w.set(liquid_psi(shape, step, 5))
    P = gpu.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    p = P.get()
    ot.run(w, wp, P, None, ot.bulk_chempot(0.0), 41.3 + 0j, 3, False)
    psi = w.get()
    for o in (P, ot, wp, w):
        o.free()
    gpu.set_precision(0)
    return p, psi


@pytest.mark.parametrize("env", [{"DFTGPU_PREFETCH_AHEAD": "0"}, {"DFTGPU_STREAMS": "1"}, {"DFTGPU_TMA": "0"}])
def test_scheduling_switches_do_not_change_results(gpu, tmp_path, env):
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(CASES), str(tmp_path)],
                       env=dict(os.environ, **env), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]
    for shape, step, model, prec in CASES:
        p, psi = run_here(gpu, tuple(shape), step, model, prec)
        assert np.array_equal(np.load(tmp_path / ("pot_%d_%d.npy" % (shape[0], prec))), p)
        assert np.array_equal(np.load(tmp_path / ("psi_%d_%d.npy" % (shape[0], prec))), psi)
