"""The factorised propagation (DFTGPU_FACTORISED_PROP=1: one kinetic pass per
axis, the wave function kept in its own [x][y][z] layout) against the default
five-pass propagation through the spectral layout.  Both evaluate the same
operator exp(-iV dt/2) F^-1 K F exp(-iV dt/2) -- K factorises per axis -- in
another order, so they agree to FP32 rounding.  The switch is read once per
process: the factorised side runs in a child process.  One shape has no
factorised instantiation (ny not a multiple of a pass's lines) and checks the
fallback; one sets a moving-background momentum (the per-axis factors use
k - k0)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, liquid_psi, relerr

pytestmark = pytest.mark.gpu

# shape, step, model, momentum (bohr^-1)
CASES = [((64, 64, 64), 0.8, 9, (0.0, 0.0, 0.0)), ((32, 64, 128), 0.9, 9, (0.0, 0.0, 0.0)),
         ((128, 32, 256), 0.7, 9, (0.05, -0.02, 0.11)), ((64, 48, 64), 0.8, 9, (0.0, 0.0, 0.0)),
         ((64, 64, 128), 0.8, 8, (0.0, 0.0, 0.0)), ((64, 64, 64), 0.8, 1, (0.0, 0.0, 0.0))]

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
import libdft_gb300 as G
from conftest import liquid_psi
G.check(G.lib().dftgpu_init(0), "init")
G.set_precision(1)
for i, (shape, step, model, k0) in enumerate(json.loads(sys.argv[2])):
    shape = tuple(shape)
    w, wp = G.Wf(shape, step), G.Wf(shape, step)
    ot = G.OT(model, w)
    w.set(liquid_psi(shape, step, 5))
    w.set_momentum(*k0)
    wp.set_momentum(*k0)
    P = G.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    np.save(sys.argv[3] + "/pot_%d.npy" % i, P.get())
    ot.run(w, wp, P, None, ot.bulk_chempot(0.0), 41.3 - 3.0j, 3, False)
    np.save(sys.argv[3] + "/psi_%d.npy" % i, w.get())
    for o in (P, ot, wp, w):
        o.free()
print("ok")
"""


def run_here(gpu, shape, step, model, k0):
    gpu.set_precision(1)
    w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    w.set(liquid_psi(shape, step, 5))
    w.set_momentum(*k0)
    wp.set_momentum(*k0)
    P = gpu.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    p = P.get()
    ot.run(w, wp, P, None, ot.bulk_chempot(0.0), 41.3 - 3.0j, 3, False)
    psi = w.get()
    for o in (P, ot, wp, w):
        o.free()
    gpu.set_precision(0)
    return p, psi


@pytest.fixture(scope="module")
def factorised(tmp_path_factory):
    out = tmp_path_factory.mktemp("long")
    env = dict(os.environ, DFTGPU_FACTORISED_PROP="1")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(CASES), str(out)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]
    return out


@pytest.mark.parametrize("i", range(len(CASES)))
def test_factorised_propagation_matches_five_pass(gpu, factorised, i):
    shape, step, model, k0 = CASES[i]
    p, psi = run_here(gpu, shape, step, model, k0)
    p_ref = np.load(factorised / ("pot_%d.npy" % i))
    psi_ref = np.load(factorised / ("psi_%d.npy" % i))
    assert relerr(p, p_ref) < 2e-6, relerr(p, p_ref)
    assert relerr(psi, psi_ref) < 5e-6, relerr(psi, psi_ref)
