"""The fused z + y plane passes (thread-block clusters exchanging the (y, kz)
plane through bulk copies between their shared memories), selected with
DFTGPU_FUSED_ZY=1, against the default separate passes: real spectra and
full OT potentials on grids whose y-z planes are 128^2 and 256^2.  The
selection is read once per process, so the fused side runs in a child
process."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, liquid_psi, relerr

pytestmark = pytest.mark.gpu

CASES = [((32, 128, 128), 0.8, 9), ((16, 256, 256), 0.8, 9), ((8, 256, 256), 0.8, 0)]

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
import libdft_gb300 as G
from conftest import liquid_psi
G.check(G.lib().dftgpu_init(0), "init")
G.set_precision(1)
out = {}
for shape, step, model in json.loads(sys.argv[2]):
    shape = tuple(shape)
    f = np.random.default_rng(7).standard_normal(shape)
    r = G.RGrid(shape, step); r.set(f); s = r.spectrum(); r.free()
    w = G.Wf(shape, step); ot = G.OT(model, w); w.set(liquid_psi(shape, step, 2))
    P = G.CGrid(shape, step); P.zero(); ot.potential(P, w); p = P.get()
    np.save(sys.argv[3] + "/spec_%d_%d.npy" % (shape[1], shape[0]), s)
    np.save(sys.argv[3] + "/pot_%d_%d.npy" % (shape[1], shape[0]), p)
    for o in (P, ot, w): o.free()
print("ok")
"""


def test_fused_plane_passes_match_separate_passes(gpu, tmp_path):
    env = dict(os.environ, DFTGPU_FUSED_ZY="1")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(CASES), str(tmp_path)], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]
    gpu.set_precision(1)
    try:
        for shape, step, model in CASES:
            f = np.random.default_rng(7).standard_normal(shape)
            rg = gpu.RGrid(shape, step)
            rg.set(f)
            s = rg.spectrum()
            rg.free()
            w = gpu.Wf(shape, step)
            ot = gpu.OT(model, w)
            w.set(liquid_psi(shape, step, 2))
            P = gpu.CGrid(shape, step)
            P.zero()
            ot.potential(P, w)
            p = P.get()
            for o in (P, ot, w):
                o.free()
            tag = "%d_%d" % (shape[1], shape[0])
            assert relerr(np.load(tmp_path / ("spec_%s.npy" % tag)), s) < 3e-6
            assert relerr(np.load(tmp_path / ("pot_%s.npy" % tag)).real, p.real) < 2e-6
            if model & 8:
                assert relerr(np.load(tmp_path / ("pot_%s.npy" % tag)).imag, p.imag) < 2e-5
    finally:
        gpu.set_precision(0)
