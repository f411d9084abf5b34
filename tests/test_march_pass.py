"""The x-marching form of the second OT pointwise pass (FP32; nz = 128, 256
or 512 and an even ny): the kinetic-correlation stencil terms and the
backflow real and imaginary parts with each field loaded once per plane.

It computes what the one-CTA-per-row form computes: the same expressions per
element, the stencil neighbours taken from registers (x), the CTA's own rows
or a halo row (y) and a shared-memory plane (z) instead of from global
memory.  DFTGPU_MARCH=0 selects the per-row form; it is read once per process,
so that side runs in a child process.  Cases: KC + BF, KC alone, BF alone,
the high-density models (cut-off density in the backflow), a clamped and
weighted backflow, the w_a outputs of dft_ot_potential2, nz = 128 / 256 /
512, and predict-correct steps; plus the clamped case against the FP64 CPU
oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, liquid_psi, relerr
from oracle import Grids

pytestmark = pytest.mark.gpu

# shape, step, model, clamp limits (0/1), dft_ot_potential2 (0/1)
CASES = [((24, 18, 128), 0.8, 9, 0, 0), ((20, 16, 128), 0.9, 1, 0, 0), ((18, 20, 128), 0.8, 8, 0, 0),
         ((16, 32, 128), 0.6, 11, 0, 0), ((16, 32, 128), 0.6, 13, 0, 0), ((24, 18, 128), 0.8, 9, 1, 0),
         ((24, 18, 128), 0.8, 9, 0, 1), ((10, 12, 256), 0.7, 9, 0, 0), ((5, 6, 512), 0.5, 9, 0, 0)]

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
import numpy as np
import libdft_gb300 as G
from test_march_pass import run_case
G.check(G.lib().dftgpu_init(0), "init")
G.set_precision(1)
for k, case in enumerate(json.loads(sys.argv[2])):
    for j, a in enumerate(run_case(G, *case)):
        np.save(sys.argv[3] + "/case%d_%d.npy" % (k, j), a)
print("ok")
"""


def psi_of(shape, step, model):
    psi = liquid_psi(shape, step, 11)
    if model & 6:   # high-density models: a compressed centre crosses the backflow cut-off
        X = [(np.arange(n) - n // 2) * step for n in shape]
        r2 = X[0][:, None, None] ** 2 + X[1][None, :, None] ** 2 + X[2][None, None, :] ** 2
        psi = psi * np.sqrt(1 + 14.0 * np.exp(-r2 / (2 * 1.5 ** 2)))
    return psi


def limits(G, psi, step, pcap=2e-6):
    """a velocity cap that binds on part of the grid, a backflow-potential cap and c_bfpot = 0.7"""
    vmax = 0.6 * np.abs(np.gradient(np.angle(psi), step, axis=0)).max() / G.HELIUM_MASS
    return vmax, pcap, 0.7


def run_case(G, shape, step, model, clamp, pot2):
    """FP32 potential (and w_a for dft_ot_potential2), then 3 predict-correct steps"""
    shape = tuple(shape)
    psi = psi_of(shape, step, model)
    w, wp = G.Wf(shape, step), G.Wf(shape, step)
    ot = G.OT(model, w)
    if clamp:
        ot.params.max_veloc, ot.params.max_bfpot, ot.params.c_bfpot = limits(G, psi, step)
    w.set(psi)
    P = G.CGrid(shape, step)
    P.zero()
    out = []
    if pot2:
        rho = G.RGrid(shape, step)
        rho.set(np.abs(psi) ** 2)
        v = [G.RGrid(shape, step) for _ in range(3)]
        gx = np.gradient(np.angle(psi), step)
        for g, a in zip(v, gx):
            g.set(a / G.HELIUM_MASS)
        G.lib().dft_ot_potential2(ot.ptr, P.ptr, rho.ptr, v[0].ptr, v[1].ptr, v[2].ptr)
        G.check(what="dft_ot_potential2")
        out += [P.get()] + [g.get() for g in v]
        for o in v + [rho]:
            o.free()
    else:
        ot.potential(P, w)
        out.append(P.get())
    ot.run(w, wp, P, None, ot.bulk_chempot(0.0), 41.3 + 0j, 3, False)
    out.append(w.get())
    for o in (P, ot, wp, w):
        o.free()
    return out


def test_marching_pass_matches_per_row_pass(gpu, tmp_path):
    """Potentials and w_a within 1e-6 of the per-row form.  After the three
    steps the two FP32 wave functions may part by more where the potential
    is large (the compressed liquid of the high-density cases: V dt of
    hundreds of radians turns one-ulp differences of V into phase
    differences of 1e-4): there they agree within twice the per-row form's
    own distance from the FP64 run (FP64 takes the per-row form)."""
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(CASES), str(tmp_path)],
                       env=dict(os.environ, DFTGPU_MARCH="0"), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]
    try:
        for k, case in enumerate(CASES):
            gpu.set_precision(0)
            ref64 = run_case(gpu, *case)
            gpu.set_precision(1)
            got = run_case(gpu, *case)
            for j, a in enumerate(got):
                ref = np.load(tmp_path / ("case%d_%d.npy" % (k, j)))
                err = relerr(a, ref)
                tol = 1e-6
                if j == len(got) - 1:
                    tol = max(tol, 2 * relerr(ref, ref64[j]))
                print("case %s output %d: rel. difference %.2e (tolerance %.1e)" % (case, j, err, tol))
                assert err < tol, (case, j, err, tol)
    finally:
        gpu.set_precision(0)


def test_marching_clamped_backflow_vs_oracle(gpu, port):
    """the clamped, weighted backflow on a marching grid against the FP64 oracle"""
    shape, step, model = (24, 18, 128), 0.8, 9
    psi = psi_of(shape, step, model)
    gpu.set_precision(1)
    try:
        with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
            wo = g.wf(psi)
            full, plain = g.ot(model, wo), g.ot(1, wo)
            bf_part = g.potential(full, wo) - g.potential(plain, wo)
            lim = limits(gpu, psi, step, 0.4 * np.abs(bf_part.real).max())   # binds on part of the grid
            p = g.params(full)
            port.lib.orc_ot_set_limits(full, p["div_epsilon"], *lim)
            Pref = g.potential(full, wo)
        w = gpu.Wf(shape, step)
        ot = gpu.OT(model, w)
        ot.params.max_veloc, ot.params.max_bfpot, ot.params.c_bfpot = lim
        w.set(psi)
        P = gpu.CGrid(shape, step)
        P.zero()
        ot.potential(P, w)
        got = P.get()
        assert relerr(got.real, Pref.real) < 2e-5
        assert relerr(got.imag, Pref.imag) < 2e-4
        for o in (P, ot, w):
            o.free()
    finally:
        gpu.set_precision(0)
