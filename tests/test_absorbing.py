"""Absorbing boundary (grid_wf_boundary / grid_wf_absorb_potential; libdft's
callers examples/gas-bubble/bubble.c:149-157, examples/1d-bubble/
bubble-1d.c:192,222).  libgrid's arithmetic is not in the reference tree; the
library and the oracle restate the same documented form: outside
[lx, hx) x [ly, hy) x [lz, hz) a weight lambda rises linearly to 1 at the grid's
edge, and the absorbing potential -i amp lambda (|psi|^2 / rho0 - 1) is added
to the potential of predict / correct steps (evaluated from the step's input)
or by grid_wf_absorb_potential.

CPU: the weight profile, and that the layer removes an excess of liquid
(real-time steps lose norm there, none without the boundary).  GPU: the
absorbing potential and predict-correct steps (single calls and the captured
step graph) against the oracle in FP64 and FP32; the adjoint refuses a wave
function with a boundary."""
import numpy as np
import pytest

from conftest import coords, relerr
from oracle import Grids

SHAPE, STEP = (24, 20, 32), 0.9
LAYER = (3, 21, 0, 20, 5, 27)          # lx, hx, ly, hy, lz, hz (no layer along y)
AMP = 20.0 / 3.1577502480407e5          # 20 K


def weight(shape, layer):
    lam = np.zeros(shape)
    for ax, (n, l, h) in enumerate(zip(shape, layer[0::2], layer[1::2])):
        i = np.arange(n, dtype=float)
        r = np.where(i < l, (l - i) / max(l, 1), np.where(i >= h, (i - h + 1) / max(n - h, 1), 0.0))
        sh = [1, 1, 1]
        sh[ax] = n
        lam = np.maximum(lam, r.reshape(sh))
    return lam


def excess_psi(shape, step, rho0, seed=4):
    """bulk liquid with a 30 % density excess reaching into the absorbing layer along x and z"""
    rng = np.random.default_rng(seed)
    X, Y, Z = coords(shape, step)
    bump = np.exp(-((np.abs(X) - 9.0) ** 2 + Y ** 2 + (np.abs(Z) - 11.0) ** 2) / (2 * 2.5 ** 2))
    rho = rho0 * (1 + 0.3 * bump) * (1 + 0.01 * rng.random(shape))
    return np.sqrt(rho) * np.exp(0.05j * np.sin(2 * np.pi * X / (shape[0] * step)))


def oracle_steps(port, psi, rho0, model, nsteps, dt, boundary):
    with Grids(port, SHAPE, STEP, 4.002602 / port.AUTOAMU) as g:
        wo, wpo, Po = g.wf(psi), g.wf(), g.cgrid()
        if boundary:
            port.lib.orc_wf_boundary(wo, wpo, AMP, rho0, *LAYER)
        oo = g.ot(model, wo)
        mu0 = port.lib.orc_bulk_chempot(oo, 0.0)
        for _ in range(nsteps):
            port.lib.orc_pc_step(oo, wo, wpo, Po, None, mu0, dt.real, dt.imag)
        return g.get_wf(wo), mu0


def test_absorbing_weight_profile(port):
    rho0 = 0.0218360 * port.AUTOANG ** 3
    with Grids(port, SHAPE, STEP, 4.002602 / port.AUTOAMU) as g:
        w = g.wf(np.full(SHAPE, np.sqrt(2 * rho0), dtype=complex))      # |psi|^2 / rho0 - 1 = 1
        port.lib.orc_wf_boundary(w, None, AMP, rho0, *LAYER)
        P = g.cgrid(np.zeros(SHAPE, dtype=complex))
        port.lib.orc_wf_absorb_potential(w, P, AMP, rho0)
        V = g.get_c(P)
    assert np.abs(V.real).max() == 0.0
    assert np.allclose(-V.imag / AMP, weight(SHAPE, LAYER), rtol=0, atol=1e-14)


def test_absorbing_layer_removes_excess_liquid(port):
    rho0 = 0.0218360 * port.AUTOANG ** 3
    psi = excess_psi(SHAPE, STEP, rho0)
    n0 = np.sum(np.abs(psi) ** 2)
    dt = 2.0 / port.AUTOFS + 0j
    with_b, _ = oracle_steps(port, psi, rho0, 0, 6, dt, True)
    without, _ = oracle_steps(port, psi, rho0, 0, 6, dt, False)
    loss_b = 1 - np.sum(np.abs(with_b) ** 2) / n0
    loss_0 = 1 - np.sum(np.abs(without) ** 2) / n0
    assert abs(loss_0) < 1e-12          # real time without the layer: unitary
    assert loss_b > 1e-4, loss_b        # the layer absorbs the excess


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
def test_absorbing_boundary_matches_oracle(gpu, port, prec):
    tol = 1e-10 if prec == 0 else 1e-5
    rho0 = 0.0218360 * gpu.AUTOANG ** 3
    psi = excess_psi(SHAPE, STEP, rho0)
    dt = 2.0 / gpu.AUTOFS + 0j
    ref, mu0 = oracle_steps(port, psi, rho0, 9, 4, dt, True)
    with Grids(port, SHAPE, STEP, gpu.HELIUM_MASS) as g:   # absorbing potential of a non-uniform liquid
        w = g.wf(psi)
        port.lib.orc_wf_boundary(w, None, AMP, rho0, *LAYER)
        P0 = np.exp(1j * np.linspace(0, 1, psi.size)).reshape(SHAPE) * 1e-5
        Po = g.cgrid(P0)
        port.lib.orc_wf_absorb_potential(w, Po, AMP, rho0)
        Vref = g.get_c(Po)
    L = gpu.lib()
    gpu.set_precision(prec)
    w, wp = gpu.Wf(SHAPE, STEP), gpu.Wf(SHAPE, STEP)
    w.set(psi)
    L.grid_wf_boundary(w.ptr, wp.ptr, AMP, rho0, *LAYER)
    gpu.check(what="grid_wf_boundary")
    P = gpu.CGrid(SHAPE, STEP)
    P.set(P0)
    L.grid_wf_absorb_potential(w.ptr, P.ptr, AMP, rho0)
    gpu.check(what="grid_wf_absorb_potential")
    assert relerr(P.get(), Vref) < tol
    ot = gpu.OT(9, w)
    for _ in range(4):
        ot.pc_step(w, wp, P, None, mu0, dt)
    assert relerr(w.get(), ref) < 3 * tol
    w.set(psi)
    ot.run(w, wp, P, None, mu0, dt, 4, False)           # the captured step graph
    assert relerr(w.get(), ref) < 3 * tol
    # the adjoint does not differentiate the layer
    rt, gv = gpu.RGrid(SHAPE, STEP), gpu.RGrid(SHAPE, STEP)
    rt.set(np.abs(psi) ** 2)
    with pytest.raises(gpu.DftGpuError):
        ot.adjoint_run(w, None, mu0, dt, 2, False, rt, gv)
    for o in (gv, rt, P, ot, wp, w):
        o.free()
    gpu.set_precision(0)
