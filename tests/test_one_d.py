"""The 1-D effective model on the GPU (grids with nx = ny = 1: libdft's
DFT_OT_1D branch, src/ot.c:133-217, src/ot.h:146; its driver
examples/1d-bubble/bubble-1d.c runs 1 x 1 x 4096 with step 0.2 bohr).

The kernels are libdft's 1-D forms, integrated over the x-y plane and not
rescaled; the convolutions use the line element dz (the oracle's shim
restates that libgrid detail; the oracle's 1-D branch equals libdft's own
ot.c on the shim, tests/test_oracle.py).  Here the GPU against the FP64 oracle:
potential, energy density and three predict-correct steps, FP64 and FP32, on
lengths of the register-resident path (64, 96, 128) and of the long-line
generic path (4096)."""
import numpy as np
import pytest

from conftest import line_psi, relerr
from oracle import Grids

pytestmark = pytest.mark.gpu

TOL = {0: 1e-10, 1: 1e-5}


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("n,step,model", [(64, 0.8, 9), (96, 0.8, 1), (128, 0.8, 8), (4096, 0.2, 0),
                                          (4096, 0.2, 9)])
def test_one_d_potential_and_steps_vs_oracle(gpu, port, prec, n, step, model):
    shape = (1, 1, n)
    psi = line_psi(port, n, step)
    dt = 2.0 / gpu.AUTOFS + 0j
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo = g.wf(psi)
        oo = g.ot(model, wo)
        Pref = g.potential(oo, wo)
        edref = g.energy_density(oo, wo)
        mu0 = port.lib.orc_bulk_chempot(oo, 0.0)
        wpo, Po = g.wf(), g.cgrid()
        for _ in range(3):
            port.lib.orc_pc_step(oo, wo, wpo, Po, None, mu0, dt.real, dt.imag)
        ref = g.get_wf(wo)
    gpu.set_precision(prec)
    try:
        w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
        ot = gpu.OT(model, w)
        w.set(psi)
        P = gpu.CGrid(shape, step)
        P.zero()
        ot.potential(P, w)
        got = P.get()
        assert relerr(got.real, Pref.real) < 2 * TOL[prec]
        if model & 8:   # the imaginary part, relative to the potential (it can be 1e-6 of it)
            err = min(relerr(got.imag, Pref.imag), np.abs(got.imag - Pref.imag).max() / np.abs(Pref).max())
            assert err < 20 * TOL[prec]
        ed = gpu.RGrid(shape, step)
        ot.energy_density(ed, w)
        assert relerr(ed.get(), edref) < 2 * TOL[prec]
        for _ in range(3):
            ot.pc_step(w, wp, P, None, mu0, dt)
        assert relerr(w.get(), ref) < 3 * TOL[prec]
        for o in (ed, P, ot, wp, w):
            o.free()
    finally:
        gpu.set_precision(0)


def test_one_d_grid_limits(gpu):
    """nz up to 4096 on a 1-D grid; 3-D grids keep each dimension in [2, 1024]"""
    w = gpu.Wf((1, 1, 4096), 0.2)
    w.free()
    with pytest.raises(gpu.DftGpuError):
        gpu.Wf((1, 1, 8192), 0.2)
    with pytest.raises(gpu.DftGpuError):
        gpu.Wf((2, 2, 2048), 0.2)
    with pytest.raises(gpu.DftGpuError):
        gpu.Wf((1, 4, 16), 0.2)
