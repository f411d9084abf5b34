"""The thermal OT models on the GPU (DFT_OT_T0MK ... T3000MK: the parameter
sets of src/ot.c:1038-1222 and, from T400MK on, the ideal Bose gas term of
src/ot.c:402-407, 804-809 and src/ot-energy.c:101-105).

libdft's form of the term (src/common.c:253-529) finds the fugacity z by a
golden-section search to a bracket of 1e-6; the GPU solves the same
truncated series for z to its working precision.  On a droplet over a
1e-4 rho0 vapour the two potentials differ by at most a few 1e-6 K (where z
is smallest), so FP64 is held to 1e-6 relative here instead of the 1e-10 of
the other terms.  The oracle's restatement equals libdft's own code on the
same shim and libdft's bulk relations (tests/test_oracle.py)."""
import numpy as np
import pytest

from conftest import relerr, thermal_psi
from oracle import Grids

pytestmark = pytest.mark.gpu

TOL = {0: 1e-6, 1: 2e-5}


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("model", [16, 32, 32 | 9, 4096 | 1, 262144 | 8])
def test_thermal_potential_energy_and_steps_vs_oracle(gpu, port, prec, model):
    shape, step = (16, 18, 20), 0.8
    psi = thermal_psi(port, shape, step)
    dt = 1.0 / gpu.AUTOFS + 0j
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo = g.wf(psi)
        oo = g.ot(model, wo)
        Pref = g.potential(oo, wo)
        edref = g.energy_density(oo, wo)
        mu0 = port.lib.orc_bulk_chempot(oo, 0.0)
        wpo, Po = g.wf(), g.cgrid()
        for _ in range(2):
            port.lib.orc_pc_step(oo, wo, wpo, Po, None, mu0, dt.real, dt.imag)
        ref = g.get_wf(wo)
    gpu.set_precision(prec)
    try:
        w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
        ot = gpu.OT(model, w)
        assert abs(ot.bulk_chempot(0.0) - mu0) <= 1e-12 * abs(mu0)
        w.set(psi)
        P = gpu.CGrid(shape, step)
        P.zero()
        ot.potential(P, w)
        got = P.get()
        assert relerr(got.real, Pref.real) < TOL[prec]
        if model & 8:
            assert relerr(got.imag, Pref.imag) < 20 * TOL[prec]
        ed = gpu.RGrid(shape, step)
        ot.energy_density(ed, w)
        assert relerr(ed.get(), edref) < TOL[prec]
        for _ in range(2):
            ot.pc_step(w, wp, P, None, mu0, dt)
        assert relerr(w.get(), ref) < 3 * TOL[prec]
        for o in (ed, P, ot, wp, w):
            o.free()
    finally:
        gpu.set_precision(0)


@pytest.mark.parametrize("model", [32, 4096, 262144])
@pytest.mark.parametrize("frac", [1.0, 0.05, 1e-3])
def test_thermal_uniform_liquid_is_the_bulk_derivative(gpu, model, frac):
    """the potential and energy density of a uniform liquid equal the bulk
    relations (the library's host form, equal to libdft's): exactly in the
    condensed branch, within the golden-section resolution in the dilute one"""
    shape, step = (12, 10, 8), 0.9
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    L = gpu.lib()
    rho = frac * L.dft_ot_bulk_density(ot.ptr)
    w.set(np.full(shape, np.sqrt(rho), dtype=complex))
    P = gpu.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    mu = L.dft_ot_bulk_dEdRho(ot.ptr, rho)
    assert relerr(P.get().real, np.full(shape, mu)) < 1e-9
    ed = gpu.RGrid(shape, step)
    ot.energy_density(ed, w)
    assert relerr(ed.get(), np.full(shape, L.dft_ot_bulk_energy(ot.ptr, rho))) < 1e-9
    for o in (ed, P, ot, w):
        o.free()


def test_thermal_adjoint_is_refused(gpu):
    shape, step = (8, 8, 8), 0.9
    w = gpu.Wf(shape, step)
    ot = gpu.OT(32 | 9, w)
    w.set(np.full(shape, 0.05 + 0j))
    rt, gv = gpu.RGrid(shape, step), gpu.RGrid(shape, step)
    rt.set(np.full(shape, 0.0025))
    with pytest.raises(gpu.DftGpuError):
        ot.adjoint_run(w, None, ot.bulk_chempot(0.0), 1.0 + 0j, 2, False, rt, gv)
    for o in (gv, rt, ot, w):
        o.free()
