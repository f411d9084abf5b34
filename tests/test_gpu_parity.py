"""GPU parity: libdftgpu (through its C ABI) against the FP64 CPU oracle and
the fixtures produced by libdft's own source (tests/golden).

Tolerances (max-norm error relative to the max-norm of the reference):
  FP64 grids: 1e-10 (the oracle and the GPU code differ only in rounding order)
  FP32 grids: 1e-5 for spectra / potentials / energy densities (a few FP32
              ulps times log2 N accumulation through the 3-D transforms).
"""
import numpy as np
import pytest

from conftest import coords, golden, liquid_psi, relerr
from oracle import Grids

pytestmark = pytest.mark.gpu

TOL = {0: 1e-10, 1: 1e-5}
PRECS = [0, 1]


@pytest.fixture(params=PRECS, ids=["fp64", "fp32"])
def prec(request, gpu):
    gpu.set_precision(request.param)
    yield request.param
    gpu.set_precision(0)


@pytest.mark.parametrize("shape", [(16, 16, 16), (16, 18, 20), (32, 24, 40), (64, 64, 64), (30, 36, 50),
                                   (8, 16, 512), (64, 256, 32), (128, 128, 128), (96, 120, 160),
                                   (16, 256, 256), (6, 512, 512),
                                   # smallest and largest axes (2 and 1024: generic kernels in FP32 too)
                                   (2, 4, 6), (4, 6, 2), (1024, 8, 4), (4, 6, 1024), (8, 1024, 2),
                                   # 3 * 2^k lengths (96, 192, 384: register-resident in FP32), an odd
                                   # axis of 729 (partial tiles of the generic y pass) and 240 / 120
                                   (96, 64, 384), (192, 96, 192), (384, 16, 192), (32, 384, 96),
                                   (729, 8, 6), (9, 729, 4), (240, 16, 240)])
def test_rfft_spectrum(gpu, prec, shape):
    rng = np.random.default_rng(1)
    f = rng.standard_normal(shape)
    r = gpu.RGrid(shape, 1.0)
    r.set(f)
    s = r.spectrum()
    r.free()
    assert relerr(s, np.fft.rfftn(f)) < TOL[prec] * 3


def octant(full, shape, odd_axis=None, scale=1.0):
    """oracle half spectrum [x][y][kz] -> stored octant [kz][kx][ky] with centring sign"""
    nx, ny, nz = shape
    ix, iy, iz = np.arange(nx // 2 + 1), np.arange(ny // 2 + 1), np.arange(nz // 2 + 1)
    sub = full[np.ix_(ix, iy, iz)]                    # [kx][ky][kz]
    val = sub.imag if odd_axis is not None else sub.real
    sign = (-1.0) ** (ix[:, None, None] + iy[None, :, None] + iz[None, None, :])
    return np.transpose(val * sign * scale, (2, 0, 1))


@pytest.mark.parametrize("fixture", ["full_mixed.npz"])
def test_kernels_match_reference(gpu, prec, fixture):
    fx = golden(fixture)
    shape, step = tuple(int(s) for s in fx["shape"]), float(fx["step"])
    w = gpu.Wf(shape, step)
    ot = gpu.OT(int(fx["model"]), w)
    n = np.prod(shape)
    for i in range(7):
        ref = octant(fx["kernels"][i], shape, odd_axis=(i - 3) if 3 <= i <= 5 else None, scale=step ** 3 / n)
        got = ot.kernel(i)
        assert relerr(got, ref) < max(TOL[prec], 1e-7), i
    ot.free()
    w.free()


@pytest.mark.parametrize("fixture", ["plain_16.npz", "full_mixed.npz", "full_lg11.npz"])
def test_potential_and_energy_density_match_reference(gpu, prec, fixture):
    fx = golden(fixture)
    shape, step = tuple(int(s) for s in fx["shape"]), float(fx["step"])
    w = gpu.Wf(shape, step)
    lg = float(fx["lg"]) if "lg" in fx else None
    ot = gpu.OT(int(fx["model"]), w, lg_bohr=lg)
    w.set(fx["psi"])
    P = gpu.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    got = P.get()
    ref = fx["P"]
    assert relerr(got.real, ref.real) < TOL[prec]
    if np.abs(ref.imag).max() > 0:
        assert relerr(got.imag, ref.imag) < 10 * TOL[prec]
    ed = gpu.RGrid(shape, step)
    ot.energy_density(ed, w)
    assert relerr(ed.get(), fx["ed"]) < TOL[prec]
    for o in (ed, P, ot, w):
        o.free()


@pytest.mark.parametrize("shape,step,model", [((32, 32, 32), 0.8, 9), ((40, 36, 30), 0.7, 1), ((48, 32, 40), 1.0, 8),
                                              ((96, 80, 128), 0.8, 9), ((64, 64, 64), 0.8, 9),
                                              ((128, 64, 80), 0.8, 9), ((64, 128, 128), 0.8, 1),
                                              ((16, 256, 256), 0.8, 9), ((4, 512, 512), 0.5, 0),
                                              ((2, 4, 6), 1.0, 9), ((1024, 6, 4), 0.6, 9), ((6, 4, 1024), 0.6, 9),
                                              # odd x / y sizes (2^a 3^b 5^c; libdft's 729 x 384 x 384 grid,
                                              # examples/gas-bubble/config.h:56): kernels rotated by
                                              # exp(2 pi i k c / n) instead of the sign (-1)^k
                                              ((9, 10, 8), 0.8, 9), ((15, 9, 12), 0.9, 9), ((27, 25, 16), 0.8, 9),
                                              ((45, 3, 10), 0.8, 1), ((243, 16, 16), 0.8, 9),
                                              # 3 * 2^k lengths on the register-resident FP32 path: z passes
                                              # of 192 (nz = 384), y pass 96, x convolutions 192 / 96 / 384
                                              ((16, 96, 384), 0.8, 9), ((192, 32, 32), 0.8, 9),
                                              ((96, 64, 96), 0.8, 1), ((384, 16, 16), 0.6, 8)])
def test_potential_vs_oracle_live(gpu, port, prec, shape, step, model):
    psi = liquid_psi(shape, step, 3)
    ns = (2, 4) if np.prod(shape) > 200000 else (4, 32)      # coarser kernel sampling on big grids (CPU time)
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo = g.wf(psi)
        oo = g.ot(model, wo, min_ns=ns[0], max_ns=ns[1])
        Pref = g.potential(oo, wo, base=2e-5 + 1e-5j)
        edref = g.energy_density(oo, wo)
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w, min_ns=ns[0], max_ns=ns[1])
    w.set(psi)
    P = gpu.CGrid(shape, step)
    P.set(np.full(shape, 2e-5 + 1e-5j))      # the potential is accumulated into P
    ot.potential(P, w)
    got = P.get()
    assert relerr(got.real - 2e-5, Pref.real - 2e-5) < TOL[prec] * 2
    if model & 8:
        assert relerr(got.imag - 1e-5, Pref.imag - 1e-5) < 20 * TOL[prec]
    ed = gpu.RGrid(shape, step)
    ot.energy_density(ed, w)
    assert relerr(ed.get(), edref) < TOL[prec] * 2
    for o in (ed, P, ot, w):
        o.free()


def test_potential_with_backflow_limits_vs_oracle(gpu, port, prec):
    """max_veloc, max_bfpot and c_bfpot != 1 (src/ot.c:391-394, 911-914, 985-988)."""
    shape, step, model = (32, 32, 32), 0.8, 9
    psi = liquid_psi(shape, step, 5)
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo = g.wf(psi)
        full, plain = g.ot(model, wo), g.ot(1, wo)
        bf_part = g.potential(full, wo) - g.potential(plain, wo)
        p = g.params(full)
        vmax = 0.6 * np.abs(np.gradient(np.angle(psi), step, axis=0)).max() / gpu.HELIUM_MASS
        lim = (p["div_epsilon"], vmax, 0.4 * np.abs(bf_part.real).max(), 0.7)
        port.lib.orc_ot_set_limits(full, *lim)
        Pref = g.potential(full, wo)
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    ot.params.max_veloc, ot.params.max_bfpot, ot.params.c_bfpot = lim[1], lim[2], lim[3]
    w.set(psi)
    P = gpu.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    got = P.get()
    assert relerr(got.real, Pref.real) < TOL[prec] * 2
    assert relerr(got.imag, Pref.imag) < 20 * TOL[prec]
    for o in (P, ot, w):
        o.free()


def test_term_entry_points_match_reference(gpu, prec):
    """dft_ot_potential2 (with the velocities it overwrites), the single-term
    entry points and the KC / backflow energy-density parts against libdft's
    own functions (tests/golden/terms.npz)."""
    fx = golden("terms.npz")
    shape, step = tuple(int(s) for s in fx["shape"]), float(fx["step"])
    L = gpu.lib()
    w = gpu.Wf(shape, step)
    ot = gpu.OT(int(fx["model"]), w)
    w.set(fx["psi"])
    rho = gpu.RGrid(shape, step)
    rho.set(fx["rho"])
    v = [gpu.RGrid(shape, step) for _ in range(3)]
    P = gpu.CGrid(shape, step)

    def setv():
        for g, a in zip(v, fx["vel"]):
            g.set(a)

    def check_pot(ref, what):
        got = P.get()
        assert relerr(got.real, ref.real) < TOL[prec] * 3, what
        if np.abs(ref.imag).max() > 0:
            assert relerr(got.imag, ref.imag) < 20 * TOL[prec], what

    setv()
    P.zero()
    L.dft_ot_potential2(ot.ptr, P.ptr, rho.ptr, v[0].ptr, v[1].ptr, v[2].ptr)
    gpu.check(what="dft_ot_potential2")
    check_pot(fx["P2"], "potential2")
    for g, ref in zip(v, fx["w2"]):
        assert relerr(g.get(), ref) < 20 * TOL[prec]
    P.zero()
    L.dft_ot_add_lennard_jones_potential(ot.ptr, P.ptr, rho.ptr, None, None)
    check_pot(fx["Plj"], "lennard-jones")
    P.zero()
    L.dft_ot_add_local_correlation_potential(ot.ptr, P.ptr, rho.ptr, None, None, None)
    check_pot(fx["Ploc"], "local correlation")
    setv()
    P.zero()
    L.dft_ot_backflow_potential(ot.ptr, P.ptr, rho.ptr, v[0].ptr, v[1].ptr, v[2].ptr, *([None] * 6))
    gpu.check(what="dft_ot_backflow_potential")
    check_pot(fx["Pbf"], "backflow")
    for g, ref in zip(v, fx["wbf"]):
        assert relerr(g.get(), ref) < 20 * TOL[prec]
    ed = gpu.RGrid(shape, step)
    for fn, key in ((L.dft_ot_energy_density_kc, "edkc"), (L.dft_ot_energy_density_bf, "edbf")):
        ed.set(np.zeros(shape))
        fn(ot.ptr, ed.ptr, w.ptr, rho.ptr)
        gpu.check(what=key)
        assert relerr(ed.get(), fx[key]) < 20 * TOL[prec], key
    for o in [ed, P, rho, ot, w] + v:
        o.free()


@pytest.mark.parametrize("model", [0, 1, 8, 9])
def test_uniform_liquid_potential_is_chemical_potential(gpu, prec, model):
    shape, step = (32, 32, 32), 0.8
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    rho0 = ot.bulk_density(0.0)
    mu0 = ot.bulk_chempot(0.0)
    assert abs(mu0 * gpu.AUTOK + 7.149933) < 1e-6
    w.set(np.full(shape, np.sqrt(rho0), dtype=complex))
    P = gpu.CGrid(shape, step)
    P.zero()
    ot.potential(P, w)
    got = P.get()
    assert relerr(got.real, np.full(shape, mu0)) < (1e-12 if prec == 0 else 2e-6)
    assert np.abs(got.imag).max() < (1e-14 if prec == 0 else 1e-6) * abs(mu0)
    for o in (P, ot, w):
        o.free()


@pytest.mark.parametrize("shape", [(24, 20, 30), (128, 128, 128), (64, 96, 160),
                                   (2, 6, 4), (1024, 4, 6), (6, 4, 1024), (4, 1024, 2), (9, 15, 10), (27, 5, 8),
                                   (96, 48, 384), (384, 8, 12), (27, 96, 192)])
def test_propagate_matches_oracle(gpu, port, prec, shape):
    step = 0.9
    rng = np.random.default_rng(9)
    psi = liquid_psi(shape, step, 9)
    V = (rng.standard_normal(shape) + 0.2j * rng.standard_normal(shape)) * 1e-5
    dts = [41.3 + 0j, -20j, 30 - 5j]
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo, Po = g.wf(psi), g.cgrid(V)
        ref = []
        for dt in dts:
            port.lib.orc_propagate(wo, Po, dt.real, dt.imag)
            ref.append(g.get_wf(wo))
        wp = g.wf()
        port.lib.orc_predict(wo, wp, Po, 10.0, -1.0)
        refp, refk, refn = g.get_wf(wp), port.lib.orc_wf_kinetic_energy(wo), port.lib.orc_wf_norm(wo)
    w = gpu.Wf(shape, step)
    P = gpu.CGrid(shape, step)
    w.set(psi)
    P.set(V)
    for dt, r in zip(dts, ref):
        w.propagate(P, dt)
        assert relerr(w.get(), r) < TOL[prec] * 3
    wp = gpu.Wf(shape, step)
    w.predict(wp, P, 10.0 - 1.0j)
    assert relerr(wp.get(), refp) < TOL[prec] * 3
    assert abs(w.kinetic_energy() / refk - 1) < TOL[prec] * 3
    assert abs(w.norm() / refn - 1) < TOL[prec] * 3        # FP64 runs of 8 (and a short last run)
    for o in (wp, P, w):
        o.free()


@pytest.mark.parametrize("shape", [(24, 20, 30), (64, 96, 32)])
def test_velocity_matches_oracle(gpu, port, prec, shape):
    """grid_wf_velocity (the exported entry point, src/ot.c:387-390) against
    the oracle: v = (hbar/m) Im(psi* D psi) / max(|psi|^2, eps), central
    differences, with a region of near-zero density so that eps is active."""
    step = 0.9
    psi = liquid_psi(shape, step, 13)
    X, Y, Z = coords(shape, step)
    psi = psi * np.tanh(np.sqrt(X ** 2 + (Y - 3.0) ** 2 + Z ** 2) / 2.0) ** 3   # a cavity: |psi|^2 -> 0
    eps = 1e-4 * float(np.max(np.abs(psi) ** 2))
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo, vx, vy, vz = g.wf(psi), g.rgrid(), g.rgrid(), g.rgrid()
        port.lib.orc_wf_velocity(wo, vx, vy, vz, eps)
        ref = [g.get_r(v) for v in (vx, vy, vz)]
    w = gpu.Wf(shape, step)
    w.set(psi)
    out = [gpu.RGrid(shape, step) for _ in range(3)]
    L = gpu.lib()
    L.grid_wf_velocity(w.ptr, out[0].ptr, out[1].ptr, out[2].ptr, eps)
    assert L.dftgpu_last_error() == 0
    for o, r in zip(out, ref):
        assert relerr(o.get(), r) < (1e-12 if prec == 0 else 2e-5)
    for o in out + [w]:
        o.free()


def test_pc_steps_match_reference_plain(gpu, prec):
    fx = golden("plain_16.npz")
    shape, step = tuple(int(s) for s in fx["shape"]), float(fx["step"])
    w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
    ot = gpu.OT(0, w)
    w.set(fx["psi"])
    w.norm_target = float(fx["norm0"])
    P, ve = gpu.CGrid(shape, step), gpu.RGrid(shape, step)
    ve.set(fx["vext"])
    for _ in range(3):
        ot.pc_step(w, wp, P, ve, float(fx["mu0"]), complex(fx["dt"]))
        w.normalize()
    assert relerr(w.get(), fx["psi3"]) < TOL[prec] * 3
    e, n, mu = ot.energy_report(w, ve)
    assert abs(e / float(fx["etot3"]) - 1) < (1e-10 if prec == 0 else 1e-5)
    assert abs(n / float(fx["norm0"]) - 1) < (1e-12 if prec == 0 else 1e-6)
    for o in (ve, P, ot, wp, w):
        o.free()


def test_pc_steps_match_reference_full(gpu, prec):
    fx = golden("full_mixed.npz")
    shape, step = tuple(int(s) for s in fx["shape"]), float(fx["step"])
    w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
    ot = gpu.OT(int(fx["model"]), w)
    w.set(fx["psi"])
    P = gpu.CGrid(shape, step)
    for _ in range(2):
        ot.pc_step(w, wp, P, None, float(fx["mu0"]), complex(fx["dt"]))
    assert relerr(w.get(), fx["psi2"]) < TOL[prec] * 3
    for o in (P, ot, wp, w):
        o.free()


def test_run_graph_is_bitwise_equal_to_steps(gpu, prec):
    shape, step = (32, 32, 32), 0.8
    psi = liquid_psi(shape, step, 4)
    out = []
    for use_run in (False, True):
        w, wp = gpu.Wf(shape, step), gpu.Wf(shape, step)
        ot = gpu.OT(9, w)
        w.set(psi)
        w.norm_target = 3.0
        P = gpu.CGrid(shape, step)
        mu0 = ot.bulk_chempot(0.0)
        if use_run:
            ot.run(w, wp, P, None, mu0, -10j / gpu.AUTOFS, 5, True)
        else:
            for _ in range(5):
                ot.pc_step(w, wp, P, None, mu0, -10j / gpu.AUTOFS)
                w.normalize()
        out.append(w.get())
        for o in (P, ot, wp, w):
            o.free()
    assert np.array_equal(out[0], out[1])


def test_energy_report_matches_oracle(gpu, port, prec):
    shape, step, model = (24, 24, 24), 0.8, 9
    psi = liquid_psi(shape, step, 12)
    X, Y, Z = coords(shape, step)
    vext = 5.0 / gpu.AUTOK * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 8.0)
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo, vo, work = g.wf(psi), g.rgrid(vext), g.rgrid()
        oo = g.ot(model, wo)
        eref = port.lib.orc_total_energy(oo, wo, vo, work)
        nref = port.lib.orc_wf_norm(wo)
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    w.set(psi)
    ve = gpu.RGrid(shape, step)
    ve.set(vext)
    e, n, mu = ot.energy_report(w, ve)
    assert abs(e / eref - 1) < (1e-10 if prec == 0 else 1e-5)
    assert abs(n / nref - 1) < (1e-12 if prec == 0 else 1e-6)
    assert np.isfinite(mu)
    for o in (ve, ot, w):
        o.free()


def test_errors_are_reported(gpu):
    L = gpu.lib()
    assert not L.grid_wf_alloc(17, 16, 16, 1.0, 7000.0, 3, 1, b"prime17")  # factor 17
    assert L.dftgpu_last_error() == 2
    assert not L.grid_wf_alloc(16, 16, 15, 1.0, 7000.0, 3, 1, b"oddz")     # odd z (packed real rows)
    assert L.dftgpu_last_error() == 2
    assert not L.grid_wf_alloc(14, 16, 16, 1.0, 7000.0, 3, 1, b"prime7")   # factor 7
    assert L.dftgpu_last_error() == 2
    assert not L.grid_wf_alloc(16, 16, 16, 1.0, 7000.0, 1, 1, b"dirichlet")
    assert L.dftgpu_last_error() == 6
    w = gpu.Wf((16, 16, 16), 1.0)
    assert not L.dft_ot_alloc(1048576, w.ptr, 4, 32)                       # DFT_DR (Dupont-Roc)
    assert L.dftgpu_last_error() == 6
    psi = np.ones((16, 16, 16), dtype=complex)
    psi[3, 4, 5] = np.nan
    w.set(psi)
    v = L.grid_wf_norm(w.ptr)
    assert np.isnan(v)
    assert L.dftgpu_last_error() == 5
    w.free()
