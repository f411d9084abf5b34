"""Crank-Nicolson propagator (WF_2ND_ORDER_CN, examples/gas-bubble/config.h:66,
examples/imag_time_rot/imag_time.c:102).  libgrid, which implements it for the
reference, is absent; the restatement both sides share is Crank-Nicolson on
the 3-point finite-difference kinetic operator, applied axis by axis (x, y, z)
inside the same Strang step as the FFT propagator, on the periodic grid, with
the moving background entering as the phase of the off-diagonal couplings
(T f[j] = (2 f[j] - e^{-i k0 h} f[j+1] - e^{i k0 h} f[j-1]) hbar^2 / (2 m h^2)).
Each axis operator is then diagonal in k, so the library and the oracle apply
(1 - i dt Q / 4m) / (1 + i dt Q / 4m), Q = (2 sin((k - k0) h / 2) / h)^2, per
axis in k space.

* CPU: the oracle's step equals the definition computed directly -- dense
  cyclic tridiagonal solves along each axis -- for real, imaginary and complex
  dt with a momentum off the reciprocal grid; its kinetic energy equals
  <psi|T|psi> with T applied as the second difference; real-time steps keep
  the norm; for a smooth state and a small step it approaches the FFT
  propagator.
* GPU against the oracle: the bare propagator (generic kinetic pass in FP64
  and FP32, register kinetic pass in FP32, a 1-D line), the kinetic energy,
  predict-correct steps of the full functional; the adjoint identity of the
  propagator and a trajectory gradient against finite differences.
"""
import numpy as np
import pytest

from conftest import liquid_psi, relerr
from oracle import Grids

FFT, CN = 1, 3


def second_difference(n, h, k0):
    """T / (hbar^2 / 2m) on a periodic line: the cyclic tridiagonal matrix"""
    T = np.zeros((n, n), dtype=np.complex128)
    for j in range(n):
        T[j, j] += 2.0 / h ** 2
        T[j, (j + 1) % n] += -np.exp(-1j * k0 * h) / h ** 2
        T[j, (j - 1) % n] += -np.exp(1j * k0 * h) / h ** 2
    return T


def cn_direct(psi, V, h, mass, dt, k0):
    """exp(-i V dt/2) CN_z CN_y CN_x exp(-i V dt/2) psi by dense solves"""
    half = np.exp(-1j * V * dt / 2)
    out = psi * half
    for ax in range(3):
        n = psi.shape[ax]
        A = 1j * dt / (4 * mass) * second_difference(n, h, k0[ax])
        M = np.linalg.solve(np.eye(n) + A, np.eye(n) - A)   # (1 + A)^-1 (1 - A)
        out = np.moveaxis(np.tensordot(M, np.moveaxis(out, ax, 0), axes=(1, 0)), 0, ax)
    return out * half


def oracle_propagate(port, shape, h, mass, psi, V, dt, k0, propagator, nsteps=1):
    with Grids(port, shape, h, mass) as g:
        w, P = g.wf(psi, propagator), g.cgrid(V)
        port.lib.orc_wf_set_momentum(w, *k0)
        for _ in range(nsteps):
            port.lib.orc_propagate(w, P, dt.real, dt.imag)
        return g.get_wf(w), port.lib.orc_wf_kinetic_energy(w)


def off_grid_momentum(shape, h):
    dk = [2 * np.pi / (n * h) for n in shape]
    return (0.37 * dk[0], -1.3 * dk[1], 2.2 * dk[2])


@pytest.mark.parametrize("dt", [41.3 + 0j, -300j, 30 - 5j])
def test_oracle_cn_equals_direct_tridiagonal_solves(port, dt):
    shape, h, mass = (6, 8, 10), 0.7, 7296.3
    rng = np.random.default_rng(1)
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    V = 1e-3 * (rng.standard_normal(shape) + 0.2j * rng.standard_normal(shape))
    k0 = off_grid_momentum(shape, h)
    out, _ = oracle_propagate(port, shape, h, mass, psi, V, dt, k0, CN)
    ref = cn_direct(psi, V, h, mass, dt, k0)
    assert relerr(out, ref) < 1e-12
    # and it is not the FFT propagator (a rough state differs at first order)
    fft, _ = oracle_propagate(port, shape, h, mass, psi, V, dt, k0, FFT)
    assert relerr(fft, ref) > 1e-3


def test_oracle_cn_kinetic_energy_is_the_finite_difference_one(port):
    shape, h, mass = (6, 8, 10), 0.7, 7296.3
    rng = np.random.default_rng(2)
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    k0 = off_grid_momentum(shape, h)
    _, t = oracle_propagate(port, shape, h, mass, psi, np.zeros(shape), 0j, k0, CN, nsteps=0)
    Tpsi = np.zeros_like(psi)
    for ax in range(3):
        T = second_difference(shape[ax], h, k0[ax])
        Tpsi += np.moveaxis(np.tensordot(T, np.moveaxis(psi, ax, 0), axes=(1, 0)), 0, ax)
    ref = float(np.real(np.vdot(psi, Tpsi))) / (2 * mass) * h ** 3
    assert abs(t / ref - 1) < 1e-12


def test_oracle_cn_keeps_norm_and_approaches_fft_for_smooth_states(port):
    shape, h, mass = (24, 20, 16), 0.8, 7296.3
    psi = liquid_psi(shape, h, 3, amp=0.05)
    V = np.zeros(shape)
    k0 = (0.0, 0.0, 0.0)
    n0 = np.sum(np.abs(psi) ** 2)
    cn, _ = oracle_propagate(port, shape, h, mass, psi, V, 41.3 + 0j, k0, CN, nsteps=5)
    assert abs(np.sum(np.abs(cn) ** 2) / n0 - 1) < 1e-12
    fft, _ = oracle_propagate(port, shape, h, mass, psi, V, 41.3 + 0j, k0, FFT, nsteps=5)
    assert relerr(cn, fft) < 2e-3


# ------------------------------------------------------------------ GPU

@pytest.mark.gpu
@pytest.mark.parametrize("prec,shape,tol", [(0, (24, 20, 16), 1e-11), (0, (30, 18, 20), 1e-11),
                                            (0, (1, 1, 256), 1e-11), (1, (27, 24, 20), 3e-5),
                                            (1, (64, 64, 64), 3e-5), (1, (96, 64, 64), 3e-5)])
@pytest.mark.parametrize("dt", [41.3 + 0j, 30 - 5j])
def test_cn_propagate_matches_oracle(gpu, port, prec, shape, tol, dt):
    h, mass = 0.9, gpu.HELIUM_MASS
    rng = np.random.default_rng(4)
    psi = liquid_psi(shape, h, 7)
    V = 1e-4 * (rng.standard_normal(shape) + 0.2j * rng.standard_normal(shape))
    k0 = off_grid_momentum(shape, h)
    ref, t_ref = oracle_propagate(port, shape, h, mass, psi, V, dt, k0, CN, nsteps=2)
    gpu.set_precision(prec)
    w, P = gpu.Wf(shape, h, propagator=gpu.WF_2ND_ORDER_CN), gpu.CGrid(shape, h)
    w.set(psi)
    w.set_momentum(*k0)
    P.set(V)
    for _ in range(2):
        w.propagate(P, dt)
    out, t = w.get(), w.kinetic_energy()
    for o in (P, w):
        o.free()
    gpu.set_precision(0)
    assert relerr(out, ref) < tol
    assert abs(t / t_ref - 1) < (1e-11 if prec == 0 else 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,shape,tol", [(0, (32, 24, 20), 1e-10), (1, (64, 64, 64), 3e-5)])
def test_cn_full_functional_matches_oracle(gpu, port, prec, shape, tol):
    """Predict-correct steps of the full functional (KC + BF) on a CN wave
    function with a moving background, imaginary then real time."""
    h = 0.9
    psi = liquid_psi(shape, h, 3)
    k0 = off_grid_momentum(shape, h)
    segments = [(-200j, 2), (41.3 + 0j, 2)]
    mass = gpu.HELIUM_MASS
    with Grids(port, shape, h, mass) as g:
        wo, wpo, Po = g.wf(psi, CN), g.wf(None, CN), g.cgrid()
        o = g.ot(9, wo)
        mu0 = port.lib.orc_bulk_chempot(o, 0.0)
        port.lib.orc_wf_set_momentum(wo, *k0)
        port.lib.orc_wf_set_momentum(wpo, *k0)
        for dt, n in segments:
            for _ in range(n):
                port.lib.orc_pc_step(o, wo, wpo, Po, None, mu0, dt.real, dt.imag)
        ref, t_ref = g.get_wf(wo), port.lib.orc_wf_kinetic_energy(wo)
    gpu.set_precision(prec)
    w = gpu.Wf(shape, h, propagator=gpu.WF_2ND_ORDER_CN)
    wp = gpu.Wf(shape, h, propagator=gpu.WF_2ND_ORDER_CN)
    P = gpu.CGrid(shape, h)
    ot = gpu.OT(9, w)
    w.set(psi)
    w.set_momentum(*k0)
    wp.set_momentum(*k0)
    for dt, n in segments:
        ot.run(w, wp, P, None, mu0, dt, n, False)
    out, t = w.get(), w.kinetic_energy()
    for x in (P, ot, wp, w):
        x.free()
    gpu.set_precision(0)
    assert relerr(out, ref) < tol
    assert abs(t / t_ref - 1) < (1e-10 if prec == 0 else 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_cn_propagator_adjoint_identity(gpu, prec):
    shape, h, dt = (64, 32, 32), 0.9, 30 - 5j
    rng = np.random.default_rng(8)
    gpu.set_precision(prec)
    psi = liquid_psi(shape, h, 5)
    V = (rng.standard_normal(shape) + 0.3j * rng.standard_normal(shape)) * 1e-3
    g_out = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    d = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    w, P = gpu.Wf(shape, h, propagator=gpu.WF_2ND_ORDER_CN), gpu.CGrid(shape, h)
    w.set_momentum(*off_grid_momentum(shape, h))
    P.set(V)
    w.set(d)
    w.propagate(P, dt)
    Sd = w.get()
    w.set(psi)
    w.propagate(P, dt)
    grids = [gpu.CGrid(shape, h) for _ in range(5)]
    gin, gout, gpi, gpo, gpot = grids
    gin.set(psi)
    gout.set(w.get())
    gpi.set(g_out)
    gpot.zero()
    w.propagate_vjp(P, dt, gin, gout, gpi, gpo, gpot)
    lhs = float(np.real(np.vdot(g_out, Sd)))
    rhs = float(np.real(np.vdot(gpo.get(), d)))
    scale = np.abs(g_out).sum() * np.abs(d).max()
    for o in grids + [P, w]:
        o.free()
    gpu.set_precision(0)
    assert abs(lhs - rhs) < (1e-12 if prec == 0 else 1e-6) * scale


@pytest.mark.gpu
def test_cn_trajectory_gradient(gpu):
    """dJ/dVext of 4 real-time steps of the full functional on a CN wave
    function with momentum, against central finite differences of the GPU
    forward map (FP64)."""
    from conftest import coords
    shape, h, nsteps = (24, 24, 24), 0.8, 4
    gpu.set_precision(0)
    rng = np.random.default_rng(21)
    psi = liquid_psi(shape, h, 6)
    w = gpu.Wf(shape, h, propagator=gpu.WF_2ND_ORDER_CN)
    w.set_momentum(*off_grid_momentum(shape, h))
    ot = gpu.OT(9, w)
    mu0 = ot.bulk_chempot(0.0)
    X, Y, Z = coords(shape, h)
    vx = 5.0 / gpu.AUTOK * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 20.0)
    vext, rt, gv = gpu.RGrid(shape, h), gpu.RGrid(shape, h), gpu.RGrid(shape, h)
    rt.set(np.abs(liquid_psi(shape, h, 9)) ** 2)
    dt = 41.3

    def J(v, grad=None):
        vext.set(v)
        w.set(psi)
        return ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, grad, checkpoint_every=2)

    J(vx, gv)
    g = gv.get()
    dv = rng.standard_normal(shape) / gpu.AUTOK
    step = 1e-2
    fd = (J(vx + step * dv) - J(vx - step * dv)) / (2 * step)
    an = float(np.sum(g * dv))
    for o in (gv, rt, vext, ot, w):
        o.free()
    assert abs(fd / an - 1) < 1e-6
