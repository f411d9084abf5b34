"""Moving background: cgrid_set_momentum (called by
examples/gas-bubble/bubble.c:104,173, examples/added_mass/added_mass.c:78,
examples/1d-bubble/bubble-1d.c:136).  A wave function whose grid carries the
momentum k0 is propagated with the kinetic operator hbar^2 |k - k0|^2 / 2m, and
its kinetic energy is <hbar^2 |k - k0|^2 / 2m>.  libgrid, which implements it
for the reference, is absent, so the checks are:

* CPU: the Galilean identity of the oracle restatement -- psi = exp(i k0.r) phi
  propagated without momentum equals exp(i k0.r) times phi propagated with
  momentum -k0 (k0 on the reciprocal grid, phi band-limited, a functional of
  the density only), and the two kinetic energies agree;
* GPU against the oracle with a momentum off the reciprocal grid: predict-
  correct steps of the full functional in FP64 (generic kinetic pass) and FP32
  (register kinetic pass), and the kinetic energy;
* the captured step graph follows a change of momentum between runs;
* the adjoint identity of the propagator and the trajectory gradient with
  momentum set.
"""
import numpy as np
import pytest

from conftest import coords, liquid_psi, relerr
from oracle import Grids

RHO0 = 0.0218360 * 0.529177210903 ** 3


def smooth_phi(shape, step):
    """A band-limited liquid state: its spectrum falls below 1e-13 well inside
    the Nyquist band, so shifting it by a few reciprocal-grid steps wraps
    nothing."""
    X, Y, Z = coords(shape, step)
    L = [n * step for n in shape]
    rho = RHO0 * (1 + 0.05 * np.cos(2 * np.pi * X / L[0]) + 0.03 * np.sin(2 * np.pi * (Y / L[1] + Z / L[2])))
    return np.sqrt(rho) * np.exp(0.2j * np.sin(2 * np.pi * X / L[0]))


def plane_wave(shape, step, k0):
    X, Y, Z = coords(shape, step)
    return np.exp(1j * (k0[0] * X + k0[1] * Y + k0[2] * Z))


def oracle_steps(port, shape, step, model, psi, segments, dt):
    """segments: [(k0, nsteps), ...] predict-correct steps of the oracle, FP64"""
    mass = 4.002602 / port.AUTOAMU
    with Grids(port, shape, step, mass) as g:
        w, wp, P = g.wf(psi), g.wf(), g.cgrid()
        o = g.ot(model, w)
        mu0 = port.lib.orc_bulk_chempot(o, 0.0)
        for k0, n in segments:
            port.lib.orc_wf_set_momentum(w, *k0)
            port.lib.orc_wf_set_momentum(wp, *k0)
            for _ in range(n):
                port.lib.orc_pc_step(o, w, wp, P, None, mu0, dt.real, dt.imag)
        return g.get_wf(w), port.lib.orc_wf_kinetic_energy(w), mu0


@pytest.mark.parametrize("dt", [41.3 + 0j, 30 - 5j])
def test_oracle_galilean_identity(port, dt):
    shape, step = (24, 20, 16), 1.0
    dk = [2 * np.pi / (n * step) for n in shape]
    k0 = (2 * dk[0], -dk[1], 3 * dk[2])
    phi = smooth_phi(shape, step)
    e = plane_wave(shape, step, k0)
    psi_n, t_psi, _ = oracle_steps(port, shape, step, 1, e * phi, [((0.0, 0.0, 0.0), 3)], dt)
    phi_n, t_phi, _ = oracle_steps(port, shape, step, 1, phi, [(tuple(-k for k in k0), 3)], dt)
    assert relerr(e * phi_n, psi_n) < 1e-11
    assert abs(t_phi / t_psi - 1) < 1e-11
    # and the momentum matters: the same state without it differs at first order
    phi_0, t_0, _ = oracle_steps(port, shape, step, 1, phi, [((0.0, 0.0, 0.0), 3)], dt)
    assert relerr(e * phi_0, psi_n) > 1e-3
    assert abs(t_0 / t_psi - 1) > 1e-2


def gpu_steps(gpu, prec, shape, step, model, psi, segments, dt):
    gpu.set_precision(prec)
    w, wp, P = gpu.Wf(shape, step), gpu.Wf(shape, step), gpu.CGrid(shape, step)
    ot = gpu.OT(model, w)
    w.set(psi)
    mu0 = ot.bulk_chempot(0.0)
    for k0, n in segments:
        w.set_momentum(*k0)
        wp.set_momentum(*k0)
        ot.run(w, wp, P, None, mu0, dt, n, False)
    out, t = w.get(), w.kinetic_energy()
    for o in (P, ot, wp, w):
        o.free()
    gpu.set_precision(0)
    return out, t


def off_grid_momentum(shape, step):
    dk = [2 * np.pi / (n * step) for n in shape]
    return (0.37 * dk[0], -1.3 * dk[1], 2.2 * dk[2])


@pytest.mark.gpu
@pytest.mark.parametrize("prec,shape,tol", [(0, (32, 24, 20), 1e-10), (1, (64, 64, 64), 2e-5)])
def test_full_functional_with_momentum_matches_oracle(gpu, port, prec, shape, tol):
    step, dt = 0.9, 41.3 + 0j
    psi = liquid_psi(shape, step, 3)
    k0 = off_grid_momentum(shape, step)
    ref, t_ref, _ = oracle_steps(port, shape, step, 9, psi, [(k0, 3)], dt)
    out, t = gpu_steps(gpu, prec, shape, step, 9, psi, [(k0, 3)], dt)
    assert relerr(out, ref) < tol
    assert abs(t / t_ref - 1) < (1e-11 if prec == 0 else 1e-5)


@pytest.mark.gpu
def test_step_graph_follows_momentum_change(gpu, port):
    """dftgpu_run replays a captured graph while its arguments repeat; a new
    momentum must be captured anew."""
    shape, step, dt = (32, 24, 20), 0.9, 41.3 + 0j
    psi = liquid_psi(shape, step, 4)
    k0 = off_grid_momentum(shape, step)
    k1 = tuple(-0.5 * k for k in k0)
    segments = [(k0, 3), (k1, 3), ((0.0, 0.0, 0.0), 2)]
    ref, _, _ = oracle_steps(port, shape, step, 9, psi, segments, dt)
    out, _ = gpu_steps(gpu, 0, shape, step, 9, psi, segments, dt)
    assert relerr(out, ref) < 1e-10


def rdot(a, b):
    return float(np.real(np.vdot(a, b)))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_propagator_adjoint_identity_with_momentum(gpu, prec):
    shape, step, dt = (64, 32, 32), 0.9, 30 - 5j
    rng = np.random.default_rng(8)
    gpu.set_precision(prec)
    psi = liquid_psi(shape, step, 5)
    V = (rng.standard_normal(shape) + 0.3j * rng.standard_normal(shape)) * 1e-3
    g_out = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    d = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    w, P = gpu.Wf(shape, step), gpu.CGrid(shape, step)
    w.set_momentum(*off_grid_momentum(shape, step))
    P.set(V)
    w.set(d)
    w.propagate(P, dt)
    Sd = w.get()
    w.set(psi)
    w.propagate(P, dt)
    grids = [gpu.CGrid(shape, step) for _ in range(5)]
    gin, gout, gpi, gpo, gpot = grids
    gin.set(psi)
    gout.set(w.get())
    gpi.set(g_out)
    gpot.zero()
    w.propagate_vjp(P, dt, gin, gout, gpi, gpo, gpot)
    lhs, rhs = rdot(g_out, Sd), rdot(gpo.get(), d)
    scale = np.abs(g_out).sum() * np.abs(d).max()
    assert abs(lhs - rhs) < (1e-12 if prec == 0 else 1e-6) * scale
    for o in grids + [P, w]:
        o.free()
    gpu.set_precision(0)


@pytest.mark.gpu
def test_trajectory_gradient_with_momentum(gpu):
    """dJ/dVext of 4 real-time steps of the full functional with momentum set,
    against central finite differences of the GPU forward map (FP64)."""
    shape, step, nsteps = (24, 24, 24), 0.8, 4
    gpu.set_precision(0)
    rng = np.random.default_rng(21)
    psi = liquid_psi(shape, step, 6)
    w = gpu.Wf(shape, step)
    w.set_momentum(*off_grid_momentum(shape, step))
    ot = gpu.OT(9, w)
    mu0 = ot.bulk_chempot(0.0)
    X, Y, Z = coords(shape, step)
    vx = 5.0 / gpu.AUTOK * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 20.0)
    vext, rt, gv = gpu.RGrid(shape, step), gpu.RGrid(shape, step), gpu.RGrid(shape, step)
    rt.set(np.abs(liquid_psi(shape, step, 9)) ** 2)
    dt = 41.3

    def J(v, grad=None):
        vext.set(v)
        w.set(psi)
        return ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, grad, checkpoint_every=2)

    J(vx, gv)
    g = gv.get()
    dv = rng.standard_normal(shape) / gpu.AUTOK
    h = 1e-2
    fd = (J(vx + h * dv) - J(vx - h * dv)) / (2 * h)
    an = float(np.sum(g * dv))
    assert abs(fd / an - 1) < 1e-6
    for o in (gv, rt, vext, ot, w):
        o.free()
