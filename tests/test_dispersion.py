"""Physics pins of the time step (no bit-level reference output exists):
a small-amplitude density wave in bulk liquid helium, propagated in real
time with the predict-correct step, must oscillate at the frequency libdft's
own runs give (examples/dispersion/plain.dat, plain-bf-kc.dat: omega(k) in
K at k in 1/Angstrom), and the real-time step must conserve the norm
(plain model: unitary) and the energy.

The set-up follows the reference's examples/dispersion/dispersion.c: 512
points of step 1 bohr along z, psi = sqrt(rho0) (1 + a cos(k z)), a = 1e-3,
dt = 15 fs, mu0 subtracted.  The reference runs a 1 x 1 x 512 grid with the
kernels integrated over the transverse plane (its 1-D mode, src/ot.c:186-190,
not provided here); this test uses a 128 x 128 bohr transverse box instead:
the 3-D kernels sampled on it miss only the Lennard-Jones tail beyond 64 bohr
(0.2 % of its integral, which the normalisation to b puts back into the
sampled part).  The frequency is fitted to the k-mode of the density,
int rho cos(kz) dV, sampled every step over 1.2 periods in FP32 (the
amplitude is far above FP32 rounding); the time-step, grid and box errors
are about 1 %.  The tables were read by hand from the period of a 15 ps run
(the comment at the top of dispersion.c): at k = 0.186 1/A that run spans
1.15 periods, at 0.742 1/A 4.6, so the tolerance is 4 % at the first and
2 % at the second.  (libdft's semi-analytic dft_ot_bulk_dispersion gives
3.71 K at 0.186 1/A against the table's 3.661 K.)  Norm and energy conservation are
checked in FP64 on a 32 x 32 x 512 box."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NZ, STEP, DT_FS, AMP = 512, 1.0, 15.0, 1e-3


def table(name):
    import os
    from conftest import GOLDEN
    return np.load(os.path.join(GOLDEN, "dispersion.npz"))[name]


def run_wave(gpu, model, kidx, nsteps, prec, ntr, every_cons=0):
    """k-mode of the density after every step; norm and energy every
    every_cons steps (0: not recorded)"""
    gpu.set_precision(prec)
    shape = (ntr, ntr, NZ)
    L = gpu.lib()
    w, wp = gpu.Wf(shape, STEP), gpu.Wf(shape, STEP)
    ot = gpu.OT(model, w)
    rho0, mu0 = ot.bulk_density(0.0), ot.bulk_chempot(0.0)
    kz = kidx * 2 * np.pi / (NZ * STEP)
    z = (np.arange(NZ) - NZ // 2) * STEP
    psi = np.sqrt(rho0) * (1 + AMP * np.cos(kz * z))
    w.set(np.broadcast_to(psi, shape).astype(complex))
    cosg, rho, tmp = gpu.RGrid(shape, STEP), gpu.RGrid(shape, STEP), gpu.RGrid(shape, STEP)
    cosg.set(np.broadcast_to(np.cos(kz * z), shape))
    P = gpu.CGrid(shape, STEP)
    dt = DT_FS / gpu.AUTOFS
    modes, norms, energies = [], [], []
    for s in range(nsteps + 1):
        if s:
            ot.run(w, wp, P, None, mu0, complex(dt), 1, False)
        L.grid_wf_density(w.ptr, rho.ptr)
        L.rgrid_product(tmp.ptr, rho.ptr, cosg.ptr)
        modes.append(tmp.integral())
        if every_cons and s % every_cons == 0:
            norms.append(w.norm())
            energies.append(ot.energy_report(w)[0])
    for o in (P, tmp, rho, cosg, ot, wp, w):
        o.free()
    gpu.set_precision(0)
    return np.array(modes), dt, np.array(norms), np.array(energies)


def fit_omega(m, dt, om_guess):
    """omega of m(t) = c0 + c1 cos(omega t) + c2 sin(omega t), least squares:
    a scan over [0.5, 2] x om_guess, then golden-section refinement"""
    t = np.arange(len(m)) * dt

    def resid(om):
        A = np.stack([np.ones_like(t), np.cos(om * t), np.sin(om * t)], 1)
        c, *_ = np.linalg.lstsq(A, m, rcond=None)
        return np.sum((A @ c - m) ** 2)

    grid = np.linspace(0.5, 2.0, 301) * om_guess
    r = [resid(om) for om in grid]
    j = int(np.argmin(r))
    lo, hi = grid[max(j - 1, 0)], grid[min(j + 1, len(grid) - 1)]
    g = (np.sqrt(5) - 1) / 2
    for _ in range(60):
        a, b = hi - g * (hi - lo), lo + g * (hi - lo)
        if resid(a) < resid(b):
            hi = b
        else:
            lo = a
    return 0.5 * (lo + hi)


@pytest.mark.parametrize("model,name", [(0, "plain"), (9, "plain_bf_kc")])
@pytest.mark.parametrize("kidx", [8, 32])
def test_density_wave_frequency_matches_reference_runs(gpu, model, name, kidx):
    k_ang = kidx * 2 * np.pi / (NZ * STEP) / gpu.AUTOANG
    tab = table(name)
    row = np.argmin(np.abs(tab[:, 0] - k_ang))
    assert abs(tab[row, 0] - k_ang) < 2e-3
    period_steps = 2 * np.pi / (tab[row, 1] / gpu.AUTOK) / (DT_FS / gpu.AUTOFS)
    m, dt, _, _ = run_wave(gpu, model, kidx, int(1.2 * period_steps) + 2, 1, 128)
    om_K = fit_omega(m, dt, tab[row, 1] / gpu.AUTOK) * gpu.AUTOK
    tol = 0.04 if kidx == 8 else 0.02
    assert abs(om_K / tab[row, 1] - 1) < tol, (om_K, tab[row, 1])


@pytest.mark.parametrize("model", [0, 9])
def test_real_time_step_conserves_norm_and_energy(gpu, model):
    m, dt, norms, energies = run_wave(gpu, model, 32, 300, 0, 32, every_cons=50)
    dn, de = np.abs(norms / norms[0] - 1).max(), np.abs(energies / energies[0] - 1).max()
    if model == 0:   # unitary step: norm conserved
        assert dn < 1e-11, dn
    assert de < 1e-6, de
