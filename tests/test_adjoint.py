"""Reverse mode: the hand-written adjoint of the split-operator step, the OT
potential and the predict-correct step (libdft has no reverse mode, so the
checks are mathematical):

* adjoint identity Re<g, S d> = Re<S^H g, d> for the propagator (linear in psi);
* central finite differences of the GPU forward map (FP64) against every
  vector-Jacobian product, for each OT model (plain, KC, backflow, KC+BF);
* central finite differences of the FP64 CPU oracle's trajectory objective
  against the GPU gradient with respect to the external potential;
* checkpoint interval independence; FP32 against FP64 gradients;
* a torch.autograd.Function over the C ABI: gradient of the objective with
  respect to the parameters of a Gaussian external potential.

Tolerances: finite differences with step h have truncation O(h^2) and
rounding O(eps_64 / h); the steps below keep both under 1e-7 of the
derivative, and the tests allow 1e-6 (2e-6 through a multi-step trajectory).
"""
import numpy as np
import pytest

from conftest import coords, liquid_psi, relerr
from oracle import Grids

pytestmark = pytest.mark.gpu

MODELS = [0, 1, 8, 9]          # plain, KC, backflow, KC + backflow


def rdot(a, b):
    """Re sum conj(a) b"""
    return float(np.real(np.vdot(a, b)))


def smooth_bump(shape, step, c, w):
    X, Y, Z = coords(shape, step)
    return np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / w ** 2)


@pytest.fixture
def fp64(gpu):
    gpu.set_precision(0)
    yield
    gpu.set_precision(0)


@pytest.mark.parametrize("dt", [41.3 + 0j, -20j, 30 - 5j])
def test_propagate_vjp_adjoint_identity_and_potential_gradient(gpu, fp64, dt):
    shape, step = (16, 20, 24), 0.9
    rng = np.random.default_rng(5)
    psi = liquid_psi(shape, step, 5)
    V = (rng.standard_normal(shape) + 0.3j * rng.standard_normal(shape)) * 1e-3
    g_out = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    d = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    w = gpu.Wf(shape, step)
    P = gpu.CGrid(shape, step)

    def S(v, x):
        P.set(v)
        w.set(x)
        w.propagate(P, dt)
        return w.get()

    psio = S(V, psi)
    grids = [gpu.CGrid(shape, step) for _ in range(5)]
    gin, gout, gpi, gpo, gpot = grids
    gin.set(psi)
    gout.set(psio)
    gpi.set(g_out)
    gpot.zero()
    P.set(V)
    w.propagate_vjp(P, dt, gin, gout, gpi, gpo, gpot)
    gpsi, gV = gpo.get(), gpot.get()
    # adjoint identity (S is linear in psi)
    lhs, rhs = rdot(g_out, S(V, d)), rdot(gpsi, d)
    assert abs(lhs - rhs) < 1e-12 * np.abs(g_out).sum() * np.abs(d).max()
    # potential gradient: f(V) = Re<g', S(V) psi>
    dV = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * 1e-3
    h = 1e-3
    fd = (rdot(g_out, S(V + h * dV, psi)) - rdot(g_out, S(V - h * dV, psi))) / (2 * h)
    an = float(np.sum(gV.real * dV.real + gV.imag * dV.imag))
    assert abs(fd - an) < 1e-6 * abs(an)
    # cot_in may alias cot_out
    P.set(V)
    gpi.set(g_out)
    gpot.zero()
    w.propagate_vjp(P, dt, gin, gout, gpi, gpi, gpot)
    assert np.array_equal(gpi.get(), gpsi)
    assert np.array_equal(gpot.get(), gV)
    for o in grids + [P, w]:
        o.free()


@pytest.mark.parametrize("model", MODELS)
def test_ot_potential_vjp_matches_finite_differences(gpu, fp64, model):
    shape, step = (24, 24, 24), 0.8
    rng = np.random.default_rng(11 + model)
    psi = liquid_psi(shape, step, 7)
    gam = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    d = 0.1 * np.abs(psi) * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    P, cot, g = gpu.CGrid(shape, step), gpu.CGrid(shape, step), gpu.CGrid(shape, step)

    def J(x):
        w.set(x)
        P.zero()
        ot.potential(P, w)
        V = P.get()
        return float(np.sum(gam.real * V.real + gam.imag * V.imag))

    w.set(psi)
    cot.set(gam)
    g.zero()
    ot.potential_vjp(w, cot, g)
    an = rdot(g.get(), d)
    errs = []
    for h in (1e-3, 3e-4):
        fd = (J(psi + h * d) - J(psi - h * d)) / (2 * h)
        errs.append(abs(fd - an) / abs(an))
    assert min(errs) < 1e-6, errs
    # accumulation: a second call adds the same product
    w.set(psi)
    ot.potential_vjp(w, cot, g)
    assert abs(rdot(g.get(), d) / an - 2) < 1e-12
    for o in (g, cot, P, ot, w):
        o.free()


def _setup_traj(gpu, shape, step, model):
    w = gpu.Wf(shape, step)
    ot = gpu.OT(model, w)
    vext = gpu.RGrid(shape, step)
    rt = gpu.RGrid(shape, step)
    return w, ot, vext, rt


def _traj_inputs(gpu, shape, step):
    psi = liquid_psi(shape, step, 21)
    V0 = 3.0 / gpu.AUTOK * smooth_bump(shape, step, (1.0, -0.5, 0.5), 4.0)
    rho_t = 0.0218360 * 0.529177210903 ** 3 * (1 + 0.05 * smooth_bump(shape, step, (-2.0, 1.0, 0.0), 5.0))
    dV = 1.0 / gpu.AUTOK * smooth_bump(shape, step, (0.5, 1.5, -1.0), 3.0)
    return psi, V0, rho_t, dV


@pytest.mark.parametrize("model,dt,renorm", [(9, 20.0, False), (0, 20.0, False), (9, -10j, True), (1, 15 - 2j, False)])
def test_adjoint_run_gradients_match_gpu_finite_differences(gpu, fp64, model, dt, renorm):
    shape, step, nsteps = (24, 24, 24), 0.8, 5
    dt = dt / gpu.AUTOFS
    psi, V0, rho_t, dV = _traj_inputs(gpu, shape, step)
    w, ot, vext, rt = _setup_traj(gpu, shape, step, model)
    mu0 = ot.bulk_chempot(0.0)
    rt.set(rho_t)
    w.norm_target = float(np.sum(np.abs(psi) ** 2) * step ** 3)
    gv, gp = gpu.RGrid(shape, step), gpu.CGrid(shape, step)

    def J(V, x):
        vext.set(V)
        w.set(x)
        return ot.adjoint_run(w, vext, mu0, dt, nsteps, renorm, rt)

    vext.set(V0)
    w.set(psi)
    J0 = ot.adjoint_run(w, vext, mu0, dt, nsteps, renorm, rt, gv, gp, checkpoint_every=2)
    assert J0 == J(V0, psi)
    G, Gp = gv.get(), gp.get()
    an = float(np.sum(G * dV))
    errs = [abs((J(V0 + h * dV, psi) - J(V0 - h * dV, psi)) / (2 * h) / an - 1) for h in (1e-1, 1e-2)]
    assert min(errs) < 2e-6, errs
    rng = np.random.default_rng(3)
    d = 0.05 * np.abs(psi) * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    an = rdot(Gp, d)
    errs = [abs((J(V0, psi + h * d) - J(V0, psi - h * d)) / (2 * h) / an - 1) for h in (1e-2, 1e-3)]
    assert min(errs) < 2e-6, errs
    for o in (gp, gv, rt, vext, ot, w):
        o.free()


def test_checkpoint_interval_does_not_change_the_gradient(gpu, fp64):
    shape, step, nsteps = (24, 24, 24), 0.8, 7
    psi, V0, rho_t, _ = _traj_inputs(gpu, shape, step)
    w, ot, vext, rt = _setup_traj(gpu, shape, step, 9)
    mu0 = ot.bulk_chempot(0.0)
    rt.set(rho_t)
    vext.set(V0)
    gv, gp = gpu.RGrid(shape, step), gpu.CGrid(shape, step)
    out = []
    for k in (1, 3, 0, 7, 100):
        w.set(psi)
        J = ot.adjoint_run(w, vext, mu0, 20.0 / gpu.AUTOFS, nsteps, False, rt, gv, gp, checkpoint_every=k)
        out.append((J, gv.get(), gp.get(), w.get()))
    for J, G, Gp, psiT in out[1:]:
        assert J == out[0][0]
        assert np.array_equal(G, out[0][1])
        assert np.array_equal(Gp, out[0][2])
        assert np.array_equal(psiT, out[0][3])
    # nsteps = 0: J of psi_0 itself, gradient w.r.t. Vext is zero
    w.set(psi)
    J = ot.adjoint_run(w, vext, mu0, 20.0 / gpu.AUTOFS, 0, False, rt, gv, gp)
    dv = step ** 3
    assert abs(J / (np.sum((np.abs(psi) ** 2 - rho_t) ** 2) * dv) - 1) < 1e-12
    assert not gv.get().any()
    assert relerr(gp.get(), 4 * (np.abs(psi) ** 2 - rho_t) * dv * psi) < 1e-13
    for o in (gp, gv, rt, vext, ot, w):
        o.free()


def test_pc_step_vjp_composes_to_adjoint_run(gpu, fp64):
    """One dftgpu_pc_step_vjp per step, driven from Python, equals dftgpu_adjoint_run."""
    shape, step, nsteps = (16, 16, 16), 0.9, 3
    dt = 20.0 / gpu.AUTOFS
    psi, V0, rho_t, _ = _traj_inputs(gpu, shape, step)
    w, ot, vext, rt = _setup_traj(gpu, shape, step, 9)
    wp, P = gpu.Wf(shape, step), gpu.CGrid(shape, step)
    mu0 = ot.bulk_chempot(0.0)
    rt.set(rho_t)
    vext.set(V0)
    gv, gp = gpu.RGrid(shape, step), gpu.CGrid(shape, step)
    w.set(psi)
    ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, gv, gp)
    states = [psi]
    w.set(psi)
    for _ in range(nsteps):
        ot.pc_step(w, wp, P, vext, mu0, dt)
        states.append(w.get())
    dv = step ** 3
    cot = gpu.CGrid(shape, step)
    cot.set(4 * (np.abs(states[-1]) ** 2 - rho_t) * dv * states[-1])
    acc = gpu.RGrid(shape, step)
    acc.set(np.zeros(shape))
    for k in range(nsteps - 1, -1, -1):
        w.set(states[k])
        ot.pc_step_vjp(w, vext, mu0, dt, False, cot, acc)
    assert relerr(acc.get(), gv.get()) < 1e-13
    assert relerr(cot.get(), gp.get()) < 1e-13
    for o in (acc, cot, gp, gv, P, wp, rt, vext, ot, w):
        o.free()


def test_gradient_matches_oracle_finite_differences(gpu, port, fp64):
    """GPU adjoint gradient against central differences of the FP64 CPU oracle's trajectory."""
    shape, step, nsteps, model = (20, 20, 20), 0.9, 4, 9
    dt = 20.0 / gpu.AUTOFS
    psi, V0, rho_t, dV = _traj_inputs(gpu, shape, step)
    dv = step ** 3
    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo, wpo, Po, vo = g.wf(psi), g.wf(), g.cgrid(), g.rgrid()
        oo = g.ot(model, wo)
        mu0 = port.lib.orc_bulk_chempot(oo, 0.0)

        def J_oracle(V):
            g.set_r(vo, V)
            g.set_wf(wo, psi)
            for _ in range(nsteps):
                port.lib.orc_pc_step(oo, wo, wpo, Po, vo, mu0, dt, 0.0)
            return float(np.sum((np.abs(g.get_wf(wo)) ** 2 - rho_t) ** 2) * dv)

        h = 1e-2
        J_ref = J_oracle(V0)
        fd = (J_oracle(V0 + h * dV) - J_oracle(V0 - h * dV)) / (2 * h)
    w, ot, vext, rt = _setup_traj(gpu, shape, step, model)
    rt.set(rho_t)
    vext.set(V0)
    w.set(psi)
    gv = gpu.RGrid(shape, step)
    J = ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, gv)
    assert abs(J / J_ref - 1) < 1e-9
    an = float(np.sum(gv.get() * dV))
    assert abs(fd - an) < 2e-6 * abs(an), (fd, an)
    for o in (gv, rt, vext, ot, w):
        o.free()


def test_fp32_gradient_tracks_fp64(gpu):
    shape, step, nsteps = (32, 32, 32), 0.8, 4
    dt = 20.0 / gpu.AUTOFS
    out = []
    for prec in (0, 1):
        gpu.set_precision(prec)
        psi, V0, rho_t, _ = _traj_inputs(gpu, shape, step)
        w, ot, vext, rt = _setup_traj(gpu, shape, step, 9)
        mu0 = ot.bulk_chempot(0.0)
        rt.set(rho_t)
        vext.set(V0)
        w.set(psi)
        gv = gpu.RGrid(shape, step)
        J = ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, gv)
        out.append((J, gv.get()))
        for o in (gv, rt, vext, ot, w):
            o.free()
    gpu.set_precision(0)
    assert abs(out[1][0] / out[0][0] - 1) < 1e-4
    assert relerr(out[1][1], out[0][1]) < 2e-3


def test_torch_autograd_gaussian_external_potential(gpu, fp64):
    """Gradient of the objective with respect to (amplitude, centre, width) of a
    Gaussian external potential, through a torch.autograd.Function whose
    forward and backward call the C ABI."""
    torch = pytest.importorskip("torch")
    shape, step, nsteps = (24, 24, 24), 0.8, 4
    dt = 20.0 / gpu.AUTOFS
    psi, _, rho_t, _ = _traj_inputs(gpu, shape, step)
    w, ot, vext, rt = _setup_traj(gpu, shape, step, 9)
    mu0 = ot.bulk_chempot(0.0)
    rt.set(rho_t)
    gv = gpu.RGrid(shape, step)
    X, Y, Z = (torch.from_numpy(a) for a in coords(shape, step))

    class Objective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, V):
            vext.set(V.detach().numpy())
            w.set(psi)
            J = ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, gv if ctx.needs_input_grad[0] else None)
            if ctx.needs_input_grad[0]:
                ctx.save_for_backward(torch.from_numpy(gv.get()))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            (G,) = ctx.saved_tensors
            return gJ * G

    def vext_of(theta):
        a, cx, width = theta[0], theta[1], theta[2]
        return a / gpu.AUTOK * torch.exp(-((X - cx) ** 2 + Y ** 2 + Z ** 2) / width ** 2)

    theta = torch.tensor([3.0, 0.7, 4.0], dtype=torch.float64, requires_grad=True)
    J = Objective.apply(vext_of(theta))
    J.backward()
    grad = theta.grad.numpy().copy()
    with torch.no_grad():
        for i, h in enumerate((1e-2, 1e-2, 1e-2)):
            e = torch.zeros(3, dtype=torch.float64)
            e[i] = h
            fd = (Objective.apply(vext_of(theta + e)) - Objective.apply(vext_of(theta - e))).item() / (2 * h)
            assert abs(fd - grad[i]) < 1e-5 * np.abs(grad).max(), (i, fd, grad[i])
        # a small step against the gradient lowers the objective
        J1 = Objective.apply(vext_of(theta - 0.1 * theta.grad / np.abs(grad).max())).item()
    assert J1 < J.item()
    for o in (gv, rt, vext, ot, w):
        o.free()


def test_adjoint_rejects_clamped_backflow_and_bad_args(gpu, fp64):
    shape, step = (16, 16, 16), 0.9
    w = gpu.Wf(shape, step)
    ot = gpu.OT(9, w)
    w.set(liquid_psi(shape, step, 1))
    cot, g = gpu.CGrid(shape, step), gpu.CGrid(shape, step)
    ot.params.max_veloc = 100.0 / gpu.AUTOMPS
    with pytest.raises(gpu.DftGpuError):
        ot.potential_vjp(w, cot, g)
    other = gpu.CGrid((16, 16, 8), step)
    with pytest.raises(gpu.DftGpuError):
        ot.potential_vjp(w, cot, other)
    for o in (other, g, cot, ot, w):
        o.free()


def _gaussians(theta, X, Y, Z, autok):
    """V = sum_g a_g exp(-((x - cx_g)^2 + y^2 + (z - cz_g)^2) / (2 w_g^2)), theta = (a [K], w, cx, cz) x 4,
    and dV/dtheta for every parameter."""
    V = np.zeros(X.shape)
    dV = []
    for a, wd, cx, cz in np.asarray(theta).reshape(4, 4):
        r2 = (X - cx) ** 2 + Y ** 2 + (Z - cz) ** 2
        e = np.exp(-r2 / (2 * wd ** 2)) / autok
        V += a * e
        dV += [e, a * e * r2 / wd ** 3, a * e * (X - cx) / wd ** 2, a * e * (Z - cz) / wd ** 2]
    return V, dV


def test_gaussian_parameter_gradient_matches_oracle_finite_differences(gpu, port):
    """The 16-parameter external potential of the adjoint workload (4 Gaussians,
    amplitude ~U(5, 50) K, width ~U(2, 6) bohr, centre ~U(-10, 10) bohr in x and
    z, seed 11) on the full-OT liquid with a 1 % density wave (l_g = 1.1 A),
    64^3, step 0.8 bohr, 40 real-time steps of 1 fs; J = int (rho_T -
    rho_target)^2 dV with rho_target the initial density shifted 2 bohr along z.
    Every parameter's derivative by central differences (h = 1e-4 relative) of
    the FP64 CPU oracle's trajectory, against the GPU adjoint in FP64 and FP32."""
    shape, step, nsteps = (64, 64, 64), 0.8, 40
    dt = 1.0 / gpu.AUTOFS
    lg = 1.1 / gpu.AUTOANG
    X, Y, Z = coords(shape, step)
    rho0 = 0.0218360 * gpu.AUTOANG ** 3
    phase = np.random.default_rng(7).uniform(0, 2 * np.pi)
    psi = np.sqrt(rho0 * (1 + 0.01 * np.cos(2 * np.pi * X / (32 * step) + phase))).astype(complex)
    rho = np.abs(psi) ** 2
    kz = 2 * np.pi * np.fft.fftfreq(shape[2], d=step)
    rho_t = np.real(np.fft.ifft(np.fft.fft(rho, axis=2) * np.exp(-1j * kz * 2.0), axis=2))
    rng = np.random.default_rng(11)
    theta0 = np.stack([rng.uniform(5, 50, 4), rng.uniform(2, 6, 4), rng.uniform(-10, 10, 4),
                       rng.uniform(-10, 10, 4)], 1).ravel()
    V0, dVs = _gaussians(theta0, X, Y, Z, gpu.AUTOK)
    dv = step ** 3

    with Grids(port, shape, step, gpu.HELIUM_MASS) as g:
        wo, wpo, Po, vo = g.wf(psi), g.wf(), g.cgrid(), g.rgrid()
        oo = g.ot(9, wo, lg_bohr=lg)
        mu0 = port.lib.orc_bulk_chempot(oo, 0.0)

        def J_oracle(th):
            g.set_r(vo, _gaussians(th, X, Y, Z, gpu.AUTOK)[0])
            g.set_wf(wo, psi)
            for _ in range(nsteps):
                port.lib.orc_pc_step(oo, wo, wpo, Po, vo, mu0, dt, 0.0)
            return float(np.sum((np.abs(g.get_wf(wo)) ** 2 - rho_t) ** 2) * dv)

        J_ref = J_oracle(theta0)
        fd = np.zeros(16)
        for k in range(16):
            e = np.zeros(16)
            e[k] = 1e-4 * abs(theta0[k])
            fd[k] = (J_oracle(theta0 + e) - J_oracle(theta0 - e)) / (2 * e[k])

    grads = {}
    for prec in (0, 1):
        gpu.set_precision(prec)
        w = gpu.Wf(shape, step)
        ot = gpu.OT(9, w, lg_bohr=lg)
        vext, rt, gv = gpu.RGrid(shape, step), gpu.RGrid(shape, step), gpu.RGrid(shape, step)
        vext.set(V0)
        rt.set(rho_t)
        w.set(psi)
        J = ot.adjoint_run(w, vext, mu0, dt, nsteps, False, rt, gv, checkpoint_every=7)
        G = gv.get()
        grads[prec] = (J, np.array([np.sum(G * d) for d in dVs]))
        for o in (gv, rt, vext, ot, w):
            o.free()
    gpu.set_precision(0)
    # FP64: every component within 1e-4 of its finite difference (components
    # below 1e-3 of the gradient's norm relative to that), the vector within
    # 1e-6.  FP32 bulk is outside the 1e-4 gradient target: its forward
    # trajectory alone moves J by ~2e-4 over these 40 real-time steps, and
    # the gradient is held to 5e-3 of its norm.
    scale = np.linalg.norm(fd)
    for prec, tol_J, tol_norm, tol_comp in ((0, 1e-9, 1e-6, 1e-4), (1, 1e-3, 5e-3, None)):
        J, an = grads[prec]
        err_norm = np.linalg.norm(an - fd) / scale
        err_comp = np.max(np.abs(an - fd) / np.maximum(np.abs(fd), 1e-3 * scale))
        print("16-parameter gradient prec=%d: J rel %.2e, |g - fd| / |fd| = %.2e, max component rel %.2e"
              % (prec, abs(J / J_ref - 1), err_norm, err_comp))
        assert abs(J / J_ref - 1) < tol_J
        assert err_norm < tol_norm, (prec, err_norm)
        if tol_comp is not None:
            assert err_comp < tol_comp, (prec, err_comp)
