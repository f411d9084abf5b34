"""Generate the golden fixtures in tests/golden/ from the reference-built oracle.

Run in a container that has the reference tree (libdft's src/ is compiled
unmodified against the oracle's libgrid restatement by ``make -C oracle ref``):

    python tests/golden/make_golden.py

Outputs (committed):
  eos.npz          pressure (bar), density (A^-3), chemical potential (K) parsed
                   from libdft examples/bulk/equation_of_state.dat
  plain_16.npz     16^3 plain OT: potential, energy density, 3 imaginary-time
                   predict-correct steps with renormalisation
  full_mixed.npz   16x18x20 (2*3^2, 2^2*5) OT+KC+BF: potential (complex),
                   energy density, kernels, 2 real-time predict-correct steps
  full_lg11.npz    24^3 OT+KC+BF with l_g = 1.1 A: potential, energy density
  terms.npz        16x18x20 OT+KC+BF: libdft's term-level and density-driven
                   entry points (dft_ot_potential2 with its overwritten
                   velocities, dft_ot_add_lennard_jones_potential,
                   dft_ot_add_local_correlation_potential,
                   dft_ot_backflow_potential, dft_ot_energy_density_kc / _bf)
  dispersion.npz   omega(k) tables (k in 1/A, omega in K) parsed from libdft
                   examples/dispersion/{plain,plain-kc,plain-bf,plain-bf-kc,
                   ot_dispersion}.dat
All inputs are seeded numpy draws stored in the fixtures themselves.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import REF_ROOT, Oracle, Grids, build  # noqa: E402

EOS_FILE = os.path.join(REF_ROOT, "examples", "bulk", "equation_of_state.dat")
DISPERSION_DIR = os.path.join(REF_ROOT, "examples", "dispersion")


def coords(shape, step):
    ax = [(np.arange(n) - n // 2) * step for n in shape]
    return np.meshgrid(*ax, indexing="ij")


def droplet_psi(shape, step, rho0, seed):
    """sqrt(rho0) (1 - exp(-r^2 / (2 * 5^2))) (1 + 1e-3 N(0,1))  (64^3 plain-OT case, scaled down)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = coords(shape, step)
    r2 = X ** 2 + Y ** 2 + Z ** 2
    psi = np.sqrt(rho0) * (1.0 - np.exp(-r2 / (2 * 5.0 ** 2)))
    return (psi * (1.0 + 1e-3 * rng.standard_normal(shape))).astype(np.complex128)


def modulated_psi(shape, step, rho0, seed, amp=0.05):
    """Uniform liquid with density modulations and a smooth phase (non-zero velocity)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = coords(shape, step)
    L = [n * step for n in shape]
    ph = rng.uniform(0, 2 * np.pi, 6)
    rho = rho0 * (1 + amp * np.cos(2 * np.pi * X / L[0] + ph[0]) + 0.5 * amp * np.cos(4 * np.pi * Y / L[1] + ph[1])
                  + 0.5 * amp * np.cos(2 * np.pi * Z / L[2] + ph[2]))
    phase = 0.3 * np.sin(2 * np.pi * X / L[0] + ph[3]) + 0.2 * np.cos(2 * np.pi * Y / L[1] + ph[4]) \
        + 0.2 * np.sin(4 * np.pi * Z / L[2] + ph[5])
    psi = np.sqrt(rho) * np.exp(1j * phase) * (1 + 1e-3 * rng.standard_normal(shape))
    return psi.astype(np.complex128)


def main():
    build("ref")
    o = Oracle("ref")
    assert o.lib.orc_kind() == 2
    mass = 4.002602 / o.AUTOAMU
    out = {}

    # ---- EOS table from the reference's own data file
    rows = []
    with open(EOS_FILE) as f:
        for line in f:
            m = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", line)
            if len(m) >= 3:
                rows.append([float(v) for v in m[:3]])
    eos = np.array(rows)
    np.savez_compressed(os.path.join(HERE, "eos.npz"), pressure_bar=eos[:, 0], density_A3=eos[:, 1],
                        chempot_K=eos[:, 2])

    # ---- dispersion tables from the reference's own data files
    tabs = {}
    for name, key in (("plain", "plain"), ("plain-kc", "plain_kc"), ("plain-bf", "plain_bf"),
                      ("plain-bf-kc", "plain_bf_kc"), ("ot_dispersion", "experiment")):
        tabs[key] = np.loadtxt(os.path.join(DISPERSION_DIR, name + ".dat"))
    np.savez(os.path.join(HERE, "dispersion.npz"), **tabs)

    # ---- plain 16^3, imaginary time
    shape, step = (16, 16, 16), 1.0
    with Grids(o, shape, step, mass) as g:
        w0 = g.wf(np.ones(shape))
        otf = g.ot(0, w0)
        prm = g.params(otf)
        rho0 = o.lib.orc_bulk_density(otf, 0.0)
        mu0 = o.lib.orc_bulk_chempot(otf, 0.0)
        psi = droplet_psi(shape, step, rho0, 42)
        X, Y, Z = coords(shape, step)
        vext = 10.0 / o.AUTOK * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 3.0 ** 2))
        w = g.wf(psi)
        P = g.potential(otf, w)
        ed = g.energy_density(otf, w)
        ekin = o.lib.orc_wf_kinetic_energy(w)
        wp, Pc, ve, work = g.wf(), g.cgrid(), g.rgrid(vext), g.rgrid()
        norm0 = o.lib.orc_wf_norm(w)
        o.lib.orc_wf_set_norm(w, norm0)
        dt = -1j * 10.0 / o.AUTOFS
        for _ in range(3):
            o.lib.orc_pc_step(otf, w, wp, Pc, ve, mu0, dt.real, dt.imag)
            o.lib.orc_wf_normalize(w)
        psi3 = g.get_wf(w)
        etot = o.lib.orc_total_energy(otf, w, ve, work)
        np.savez_compressed(os.path.join(HERE, "plain_16.npz"), shape=shape, step=step, model=0, psi=psi, vext=vext,
                            mu0=mu0, rho0=rho0, P=P, ed=ed, ekin=ekin, dt=dt, psi3=psi3, etot3=etot,
                            norm0=norm0, params=np.array([prm[k] for k in sorted(prm)]),
                            param_names=np.array(sorted(prm)))
    # ---- full model, mixed radix, real time
    shape, step, model = (16, 18, 20), 0.8, 1 | 8
    with Grids(o, shape, step, mass) as g:
        w0 = g.wf(np.ones(shape))
        otf = g.ot(model, w0)
        rho0 = o.lib.orc_bulk_density(otf, 0.0)
        mu0 = o.lib.orc_bulk_chempot(otf, 0.0)
        psi = modulated_psi(shape, step, rho0, 7)
        w = g.wf(psi)
        P = g.potential(otf, w)
        ed = g.energy_density(otf, w)
        kers = np.stack([g.kernel(otf, i) for i in range(7)])
        wp, Pc = g.wf(), g.cgrid()
        dt = 1.0 / o.AUTOFS + 0j
        for _ in range(2):
            o.lib.orc_pc_step(otf, w, wp, Pc, None, mu0, dt.real, dt.imag)
        psi2 = g.get_wf(w)
        np.savez_compressed(os.path.join(HERE, "full_mixed.npz"), shape=shape, step=step, model=model, psi=psi,
                            mu0=mu0, P=P, ed=ed, kernels=kers, dt=dt, psi2=psi2)
    # ---- full model with l_g = 1.1 A
    shape, step, model = (24, 24, 24), 0.8, 1 | 8
    with Grids(o, shape, step, mass) as g:
        w0 = g.wf(np.ones(shape))
        lg = 1.1 / o.AUTOANG
        otf = g.ot(model, w0, lg_bohr=lg)
        rho0 = o.lib.orc_bulk_density(otf, 0.0)
        psi = modulated_psi(shape, step, rho0, 11, amp=0.1)
        w = g.wf(psi)
        P = g.potential(otf, w)
        ed = g.energy_density(otf, w)
        np.savez_compressed(os.path.join(HERE, "full_lg11.npz"), shape=shape, step=step, model=model, lg=lg,
                            psi=psi, P=P, ed=ed)
    print("golden fixtures written to", HERE)


def terms():
    """terms.npz (python tests/golden/make_golden.py terms)"""
    build("ref")
    o = Oracle("ref")
    assert o.lib.orc_kind() == 2
    mass = 4.002602 / o.AUTOAMU
    shape, step, model = (16, 18, 20), 0.8, 1 | 8
    L = o.lib
    with Grids(o, shape, step, mass) as g:
        w0 = g.wf(np.ones(shape))
        otf = g.ot(model, w0)
        rho0 = L.orc_bulk_density(otf, 0.0)
        psi = modulated_psi(shape, step, rho0, 5, amp=0.08)
        w = g.wf(psi)
        rho_g, v = g.rgrid(), [g.rgrid() for _ in range(3)]
        L.orc_wf_density(w, rho_g)
        p = g.params(otf)
        L.orc_wf_velocity(w, v[0], v[1], v[2], p["div_epsilon"])
        rho, vel = g.get_r(rho_g), np.stack([g.get_r(x) for x in v])
        out = dict(shape=shape, step=step, model=model, psi=psi, rho=rho, vel=vel)
        P = g.cgrid(0.0)
        L.orc_ref_potential2(otf, P, rho_g, v[0], v[1], v[2])
        out["P2"], out["w2"] = g.get_c(P), np.stack([g.get_r(x) for x in v])
        for x, val in zip(v, vel):
            g.set_r(x, val)
        P = g.cgrid(0.0)
        L.orc_ref_add_lj(otf, P, rho_g)
        out["Plj"] = g.get_c(P)
        P = g.cgrid(0.0)
        L.orc_ref_add_local(otf, P, rho_g)
        out["Ploc"] = g.get_c(P)
        P = g.cgrid(0.0)
        L.orc_ref_backflow(otf, P, rho_g, v[0], v[1], v[2])
        out["Pbf"], out["wbf"] = g.get_c(P), np.stack([g.get_r(x) for x in v])
        ed = g.rgrid(0.0)
        L.orc_ref_energy_density_kc(otf, ed, w, rho_g)
        out["edkc"] = g.get_r(ed)
        ed = g.rgrid(0.0)
        L.orc_ref_energy_density_bf(otf, ed, w, rho_g)
        out["edbf"] = g.get_r(ed)
    np.savez_compressed(os.path.join(HERE, "terms.npz"), **out)
    print("terms.npz written to", HERE)


def compressed_psi(shape, step, rho0, seed):
    """A liquid compressed to ~15 rho0 (0.33 A^-3) at the centre: it crosses the
    backflow cut-off density (0.033 A^-3) and reaches the range of the
    high-density penalty (rho_m = 0.37 A^-3); with a phase (non-zero velocity)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = coords(shape, step)
    bump = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 1.5 ** 2))
    rho = rho0 * (1 + 0.2 * rng.random(shape)) * (1 + 14.0 * bump)
    phase = 0.3 * np.sin(2 * np.pi * X / (shape[0] * step)) + 0.2 * rng.random(shape)
    return (np.sqrt(rho) * np.exp(1j * phase)).astype(np.complex128)


def hd():
    """hd.npz (python tests/golden/make_golden.py hd): the high-density models
    from libdft's own ot.c / ot-energy.c over the shim's grid_func1..5."""
    build("ref")
    o = Oracle("ref")
    assert o.lib.orc_kind() == 2
    mass = 4.002602 / o.AUTOAMU
    L = o.lib
    shape, step = (16, 18, 20), 0.8
    out = dict(shape=shape, step=step)
    rho0 = 0.0218360 * o.AUTOANG ** 3
    psi = compressed_psi(shape, step, rho0, 3)
    out["psi"] = psi
    for model in (2, 11, 13):
        with Grids(o, shape, step, mass) as g:
            w = g.wf(psi)
            otf = g.ot(model, w)
            out["P_%d" % model] = g.potential(otf, w)
            out["ed_%d" % model] = g.energy_density(otf, w)
            if model == 11:
                mu0 = L.orc_bulk_chempot(otf, 0.0)
                wp, Pc = g.wf(), g.cgrid()
                dt = 0.2 / o.AUTOFS + 0j
                for _ in range(2):
                    L.orc_pc_step(otf, w, wp, Pc, None, mu0, dt.real, dt.imag)
                out["psi2_11"], out["mu0"], out["dt"] = g.get_wf(w), mu0, dt
                g.set_wf(w, psi)
                rho_g, v = g.rgrid(), [g.rgrid() for _ in range(3)]
                L.orc_wf_density(w, rho_g)
                p = g.params(otf)
                L.orc_wf_velocity(w, v[0], v[1], v[2], p["div_epsilon"])
                vel = np.stack([g.get_r(x) for x in v])
                out["vel"] = vel
                P = g.cgrid(0.0)
                L.orc_ref_potential2(otf, P, rho_g, v[0], v[1], v[2])
                out["P2_11"], out["w2_11"] = g.get_c(P), np.stack([g.get_r(x) for x in v])
                for x, val in zip(v, vel):
                    g.set_r(x, val)
                P = g.cgrid(0.0)
                L.orc_ref_backflow(otf, P, rho_g, v[0], v[1], v[2])
                out["Pbf_11"], out["wbf_11"] = g.get_c(P), np.stack([g.get_r(x) for x in v])
                ed = g.rgrid(0.0)
                L.orc_ref_energy_density_bf(otf, ed, w, rho_g)
                out["edbf_11"] = g.get_r(ed)
    np.savez_compressed(os.path.join(HERE, "hd.npz"), **out)
    print("hd.npz written to", HERE)


if __name__ == "__main__":
    if sys.argv[1:] == ["terms"]:
        terms()
    elif sys.argv[1:] == ["hd"]:
        hd()
    else:
        main()
