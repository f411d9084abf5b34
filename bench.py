#!/usr/bin/env python
"""OT-DFT time-step throughput on GB300 (steps/s, full OT).

Default workload (the helium-nanodroplet relaxation the headline metric is
quoted on, "cfg2"): 256^3 grid, step 0.8 bohr, full Orsay-Trento functional
(kinetic correlation + backflow), a droplet of N = 2000 atoms (radius
(3N / 4 pi rho0)^(1/3), 1.5 bohr tanh surface, 1e-3 multiplicative noise,
seed 3), imaginary-time predict-correct steps of 20 fs with the particle
number renormalised to N after every step.  One "step" is one
predict-correct step: two OT potential evaluations and two split-operator
propagations.  --workload selects the specification's other cases (cfg0:
64^3 plain OT with an external potential; cfg1: 128^3 real time; cfg4: the
512^3 vortex ring); --grid overrides the grid size, N or NXxNYxNZ (profiling of smaller
cases).  Data are synthetic; at 256^3 and above every input (psi: 134 MB in
FP32 at 256^3) is larger than L2, so no L2 flush is needed between steps.

The JSON line reports the FP32-bulk path (value, e2e, roofline) and, in the
same run, the FP64 path's steps/s and the FP32-vs-FP64 energy-per-atom error
after the same steps.  --impl reference times the FP64 CPU oracle (the
restatement of the reference's CPU path) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

AUTOFS = 0.024188843265857
AUTOANG = 0.529177210903
AUTOK = 3.1577502480407e5
RHO0 = 0.0218360 * AUTOANG ** 3       # bulk liquid density at P = 0 (bohr^-3)
NATOMS = 2000.0


def _shape(n):
    """a grid size: N (cubic) or (nx, ny, nz)"""
    return tuple(n) if isinstance(n, (tuple, list)) else (n, n, n)


def _centred(n, step):
    nx, ny, nz = _shape(n)
    return ((np.arange(nx) - nx // 2) * step)[:, None, None], ((np.arange(ny) - ny // 2) * step)[None, :, None], \
        ((np.arange(nz) - nz // 2) * step)[None, None, :]


def droplet_psi(n=256, step=0.8, seed=3):
    rho0 = RHO0
    R = (3.0 * NATOMS / (4.0 * np.pi * rho0)) ** (1.0 / 3.0)
    X, Y, Z = _centred(n, step)
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    rho = 0.5 * rho0 * (1.0 - np.tanh((r - R) / 1.5))
    rng = np.random.default_rng(seed)
    psi = np.sqrt(rho) * (1.0 + 1e-3 * rng.standard_normal(_shape(n)))
    return psi.astype(np.complex128)


def bubble_psi(n, step):
    """sqrt(rho0) (1 - exp(-r^2 / (2 * 5^2))) (1 + 1e-3 N(0,1)), seed 42 (r in bohr)."""
    X, Y, Z = _centred(n, step)
    r2 = X ** 2 + Y ** 2 + Z ** 2
    rng = np.random.default_rng(42)
    return (np.sqrt(RHO0) * (1 - np.exp(-r2 / (2 * 5.0 ** 2))) * (1 + 1e-3 * rng.standard_normal(_shape(n)))).astype(complex)


def gaussian_vext(n, step):
    """10 K exp(-r^2 / (2 * 3^2)) at the grid centre."""
    X, Y, Z = _centred(n, step)
    return 10.0 / AUTOK * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 3.0 ** 2)) * np.ones(_shape(n))


def wave_psi(n, step):
    """rho0 (1 + 0.01 cos(2 pi x / (32 step) + phi)), phi ~ U(0, 2 pi) from seed 7."""
    X, _, _ = _centred(n, step)
    phase = np.random.default_rng(7).uniform(0, 2 * np.pi)
    return (np.sqrt(RHO0 * (1 + 0.01 * np.cos(2 * np.pi * X / (32 * step) + phase))) * np.ones(_shape(n))).astype(complex)


def ring_psi(n, step, R=40.0, core=1.0):
    """Uniform rho0 with a phase-imprinted vortex ring of radius R about the z axis, tanh(d / core) core."""
    X, Y, Z = _centred(n, step)
    rc = np.sqrt(X ** 2 + Y ** 2)
    d = np.sqrt((rc - R) ** 2 + Z ** 2)
    theta = np.arctan2(Z, rc - R)
    return (np.sqrt(RHO0) * np.tanh(d / core) * np.exp(1j * theta)).astype(np.complex64).astype(complex)


# name: grid, step (bohr), OT model (DFT_OT_KC = 1, DFT_OT_BACKFLOW = 8), dt (fs; imaginary
# time negative-imaginary), renormalisation, l_g (A; None = default), initial state, external potential
WORKLOADS = {
    "cfg0": dict(n=64, step=1.0, model=0, dt_fs=-10j, renorm=True, lg=None, psi=bubble_psi, vext=gaussian_vext,
                 what="plain OT, bubble around a 10 K Gaussian external potential, imaginary-time predict-correct "
                      "dt=10 fs, norm fixed"),
    "cfg1": dict(n=128, step=0.8, model=9, dt_fs=1.0 + 0j, renorm=False, lg=1.1, psi=wave_psi, vext=None,
                 what="full OT (KC+BF, l_g=1.1 A), 1 % density wave, real-time predict-correct dt=1 fs"),
    "cfg2": dict(n=256, step=0.8, model=9, dt_fs=-20j, renorm=True, lg=None, psi=droplet_psi, vext=None,
                 what="He droplet N=2000, full OT (KC+BF), imaginary-time predict-correct dt=20 fs, "
                      "renormalised each step"),
    "cfg4": dict(n=512, step=0.6, model=9, dt_fs=0.5 + 0j, renorm=False, lg=None, psi=ring_psi, vext=None,
                 what="vortex ring R=40 bohr in bulk liquid, full OT (KC+BF), real-time predict-correct dt=0.5 fs"),
}
W = dict(WORKLOADS["cfg2"], name="cfg2")


PROPAGATORS = {"fft": 1, "cn": 3}   # WF_2ND_ORDER_FFT, WF_2ND_ORDER_CN


def set_workload(name, grid=None, propagator="fft"):
    global W
    W = dict(WORKLOADS[name], name=name, propagator=PROPAGATORS[propagator])
    if grid:
        W["n"] = grid if isinstance(grid, int) or len(grid) != 1 else grid[0]


def shape():
    return _shape(W["n"])


def npoints():
    nx, ny, nz = shape()
    return nx * ny * nz


def metric_name():
    return "OT-DFT steps/s at 256\u00b3, FP32-bulk vs FP64 plain on 1 GB300 @ \u22641e-6 rel. energy err"


def initial_state():
    n, step = W["n"], W["step"]
    psi = W["psi"](n, step)
    vext = W["vext"](n, step) if W["vext"] else None
    norm = None
    if W["renorm"]:
        norm = NATOMS if W["psi"] is droplet_psi else float(np.sum(np.abs(psi) ** 2) * step ** 3)
    return psi, vext, norm


def dt_au():
    return W["dt_fs"] / AUTOFS


def finite_or_null(obj):
    """NaN / inf (phases a run skipped) as JSON null, so the line is strict JSON."""
    if isinstance(obj, float):
        return obj if np.isfinite(obj) else None
    if isinstance(obj, dict):
        return {k: finite_or_null(v) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [finite_or_null(v) for v in obj]
    return obj


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5).stdout
                f = [x.strip() for x in out.strip().split(",")]
                if len(f) >= 9:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------------------- GPU arm
class Setup:
    """Wave functions, functional, potential and external potential of one precision."""

    def __init__(self, G, prec, psi0, vext0, norm):
        G.set_precision(prec)
        step, shp = W["step"], shape()
        self.w = G.Wf(shp, step, propagator=W["propagator"])
        self.wp = G.Wf(shp, step, propagator=W["propagator"])
        lg = W["lg"] / AUTOANG if W["lg"] else None
        self.ot = G.OT(W["model"], self.w, lg_bohr=lg)
        self.w.set(psi0)
        if norm is not None:
            self.w.norm_target = norm
            self.w.normalize()
        self.P = G.CGrid(shp, step)
        self.vext = None
        if vext0 is not None:
            self.vext = G.RGrid(shp, step)
            self.vext.set(vext0)
        self.mu0 = self.ot.bulk_chempot(0.0)

    def run(self, nsteps):
        self.ot.run(self.w, self.wp, self.P, self.vext, self.mu0, dt_au(), nsteps, W["renorm"])

    def free(self):
        for o in (self.vext, self.P, self.ot, self.wp, self.w):
            if o is not None:
                o.free()


def time_steps(G, torch, S, steps, dist):
    """K graph-replayed steps bracketed by barrier + synchronize; CUDA events on
    the library's stream (the legacy default stream, torch's current stream)."""
    G.synchronize()
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_steps")
    t0.record()
    S.run(steps)
    t1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = t0.elapsed_time(t1)
    if dist:
        ms = max_over_ranks(torch, ms, "cuda")
    return ms


def max_over_ranks(torch, ms, device):
    """Replica timing: the slowest rank's milliseconds (all ranks get it)."""
    x = torch.tensor([ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(x, op=torch.distributed.ReduceOp.MAX)
    return float(x.item())


def profile_step(G, S):
    """One eager predict-correct step (+ renormalisation) with the kernel profiler on."""
    L = G.lib()
    G.check(L.dftgpu_profile(1), "dftgpu_profile")
    S.ot.pc_step(S.w, S.wp, S.P, S.vext, S.mu0, dt_au())
    if W["renorm"]:
        S.w.normalize()
    buf = __import__("ctypes").create_string_buffer(1 << 16)
    G.check(L.dftgpu_profile_report(buf, len(buf)), "profile_report")
    G.check(L.dftgpu_profile(0), "dftgpu_profile")
    return json.loads(buf.value.decode())


def time_adjoint(G, torch, S, nsteps, every):
    """dJ/dVext and dJ/dpsi_0 of J = int (|psi_T|^2 - rho_t)^2 dV over nsteps
    steps (forward sweep, checkpoints every `every` steps, reverse sweep
    recomputing each segment), timed with CUDA events on the library's stream."""
    step, shp = W["step"], shape()
    psi = S.w.get()
    vext, rt, gv = G.RGrid(shp, step), G.RGrid(shp, step), G.RGrid(shp, step)
    gp = G.CGrid(shp, step)
    vext.set(np.zeros(shp))
    rt.set(np.abs(psi) ** 2 * 1.01)
    S.ot.adjoint_run(S.w, vext, S.mu0, dt_au(), 2, W["renorm"], rt, gv, gp, checkpoint_every=every)   # allocations
    S.w.set(psi)
    G.synchronize()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    S.ot.adjoint_run(S.w, vext, S.mu0, dt_au(), nsteps, W["renorm"], rt, gv, gp, checkpoint_every=every)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    ok = bool(np.isfinite(gv.get()).all())
    for o in (gp, gv, rt, vext):
        o.free()
    return ms, ok


def model_bytes():
    """Algorithmic bytes of one FP32 step: (4 T + 28) N P, T = 3-D real transforms per potential
    (plain 5, + KC 24, full 34), P = 4 bytes."""
    T = {0: 5, 1: 24, 8: 15, 9: 34}[W["model"]]
    return (4 * T + 28) * npoints() * 4


def run_gpu(args):
    import torch
    import libdft_gb300 as G

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    torch.cuda.init()
    G.check(G.lib().dftgpu_init(local), "dftgpu_init")

    psi0, vext0, norm = initial_state()
    K, Wu = args.steps, args.warmup
    n = W["n"]
    N = npoints()

    # ---- FP32-bulk headline
    S = Setup(G, G.FP32, psi0, vext0, norm)
    S.run(Wu)                                                   # warm-up (captures the step graph)
    with ClockSampler(local) as clk:
        ms = time_steps(G, torch, S, K, dist)
    clocks = clk.summary()
    prof = profile_step(G, S)

    # e2e through the public API with host buffers: H2D psi, one step, D2H psi
    host = torch.empty(2 * N, dtype=torch.float32, pin_memory=True)
    L = G.lib()
    G.check(L.cgrid_copy_to_host_raw(S.w.grid_ptr, host.data_ptr()), "d2h")
    ke = max(3, K // 5)
    S.run(1)
    G.synchronize()
    te = time.perf_counter()
    for _ in range(ke):
        G.check(L.cgrid_copy_from_host_raw(S.w.grid_ptr, host.data_ptr()), "h2d")
        S.run(1)
        G.check(L.cgrid_copy_to_host_raw(S.w.grid_ptr, host.data_ptr()), "d2h")
    e2e_s = time.perf_counter() - te
    adj_steps, adj_every = 9, 3
    ms_adj32, adj_ok32 = time_adjoint(G, torch, S, adj_steps, adj_every)
    S.free()

    # ---- accuracy: FP32 vs FP64 energy per atom after the same steps from psi0
    acc_steps = args.acc_steps
    energies = {G.FP32: (float("nan"), float("nan")), G.FP64: (float("nan"), float("nan"))}
    rho = {}
    ms64, k64 = float("nan"), 1
    ms_adj, adj_ok = float("nan"), False
    for prec in (() if args.fp32_only else (G.FP32, G.FP64)):
        S = Setup(G, prec, psi0, vext0, norm)
        S.run(acc_steps)
        e, nrm, mu = S.ot.energy_report(S.w, S.vext)
        energies[prec] = (e / nrm, mu)
        rho[prec] = np.abs(S.w.get()) ** 2
        if prec == G.FP64:
            # ---- FP64 path throughput on the same workload, and its adjoint
            # (the precision whose gradients meet the 1e-4 finite-difference target)
            k64 = max(2, K // 10)
            ms64 = time_steps(G, torch, S, k64, dist)
            ms_adj, adj_ok = time_adjoint(G, torch, S, adj_steps, adj_every)
        S.free()
    l2 = (float(np.linalg.norm(rho[G.FP32] - rho[G.FP64]) / np.linalg.norm(rho[G.FP64]))
          if len(rho) == 2 else float("nan"))

    if rank != 0:
        if dist:
            torch.distributed.destroy_process_group()
        return None

    per_step = sum(v["launches"] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    dom_name, dom_v = dom
    achieved = dom_v["bytes"] / (dom_v["ms"] * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic, step_dram = None, None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if tj.get("workload") == W["name"] and tj.get("grid") == n:
            traffic = tj.get("per_launch_bytes", {}).get(dom_name)
            step_dram = tj.get("dram_bytes_per_step")

    steps_s = world * K / (ms * 1e-3)
    steps_s64 = world * k64 / (ms64 * 1e-3)
    e32, e64 = energies[G.FP32][0], energies[G.FP64][0]
    ms_step = ms / K
    alg = model_bytes()
    line = {
        "metric": metric_name(),
        "value": steps_s,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": Wu,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": workload_name(), "grid": list(shape()), "model": model_name(),
                   "precision": "FP32 bulk, FP64 reductions", "l2": l2_note(), "parallelism": "replicas"},
        "e2e": {"value": world * ke / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": 2 * N * 4,
                "d2h_bytes_per_step": 2 * N * 4},
        "adjoint": {"value": world * adj_steps / (ms_adj * 1e-3), "unit": "trajectory steps/s",
                    "what": "gradient of a final-density objective w.r.t. Vext and psi_0: forward sweep + "
                            "checkpointed reverse sweep (dftgpu_adjoint_run), FP64 (the precision whose "
                            "gradients meet the 1e-4 finite-difference target)",
                    "nsteps": adj_steps, "checkpoint_every": adj_every, "ms_per_step": ms_adj / adj_steps,
                    "cost_over_forward_step": (ms_adj / adj_steps) / (ms64 / k64), "finite": adj_ok,
                    "fp32": {"value": world * adj_steps / (ms_adj32 * 1e-3), "ms_per_step": ms_adj32 / adj_steps,
                             "cost_over_forward_step": (ms_adj32 / adj_steps) / ms_step, "finite": adj_ok32,
                             "note": "FP32 bulk: gradients within ~3e-3 of finite differences, outside the "
                                     "1e-4 target"}},
        "fp64": {"value": steps_s64, "unit": "steps/s", "steps": k64, "ms_per_step": ms64 / k64},
        "fp32_over_fp64": steps_s / steps_s64,
        "accuracy": {"steps": acc_steps, "E_per_atom_K_fp32": e32 * AUTOK, "E_per_atom_K_fp64": e64 * AUTOK,
                     "rel_err_E_per_atom": abs(e32 - e64) / abs(e64),
                     "mu_K_fp32": energies[G.FP32][1] * AUTOK, "mu_K_fp64": energies[G.FP64][1] * AUTOK,
                     "rel_err_mu": abs(energies[G.FP32][1] / energies[G.FP64][1] - 1),
                     "density_rel_L2": l2},
        "algorithmic_GBps_step_model": alg / (ms_step * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "launches_per_step": dom_v["launches"],
                     "share_of_step": dom_v["ms"] / sum(v["ms"] for v in prof.values()),
                     "step_model_bytes": alg, "step_frac": alg / (ms_step * 1e-3) / 1e9 / peak,
                     "step_dram_bytes": step_dram,
                     "step_dram_frac": (step_dram / (ms_step * 1e-3) / 1e9 / peak) if step_dram else None},
        "kernel_profile": {k: {"launches": v["launches"], "ms": round(v["ms"], 4),
                               "GBps": (v["bytes"] / (v["ms"] * 1e-3) / 1e9 if v["ms"] > 0 and v["bytes"] > 0 else None)}
                           for k, v in prof.items()},
        "gpu_launches": per_step * K,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(1, args.cpu_steps)
    if dist:
        torch.distributed.destroy_process_group()
    return line


def model_name():
    return {0: "OT plain", 1: "OT+KC", 8: "OT+BF", 9: "OT+KC+BF"}[W["model"]]


def workload_name():
    nx, ny, nz = shape()
    g = "%d^3" % nx if nx == ny == nz else "%dx%dx%d" % (nx, ny, nz)
    cn = ", Crank-Nicolson kinetic step" if W["propagator"] == PROPAGATORS["cn"] else ""
    return "%s: %s%s, %s, step %g bohr" % (W["name"], W["what"], cn, g, W["step"])


def l2_note():
    """whether one wave function (FP32) outruns the 129 MB L2 between steps"""
    mb = 8 * npoints() / 1e6
    if mb > 129:
        return "inputs larger than L2 (psi %.0f MB FP32); no flush" % mb
    return "psi %.1f MB FP32 fits in L2 (smaller than the headline workload); no flush" % mb


# ---------------------------------------------------------------------- CPU oracle
def cpu_baseline(warmup=1, steps=5):
    """The FP64 CPU oracle on the same workload, all host cores: `warmup`
    untimed steps, then `steps` timed steps."""
    from oracle import Grids, Oracle
    o = Oracle("port")
    psi0, vext0, norm = initial_state()
    step = W["step"]
    mass = 4.002602 / o.AUTOAMU
    with Grids(o, shape(), step, mass) as g:
        w = g.wf(psi0, W["propagator"])
        vext = g.rgrid(vext0) if vext0 is not None else None
        # kernels sampled with one sub-point per cell: the step's cost does not
        # depend on the kernel values and full adaptive sampling takes minutes
        lg = W["lg"] / AUTOANG if W["lg"] else 0.0
        otf = g.ot(W["model"], w, min_ns=1, max_ns=1, lg_bohr=lg)
        mu0 = o.lib.orc_bulk_chempot(otf, 0.0)
        wp, P = g.wf(None, W["propagator"]), g.cgrid()
        if norm is not None:
            o.lib.orc_wf_set_norm(w, norm)
            o.lib.orc_wf_normalize(w)
        dt = dt_au()

        def one():
            o.lib.orc_pc_step(otf, w, wp, P, vext, mu0, dt.real, dt.imag)
            if norm is not None:
                o.lib.orc_wf_normalize(w)

        for _ in range(warmup):
            one()
        t = time.perf_counter()
        for _ in range(steps):
            one()
        el = time.perf_counter() - t
    return {"value": steps / el, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d warm-up + %d timed predict-correct step(s) of the %s workload (%s), FP64, OpenMP over "
                      "all host cores (%.1f s timed)" % (warmup, steps, W["name"], "x".join(map(str, shape())), el)}


def run_reference(args):
    """The reference arm: the FP64 CPU oracle (the restatement of libdft's CPU
    path, OpenMP over all host cores) on this workload; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    warm = min(getattr(args, "warmup", 1), 5)
    steps = max(1, min(getattr(args, "steps", 1), 30))
    cb = cpu_baseline(warm, steps)
    return {"impl": "reference", "metric": metric_name(), "value": cb["value"], "unit": "steps/s", "n_gpus": 0,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(), "grid": list(shape())},
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS))
    ap.add_argument("--acc-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=5, help="timed steps of the CPU baseline (after 1 warm-up)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", default="", help="grid size N (cubic) or NXxNYxNZ (default: the workload's)")
    ap.add_argument("--fp32-only", action="store_true", help="skip the FP64 and accuracy phases (profiling runs)")
    ap.add_argument("--propagator", default="fft", choices=sorted(PROPAGATORS),
                    help="kinetic step of the wave functions: FFT (default) or Crank-Nicolson")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    grid = tuple(int(v) for v in args.grid.lower().split("x")) if args.grid else None
    set_workload(args.workload, grid, args.propagator)
    line = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if line is not None:
        print(json.dumps(finite_or_null(line)))


if __name__ == "__main__":
    main()
