#!/usr/bin/env python
"""OT-DFT time-step throughput on GB300 (steps/s at 256^3, full OT).

Workload (the helium-nanodroplet relaxation the headline metric is quoted
on): 256^3 grid, step 0.8 bohr, full Orsay-Trento functional (kinetic
correlation + backflow), a droplet of N = 2000 atoms (radius
(3N / 4 pi rho0)^(1/3), 1.5 bohr tanh surface, 1e-3 multiplicative noise,
seed 3), imaginary-time predict-correct steps of 20 fs with the particle
number renormalised to N after every step.  One "step" is one
predict-correct step: two OT potential evaluations and two split-operator
propagations.  Data are synthetic; every input (psi: 134 MB in FP32) is
larger than L2, so no L2 flush is needed between steps.

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

NX = 256
STEP = 0.8
NATOMS = 2000.0
DT_FS = 20.0
MODEL = 1 | 8          # DFT_OT_KC | DFT_OT_BACKFLOW


def metric_name():
    try:
        with open(os.path.join(ROOT, "BASELINE.json")) as f:
            return json.load(f)["metric"]
    except Exception:
        return "OT-DFT steps/s at 256^3, FP32-bulk vs FP64 plain on 1 GB300"


def droplet_psi(n=NX, step=STEP, seed=3):
    rho0 = 0.0218360 * 0.529177210903 ** 3
    R = (3.0 * NATOMS / (4.0 * np.pi * rho0)) ** (1.0 / 3.0)
    ax = (np.arange(n) - n // 2) * step
    r = np.sqrt(ax[:, None, None] ** 2 + ax[None, :, None] ** 2 + ax[None, None, :] ** 2)
    rho = 0.5 * rho0 * (1.0 - np.tanh((r - R) / 1.5))
    rng = np.random.default_rng(seed)
    psi = np.sqrt(rho) * (1.0 + 1e-3 * rng.standard_normal((n, n, n)))
    return psi.astype(np.complex128)


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
def gpu_setup(G, prec, psi0):
    G.set_precision(prec)
    shape = (NX, NX, NX)
    w, wp = G.Wf(shape, STEP), G.Wf(shape, STEP)
    ot = G.OT(MODEL, w)
    w.set(psi0)
    w.norm_target = NATOMS
    w.normalize()
    P = G.CGrid(shape, STEP)
    mu0 = ot.bulk_chempot(0.0)
    return w, wp, ot, P, mu0


def free_all(*objs):
    for o in objs:
        o.free()


def time_steps(G, torch, w, wp, ot, P, mu0, dt, steps, dist):
    """K graph-replayed steps bracketed by barrier + synchronize; CUDA events on
    the library's stream (the legacy default stream, torch's current stream)."""
    G.synchronize()
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_steps")
    t0.record()
    ot.run(w, wp, P, None, mu0, dt, steps, True)
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


def profile_step(G, w, wp, ot, P, mu0, dt):
    """One eager predict-correct step + renormalisation with the kernel profiler on."""
    L = G.lib()
    G.check(L.dftgpu_profile(1), "dftgpu_profile")
    ot.pc_step(w, wp, P, None, mu0, dt)
    w.normalize()
    buf = __import__("ctypes").create_string_buffer(1 << 16)
    G.check(L.dftgpu_profile_report(buf, len(buf)), "profile_report")
    G.check(L.dftgpu_profile(0), "dftgpu_profile")
    return json.loads(buf.value.decode())


def time_adjoint(G, torch, w, ot, mu0, dt, nsteps, every):
    """dJ/dVext and dJ/dpsi_0 of J = int (|psi_T|^2 - rho_t)^2 dV over nsteps
    renormalised steps (forward sweep, checkpoints every `every` steps, reverse
    sweep recomputing each segment), timed with CUDA events on the library's stream."""
    shape = (NX, NX, NX)
    psi = w.get()
    vext, rt, gv = G.RGrid(shape, STEP), G.RGrid(shape, STEP), G.RGrid(shape, STEP)
    gp = G.CGrid(shape, STEP)
    vext.set(np.zeros(shape))
    rt.set(np.abs(psi) ** 2 * 1.01)
    ot.adjoint_run(w, vext, mu0, dt, 2, True, rt, gv, gp, checkpoint_every=every)    # allocations
    w.set(psi)
    G.synchronize()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    ot.adjoint_run(w, vext, mu0, dt, nsteps, True, rt, gv, gp, checkpoint_every=every)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    ok = bool(np.isfinite(gv.get()).all())
    free_all(gp, gv, rt, vext)
    return ms, ok


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

    dt = -1j * DT_FS / 0.024188843265857
    psi0 = droplet_psi(NX)
    K, W = args.steps, args.warmup

    # ---- FP32-bulk headline
    w, wp, ot, P, mu0 = gpu_setup(G, G.FP32, psi0)
    ot.run(w, wp, P, None, mu0, dt, W, True)                   # warm-up (captures the step graph)
    with ClockSampler(local) as clk:
        ms = time_steps(G, torch, w, wp, ot, P, mu0, dt, K, dist)
    clocks = clk.summary()
    prof = profile_step(G, w, wp, ot, P, mu0, dt)

    # e2e through the public API with host buffers: H2D psi, one step, D2H psi
    host = torch.empty(2 * NX ** 3, dtype=torch.float32, pin_memory=True)
    L = G.lib()
    G.check(L.cgrid_copy_to_host_raw(w.grid_ptr, host.data_ptr()), "d2h")
    ke = max(3, K // 5)
    ot.run(w, wp, P, None, mu0, dt, 1, True)
    G.synchronize()
    te = time.perf_counter()
    for _ in range(ke):
        G.check(L.cgrid_copy_from_host_raw(w.grid_ptr, host.data_ptr()), "h2d")
        ot.run(w, wp, P, None, mu0, dt, 1, True)
        G.check(L.cgrid_copy_to_host_raw(w.grid_ptr, host.data_ptr()), "d2h")
    e2e_s = time.perf_counter() - te
    adj_steps, adj_every = 9, 3
    ms_adj, adj_ok = time_adjoint(G, torch, w, ot, mu0, dt, adj_steps, adj_every)
    free_all(P, ot, wp, w)

    # ---- accuracy: FP32 vs FP64 energy per atom after the same steps from psi0
    acc_steps = args.acc_steps
    energies = {G.FP32: (float("nan"), float("nan")), G.FP64: (float("nan"), float("nan"))}
    ms64, k64 = float("nan"), 1
    for prec in (() if args.fp32_only else (G.FP32, G.FP64)):
        w, wp, ot, P, mu0 = gpu_setup(G, prec, psi0)
        ot.run(w, wp, P, None, mu0, dt, acc_steps, True)
        e, n, mu = ot.energy_report(w)
        energies[prec] = (e / n, mu)
        if prec == G.FP64:
            # ---- FP64 path throughput on the same workload
            k64 = max(2, K // 10)
            ms64 = time_steps(G, torch, w, wp, ot, P, mu0, dt, k64, dist)
        free_all(P, ot, wp, w)

    if rank != 0:
        if dist:
            torch.distributed.destroy_process_group()
        return None

    per_step = sum(v["launches"] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    dom_name, dom_v = dom
    achieved = dom_v["bytes"] / (dom_v["ms"] * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if dom_name in tj.get("per_launch_bytes", {}):
            traffic = tj["per_launch_bytes"][dom_name]

    steps_s = world * K / (ms * 1e-3)
    steps_s64 = world * k64 / (ms64 * 1e-3)
    e32, e64 = energies[G.FP32][0], energies[G.FP64][0]
    N = NX ** 3
    T = 34
    alg_bytes = (4 * T + 28) * N * 4
    line = {
        "metric": metric_name(),
        "value": steps_s,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": workload_name(), "grid": [NX, NX, NX], "model": "OT+KC+BF",
                   "precision": "FP32 bulk, FP64 reductions", "l2": l2_note(), "parallelism": "replicas"},
        "e2e": {"value": world * ke / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": 2 * N * 4,
                "d2h_bytes_per_step": 2 * N * 4},
        "adjoint": {"value": world * adj_steps / (ms_adj * 1e-3), "unit": "trajectory steps/s",
                    "what": "gradient of a final-density objective w.r.t. Vext and psi_0: forward sweep + "
                            "checkpointed reverse sweep (dftgpu_adjoint_run), FP32",
                    "nsteps": adj_steps, "checkpoint_every": adj_every, "ms_per_step": ms_adj / adj_steps,
                    "cost_over_forward_step": (ms_adj / adj_steps) / (ms / K), "finite": adj_ok},
        "fp64": {"value": steps_s64, "unit": "steps/s", "steps": k64, "ms_per_step": ms64 / k64},
        "fp32_over_fp64": steps_s / steps_s64,
        "accuracy": {"steps": acc_steps, "E_per_atom_K_fp32": e32 * 3.1577502480407e5,
                     "E_per_atom_K_fp64": e64 * 3.1577502480407e5,
                     "rel_err_E_per_atom": abs(e32 - e64) / abs(e64),
                     "mu_K_fp32": energies[G.FP32][1] * 3.1577502480407e5,
                     "mu_K_fp64": energies[G.FP64][1] * 3.1577502480407e5},
        "algorithmic_GBps_step_model": alg_bytes / (ms / K * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "launches_per_step": dom_v["launches"], "share_of_step": dom_v["ms"] / sum(v["ms"] for v in prof.values())},
        "kernel_profile": {k: {"launches": v["launches"], "ms": round(v["ms"], 4),
                               "GBps": (v["bytes"] / (v["ms"] * 1e-3) / 1e9 if v["ms"] > 0 and v["bytes"] > 0 else None)}
                           for k, v in prof.items()},
        "gpu_launches": per_step * K,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    if dist:
        torch.distributed.destroy_process_group()
    return line


def workload_name():
    return ("He droplet N=2000, %d^3, step 0.8 bohr, full OT (KC+BF), imaginary-time predict-correct dt=20 fs, "
            "renormalised each step" % NX)


def l2_note():
    """whether one wave function (FP32) outruns the 129 MB L2 between steps"""
    mb = 8 * NX ** 3 / 1e6
    if mb > 129:
        return "inputs larger than L2 (psi %.0f MB FP32); no flush" % mb
    return "psi %.1f MB FP32 fits in L2 (profiling size, not the headline workload); no flush" % mb


# ---------------------------------------------------------------------- CPU oracle
def cpu_baseline(args, steps=1):
    """The FP64 CPU oracle on the same workload, all host cores."""
    from oracle import Grids, Oracle
    o = Oracle("port")
    psi0 = droplet_psi(NX)
    mass = 4.002602 / o.AUTOAMU
    with Grids(o, (NX, NX, NX), STEP, mass) as g:
        w = g.wf(psi0)
        # kernels sampled with one sub-point per cell: the step's cost does not
        # depend on the kernel values and full adaptive sampling takes minutes
        otf = g.ot(MODEL, w, min_ns=1, max_ns=1)
        mu0 = o.lib.orc_bulk_chempot(otf, 0.0)
        wp, P = g.wf(), g.cgrid()
        o.lib.orc_wf_set_norm(w, NATOMS)
        o.lib.orc_wf_normalize(w)
        dt = -1j * DT_FS / o.AUTOFS
        t = time.perf_counter()
        for _ in range(steps):
            o.lib.orc_pc_step(otf, w, wp, P, None, mu0, dt.real, dt.imag)
            o.lib.orc_wf_normalize(w)
        el = time.perf_counter() - t
    return {"value": steps / el, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d predict-correct step(s) of the %d^3 full-OT droplet workload, FP64, OpenMP over all "
                      "host cores (%.1f s)" % (steps, NX, el)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    cb = cpu_baseline(args, steps=max(1, min(args.steps, 2)))
    return {"impl": "reference", "metric": metric_name(), "value": cb["value"], "unit": "steps/s", "n_gpus": 0,
            "steps": max(1, min(args.steps, 2)), "warmup": 0, "ms_per_step": 1e3 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(), "grid": [NX, NX, NX]},
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--acc-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=256, help="grid points per axis (profiling of smaller cases)")
    ap.add_argument("--fp32-only", action="store_true", help="skip the FP64 and accuracy phases (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global NX
    NX = args.grid
    line = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if line is not None:
        print(json.dumps(finite_or_null(line)))


if __name__ == "__main__":
    main()
