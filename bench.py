#!/usr/bin/env python
"""agent-steps/s of the chili mechanics/interaction step on GB300.

One bench step = one complete run of the workload from its initial state: for the default
workload (rods_2d) 100,000 bacterial rods x 6 vertices, the first 400 of its 500
explicit-Euler steps in FP64 (RODS_TIMED_STEPS below says why).
  value  device-resident throughput: the initial state is restored on the device (crg_snapshot)
         and the 400 steps run from CUDA graphs; CUDA events on the library's stream bracket
         the K timed steps; L2 is flushed (256 MiB write) between timed steps.
  e2e    the same run through the public C ABI with host buffers: crg_upload from pinned
         host memory, crg_step, crg_download to host, every bench step.
  cpu_baseline  the oracle (a C++ restatement of chili, multi-threaded by subdomains like
         chili) on this host's cores: all usable cores (one chili subdomain per thread) and
         one thread, each over the first steps of the same run that fit in about
         --cpu-seconds (the count is stated in `sample`), with the core count and CPU model
         of the host.  The GPU arm runs the same subdomain weight map.
--impl reference times that CPU implementation alone, with all usable host cores, on the
whole timed run when it takes at most ~20 s on the host, else on its first steps.

Multi-GPU: the path is replicated, not sharded (independent simulations); each rank runs
the workload on its own GPU and rank 0 reports the sum of agent-steps over the max time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "agent-steps/s on 1 GB300: FP64 plain vs mixed/batched; served p50/p99 latency"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="crg", choices=["crg", "reference"])
    p.add_argument("--workload", default="rods_2d", choices=["rods_2d", "spheres_3d"])
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the mixed-precision, ensemble and served measurements")
    p.add_argument("--extras", default="rods_mixed,mixed_large,ensemble,served,cell_cycle",
                   help="comma-separated extras to run (default: all)")
    # a small run for profilers (ncu): direct launches, every kernel a separate launch
    p.add_argument("--profile-case", action="store_true",
                   help="run --case-steps steps of the workload with direct launches (no CUDA "
                        "graphs), print the wall time and exit")
    p.add_argument("--case-steps", type=int, default=10)
    p.add_argument("--case-n", type=int, default=0, help="agents (0: the workload's size)")
    p.add_argument("--case-side", type=float, default=0.0,
                   help="box side (rod_colony; 0: the workload's default)")
    p.add_argument("--case-subdomains", type=int, default=16)
    p.add_argument("--case-precision", default=None, choices=[None, "f64", "mixed"])
    p.add_argument("--case-variant", type=int, default=0, help="CRG_OPT_KERNEL_VARIANT")
    p.add_argument("--case-workload", default=None,
                   choices=[None, "rods_2d", "spheres_3d", "spheres_3d_large", "rod_colony"])
    # the served form over several arrival rates (minutes of GPU time: not in the default run)
    p.add_argument("--served-sweep", action="store_true",
                   help="run the request stream at --sweep-rates and print one JSON line")
    p.add_argument("--sweep-rates", default="15,25,40,80")
    p.add_argument("--sweep-requests", type=int, default=1000)
    # every force-kernel shape the autotuner tries, timed on the ensemble and at 2^23
    p.add_argument("--tile-sweep", action="store_true",
                   help="time every mixed sphere force-kernel shape (block x tile) on the "
                        "1,024-simulation ensemble and on 2^23 spheres; one JSON line")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# The rods workload is unstable under the reference's own RodMechanics: crushed rods fold
# to angles where the tan(angle/2) curvature force diverges and the run ends with a
# BoundaryError near step 450 (the oracle and the GPU stop at the same rod and step,
# tests/test_gpu_fullsize.py).  The timed run therefore covers the first 400 of the 500
# configured steps.
RODS_TIMED_STEPS = 400


def n_subdomains():
    """chili's n_threads for every arm: one subdomain per usable host core, the run the CPU
    arm makes on all cores.  The number of subdomains fixes chili's pair weights, so the GPU
    arm runs the same weight map (the same physics) as the all-core CPU run."""
    from cellular_raza_gb300 import workloads as W

    return W.host_threads()


def host_cpu():
    """Processor count, usable cores and CPU model of this host (where the CPU arms run)."""
    import platform

    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=20).stdout
        f = {}
        for ln in out.splitlines():
            if ":" in ln:
                k, v = ln.split(":", 1)
                f.setdefault(k.strip(), v.strip())
        model = f.get("Model name")
        vendor = f.get("Vendor ID")
        if model and vendor and vendor not in model:
            model = f"{vendor} {model}"
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as fh:
                for ln in fh:
                    if ln.lower().startswith("model name"):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    from cellular_raza_gb300 import workloads as W

    return {"nproc": os.cpu_count(), "usable_cores": W.host_threads(),
            "cpu_model": model or "unknown", "arch": platform.machine()}


def make_workload(name, n_sub=None):
    n_sub = n_subdomains() if n_sub is None else n_sub
    from cellular_raza_gb300 import workloads as W

    if name == "rods_2d":
        w = W.rods_2d(seed=2024, n_subdomains=n_sub)
        w.n_steps = RODS_TIMED_STEPS
        return w
    return W.spheres_3d(seed=2024, n_subdomains=n_sub)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def committed_traffic(kernel_key):
    """Per-launch DRAM bytes of the force kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel_key)
    except (OSError, ValueError):
        return None


# ----------------------------------------------------------------------------- CPU arms

def oracle_rate(w, threads, seconds):
    """The oracle on `threads` threads (= chili subdomains) over the first steps of the
    workload, as many as fit in about `seconds` (all of them when they fit)."""
    import pyoracle

    pyoracle.build()
    m = w.model.replace(n_subdomains=threads)
    probe = pyoracle.run(m, w.pos, w.vel, 1)["elapsed_s"]
    steps = int(max(1, min(w.n_steps, seconds / max(probe, 1e-6))))
    r = pyoracle.run(m, w.pos, w.vel, steps)
    return w.n * steps / r["elapsed_s"], steps, r["elapsed_s"]


def cpu_run(w, n_threads, seconds):
    """CPU baseline on this host: all usable cores (one subdomain each, the GPU arm's weight
    map) and one thread, each on a bounded sample of the same workload."""
    host = host_cpu()
    v_all, s_all, t_all = oracle_rate(w, n_threads, seconds)
    v_one, s_one, t_one = oracle_rate(w, 1, seconds)
    return {"value": v_all, "unit": "agent-steps/s", "cores": n_threads, "threads": n_threads,
            "kind": "port", **host,
            "sample": f"{w.name}: {w.n} agents x {s_all} of {w.n_steps} steps, {n_threads} "
                      f"threads = {n_threads} chili subdomains ({t_all:.1f} s)",
            "single_thread": {"value": v_one, "unit": "agent-steps/s", "threads": 1,
                              "sample": f"{w.name}: {w.n} agents x the first {s_one} of "
                                        f"{w.n_steps} steps, 1 thread = 1 subdomain "
                                        f"({t_one:.1f} s)"}}


def workload_config(w, n_subdomains, world):
    """The `config` object both arms print: the workload, its sizes and the step it runs
    (each arm's sampling and timing details go in its own keys)."""
    return {"workload": w.name, "agents": w.n, "vertices_per_agent": w.model.n_vertices,
            "dim": w.model.dim, "sim_steps_per_bench_step": w.n_steps, "solver": "euler",
            "precision": "f64", "n_subdomains": n_subdomains,
            "l2": "GPU arm: flushed between timed steps (256 MiB write)",
            "parallelism": f"replicas x{world}"}


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n_threads = n_subdomains()  # chili runs one OS thread per subdomain
    w = make_workload(args.workload)
    import pyoracle

    pyoracle.build()
    m = w.model.replace(n_subdomains=n_threads)
    probe = pyoracle.run(m, w.pos, w.vel, 1)["elapsed_s"]
    # a bench step is the whole timed run when it takes at most ~20 s on this host, else the
    # first steps of it that do (stated in `sample`)
    steps = int(max(1, min(w.n_steps, 20.0 / max(probe, 1e-6))))
    for _ in range(args.warmup):
        pyoracle.run(m, w.pos, w.vel, 1)
    t_total = 0.0
    for _ in range(args.steps):
        t_total += pyoracle.run(m, w.pos, w.vel, steps)["elapsed_s"]
    value = w.n * steps * args.steps / t_total
    sample = (f"{w.name}: {w.n} agents x {steps} of {w.n_steps} steps per bench step "
              f"({'the whole run' if steps == w.n_steps else 'its first steps'}), "
              f"{n_threads} threads = {n_threads} chili subdomains")
    line = {
        "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded PCG64)", "impl": "reference",
        "config": workload_config(w, n_threads, 1),
        "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": n_threads,
                         "threads": n_threads, "kind": "port", **host_cpu(),
                         "sample": sample},
        "e2e": {"value": value, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm

def mean_interactions(sim, w, every):
    """In-range pair evaluations per step averaged over the run that is timed: the neighbour
    statistics of the state before step 1, 1 + every, ..., and after the last step
    (trapezoidal mean), from a separate untimed pass over the same steps."""
    import numpy as np

    sim.snapshot(restore=True)
    done, samples = 0, []
    while True:
        st = sim.neighbor_stats()
        samples.append((done, float(st["n_inter"].astype(np.float64).sum())))
        if done >= w.n_steps:
            break
        k = min(every, w.n_steps - done)
        sim.step(k)
        done += k
    area = sum((b[0] - a[0]) * (a[1] + b[1]) / 2.0 for a, b in zip(samples, samples[1:]))
    return area / w.n_steps, len(samples)


def algorithmic_flops(w, n_inter):
    """FP64 work of one step's force stage once the FP32 prefilter has removed the
    evaluations beyond the cutoff (sqrt, exp, division count one flop each), as
    (whole force stage, dominant kernel).
    spheres: 30 flop per interacting ordered pair (8 distance + 22 force) + 21 per agent
    (update), all in one kernel; rods: 45 flop per in-range vertex-segment evaluation of
    a.calc(a, b) (18 nearest point, 6 distance, 21 force) in the pass kernel (a lower bound:
    the ext halves of weight-1 pairs come on top) + 250 per rod (springs, curvature,
    update) in the update kernel."""
    if w.model.kind == "rod":
        return 45.0 * n_inter + 250.0 * w.n, 45.0 * n_inter
    f = 30.0 * n_inter + 21.0 * w.n
    return f, f


def replica_throughput(dist, local_ms, local_agent_steps):
    """Whole-job throughput of independent replicas: the agent-steps of all ranks over the
    slowest rank's time.  Returns (max ms, total agent-steps, agent-steps/s)."""
    import torch

    t_max, total = float(local_ms), float(local_agent_steps)
    if dist is not None:
        t = torch.tensor([t_max], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        s = torch.tensor([total], dtype=torch.float64)
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
        t_max, total = float(t.item()), float(s.item())
    return t_max, total, total / (t_max / 1e3)


def timed_run(torch, sim, steps, restore=True):
    """Device time (ms) of `steps` steps of a handle, CUDA events on its stream."""
    ext = torch.cuda.ExternalStream(sim.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if restore:
        sim.snapshot(restore=True)
    torch.cuda.synchronize()
    e0.record(ext)
    sim.step(steps)
    e1.record(ext)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def extra_mixed_large(torch):
    """2^23 spheres at the density of spheres_3d, 200 steps: mixed precision against the FP64
    path (throughput and the relative position error of mixed against FP64)."""
    import numpy as np
    from cellular_raza_gb300 import engine as E
    from cellular_raza_gb300 import workloads as W

    w = W.spheres_3d_large(seed=2024)
    out = {"workload": "spheres_3d_large", "agents": w.n, "steps": w.n_steps}
    finals = {}
    for prec in ("mixed", "f64"):
        sim = E.Simulation.single(w.model.replace(precision=prec), w.n)
        sim.upload(w.pos, w.vel)
        sim.snapshot()
        sim.step(3)  # warm-up (graph instantiation)
        ms = timed_run(torch, sim, w.n_steps)
        out[f"{prec}_agent_steps_per_s"] = w.n * w.n_steps / (ms / 1e3)
        out[f"{prec}_ms_per_step"] = ms / w.n_steps
        finals[prec] = sim.download(order="id")["pos"]
        sim.close()
    a, b = finals["f64"], finals["mixed"]
    dx = np.linalg.norm(b - a, axis=-1).ravel()
    x = np.linalg.norm(a, axis=-1).ravel()
    err = dx / x
    worst = int(np.argmax(err))
    out["speedup_mixed_over_f64"] = out["mixed_agent_steps_per_s"] / out["f64_agent_steps_per_s"]
    out["max_rel_pos_err"] = float(err.max())  # per agent |dx| / |x|
    out["p9999_rel_pos_err"] = float(np.percentile(err, 99.99))
    out["mean_rel_pos_err"] = float(err.mean())
    out["normwise_rel_pos_err"] = float(dx.max() / x.max())  # max |dx| / max |x|
    out["l2_rel_pos_err"] = float(np.linalg.norm(b - a) / np.linalg.norm(a))
    out["max_abs_pos_err"] = float(dx.max())
    out["worst_agent_abs_pos"] = float(x[worst])
    out["agents_above_1e-5"] = int((err > 1e-5).sum())
    # chili's pair weights (1 inside a voxel, 1/2 across neighbour voxels of one subdomain)
    # make the force jump when an agent changes voxel, so an agent within rounding distance
    # of a voxel face can take a different branch in the two runs; the same comparison with
    # the continuous physical weights isolates the precision error itself
    phys = {}
    for prec in ("mixed", "f64"):
        m = w.model.replace(precision=prec, weight_mode=1)
        phys[prec] = E.run(w.__class__(w.name, m, w.pos, w.vel, w.n_steps), w.n_steps)["pos"]
    pe = (np.linalg.norm(phys["mixed"] - phys["f64"], axis=-1).ravel() /
          np.linalg.norm(phys["f64"], axis=-1).ravel())
    out["physical_weights"] = {"max_rel_pos_err": float(pe.max()),
                               "p9999_rel_pos_err": float(np.percentile(pe, 99.99)),
                               "agents_above_1e-5": int((pe > 1e-5).sum())}
    return out


def extra_rods_mixed(torch, n_sub):
    """The headline rod workload (100,000 rods x 6 vertices, 2D, chili's weights for n_sub
    subdomains) in mixed precision against FP64 over its first 200 steps (the unstable rods
    of this input end both runs in a BoundaryError later, at a step that depends on the last
    bits): throughput, the force error on the initial state and the position error after
    one, ten and 200 steps (normwise: max |mixed - f64| / max |f64|)."""
    import numpy as np
    from cellular_raza_gb300 import _native as N
    from cellular_raza_gb300 import engine as E

    w = make_workload("rods_2d", n_sub)
    w.n_steps = 200
    out = {"workload": "rods_2d", "agents": w.n, "steps": w.n_steps, "n_subdomains": n_sub}
    res = {}
    for prec in ("mixed", "f64"):
        m = w.model.replace(precision=prec)
        sim = E.Simulation.single(m, w.n)
        res[(prec, "force")] = sim.forces(w.pos)
        sim.upload(w.pos, w.vel)
        sim.snapshot()
        sim.step(3)  # warm-up (graph instantiation)
        ms = timed_run(torch, sim, w.n_steps)
        out[f"{prec}_agent_steps_per_s"] = w.n * w.n_steps / (ms / 1e3)
        out[f"{prec}_ms_per_step"] = ms / w.n_steps
        res[(prec, w.n_steps)] = sim.download(order="id")["pos"]
        sim.set_option(N.OPT_PROFILE, 1)  # per-phase device times of the same run
        sim.snapshot(restore=True)
        sim.step(w.n_steps)
        p = sim.profile()
        out[f"{prec}_force_stage_ms_per_step"] = p["force_ms"] / w.n_steps
        out[f"{prec}_pair_kernel_ms_per_step"] = p["kernel_ms"] / w.n_steps
        out[f"{prec}_update_ms_per_step"] = p["update_ms"] / w.n_steps
        sim.set_option(N.OPT_PROFILE, 0)
        for k in (1, 10):
            sim.snapshot(restore=True)
            sim.step(k)
            res[(prec, k)] = sim.download(order="id")["pos"]
        sim.close()

    def normwise(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    fa, fb = res[("mixed", "force")], res[("f64", "force")]
    out["force_normwise_rel_err"] = normwise(fa, fb)
    per_rod = (np.linalg.norm((fa - fb).reshape(w.n, -1), axis=1) /
               np.maximum(np.linalg.norm(fb.reshape(w.n, -1), axis=1), 1e-300))
    out["force_per_rod_rel_err_p50"] = float(np.median(per_rod))
    out["force_per_rod_rel_err_p9999"] = float(np.percentile(per_rod, 99.99))
    for k in (1, 10, w.n_steps):
        out[f"pos_normwise_rel_err_{k}_steps"] = normwise(res[("mixed", k)], res[("f64", k)])
        a, b = res[("mixed", k)], res[("f64", k)]
        per_rod = (np.linalg.norm((a - b).reshape(w.n, -1), axis=1) /
                   np.linalg.norm(b.reshape(w.n, -1), axis=1))
        out[f"pos_max_rel_err_per_rod_{k}_steps"] = float(per_rod.max())
    # the same comparison under physical pair weights (every pair weight 1)
    for k in (10, w.n_steps):
        ph = {}
        try:
            for prec in ("mixed", "f64"):
                m = w.model.replace(precision=prec, weight_mode=1)
                ph[prec] = E.run(w.__class__(w.name, m, w.pos, w.vel, k), k)["pos"]
            err = normwise(ph["mixed"], ph["f64"])
        except Exception as e:  # this input can end in a BoundaryError under other weights
            err = f"{type(e).__name__}: {e}"
        out[f"physical_weights_pos_normwise_rel_err_{k}_steps"] = err
    out["speedup_mixed_over_f64"] = out["mixed_agent_steps_per_s"] / out["f64_agent_steps_per_s"]
    return out


def extra_ensemble(torch):
    """1,024 independent 3D Morse simulations (log-uniform sizes, varied strength/damping),
    mixed precision, packed into the same launches (graph-captured step loop, autotuned force
    kernel shape), 500 steps; against sequential plain FP64 runs timed on a stratified
    sample of 24 of the simulations and scaled to all 1,024."""
    import numpy as np
    from cellular_raza_gb300 import engine as E
    from cellular_raza_gb300 import workloads as W

    ws = W.ensemble(seed=2024)
    steps = ws[0].n_steps
    n_total = sum(w.n for w in ws)
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    sim.snapshot()
    tune = sim.autotune(5)
    sim.step(3)
    ms = timed_run(torch, sim, steps)  # restores the snapshot first: ends after `steps`
    final = sim.download(order="id")["pos"]
    sim.close()
    batched = n_total * steps / (ms / 1e3)
    stride = len(ws) // 24
    sample_idx = list(range(0, len(ws), stride))[:24]
    off = np.cumsum([0] + [w.n for w in ws])
    t_seq = 0.0
    errs, errs_norm = [], []
    for s in sample_idx:
        w = ws[s]
        s1 = E.Simulation.single(w.model.replace(precision="f64"), w.n)
        s1.upload(w.pos, w.vel)
        s1.snapshot()
        s1.step(3)
        t_seq += timed_run(torch, s1, steps) / 1e3
        ref = s1.download(order="id")["pos"]
        s1.close()
        mixed = final[off[s]:off[s + 1]]
        dx = np.linalg.norm((mixed - ref).reshape(w.n, -1), axis=1)
        x = np.linalg.norm(ref.reshape(w.n, -1), axis=1)
        errs.append(float((dx / x).max()))
        errs_norm.append(float(dx.max() / x.max()))
    seq_total_s = t_seq * len(ws) / len(sample_idx)
    sequential = n_total * steps / seq_total_s
    return {"workload": "ensemble", "sims": len(ws), "agents": n_total, "steps": steps,
            "precision": "mixed", "autotune": tune, "batched_agent_steps_per_s": batched,
            "batched_ms_per_step": ms / steps,
            "sequential_f64_agent_steps_per_s": sequential,
            "sequential_sample": f"{len(sample_idx)} of {len(ws)} simulations, scaled",
            "speedup": batched / sequential,
            "mixed_vs_f64_error": {
                "definition": "final positions of the batched mixed run against the sampled "
                              "simulations run alone in FP64, after all steps",
                "max_rel_pos_err": max(errs),  # per agent |dx| / |x|, worst simulation
                "max_normwise_rel_pos_err": max(errs_norm),  # max |dx| / max |x|
                "median_sim_max_rel_pos_err": float(np.median(errs))}}


def extra_cycle(n_rods=2000, steps=600):
    """A growing colony of the bacterial-rods agent (cell cycle: neighbour sensing, growth
    limited by the neighbour count, division), 2,000 rods at the density of
    workloads.rod_colony's 150-rod colony, 600 steps.  Cycle handles run one step per launch
    sequence (each step reads its division count back); the wall time around the calls
    covers that.  Agent-steps sum the agent count of every step."""
    import math
    import time

    from cellular_raza_gb300 import engine as E
    from cellular_raza_gb300 import workloads as W

    w = W.rod_colony(n=n_rods, side=300.0 * math.sqrt(n_rods / 150.0), seed=2024,
                     n_subdomains=n_subdomains())
    with E.Simulation.single(w.model, 8 * w.n) as sim:
        sim.upload(w.pos, w.vel)
        sim.set_spring_lengths(w.spring_length)
        agent_steps = 0
        t0 = time.perf_counter()
        for _ in range(steps):
            agent_steps += sim.n_agents
            sim.step(1)
        dt = time.perf_counter() - t0
        n_end = sim.n_agents
    out = {"workload": "rod_colony", "agents_start": w.n, "agents_end": n_end,
           "steps": steps, "dim": w.model.dim, "vertices_per_agent": w.model.n_vertices,
           "agent_steps_per_s": agent_steps / dt, "ms_per_step": dt * 1e3 / steps,
           "timing": "wall clock around the crg_step calls"}
    # the oracle's colony on the host's cores (one chili subdomain per thread), the same run
    try:
        import pyoracle

        pyoracle.build()
        t0 = time.perf_counter()
        res = pyoracle.run_cycle(w.model, w.pos, w.vel, steps, spring_length=w.spring_length)
        cpu_s = time.perf_counter() - t0
        # agent-steps of the oracle's run: its count grows like the GPU's (same final count)
        out["cpu_oracle"] = {"agents_end": int(len(res["ids"])), "seconds": cpu_s,
                             "agent_steps_per_s": agent_steps / cpu_s,
                             "threads": n_subdomains(), **host_cpu(),
                             "note": "wall clock of the oracle's whole run, agent-steps "
                                     "counted on the GPU run"}
    except Exception as e:  # reported, not fatal
        out["cpu_oracle"] = {"error": f"{type(e).__name__}: {e}"}
    return out


def served_stream(n_requests, rate_hz, seed=2024):
    """Poisson stream of simulation requests (N log-uniform [128, 262144], steps uniform
    [100, 2000], 2D/3D and FP64/mixed 50/50) through the request server (continuous batching,
    160 GB admission budget): p50/p99 submit-to-result latency and served agent-steps/s."""
    import numpy as np
    from cellular_raza_gb300 import serve as SV
    from cellular_raza_gb300 import workloads as W

    reqs = W.request_stream(seed=seed, n_requests=n_requests, rate_hz=rate_hz)
    lat = []
    with SV.Server(hbm_budget_bytes=160 << 30, steps_per_tick=32) as srv:
        t0 = time.perf_counter()
        tickets = []
        for r in reqs:
            delay = r.arrival_s - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets.append((r, srv.submit(r.workload)))
        work = 0
        for r, t in tickets:
            res = srv.wait(t)
            lat.append(res["latency_s"])
            work += r.workload.n * r.workload.n_steps
        makespan = time.perf_counter() - t0
    lat = np.array(lat)
    offered = sum(r.workload.n * r.workload.n_steps for r in reqs) / reqs[-1].arrival_s
    return {"rate_hz": rate_hz, "requests": n_requests,
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()),
            "served_agent_steps_per_s": work / makespan,
            "offered_agent_steps_per_s": offered, "makespan_s": makespan}


def sequential_plain(n_requests, sample, seed=2024):
    """The same request stream run one request at a time as plain FP64 simulations (one
    handle each: upload, every step, download), timed on a sample of `sample` requests spread
    evenly over the stream and scaled to all of them."""
    from cellular_raza_gb300 import engine as E
    from cellular_raza_gb300 import workloads as W

    reqs = W.request_stream(seed=seed, n_requests=n_requests, rate_hz=1.0)
    stride = max(1, len(reqs) // sample)
    pick = reqs[::stride][:sample]
    t_sum, work_sum = 0.0, 0
    for r in pick:
        w = r.workload
        t0 = time.perf_counter()
        E.run(W.Workload(w.name, w.model.replace(precision="f64"), w.pos, w.vel, w.n_steps))
        t_sum += time.perf_counter() - t0
        work_sum += w.n * w.n_steps
    total_work = sum(r.workload.n * r.workload.n_steps for r in reqs)
    return {"agent_steps_per_s": work_sum / t_sum,
            "seconds_for_the_stream": t_sum * total_work / work_sum,
            "sample": f"{len(pick)} of {n_requests} requests (every {stride}th), plain FP64, "
                      f"wall clock per request including upload and download, scaled by "
                      f"agent-steps"}


def extra_served(n_requests=1000, rate_hz=40.0):
    """The request stream at one arrival rate, beside sequential plain runs of it."""
    out = served_stream(n_requests, rate_hz)
    seq = sequential_plain(n_requests, 40)
    out["sequential_plain_f64"] = seq
    out["speedup_over_sequential"] = out["served_agent_steps_per_s"] / seq["agent_steps_per_s"]
    out["note"] = (f"{n_requests} requests of the 20,000-request stream at {rate_hz} Hz; "
                   "bench.py --served-sweep runs four rates")
    return out


def served_sweep(args):
    """Four arrival rates x 1,000 requests of the request stream, and the sequential plain
    comparison (one JSON line)."""
    rates = [float(x) for x in args.sweep_rates.split(",")]
    rows = [served_stream(args.sweep_requests, r) for r in rates]
    seq = sequential_plain(args.sweep_requests, 60)
    for row in rows:
        row["speedup_over_sequential"] = row["served_agent_steps_per_s"] / seq["agent_steps_per_s"]
    print(json.dumps({"workload": "request_stream", "sweep": rows,
                      "sequential_plain_f64": seq, "hbm_budget_bytes": 160 << 30,
                      "steps_per_tick": 32}), flush=True)


TILE_SHAPES = [(1, 64, 0), (1, 128, 0), (1, 256, 0), (1, 64, 2), (1, 128, 1), (1, 128, 2),
               (1, 128, 4), (1, 256, 1), (1, 256, 2), (3, 0, 0)]


def tile_sweep(args):
    """Wall time per step of each (variant, block, tile) shape of the mixed sphere force
    kernel: one-shot thread-per-agent grids, the persistent tile kernel and the warp-packed
    kernel (32 graph-captured steps after 32 warm-up steps per shape; the state runs on
    from shape to shape), then what crg_autotune picks."""
    import numpy as np

    from cellular_raza_gb300 import _native as N
    from cellular_raza_gb300 import engine as E
    from cellular_raza_gb300 import workloads as W

    def shapes_on(ws, shapes, steps):
        sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
        sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
                   counts=[w.n for w in ws])
        out = {}
        for v, b, t in shapes:
            sim.set_option(N.OPT_KERNEL_VARIANT, v)
            sim.set_option(N.OPT_BLOCK, b)
            sim.set_option(N.OPT_TILE, t)
            sim.step(steps)
            t0 = time.perf_counter()
            sim.step(steps)
            out[f"variant {v} block {b} tile {t}"] = 1e3 * (time.perf_counter() - t0) / steps
        tune = sim.autotune(5)
        sim.close()
        return {"ms_per_step": out, "autotune": tune}

    ens = W.ensemble(seed=0, precision="mixed", n_steps=500)
    res = {"ensemble_1024_mixed": shapes_on(ens, TILE_SHAPES, 32),
           "spheres_2^23_mixed": shapes_on([W.spheres_3d_large()], TILE_SHAPES, 32)}
    print(json.dumps({"workload": "tile_sweep", **res}), flush=True)


def crg_arm(args):
    rank, world, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    from cellular_raza_gb300 import _native as N
    from cellular_raza_gb300 import engine as E

    n_cpu = n_subdomains()
    w = make_workload(args.workload, n_cpu)
    sim = E.Simulation.single(w.model, w.n)
    sim.upload(w.pos, w.vel)
    sim.snapshot()
    ext = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")

    def barrier():
        if dist is not None:
            dist.barrier()

    def run_once():
        sim.snapshot(restore=True)
        sim.step(w.n_steps)

    for _ in range(max(args.warmup, 3)):
        run_once()
        with torch.cuda.stream(ext):  # the flush kernel's first launch stays out of the timing
            flush.zero_()
    torch.cuda.synchronize()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        ev0.record(ext)
        for k in range(args.steps):
            run_once()
            if k + 1 < args.steps:
                with torch.cuda.stream(ext):
                    flush.zero_()
        ev1.record(ext)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    t_max, agent_steps, value = replica_throughput(dist, ms, w.n * w.n_steps * args.steps)

    # e2e through the C ABI with host buffers (pinned)
    nbytes = w.pos.size * 8
    pin_pos = torch.from_numpy(w.pos.reshape(-1).copy()).pin_memory()
    pin_vel = torch.from_numpy(w.vel.reshape(-1).copy()).pin_memory()
    out_pos = torch.empty(w.pos.size, dtype=torch.float64).pin_memory()
    out_vel = torch.empty(w.pos.size, dtype=torch.float64).pin_memory()
    out_ids = torch.empty(w.n, dtype=torch.int64).pin_memory()
    out_vox = torch.empty(w.n, dtype=torch.int32).pin_memory()
    L = N.load()
    dp = C.POINTER(C.c_double)

    def e2e_once():
        rc = L.crg_upload(sim._h, w.n, None, C.cast(pin_pos.data_ptr(), dp),
                          C.cast(pin_vel.data_ptr(), dp), None)
        N.check(rc, "crg_upload", sim._h)
        sim.step(w.n_steps)
        rc = L.crg_download(sim._h, C.cast(out_pos.data_ptr(), dp),
                            C.cast(out_vel.data_ptr(), dp),
                            C.cast(out_ids.data_ptr(), C.POINTER(C.c_uint64)),
                            C.cast(out_vox.data_ptr(), C.POINTER(C.c_uint32)))
        N.check(rc, "crg_download", sim._h)

    for _ in range(max(args.warmup, 3)):
        e2e_once()
        with torch.cuda.stream(ext):
            flush.zero_()
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for k in range(args.steps):
        e2e_once()
        if k + 1 < args.steps:
            with torch.cuda.stream(ext):
                flush.zero_()
    e1.record(ext)
    torch.cuda.synchronize()
    e2e_ms, _, e2e_value = replica_throughput(dist, e0.elapsed_time(e1),
                                              w.n * w.n_steps * args.steps)
    h2d = 2 * nbytes
    d2h = 2 * nbytes + 8 * w.n + 4 * w.n

    # Per-kernel device time from a profiled pass over the same run: the steps run from the
    # same captured graphs, which then hold event nodes between the phases and around the
    # dominant force kernel and the rod update kernel (CUDA events on the library's stream)
    sim.set_option(N.OPT_PROFILE, 1)
    sim.snapshot(restore=True)
    sim.step(w.n_steps)
    prof = sim.profile()
    sim.set_option(N.OPT_PROFILE, 0)
    prof_steps = w.n_steps
    force_ms = prof["force_ms"] / prof_steps
    sort_ms = prof["sort_ms"] / prof_steps
    kernel_ms = prof["kernel_ms"] / prof_steps
    update_ms = prof["update_ms"] / prof_steps
    # the work those steps did: in-range evaluations averaged over the same steps
    n_inter, n_samples = mean_interactions(sim, w, every=25 if w.n_steps <= 500 else 50)
    flops, kernel_flops = algorithmic_flops(w, n_inter)
    peaks = measured_peaks()
    fma = E.measure_fma_peaks()
    fp64_peak = fma["fp64_tflops"]
    achieved = kernel_flops / (kernel_ms * 1e-3) / 1e12
    if w.model.kind == "rod":
        kernel = "k_rods_passq"
    else:  # FP64 spheres: agent groups up to 38,912 agents, lane per agent above
        kernel = "k_spheres_groups" if w.n <= 38912 else "k_spheres_pass"
    roofline = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak if fp64_peak else None,
                "traffic": committed_traffic(f"{args.workload}_{kernel}"),
                "peak_source": "measured DFMA microbenchmark (crg_measure_fma_peaks) on this GPU",
                "kernel": kernel, "kernel_ms_per_launch": kernel_ms,
                "algorithmic_flop_per_launch": kernel_flops,
                "in_range_evaluations_per_step": n_inter,
                "work_samples": f"{n_samples} states over the {w.n_steps} timed steps",
                "timing": "CUDA event nodes in the captured step graphs, all timed steps",
                "force_stage_ms_per_step": force_ms, "force_stage_flop_per_step": flops,
                "force_stage_tflops": flops / (force_ms * 1e-3) / 1e12,
                "sort_ms_per_step": sort_ms}
    # the sort kernels are HBM-bound.  Algorithmic bytes per agent and step: pos and vel
    # read and written (2 x 2 x 8 x nc), ids read and written (2 x 8), old and new key,
    # count and slot (4 x 4), FP32 offsets written (4 x nc), the 64-bit slot entry written,
    # sorted and read (8 x 3)
    nc = w.model.nc
    sort_bytes = w.n * (2 * 2 * 8 * nc + 2 * 8 + 4 * 4 + 4 * nc + 8 * 3)
    hbm = peaks.get("hbm_gbs")

    def hbm_line(nbytes, ms):
        gbs = nbytes / (ms * 1e-3) / 1e9 if ms > 0 else None
        return {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                "frac": (gbs / hbm) if (hbm and gbs) else None, "bytes_per_step": nbytes,
                "ms_per_step": ms, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}

    roofline_sort = hbm_line(sort_bytes, sort_ms)
    roofline_update = None
    if w.model.kind == "rod" and update_ms > 0:
        # k_rods_update, algorithmic bytes per rod: positions, velocities and the interaction
        # force read, next positions and velocities written (5 x 8 x nc), key and id read and
        # written (2 x (4 + 8))
        roofline_update = hbm_line(w.n * (5 * 8 * nc + 2 * 12), update_ms)
        roofline_update["kernel"] = "k_rods_update"
    gpu_launches = prof["kernels"] // prof_steps * w.n_steps * args.steps if prof_steps else None

    sim.close()
    extras = {}
    if world == 1 and not args.no_extras:
        wanted = set(args.extras.split(","))
        for name, fn in (("rods_mixed", lambda: extra_rods_mixed(torch, n_cpu)),
                         ("mixed_large", lambda: extra_mixed_large(torch)),
                         ("ensemble", lambda: extra_ensemble(torch)),
                         ("served", extra_served),
                         ("cell_cycle", extra_cycle)):
            if name not in wanted:
                continue
            try:
                extras[name] = fn()
            except Exception as e:  # reported, not fatal for the headline line
                extras[name] = {"error": f"{type(e).__name__}: {e}"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_run(w, n_cpu, args.cpu_seconds)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "config": workload_config(w, n_cpu, world),
            "e2e": {"value": e2e_value, "unit": "agent-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": roofline,
            "roofline_sort": roofline_sort,
            "roofline_update": roofline_update,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": gpu_launches,
            "fma_peaks_tflops": fma,
            "rods_mixed": extras.get("rods_mixed"),
            "mixed_large": extras.get("mixed_large"),
            "ensemble": extras.get("ensemble"),
            "served": extras.get("served"),
            "cell_cycle": extras.get("cell_cycle"),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def profile_case(args):
    """The command the ncu captures summarised under profiles/ run: the seeded workload
    (`--case-workload`, default `--workload`) for `--case-steps` steps through the C ABI with
    direct launches, so each kernel of a step is its own launch."""
    from cellular_raza_gb300 import _native as N
    from cellular_raza_gb300 import engine as E
    from cellular_raza_gb300 import workloads as W

    kw = {"n_subdomains": args.case_subdomains}
    if args.case_n:
        kw["n"] = args.case_n
    if args.case_precision:
        kw["precision"] = args.case_precision
    if args.case_side:
        kw["side"] = args.case_side
    w = getattr(W, args.case_workload or args.workload)(seed=2024, **kw)
    cycle = getattr(w.model, "cycle", False)
    with E.Simulation.single(w.model, 16 * w.n if cycle else w.n) as sim:
        sim.set_option(N.OPT_GRAPH_CHUNK, 0)
        sim.set_option(N.OPT_KERNEL_VARIANT, args.case_variant)
        sim.upload(w.pos, w.vel)
        if cycle:
            sim.set_spring_lengths(w.spring_length)
        t = time.perf_counter()
        sim.step(args.case_steps)
        sim.download()
        print(f"{w.name}: {w.n} agents x {args.case_steps} steps in "
              f"{time.perf_counter() - t:.3f} s")


def main():
    args = parse()
    if args.profile_case:
        profile_case(args)
    elif args.served_sweep:
        served_sweep(args)
    elif args.tile_sweep:
        tile_sweep(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        crg_arm(args)


if __name__ == "__main__":
    main()
