#!/usr/bin/env python3
"""Benchmark: SPH pair-interactions/s of one density -> ghost -> force step.

Workload (default): the 384^3 = 56,623,104-particle periodic box drawn from a
strongly clustered density field (lattice displaced by a seeded Gaussian
random field with P(k) ~ k^-2, rms displacement 1.0 of the spacing, density
contrast rms ~5), Minimal SPH with the Wendland C2 kernel, all particles
active -- the largest of the workloads that fits one GPU.  A step is one full
pass -- density loop, the ghost's Newton iterations on h with density
re-runs, force loop -- starting from h0 = eta * spacing, run by the batched
form (one persistent gather launch per loop, CUDA graphs per step).
The same line carries the two targets of the batched and serving forms
(`targets`): the sparse-activity 256^3 Sedov box in the batched and the plain
per-task forms, and the serving loop's boxes/s and p50/p99 latency.

  value   interactions/s with the particle state resident in HBM;
  e2e     the same through the C ABI with host buffers: every step copies the
          inputs from pinned host memory and the 24 result fields back;
  metric  directed pair interactions (H_d + H_f) / t: H_d = pairs with
          r^2 < gamma^2 h_i^2 at the converged h, H_f = pairs with
          r^2 < gamma^2 max(h_i, h_j)^2, over active i.

--impl reference times the CPU restatement of the reference loops
(oracle/sph_oracle.c) on the host cores instead: one independent box per core.
With N > 1 ranks (torchrun) every rank runs its own replica box (the path has
no cross-box exchange), value = all ranks' interactions / max rank time.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_DENSITY = 71   # per directed density hit (hydro_iact.h:137-189 tally)
FLOPS_FORCE = 132    # per directed force hit (hydro_iact.h:378-490 tally)
METRIC = "SPH pair-interactions/s (density+ghost+force step)"
UNIT = "interactions/s"

WORKLOADS = {
    "clustered128": ("clustered", 128, 0.3,
                     "128^3=2,097,152 particles, lattice displaced by a P(k)~k^-2 "
                     "Gaussian random field (rms 0.3 spacing), periodic unit box"),
    "large384": ("clustered", 384, 1.0,
                 "384^3=56,623,104 particles, lattice displaced by a P(k)~k^-2 "
                 "Gaussian random field (rms 1.0 spacing), periodic unit box"),
    "plain32": ("lattice", 32, None,
                "32^3=32,768 particles, jittered lattice (+/-0.1 spacing), "
                "Gaussian velocities sigma 0.05"),
    "sedov256": ("sedov", 256, None,
                 "256^3=16,777,216 particles, jittered lattice, Sedov blast "
                 "(E=1 in the 33 central particles, u=1e-6 elsewhere), 8 time bins"),
    "serve2000": ("serve", 2000, None,
                  "stream of 2,000 independent boxes, N log-uniform in [4,096, 262,144] "
                  "(rounded to n^3), lattice or clustered (coin flip), u uniform in "
                  "[0.5, 2], 10 steps each, Poisson arrivals at 80% of measured capacity"),
    "serve200": ("serve", 200, None, "stream of 200 boxes drawn as serve2000"),
    "sedov64": ("sedov", 64, None,
                "64^3=262,144 particles, jittered lattice, Sedov blast, 8 time bins"),
    "integrate384": ("integrate", 384, None,
                     "time integration kernels (drift, kick2, timestep, kick1) over "
                     "384^3=56,623,104 particles of device-resident state; plus the "
                     "engine sequence on a 128^3 jittered lattice"),
    "sort128": ("sort", 128, 0.3,
                "per-cell 13-axis sort arrays (runner_do_hydro_sort) of every cell of the "
                "128^3=2,097,152-particle clustered box (rms 0.3 spacing): leaves sorted, "
                "split cells merged, deepest first"),
    "rebuild384": ("rebuild", 384, 1.0,
                   "device-resident cell assignment (top-level grid, top cell per particle, "
                   "octree split, depth_h) of 384^3=56,623,104 particles, lattice displaced "
                   "by a P(k)~k^-2 Gaussian random field (rms 1.0 spacing), periodic unit box"),
}

# Algorithmic bytes per particle of the integration kernels (loads + stores
# of the state fields each one touches; time bins 1 B, positions 24 B).
INTEG_BYTES = {
    # x, v_full, v, a, u, u_dt, h, h_dt, rho, v_sig in; x, v, u, h, rho, P, c, v_sig out
    "drift": (24 + 12 + 12 + 12 + 4 * 6) + (24 + 12 + 4 * 6),
    # time_bin, v_full, a, u_dt, u_full, rho, v_sig in; v_full, u_full, v, u, P, c, v_sig out
    "kick2": (1 + 12 + 12 + 4 * 4) + (12 + 4 + 12 + 4 * 4),
    # time_bin, h, v_sig, h_dt, min_ngb_bin in; time_bin out
    "timestep": (1 + 4 + 4 + 4 + 1) + 1,
    # time_bin, v_full, a, u_dt, u_full in; v_full, u_full out
    "kick1": (1 + 12 + 12 + 4 + 4) + (12 + 4),
}


def make_box(name, seed):
    from swift_gb300 import ics
    kind, n, rms, _ = WORKLOADS[name]
    if kind == "clustered":
        return ics.clustered(n, seed=seed, rms=rms)
    if kind == "sedov":
        return ics.sedov(n, seed=seed)
    return ics.lattice(n, seed=seed)


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def sm_count(device=0):
    """Streaming multiprocessors of the GPU (cudaDevAttrMultiProcessorCount)."""
    import torch
    return int(torch.cuda.get_device_properties(device).multi_processor_count)


def fp32_peak_tflops(pk, sms):
    """FP32 issue peak: SMs x 128 FP32 lanes x 2 flop (FMA) x SM clock.
    MEASURED_PEAKS.json carries no FP32 figure; its measured maximum SM clock
    is used, else the nominal 2070 MHz."""
    mhz = float(pk.get("sm_max_mhz", 2070.0))
    return sms * 128 * 2 * mhz * 1e6 / 1e12, mhz


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, gpu_index):
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU leg: the oracle's restatement of the reference loops, one box per core.
# The reference itself cannot run on the GPU host (its tree is not there), so
# the timed CPU path is the restatement built with the reference's stock
# optimisation flags (-O3 -ffast-math -funroll-loops -fomit-frame-pointer and
# the host CPU's own tuning).

# Per workload: the sample the CPU times -- a box of the same generator and
# parameters (same neighbour-count distribution per particle), at the size one
# core finishes in a few seconds.
CPU_SAMPLE = {"large384": "clustered:64:1.0", "clustered128": "clustered:64:0.3"}


def _parse_sample(spec):
    parts = spec.split(":")
    kind, n = parts[0], int(parts[1])
    rms = float(parts[2]) if len(parts) > 2 else 0.3
    return kind, n, rms


def _cpu_box_worker(args):
    spec, seed = args
    sys.path.insert(0, ROOT)
    from swift_gb300 import ics
    from oracle import oracle
    kind, n, rms = _parse_sample(spec)
    box = (ics.clustered(n, seed=seed, rms=rms) if kind == "clustered"
           else ics.lattice(n, seed=seed))
    t0 = time.perf_counter()
    out = oracle.run(box, stock=True)
    dt = time.perf_counter() - t0
    hits = int(out["ngb_final"].sum()) + int(out["ngb_force"].sum())
    return hits, dt, box["x"].shape[0]


def cpu_baseline(spec="clustered:64:1.0", boxes_per_core=1, cores=None):
    """Interactions/s of the reference loops restated in C (oracle, stock
    flags), run as independent boxes on all host cores (spawned workers)."""
    from oracle import oracle
    oracle.build(stock=True)
    cores = cores or os.cpu_count() or 1
    jobs = [(spec, 1000 + k) for k in range(cores * boxes_per_core)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_box_worker, jobs)
    wall = time.perf_counter() - t0
    hits = sum(r[0] for r in res)
    cpu_s = sum(r[1] for r in res)
    # throughput over the loops' own time: all workers run concurrently, the
    # slowest one bounds the sample (process start-up and IC generation are
    # excluded)
    loop_s = max(r[1] for r in res) * boxes_per_core
    kind, n, rms = _parse_sample(spec)
    gen = f"clustered rms {rms:g} spacing" if kind == "clustered" else kind
    return {"value": hits / loop_s, "unit": UNIT, "cores": cores, "kind": "port",
            "build": "oracle/sph_oracle.c with " + " ".join(oracle.stock_flags()),
            "sample": f"{len(jobs)} independent {n}^3 = {res[0][2]:,}-particle boxes of "
                      f"the workload's generator ({gen}), one per worker process; "
                      f"{cpu_s:.1f} s of CPU work, {wall:.1f} s wall"}


# ---------------------------------------------------------------------------

def run_reference_arm(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    t0 = time.perf_counter()
    vals = []
    spec = args.cpu_sample or CPU_SAMPLE.get(args.workload, "clustered:64:1.0")
    for _ in range(max(1, args.steps)):
        cb = cpu_baseline(spec)
        vals.append(cb["value"])
    value = statistics.median(vals)
    wall = time.perf_counter() - t0
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 positions)",
        "data": "synthetic (seeded generators)",
        "config": {"workload": WORKLOADS[args.workload][3],
                   "sample": spec, "parallelism": "replicas"},
        "cpu_baseline": {**cb, "value": value},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    return 0


def traffic_from_profile(kernel, workload, tuning):
    """DRAM bytes per launch of a gather (kernel "density_gather" or
    "force_gather") from the committed ncu summary of this workload: the
    capture made with the same j-block depth and lanes per particle (lines
    "traffic_bytes_per_launch: N (...) — jtile J, threads_per_particle T,
    row_widen W")."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    rw = float(tuning.get("row_widen") or 1.21)
    want = (f"jtile {tuning.get('jtile')}",
            f"threads_per_particle {tuning.get('threads_per_particle', 1)}",
            f"row_widen {rw:g}")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:") and all(w in line for w in want):
                    return float(line.split(":")[1].strip().split()[0])
    except Exception:
        pass
    return None


def sparse_record(workload, steps, warmup, plain_steps, seed):
    """Sparse activity (256^3 Sedov blast, 8 time bins): after one step with
    every particle active (untimed, it gives every particle a density and
    force state), each step activates the bins the power-of-two time-line
    makes active at that step (1-3% of the particles over steps 1-8) and runs
    density -> ghost -> force on them, reading the carried state of their
    inactive neighbours.  A step is timed on the host clock from the
    activation (host planning included) to the end of the force loop, for
    the batched form and for the plain per-task form on the same sequence of
    steps."""
    import numpy as np
    import torch
    from swift_gb300 import api, ics
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    box = make_box(workload, seed=seed + rank)
    n = box["x"].shape[0]
    sp = api.Space(box)
    nb = int(box.get("bin_base", 20))
    seq = [ics.max_active_bin_for_step(k, base=nb) for k in range(1, 1 + warmup + steps)]
    active_frac = {b: float(np.mean(box["time_bin"] <= b)) for b in set(seq)}

    def prime():
        sp.set_active(api.ALL_ACTIVE)
        sp.step()

    def one(b, plain):
        t0 = time.perf_counter()
        sp.set_active(b)
        if plain:
            sp.step_plain()
        else:
            sp.step()
        return time.perf_counter() - t0

    prime()
    for b in seq[:warmup]:
        one(b, False)
    sp.phase_times(reset=True)
    sp.host_times(reset=True)
    sp.step_stats(reset=True)
    sp.plan_times(reset=True)
    clocks = ClockSampler(local_rank)
    t_b, inter = [], []
    graphs = {"graph_steps": 0, "force_replans": 0, "late_rounds": 0, "captures": 0}
    for b in seq[warmup:]:
        t_b.append(one(b, False))
        for k, v in sp.step_stats(reset=True).items():
            graphs[k] += v
        hits = sp.count_hits()  # untimed replay of the same step, instrumented
        inter.append(int(hits[3]) + int(hits[2]))
    clk = clocks.stop()
    phase_ms, nsteps = sp.phase_times(reset=True)
    host_ms = {k: v / max(1, len(t_b)) for k, v in sp.host_times(reset=True).items()}
    dp_ms, dp_steps = sp.plan_times(reset=True)
    # plain form: same state origin, same steps
    prime()
    for b in seq[:min(warmup, 1)]:
        one(b, True)
    t_p = [one(b, True) for b in seq[warmup:][:plain_steps]]
    sp.close()
    ms_b = 1e3 * sum(t_b) / len(t_b)
    ms_p = 1e3 * sum(t_p) / len(t_p)
    ms_p_same = 1e3 * sum(t_b[:len(t_p)]) / len(t_p)
    out = {
        "metric": METRIC, "value": sum(inter) / sum(t_b), "unit": UNIT,
        "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": ms_b, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 positions)",
        "data": "synthetic (seeded generators, no dataset)",
        "config": {"workload": WORKLOADS[workload][3], "particles": n,
                   "form": "batched persistent; steps timed on the host clock "
                           "including host planning",
                   "max_active_bin_per_step": seq[warmup:],
                   "active_fraction": {str(k): v for k, v in sorted(active_frac.items())}},
        "phases_ms_gpu": {"density": phase_ms[0] / max(1, nsteps),
                          "ghost_rounds": phase_ms[1] / max(1, nsteps),
                          "force": phase_ms[2] / max(1, nsteps)},
        "host_ms_per_step": host_ms,
        # gather lists planned inside each step's graph (device time, part of
        # phases_ms_gpu) by the steps that planned on the device
        "device_planning_ms_per_step": dp_ms / max(1, dp_steps),
        "device_planned_steps": dp_steps,
        "batched_ms_per_step": [round(1e3 * t, 3) for t in t_b],
        "plain_ms_per_step": [round(1e3 * t, 3) for t in t_p],
        "plain_over_batched": ms_p / ms_p_same,
        "step_graphs": graphs,
        "interactions_per_step": inter,
        "clocks": clk,
    }
    return out


def run_sparse(args):
    print(json.dumps(sparse_record(args.workload, args.steps, args.warmup, args.plain_steps,
                                   args.seed)), flush=True)


def run_integrate(args):
    """Time integration: (1) the four integration kernels over a 384^3
    device-resident state (inputs far larger than L2), CUDA events per
    kernel on the launching stream, every particle active; (2) the engine
    sequence (drift-all, the space drifted or rebuilt, density -> ghost ->
    force, kick2, timestep, kick1) on a 128^3 lattice, host clock per
    step."""
    import ctypes

    import numpy as np
    import torch
    from swift_gb300 import api, ics
    from swift_gb300.integrate import MAX_NR_TIMESTEPS, Integrator, default_log_max_h_change
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n = (args.integ_side or WORKLOADS[args.workload][1]) ** 3
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed)
    def rnd(*s, dtype=torch.float32):
        return torch.rand(*s, device=dev, generator=g, dtype=dtype)
    t = {"x": rnd(n, 3, dtype=torch.float64), "v_full": rnd(n, 3) - 0.5, "v": rnd(n, 3) - 0.5,
         "a": rnd(n, 3) - 0.5, "u_full": 1 + rnd(n), "u": 1 + rnd(n), "u_dt": rnd(n) - 0.5,
         "h": 0.01 * (1 + rnd(n)), "h_dt": 0.01 * (rnd(n) - 0.5), "rho": 1 + rnd(n),
         "P": torch.ones(n, device=dev), "c": torch.ones(n, device=dev),
         "v_sig": 1 + rnd(n), "time_bin": torch.full((n,), 40, dtype=torch.int8, device=dev),
         "min_ngb_bin": torch.full((n,), 57, dtype=torch.int8, device=dev)}
    st = api.IntegState()
    for k in api.INTEG_FIELDS:
        setattr(st, k, ctypes.c_void_p(t[k].data_ptr()))
    ip = api.IntegParams()
    ip.time_base, ip.dt_min, ip.dt_max = 1.0 / MAX_NR_TIMESTEPS, 0.0, 1e-2
    ip.CFL, ip.log_max_h_change = 0.1, default_log_max_h_change()
    ip.h_min, ip.h_max, ip.minimal_u = 0.0, 3.4e38, 0.0
    ip.dim[:] = [1.0, 1.0, 1.0]
    ip.periodic = 1
    L = api.lib()
    stream = torch.cuda.current_stream(dev)
    sp_ = ctypes.c_void_p(stream.cuda_stream)
    ti = 1 << 42        # bin 40 particles end their steps here: all active
    tmin, bad = ctypes.c_int64(), ctypes.c_int64()
    ops = {
        "drift": lambda: L.sphgpu_integ_drift(ctypes.byref(ip), ctypes.byref(st), n,
                                              ti - (1 << 40), ti, 1, sp_),
        "kick2": lambda: L.sphgpu_integ_kick(ctypes.byref(ip), ctypes.byref(st), n, 2, ti,
                                             56, sp_),
        "timestep": lambda: L.sphgpu_integ_timestep(ctypes.byref(ip), ctypes.byref(st), n,
                                                    ti, 56, ctypes.byref(tmin),
                                                    ctypes.byref(bad), sp_),
        "kick1": lambda: L.sphgpu_integ_kick(ctypes.byref(ip), ctypes.byref(st), n, 1, ti, 56,
                                             sp_),
    }
    for _ in range(args.warmup):
        for f in ops.values():
            api._check(f())
        t["time_bin"].fill_(40)
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    ms = {k: [] for k in ops}
    for _ in range(args.steps):
        for k, f in ops.items():
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            api._check(f())
            e1.record(stream)
            e1.synchronize()
            ms[k].append(e0.elapsed_time(e1))
        t["time_bin"].fill_(40)  # keep every particle active
    torch.cuda.synchronize()
    clk = clocks.stop()
    pk = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))
    kern = {}
    for k, v in ms.items():
        avg = statistics.mean(v) / 1e3
        gbs = INTEG_BYTES[k] * n / avg / 1e9
        kern[k] = {"ms": 1e3 * avg, "bytes_per_particle": INTEG_BYTES[k], "GB_s": gbs,
                   "frac_of_measured_hbm": gbs / hbm}
    total = sum(statistics.mean(v) for v in ms.values()) / 1e3
    # the engine sequence on a 128^3 lattice: device-resident state, the
    # space drifted until the reference's rebuild criterion fires
    del t, st
    torch.cuda.empty_cache()
    side = args.engine_side
    box = ics.lattice(side, seed=args.seed, sigma_v=0.3)
    box["u"][::5] *= 6.0
    t0 = time.perf_counter()
    it = Integrator(box, time_end=1.0, dt_max=0.05).init()
    t_init = time.perf_counter() - t0
    t_eng, act, mabs, rb = [], [], [], []
    for _ in range(args.engine_steps):
        r0 = it.rebuilds
        t0 = time.perf_counter()
        mabs.append(int(it.step()))
        t_eng.append(time.perf_counter() - t0)
        act.append(it.last_active)
        rb.append(it.rebuilds - r0)
    it.close()
    out = {
        "metric": "particle integrations/s (drift + kick2 + timestep + kick1)",
        "value": n / total, "unit": "particles/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 positions)",
        "data": "synthetic (random device state; seeded lattice for the engine sequence)",
        "config": {"workload": WORKLOADS[args.workload][3], "particles": n,
                   "l2": "inputs larger than L2 (state ~100 B/particle)"},
        "kernels": kern,
        "roofline": {"bound": "hbm", "kernel": "drift", "achieved": kern["drift"]["GB_s"],
                     "peak": hbm, "unit": "GB/s", "frac": kern["drift"]["frac_of_measured_hbm"],
                     "traffic": None, "peak_note": "hbm_gbs of MEASURED_PEAKS.json",
                     "limiter": "FP64 pipe (81-85% busy under ncu, DRAM 4-19%): the "
                                "reference's double-precision updates are kept bit-exact"},
        "engine_sequence": {
            "box": f"{side}^3={side ** 3:,} particles, jittered lattice, Gaussian velocities "
                   "sigma 0.3, every fifth particle u x 6 (several time bins)",
            "ms_per_step_host_clock": [round(1e3 * x, 2) for x in t_eng],
            "ms_per_step_mean": round(1e3 * statistics.mean(t_eng), 2),
            "active_particles": act, "max_active_bin": mabs, "rebuilds": rb,
            "init_s": round(t_init, 2),
            "host_copies_of_particle_state": "at rebuilds only (the step's state stays in HBM)"},
        "gpu_launches": 4 * args.steps,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def run_rebuild(args):
    """The rebuild's cell assignment on the device (sphgpu_cell_assign):
    positions and h resident in HBM, host clock around each call (the call
    reads the grid and the tree back, so it is synchronous).  e2e adds the
    upload of x and h from pinned host memory and the download of the order
    and depth_h.  For comparison, the host build of the same box
    (sphgpu_space_create: the same tree plus sort order and gather plans on
    the host cores) is timed once."""
    import numpy as np
    import torch
    from swift_gb300 import api
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    kind, side, rms, desc = WORKLOADS[args.workload]
    from swift_gb300 import ics
    box = ics.clustered(side, seed=args.seed + rank, rms=rms)
    n = box["x"].shape[0]
    xh = torch.from_numpy(np.ascontiguousarray(box["x"])).pin_memory()
    hh = torch.from_numpy(np.ascontiguousarray(box["h"], np.float32)).pin_memory()
    xd, hd = xh.to(dev), hh.to(dev)
    oh = torch.empty(n, dtype=torch.int32).pin_memory()
    dhh = torch.empty(n, dtype=torch.int8).pin_memory()
    for _ in range(args.warmup):
        api.cell_assign(xd, hd, box["dim"])
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    t_dev, t_e2e = [], []
    phases = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        order, dh, cells, cdim = api.cell_assign(xd, hd, box["dim"])
        torch.cuda.synchronize()
        t_dev.append(time.perf_counter() - t0)
        phases.append(api.cell_assign_times())
    for _ in range(args.steps):
        t0 = time.perf_counter()
        xd.copy_(xh, non_blocking=True)
        hd.copy_(hh, non_blocking=True)
        order, dh, cells, cdim = api.cell_assign(xd, hd, box["dim"])
        oh.copy_(order, non_blocking=True)
        dhh.copy_(dh, non_blocking=True)
        torch.cuda.synchronize()
        t_e2e.append(time.perf_counter() - t0)
    clk = clocks.stop()
    t0 = time.perf_counter()
    with api.Space(box) as sp:
        t_host = time.perf_counter() - t0
        same = bool(np.array_equal(sp.tree(), cells))
    # the same host build adopting the device's tree (order copied down)
    t0 = time.perf_counter()
    with api.Space(box, assigned=(oh.numpy(), cells)) as sp:
        t_adopt = time.perf_counter() - t0
    dt, de = statistics.median(t_dev), statistics.median(t_e2e)
    out = {
        "metric": "particles assigned to cells per second (device-resident rebuild)",
        "value": n / dt, "unit": "particles/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 positions, u64 keys",
        "data": "synthetic (seeded clustered box)",
        "config": {"workload": desc, "particles": n, "cdim": list(cdim), "cells": len(cells),
                   "max_depth": int(cells[:, 2].max()),
                   "l2": "inputs larger than L2 (x 24 B + h 4 B per particle)"},
        "e2e": {"value": n / de, "unit": "particles/s", "h2d_bytes_per_step": n * 28,
                "d2h_bytes_per_step": n * 5},
        "phases_ms": {k: statistics.median(p[k] for p in phases) for k in phases[0]
                      if k != "launches"},
        "host_space_create_s": t_host,
        "host_space_create_assigned_s": t_adopt,
        "tree_equals_host_build": same,
        "gpu_launches": int(sum(p["launches"] for p in phases)),
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def serving_record(workload, seed, plain_boxes):
    """Continuous-batching serving loop over a seeded stream of boxes.

    1. capacity: a burst of the first 300 requests, all arriving at t = 0,
       through a fresh server -> boxes/s;
    2. the 2,000-request stream with Poisson arrivals at 80% of that
       capacity -> p50 / p99 latency (arrival to completion) and boxes/s;
    3. the plain per-task form and the single-box batched form on boxes of
       the same stream taken at evenly spaced quantiles of N, one box after
       another (host planning included, as in the server) -> boxes/s."""
    import numpy as np
    import torch
    from swift_gb300 import api, serve
    torch.cuda.set_device(0)
    count = WORKLOADS[workload][1]
    specs = serve.request_stream(count, seed=seed)
    t = time.perf_counter()
    boxes = serve.make_boxes(specs, processes=min(16, os.cpu_count() or 1))
    gen_s = time.perf_counter() - t
    nparts = np.array([b["x"].shape[0] for b in boxes])
    # 1. capacity
    burst = min(300, count)
    with api.Server() as srv:
        lat_b, wall_b, _ = serve.serve(srv, boxes[:burst], np.zeros(burst), serve.STEPS)
        arena = srv.stats()
    capacity = burst / wall_b
    # 2. the stream at 80% of capacity
    rate = 0.8 * capacity
    arr = serve.poisson_arrivals(count, rate, seed=seed)
    clocks = ClockSampler(0)
    with api.Server() as srv:
        lat, wall, _ = serve.serve(srv, boxes, arr, serve.STEPS)
        st = srv.stats()
    clk = clocks.stop()
    thr = count / wall
    summ = serve.latency_summary(lat)
    # 3. one box at a time: plain per-task form and single-box batched form
    # boxes at evenly spaced quantiles of N, so that the sample's mean size
    # is the stream's
    k = min(plain_boxes, count)
    by_n = np.argsort(nparts, kind="stable")
    sample = sorted(int(by_n[int((q + 0.5) * count / k)]) for q in range(k))

    def one_by_one(plain):
        t0 = time.perf_counter()
        for i in sample:
            with api.Space(boxes[i]) as sp:
                for _ in range(serve.STEPS):
                    if plain:
                        sp.step_plain()
                    else:
                        sp.step()
        return len(sample) / (time.perf_counter() - t0)

    plain_bps = one_by_one(True)
    single_bps = one_by_one(False)
    out = {
        "metric": "served boxes/s (10 density+ghost+force steps each)",
        "value": thr, "unit": "boxes/s", "n_gpus": 1, "steps": serve.STEPS,
        "warmup": 0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 positions)",
        "data": "synthetic (seeded request stream)",
        "config": {"workload": WORKLOADS[workload][3], "requests": count,
                   "particles_total": int(nparts.sum()),
                   "particles_mean": float(nparts.mean()),
                   "box_generation_s": gen_s,
                   "arena": arena},
        "capacity_boxes_per_s": capacity,
        "arrival_rate_per_s": rate,
        "latency": summ,
        "server": st,
        "plain_boxes_per_s": plain_bps,
        "single_box_batched_boxes_per_s": single_bps,
        "serve_over_plain": thr / plain_bps,
        "one_by_one_sample": {"boxes": len(sample),
                              "particles_mean": float(nparts[sample].mean())},
        "clocks": clk,
    }
    return out


def run_sort(args):
    """The whole tree's sort arrays (sphgpu_hydro_sort, all 13 axes), CUDA
    events around each call on the launching stream.  Algorithmic bytes: a
    leaf reads its particles' positions once (24 B each) and writes 13
    arrays of count + 1 entries (8 B each); a split cell reads its
    progeny's 13 arrays and writes its own (8 B per entry each way)."""
    import numpy as np
    import torch
    from swift_gb300 import api, ics
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    kind, side, rms, desc = WORKLOADS[args.workload]
    box = ics.clustered(side, seed=args.seed, rms=rms)
    stream = torch.cuda.Stream()
    sh = ctypes_stream(stream)
    import ctypes
    with api.Space(box) as sp:
        tree = sp.tree()
        parent = tree[:, 3]
        split = np.zeros(len(tree), bool)
        split[parent[parent >= 0]] = True
        cnt = tree[:, 1].astype(np.int64)
        nonempty = cnt > 0
        leaf_b = np.sum(24 * cnt[~split & nonempty] + 13 * 8 * (cnt[~split & nonempty] + 1))
        split_b = np.sum(2 * 13 * 8 * (cnt[split & nonempty] + 1))
        algo = int(leaf_b + split_b)
        entries = int(np.sum(13 * (cnt[nonempty] + 1)))
        L = api.lib()
        for _ in range(args.warmup):
            api._check(L.sphgpu_hydro_sort(sp._h, 0x1FFF, sh))
        torch.cuda.synchronize()
        clocks = ClockSampler(local_rank)
        ms = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            api._check(L.sphgpu_hydro_sort(sp._h, 0x1FFF, sh))
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        clk = clocks.stop()
    t = statistics.median(ms) / 1e3
    hbm = float(peaks().get("hbm_gbs", 6800.0))
    gbs = algo / t / 1e9
    out = {
        "metric": "sort entries/s (13 axes, every cell of the tree)", "value": entries / t,
        "unit": "entries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 keys rounded to f32", "data": "synthetic",
        "config": {"workload": desc, "particles": int(box["x"].shape[0]),
                   "cells": int(nonempty.sum()), "split_cells": int((split & nonempty).sum()),
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "sort_leaves + sort_merge", "achieved": gbs,
                     "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                     "algorithmic_bytes": algo, "traffic": None,
                     "peak_note": "hbm_gbs of MEASURED_PEAKS.json",
                     "limiter": "one thread per (cell, axis) runs the reference's sequential "
                                "quicksort / 8-way merge, kept for the reference's tie order"},
        "gpu_launches": None,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def run_serving(args):
    print(json.dumps(serving_record(args.workload, args.seed, args.plain_boxes)), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from swift_gb300 import api

    box = make_box(args.workload, seed=args.seed + rank)
    n = box["x"].shape[0]
    sp = api.Space(box)
    stream = torch.cuda.Stream()
    sh = ctypes_stream(stream)
    # plan (first step), autotune (tile shape x j-block depth), warm-up
    sp.step(stream=sh)
    if args.tuning:
        jt, bw, *tp = (int(v) for v in args.tuning.split(","))
        sp.set_tuning(tpp=tp[0] if tp else 1, jtile=jt, block_warps=bw,
                      bulk_stage=tp[1] if len(tp) > 1 else 0,
                      row_widen=float(args.row_widen), row_cap=int(args.row_cap))
        sp.step(stream=sh)
    if args.no_tune or args.tuning:
        tuning, tune_ms = (dict(zip(("threads_per_particle", "jtile", "rerun_lists",
                                     "block_warps"), sp.tuning())), {})
        tuning["bulk_stage"] = sp.bulk_stage()
        if args.row_widen:
            tuning["row_widen"] = args.row_widen
        if args.row_cap:
            tuning["row_cap"] = args.row_cap
    else:
        tuning, tune_ms = sp.autotune(reps=2)
    for _ in range(args.warmup):
        sp.step(stream=sh)
    hits = sp.count_hits()
    inter_per_step = int(hits[3]) + int(hits[2])
    sp.phase_times(reset=True)
    sp.step_stats(reset=True)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = ClockSampler(local_rank)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        sp.step(stream=sh)
    e1.record(stream)
    barrier()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    phase_ms, nsteps = sp.phase_times(reset=True)
    step_graphs = sp.step_stats(reset=True)

    # End to end through host buffers (pinned), same step.
    pinned = {}
    for k in ("x", "v", "m", "h", "u"):
        t = torch.from_numpy(np.ascontiguousarray(box[k])).pin_memory()
        pinned[k] = t.numpy()
    # two result buffers: a step's results come down while the next computes
    fields = [torch.empty((n, 24), dtype=torch.float32).pin_memory().numpy() for _ in range(2)]
    sp.step_host(pinned, fields[0], stream=sh)
    sp.step_host_async(pinned, fields[1])
    sp.step_host_wait()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        sp.step_host_async(pinned, fields[k % 2])
    sp.step_host_wait()
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps

    t_step = ms_total / 1e3 / args.steps
    if world > 1:
        t_step, e2e_s, total_inter = reduce_over_ranks(t_step, e2e_s,
                                                       inter_per_step, "cuda")
    else:
        total_inter = float(inter_per_step)

    out = None
    sp.close()
    if rank == 0:
        pk = peaks()
        sms = sm_count(local_rank)
        peak, mhz = fp32_peak_tflops(pk, sms)
        force_ms = phase_ms[2] / max(1, nsteps)
        dens_ms = phase_ms[0] / max(1, nsteps)
        ghost_ms = phase_ms[1] / max(1, nsteps)
        step_flops = (FLOPS_DENSITY * float(hits[0] + hits[1])
                      + FLOPS_FORCE * float(hits[2]))
        # Each phase is bracketed by event-record nodes inside the step's
        # graphs (on the stream the kernels run on).  Its algorithmic work:
        # density = 71 flop x first-pass hits; ghost = 71 flop x re-run hits
        # (the per-particle solver from the rows and the catch-up gathers);
        # force = 132 flop x force hits.
        phase = {
            "density": {"ms": dens_ms, "flop": FLOPS_DENSITY * float(hits[0]),
                        "kernel": "gather_lanes<density, records rows> (first density pass)",
                        "profile": "density_gather"},
            "ghost": {"ms": ghost_ms, "flop": FLOPS_DENSITY * float(hits[1]),
                      "kernel": "solve_from_lists + catch-up gathers (ghost re-runs)",
                      "profile": None},
            "force": {"ms": force_ms, "flop": FLOPS_FORCE * float(hits[2]),
                      "kernel": "gather_lanes<force>", "profile": "force_gather"},
        }
        for v in phase.values():
            v["tflops"] = v["flop"] / (v["ms"] / 1e3) / 1e12 if v["ms"] > 0 else 0.0
            v["frac"] = v["tflops"] / peak
        dom = max(phase, key=lambda k: phase[k]["ms"])
        D = phase[dom]
        traffic = (traffic_from_profile(D["profile"], args.workload, tuning)
                   if D["profile"] else None)
        cb = None
        spec = args.cpu_sample or CPU_SAMPLE.get(args.workload, "clustered:64:1.0")
        if not args.no_cpu:
            cb = cpu_baseline(spec)
        targets = None
        if args.workload == "large384" and not args.no_targets and world == 1:
            targets = run_targets(args)
        out = {
            "metric": METRIC, "value": total_inter / t_step, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 positions)",
            "data": "synthetic (seeded generators, no dataset)",
            "config": {
                "workload": WORKLOADS[args.workload][3],
                "particles_per_gpu": n,
                "form": "batched persistent: per step one CUDA graph for density + ghost "
                        "rounds and one for the force",
                "active": "all", "h0": "eta*spacing (ghost iterates every step)",
                "l2": "inputs larger than L2 (particle state ~150 B/particle)",
                "parallelism": "replicas" if world > 1 else "single",
                "interactions_per_step": inter_per_step,
                "tuning": tuning, "autotune_ms_per_step": tune_ms,
                "sms": sms,
                "cpu_sample": spec,
            },
            "phases_ms": {"density": dens_ms, "ghost_rounds": ghost_ms,
                          "force": force_ms},
            "phases_roofline": {k: {"kernel": v["kernel"], "ms": v["ms"],
                                    "tflops": v["tflops"], "frac": v["frac"]}
                                for k, v in phase.items()},
            "hits_per_step": {"density_first": int(hits[0]),
                              "density_reruns": int(hits[1]),
                              "force": int(hits[2])},
            "step_tflops": step_flops / t_step / 1e12,
            "roofline": {
                "bound": "fp32", "kernel": D["kernel"], "phase": dom,
                "achieved": D["tflops"], "peak": peak, "unit": "TFLOP/s",
                "frac": D["frac"],
                "peak_note": f"derived: {sms} SMs x 128 FP32 lanes x 2 x {mhz:.0f} MHz "
                             "(sm_max_mhz of MEASURED_PEAKS.json; no measured FP32 "
                             "figure there)",
                "traffic": traffic,
                "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum per launch "
                                f"from profiles/{D['profile']}_{args.workload}.md"
                                if traffic else None,
            },
            "e2e": {"value": total_inter / e2e_s, "unit": UNIT,
                    "h2d_bytes_per_step": int(n * (24 + 12 + 4 + 4 + 4)),
                    "d2h_bytes_per_step": int(n * 24 * 4)},
            # per step: begin-step, density units + gather, 30 ghost rounds
            # (ghost, units, re-run gather, and the list kernel after the
            # first; gated ones return at once), block h_max, force units +
            # gather
            # per step: begin-step, density (units + gather), 8 ghost rounds in the
            # graph (ghost, units, gather; gated) -- with the lists ghost round 0
            # and the per-particle solver come first and the 8 rounds are
            # catch-up rounds -- force (h_max, units, gather)
            "gpu_launches": (7 + 8 * 3 + (2 if tuning.get("rerun_lists") else 0)) * args.steps,
            # each timed step one CUDA graph (density, ghost rounds, the force
            # plan's check, force); re-plans and late rounds count the rare
            # steps that finished outside it
            "step_graphs": step_graphs,
            "clocks": clk,
            "cpu_baseline": cb,
            "targets": targets,
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_targets(args):
    """The two targets of the batched and serving forms, each bounded to well
    under a minute: (1) the sparse-activity 256^3 Sedov box, batched form
    against the plain per-task form on the same steps; (2) the serving loop
    over the 2,000-box stream (capacity burst, Poisson arrivals at 80 % of it,
    p50/p99 latency), with two boxes timed one by one in the plain and the
    single-box batched forms."""
    out = {}
    try:
        r = sparse_record("sedov256", steps=4, warmup=3, plain_steps=2, seed=args.seed)
        out["batched_over_plain"] = {
            "workload": WORKLOADS["sedov256"][3], "target": ">= 3",
            "value": r["plain_over_batched"],
            "batched_ms_per_step": r["ms_per_step"],
            "plain_ms_per_step": r["plain_ms_per_step"],
            "host_ms_per_step": r["host_ms_per_step"],
            "phases_ms_gpu": r["phases_ms_gpu"],
            "active_fraction": r["config"]["active_fraction"],
            "step_graphs": r["step_graphs"],
            "clocks": r["clocks"]}
    except Exception as e:  # recorded, not fatal to the headline line
        out["batched_over_plain"] = {"error": repr(e)}
    try:
        r = serving_record("serve2000", seed=args.seed, plain_boxes=2)
        out["serving"] = {
            "workload": WORKLOADS["serve2000"][3], "target": ">= 2 x plain",
            "boxes_per_s": r["value"], "latency": r["latency"],
            "capacity_boxes_per_s": r["capacity_boxes_per_s"],
            "serve_over_plain": r["serve_over_plain"],
            "serve_over_single_box_batched": r["value"] / r["single_box_batched_boxes_per_s"],
            "plain_boxes_per_s": r["plain_boxes_per_s"],
            "single_box_batched_boxes_per_s": r["single_box_batched_boxes_per_s"],
            "one_by_one_sample": r["one_by_one_sample"],
            "clocks": r["clocks"]}
    except Exception as e:
        out["serving"] = {"error": repr(e)}
    return out


def reduce_over_ranks(t_step, e2e_s, interactions, device):
    """Replicas: the slowest rank's step times, all ranks' interactions."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([t_step, e2e_s], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(interactions)], device=device, dtype=torch.float64)
    dist.all_reduce(c)
    return float(t[0]), float(t[1]), float(c[0])


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


def main():
    ap = argparse.ArgumentParser(description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="large384")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-sample", default="",
                    help="KIND:SIDE[:RMS] boxes the CPU leg times (default: per workload)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-targets", action="store_true",
                    help="large384: skip the sparse-activity and serving target records")
    ap.add_argument("--plain-boxes", type=int, default=24,
                    help="serving workload: boxes timed one by one per form")
    ap.add_argument("--plain-steps", type=int, default=4,
                    help="sparse workload: steps timed in the plain form")
    ap.add_argument("--row-widen", type=float, default=0.0,
                    help="with --tuning: the first pass's row bound as a multiple of "
                         "(gamma h)^2 (0: the library's default)")
    ap.add_argument("--row-cap", type=int, default=0,
                    help="with --tuning: items per particle row (0: the library's default)")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default gather configuration")
    ap.add_argument("--engine-side", type=int, default=128,
                    help="integrate workload: lattice side of the engine-sequence box")
    ap.add_argument("--engine-steps", type=int, default=12,
                    help="integrate workload: engine steps timed")
    ap.add_argument("--integ-side", type=int, default=0,
                    help="integration workload: particles = side^3 (default 384)")
    ap.add_argument("--tuning", default="",
                    help="JTILE,BLOCK_WARPS[,TPP[,BULK]]: fixed gather configuration, no "
                         "autotune (BULK 1: j-blocks staged by bulk copies)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if WORKLOADS[args.workload][0] == "sedov":
        return run_sparse(args)
    if WORKLOADS[args.workload][0] == "serve":
        return run_serving(args)
    if WORKLOADS[args.workload][0] == "integrate":
        return run_integrate(args)
    if WORKLOADS[args.workload][0] == "rebuild":
        return run_rebuild(args)
    if WORKLOADS[args.workload][0] == "sort":
        return run_sort(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
