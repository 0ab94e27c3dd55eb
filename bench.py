#!/usr/bin/env python3
"""Throughput of the EMT6-Ro batched simulation step on GB300.

Workload (GA-scale uniform batch): 20 seeded disc tumours (radius 6-14 on the
51 x 51 lattice) x 100 random 10-Gy protocols (1-8 doses, 0.25-Gy quanta,
30-min grid in the first 48 h) x 20 replicates = 40,000 simulations, default
parameters, 6-s steps.  One bench step advances every simulation by
--sim-steps steps (default 600 = one simulated hour), continuing from the
previous bench step, so the timed window is steps W*600 .. (W+K)*600 of the
144,000-step (10-day) horizon.  Metric: site-updates/s = simulations x steps
x 2601 interior sites / time.

  value            device time (CUDA events on the batch's stream) of the
                   step kernels, state resident in HBM (7 GB >> 129 MB L2, so
                   every launch streams its state from HBM; no flush needed)
  e2e              the same through the public API (emt6ro.simulation
                   .Experiment): per step add_irradiations (doses of that hour
                   uploaded from the host), run, get_results (counts to host)
  roofline         FP32 algorithmic flops of the step kernels against the
                   device's measured FP32 FMA rate
  full_horizon     a stratified 4,864-simulation subset of the same batch run
                   over all 144,000 steps, per 14,400-step (1-day) window and
                   overall: the early-window value beside the 10-day figure
  ref_cuda_window  this project's kernels on the window the reference arm
                   times the reference's own CUDA kernels on (all 40,000
                   simulations from their initial states, steps 1,800-7,800)
  cpu_baseline     the oracle port of the reference CPU path (timing-only
                   build: -O3, FP contraction, CPU tuning) on all host cores,
                   a stratified 64-simulation sample over the same window,
                   and 16 simulations over the full horizon

--impl reference times that CPU path (all host threads) on the same window
and, where its cubin was built, the reference's own CUDA kernels on all
40,000 simulations over steps 1,800-7,800 ("ref_cuda"; the reference kernels'
fixed buffers were checked to hold this workload for 8,192 steps).
Under torchrun (--gpus N) every rank runs its own 40,000-simulation shard
(weak scaling); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (ROOT / "emt6-ro_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

import numpy as np  # noqa: E402

SITES = 51 * 51
METRIC = "site-updates/s"
FLOP_PER_SITE_SUBSTEP = 33  # 3 fields x 11 flop (9-point stencil + update)
# surrogate training, per row: forward GEMMs 2(128*512 + 2*512*512 + 512),
# input-gradient GEMMs 2(2*512*512), weight-gradient GEMMs 2(512*128 + 2*512*512)
SURROGATE_FLOP_ROW = 2 * (128 * 512 + 2 * 512 * 512 + 512) + 2 * (2 * 512 * 512) + \
    2 * (512 * 128 + 2 * 512 * 512)
BYTES_PER_SITE_SUBSTEP = 24  # 3 fields x (4 B read + 4 B write)
HORIZON = 144_000            # 10 days of 6-s steps
# the reference-CUDA comparison window: 3 untimed then 10 timed 600-step
# bench steps from the initial states (steps 1,800-7,800), inside the 8,192
# steps checked to keep the reference kernels' fixed buffers from overflowing
REF_WINDOW = (3, 10, 600)
FULL_HORIZON_SIMS = 4864
FULL_HORIZON_WINDOW = 14_400  # one simulated day


from emt6ro.ga_model.sharding import shard_range  # noqa: E402  (contiguous shard per rank)


def large_batch(n: int = 4864):
    """Simulations of the ragged-batch tumours with disc radius >= 15: their
    regions outgrow the narrow kernel, so the wide kernel does the work."""
    from emt6ro import workloads as wl
    params = wl.default_parameters()
    tumors, protocols, st, sp, _ = wl.ragged_batch(params, 30_000)
    radii = np.array([np.sqrt((t.sites["state"] == 1).sum() / np.pi) for t in tumors])
    keep = np.nonzero(radii[st] >= 14.5)[0][:n]
    return params, tumors, protocols, st[keep], sp[keep]


def ga_batch(n_reps: int = 20):
    from emt6ro import workloads as wl
    params = wl.default_parameters()
    tumors = wl.ga_tumors(params, 20)
    protocols = wl.ga_protocols(100)
    T, P = len(tumors), len(protocols)
    sim_tumor = np.repeat(np.tile(np.arange(T), P), n_reps).astype(np.int32)
    sim_protocol = np.repeat(np.arange(P), T * n_reps).astype(np.int32)
    return params, tumors, protocols, sim_tumor, sim_protocol


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms in the background."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def _stratified(n_total: int, n: int) -> np.ndarray:
    return np.unique(np.linspace(0, n_total - 1, n).astype(np.int64))


def cpu_sample(params, tumors, protocols, sim_tumor, sim_protocol, steps, warmup, sim_steps,
               n_sample=64, threads=None):
    """The oracle port of the reference CPU path (its timing-only build:
    oracle.build.fast_flags()) on a stratified sample of the workload, over
    the same step window as the GPU: `warmup` untimed then `steps` timed
    bench steps of `sim_steps` steps, all host threads, one simulation per
    thread at a time.  Returns (site-updates/s per timed step, threads, n)."""
    from oracle import pyoracle as po
    from emt6ro import workloads as wl
    threads = threads or os.cpu_count() or 1
    idx = _stratified(len(sim_tumor), n_sample)
    doses = wl.protocol_doses(protocols, 480)
    b = po.Batch(po.params_copy(params.native), len(idx), seed=1, lib=po.oracle_fast())
    for k, i in enumerate(idx):
        b.set(k, tumors[sim_tumor[i]].sites, doses[sim_protocol[i]], sim_index=int(i))
    for _ in range(warmup):
        b.run(sim_steps, nthreads=threads)
    rates = []
    for _ in range(steps):
        t = time.perf_counter()
        b.run(sim_steps, nthreads=threads)
        rates.append(len(idx) * sim_steps * SITES / (time.perf_counter() - t))
    return rates, threads, len(idx)


def cpu_full_horizon(params, tumors, protocols, sim_tumor, sim_protocol, threads=None):
    """The same CPU path on one stratified simulation per host thread over all
    144,000 steps: site-updates/s over the 10-day horizon."""
    from oracle import pyoracle as po
    from emt6ro import workloads as wl
    threads = threads or os.cpu_count() or 1
    idx = _stratified(len(sim_tumor), threads)
    doses = wl.protocol_doses(protocols, 480)
    b = po.Batch(po.params_copy(params.native), len(idx), seed=1, lib=po.oracle_fast())
    for k, i in enumerate(idx):
        b.set(k, tumors[sim_tumor[i]].sites, doses[sim_protocol[i]], sim_index=int(i))
    t = time.perf_counter()
    b.run(HORIZON, nthreads=threads)
    return len(idx) * HORIZON * SITES / (time.perf_counter() - t), len(idx)


def _cpu_kind():
    from oracle import build as ob
    return (f"oracle/emt6_oracle.c restatement of the reference CPU path, timing-only build "
            f"(gcc {' '.join(ob.fast_flags())}), pthreads over all host cores, one simulation "
            "per thread at a time")


def ref_cuda_sample(params, tumors, protocols, sim_tumor, sim_protocol):
    """The reference's own CUDA kernels (compiled from its sources for sm_103a,
    oracle/_ref/emt6ro_ref_sm103a.cubin) on the whole 40,000-simulation batch,
    launched in the order of its Simulation::step and timed with CUDA events
    on its stream over REF_WINDOW (steps 1,800-7,800 from the initial states,
    whatever --steps/--warmup say).  Returns a dict, or None when the cubin
    is absent."""
    from oracle import pyrefgpu
    from emt6ro import workloads as wl
    if not pyrefgpu.available():
        return None
    import torch
    warmup, steps, sim_steps = REF_WINDOW
    doses = wl.protocol_doses(protocols, 480)
    ref = pyrefgpu.RefGpuSimulation(params, tumors, doses, sim_tumor, sim_protocol, seed=1)
    stream = torch.cuda.ExternalStream(ref.stream)
    for _ in range(warmup):
        ref.run(sim_steps)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(stream)
        ref.run(sim_steps)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    counts = ref.counts()
    ref.close()
    n = len(sim_tumor)
    lo, hi = warmup * sim_steps, (warmup + steps) * sim_steps
    return {"value": n * sim_steps * SITES / (ms * 1e-3), "unit": METRIC, "ms_per_step": ms,
            "steps": steps, "warmup": warmup, "sim_steps_per_step": sim_steps,
            "mean_count": float(counts.mean()),
            "kind": "reference CUDA kernels built from its sources (nvcc 13, sm_103a, -O3), "
                    "host loop restating Simulation::step",
            "sample": f"all {n} simulations, steps {lo}-{hi} from the initial states",
            "compare_with": "ref_cuda_window in this project's bench line: its kernels on the "
                            "same simulations, inputs and steps"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    params, tumors, protocols, st, sp = ga_batch()
    ref_cuda = None
    if not args.no_ref_cuda:
        ref_cuda = ref_cuda_sample(params, tumors, protocols, st, sp)
    rates, threads, n = cpu_sample(params, tumors, protocols, st, sp, args.steps, args.warmup,
                                   args.sim_steps)
    v = statistics.median(rates)
    ms = n * args.sim_steps * SITES / v * 1e3
    lo, hi = args.warmup * args.sim_steps, (args.warmup + args.steps) * args.sim_steps
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded disc tumours and protocols)",
        "config": {"workload": "GA batch 20 tumours x 100 protocols x 20 runs, 53x53, 6-s "
                               f"steps {lo:,}-{hi:,} of the {HORIZON:,}-step horizon; CPU "
                               f"sample of {n} simulations",
                   "sim_steps_per_step": args.sim_steps},
        "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{n} of the 40,000 simulations (stratified), steps "
                                   f"{lo:,}-{hi:,}, {args.sim_steps} steps per bench step; "
                                   + _cpu_kind()},
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if ref_cuda is not None:
        line["ref_cuda"] = ref_cuda
    return line


def _e2e(args, params, tumors, protocols, dev, seed, world, dist, bins):
    """The same workload end to end through emt6ro.simulation.Experiment: per
    bench step the doses of that hour uploaded (add_irradiations), run, and the
    living counts read back (get_results).  Returns (value, h2d, d2h bytes)."""
    import torch
    from emt6ro import simulation as sim
    B = 20 * len(tumors) * len(protocols)
    exp = sim.Experiment(params, tumors, 20, len(protocols), gpu_id=dev, seed=seed)
    for w in range(args.warmup):
        exp.add_irradiations(_window(protocols, w, args.sim_steps))
        exp.run(args.sim_steps)
        exp.get_results()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        exp.add_irradiations(_window(protocols, args.warmup + k, args.sim_steps))
        exp.run(args.sim_steps)
        res = exp.get_results()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    value = world * B * args.sim_steps * SITES * args.steps / e2e_s
    h2d = len(protocols) * bins * 4     # dose table upload per add_irradiations
    d2h = int(res.size) * 4             # living counts per get_results
    del exp
    return value, h2d, d2h


def _ours_on_ref_window(params, tumors, protocols, st, sp, dev, seed):
    """This project's kernels on REF_WINDOW: all simulations from their initial
    states, 3 untimed then 10 timed 600-step bench steps (steps 1,800-7,800),
    CUDA events on the batch's stream."""
    import torch
    from emt6ro.batch import Batch
    warmup, steps, sim_steps = REF_WINDOW
    b = Batch(params, tumors, protocols, st, sp, device=dev, seed=seed)
    b.set_schedule(0, sim_steps)
    stream = torch.cuda.ExternalStream(b.stream())
    for _ in range(warmup):
        b.run(sim_steps)
    b.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(stream)
        b.run(sim_steps)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    b.sync()
    ms = sum(a.elapsed_time(e) for a, e in ev) / steps
    lo, hi = warmup * sim_steps, (warmup + steps) * sim_steps
    return {"value": len(st) * sim_steps * SITES / (ms * 1e-3), "unit": METRIC,
            "ms_per_step": ms, "mean_count": float(b.counts().mean()),
            "sample": f"all {len(st)} simulations, steps {lo}-{hi} from the initial states",
            "compare_with": "ref_cuda in the --impl reference line (the reference's own CUDA "
                            "kernels on the same simulations, inputs and steps)"}


def _full_horizon(params, tumors, protocols, st, sp, dev, seed):
    """A stratified FULL_HORIZON_SIMS-simulation subset of the batch over all
    144,000 steps: site-updates/s per one-day window and over the horizon
    (CUDA events on the batch's stream)."""
    import torch
    from emt6ro.batch import Batch
    idx = _stratified(len(st), FULL_HORIZON_SIMS)
    b = Batch(params, tumors, protocols, st[idx], sp[idx], device=dev, seed=seed)
    b.set_schedule(0, 1200)
    stream = torch.cuda.ExternalStream(b.stream())
    nwin = HORIZON // FULL_HORIZON_WINDOW
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(nwin + 1)]
    diffused = [b.diffused()]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for k in range(nwin):
        b.run(FULL_HORIZON_WINDOW)
        ev[k + 1].record(stream)
        diffused.append(b.diffused())  # waits for the window (outside its events)
    torch.cuda.synchronize()
    b.sync()
    win_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(nwin)]
    n = len(idx)
    per_win = [n * FULL_HORIZON_WINDOW * SITES / (ms * 1e-3) for ms in win_ms]
    per_win_tf = [(diffused[k + 1] - diffused[k]) * FLOP_PER_SITE_SUBSTEP / (ms * 1e-3) / 1e12
                  for k, ms in enumerate(win_ms)]
    flops = (diffused[-1] - diffused[0]) * FLOP_PER_SITE_SUBSTEP
    return {"value": n * HORIZON * SITES / (sum(win_ms) * 1e-3), "unit": METRIC,
            "fp32_tflops": flops / (sum(win_ms) * 1e-3) / 1e12,
            "seconds": sum(win_ms) * 1e-3, "per_day": per_win, "per_day_fp32_tflops": per_win_tf,
            "mean_count_day10": float(b.counts().mean()),
            "sample": f"{n} of the {len(st)} simulations (stratified), steps 0-{HORIZON}, "
                      "1200-step launches"}


def run_ours(args, rank, world, dist):
    import ctypes
    import torch
    from emt6ro import _native as N
    from emt6ro.batch import Batch

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    params, tumors, protocols, st, sp = large_batch() if args.workload == "large" else ga_batch()
    if args.sims:
        # a stratified subset of the batch (profiling captures of a small case)
        keep = np.unique(np.linspace(0, len(st) - 1, args.sims).astype(np.int64))
        st, sp = st[keep], sp[keep]
    B = len(st)
    seed = 0xE6E6 + rank

    # ---- device-resident run -------------------------------------------------
    b = Batch(params, tumors, protocols, st, sp, device=dev, seed=seed)
    b.set_schedule(0, args.sim_steps)
    stream = torch.cuda.ExternalStream(b.stream())
    for _ in range(args.warmup):
        b.run(args.sim_steps)
    b.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    d0, l0 = b.diffused(), b.launches()
    clocks = ClockSampler(dev)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        ev[k][0].record(stream)
        b.run(args.sim_steps)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clocks.stop()
    b.sync()
    times = [s.elapsed_time(e) for s, e in ev]
    total_ms = sum(times)
    diffused = b.diffused() - d0
    launches = b.launches() - l0
    mean_count = float(b.counts().mean())
    if dist:
        t = torch.tensor([total_ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * B * args.sim_steps * SITES / (ms_per_step * 1e-3)

    # ---- end to end through the public API -----------------------------------
    bins = (144_000 + 299) // 300
    e2e_value = None
    h2d = d2h = 0
    if not args.no_e2e and not args.sims and args.workload == "ga":
        e2e_value, h2d, d2h = _e2e(args, params, tumors, protocols, dev, seed, world, dist, bins)

    # ---- the reference-CUDA window and the 10-day horizon (one GPU only) -----
    extras = args.workload == "ga" and not args.sims and world == 1 and not args.no_extras
    ref_window = _ours_on_ref_window(params, tumors, protocols, st, sp, dev, seed + 1) \
        if extras else None
    full = _full_horizon(params, tumors, protocols, st, sp, dev, seed + 2) if extras else None

    # ---- roofline of the dominant kernel -------------------------------------
    peak = ctypes.c_double()
    N.check(N.lib().emt6_probe_fp32_peak(dev, ctypes.byref(peak)))
    # the two step kernels of a bench step together (the narrow one is 96-98% of
    # it, the launch-order kernels 0.01%): the diffused counter covers both
    kernel_ms = ms_per_step
    achieved = diffused / args.steps * FLOP_PER_SITE_SUBSTEP / (kernel_ms * 1e-3) / 1e12
    profiles = ROOT / "profiles" / "traffic.json"
    traffic = None
    if profiles.exists() and args.workload == "ga":
        try:
            cap = json.loads(profiles.read_text())["captured"]
            # per launch each simulation's state is read and written once
            traffic = (cap["dram_read_bytes"] + cap["dram_write_bytes"]) / cap["simulations"] * B
        except (ValueError, KeyError, ZeroDivisionError):
            traffic = None
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
            "frac": achieved / peak.value if peak.value else None, "traffic": traffic,
            "peak_source": "measured FP32 FMA rate of this GPU (emt6_probe_fp32_peak); "
                           "MEASURED_PEAKS.json has no FP32 figure",
            "algorithmic": f"{FLOP_PER_SITE_SUBSTEP} flop per diffused site-substep x "
                           f"{diffused // args.steps} site-substeps per bench step"}
    hbm_peak = _measured_hbm()
    state_bytes = B * (3 * 2809 * 4 + 2809 + 2 * 2857) * 2
    roof_hbm = {"bound": "hbm", "achieved": state_bytes / (kernel_ms * 1e-3) / 1e9,
                "peak": hbm_peak, "unit": "GB/s",
                "frac": state_bytes / (kernel_ms * 1e-3) / 1e9 / hbm_peak if hbm_peak else None,
                "traffic": traffic,
                "note": "resident design: each launch loads and stores each simulation's "
                        "lattice once; per-step stencil traffic stays in registers/shared "
                        f"memory ({BYTES_PER_SITE_SUBSTEP} B per site-substep on chip)"}
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded disc tumours and protocols, default parameters)",
        "config": {"workload": ("GA batch: 20 tumours x 100 protocols x 20 runs = 40,000 "
                                "simulations per GPU, 53x53 lattice, 6-s steps "
                                f"{args.warmup * args.sim_steps:,}-"
                                f"{(args.warmup + args.steps) * args.sim_steps:,} of the "
                                f"{HORIZON:,}-step horizon")
                               if args.workload == "ga" else
                               (f"large tumours: {B} simulations of the ragged batch's disc "
                                "radius >= 15 tumours (wide kernel), 53x53 lattice, 6-s steps"),
                   "sim_steps_per_step": args.sim_steps, "simulations_per_gpu": B,
                   "l2": f"state {B * 176e3 / 1e9:.1f} GB per GPU (> 129 MB L2); no flush "
                         "needed",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "roofline": roof,
        "roofline_hbm": roof_hbm,
        "diffused_site_substeps_per_step": diffused // args.steps,
        "mean_count": mean_count,
        "ref_cuda_window": ref_window,
        "full_horizon": full,
    }


def run_ragged(args):
    """Ragged batch: 30,000 simulations, disc radius 2-20, 0-12 doses, horizons
    {72k, 144k, 288k} steps (5, 10, 20 days) mixed uniformly, scaled by
    --horizon-scale; launch schedule chosen by the autotuner; reports the
    makespan (tail latency of the slowest simulation) and site-updates/s."""
    import torch
    from emt6ro import workloads as wl, autotune
    from emt6ro.batch import Batch
    params = wl.default_parameters()
    tumors, prots, st, sp, hz = wl.ragged_batch(params, 30_000)
    hz = np.maximum((hz.astype(np.float64) * args.horizon_scale).astype(np.uint32), 1)
    t0 = time.perf_counter()
    mode, chunk, lay, table = autotune.tune(params, tumors, prots, st, sp, hz, sample=2432,
                                            trial_steps=min(600, int(hz.min())))
    tune_s = time.perf_counter() - t0
    b = Batch(params, tumors, prots, st, sp, sim_horizon=hz, seed=0xC0FFEE)
    b.set_schedule(mode, chunk)
    b.set_layouts(lay)
    stream = torch.cuda.ExternalStream(b.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    e0.record(stream)
    b.run(int(hz.max()))
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.stop()
    b.sync()
    ms = e0.elapsed_time(e1)
    work = float(hz.astype(np.float64).sum()) * SITES
    steps_done = [b.step(i) for i in range(0, len(st), 997)]
    assert all(s == int(hz[i]) for s, i in zip(steps_done, range(0, len(st), 997)))
    return {
        "metric": METRIC, "value": work / (ms * 1e-3), "unit": METRIC, "n_gpus": 1,
        "steps": 1, "warmup": 0, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ragged batch)",
        "config": {"workload": "ragged batch: 30,000 simulations, disc radius 2-20, 0-12 doses, "
                               "horizons 5/10/20 days mixed",
                   "horizon_scale": args.horizon_scale,
                   "horizons_steps": sorted({int(x) for x in np.unique(hz)}),
                   "schedule_mode": mode, "steps_per_launch": chunk, "tile_shapes": lay},
        "tail_latency_s": ms * 1e-3,
        "autotune": {"seconds": tune_s,
                     "table": [[m, c, y, round(t, 4)] for m, c, y, t in table],
                     "columns": ["schedule mode", "steps per launch", "tile shapes", "seconds"]},
        "clocks": clocks.summary(), "gpu_launches": b.launches(),
    }


def _spearman(a, b):
    ra = np.argsort(np.argsort(a)).astype(np.float64)
    rb = np.argsort(np.argsort(b)).astype(np.float64)
    return float(np.corrcoef(ra, rb)[0, 1])


def run_surrogate(args):
    """Surrogate training on simulator output and one surrogate-screened GA
    generation.

    1. Training data: --train-pairs distinct GA protocols (1-8 doses, 10 Gy,
       0.25-Gy quanta, 30-min grid in the first 48 h), each paired with one
       of the 20 GA tumours at random, target the final living-cell count of
       --train-reps simulations of --horizon steps (default 144,000 = 10
       days).  5% of the pairs are held out for the reported error, 5% of the
       rest select the best epoch.
    2. Training: an ensemble of --ensemble surrogates (Adam, batch 4096, on
       the GPU by the library's tcgen05 BF16 kernels); the training step is
       also timed alone with CUDA events.
    3. GA generation: --population protocols x 20 tumours scored by the
       surrogate; the best --elite-frac re-simulated with --elite-sims
       simulations each (20 tumours x runs).
    4. Plain scoring, measured: --plain-sample protocols drawn at random
       from the population, each simulated like an elite (same simulations,
       same horizon); plain protocols/s = sample / its simulation time.  The
       same sample gives the surrogate's per-protocol error on random
       protocols.
    The screened rate is reported per generation once the surrogate exists,
    and amortised with the one-off training-data simulation and training
    over 1, 10 and 100 generations.
    """
    import torch
    from emt6ro import surrogate as S, workloads as wl
    from emt6ro.batch import Batch
    params = wl.default_parameters()
    tumors = wl.ga_tumors(params, 20)
    T = len(tumors)
    horizon = args.horizon
    clocks = ClockSampler(0)
    clocks.start()
    # 1. training data
    P = args.train_pairs
    protocols = wl.ga_protocols(P, seed=2024)
    pp = np.arange(P)
    pt = np.random.default_rng(2025).integers(0, T, P)
    t0 = time.perf_counter()
    y = S.simulate_means(params, tumors, protocols, pp, pt, args.train_reps, horizon, seed=11)
    data_s = time.perf_counter() - t0
    x = S.features(protocols, tumors, pp, pt)
    train = np.random.default_rng(2026).random(P) >= 0.05
    # 2. training: an ensemble of --ensemble members
    ens = S.SurrogateEnsemble(k=args.ensemble, max_batch=4096, seed=0)
    t0 = time.perf_counter()
    ens.fit(x[train], y[train], epochs=args.epochs, lr=args.lr, batch=4096, val_frac=0.05)
    fit_s = time.perf_counter() - t0
    net = ens.nets[0]
    pred_held = ens.predict(x[~train])
    pred_single = net.predict(x[~train])
    err = pred_held - y[~train]
    held = {"rmse_cells": float(np.sqrt(np.mean(err ** 2))),
            "rmse_over_mean": float(np.sqrt(np.mean(err ** 2)) / np.mean(y[~train])),
            "r2": float(1 - np.mean(err ** 2) / np.var(y[~train])),
            "r2_single_member": float(1 - np.mean((pred_single - y[~train]) ** 2) /
                                      np.var(y[~train])),
            "pairs": int((~train).sum())}
    # training-step throughput on one resident batch (CUDA events on the
    # surrogate's stream)
    xs = net._norm_x(x[train][:4096] if train.sum() >= 4096 else np.resize(x[train], (4096, 100)))
    ts = np.zeros(4096, np.float32)
    stream = net._stream()
    xd, td = net._to_dev(xs), net._to_dev(ts)
    from emt6ro import _native as Nat
    L = Nat.lib()
    for _ in range(5):
        Nat.check(L.emt6_mlp_train_step(net._h, xd.data_ptr(), td.data_ptr(), 4096, 0.0, None))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 50
    e0.record(stream)
    for _ in range(reps):
        Nat.check(L.emt6_mlp_train_step(net._h, xd.data_ptr(), td.data_ptr(), 4096, 0.0, None))
    e1.record(stream)
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / reps
    flop_row = SURROGATE_FLOP_ROW
    tflops = flop_row * 4096 / (step_ms * 1e-3) / 1e12
    bf16_peak = _measured_bf16()
    # 3. screened GA generation
    pop = wl.ga_protocols(args.population, seed=99)
    keep = max(1, int(round(args.elite_frac * len(pop))))
    runs = max(1, args.elite_sims // T)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    elite, pred = S.prescreen(ens, pop, tumors, keep)
    score_s = time.perf_counter() - t0
    st = np.tile(np.repeat(np.arange(T, dtype=np.int32), runs), keep)
    sp = np.repeat(np.arange(keep, dtype=np.int32), T * runs)
    elite_prots = [pop[i] for i in elite]
    t0 = time.perf_counter()
    counts = np.zeros(len(st), np.float64)
    chunk = 40_000 // (T * runs) * (T * runs)
    for lo in range(0, len(st), chunk):
        hi = min(len(st), lo + chunk)
        b = Batch(params, tumors, elite_prots, st[lo:hi], sp[lo:hi], seed=31 + lo)
        b.run(horizon)
        counts[lo:hi] = b.counts()
        del b
    sim_s = time.perf_counter() - t0
    # 4. plain scoring of a random sample of the population, measured
    nplain = max(1, min(args.plain_sample, len(pop)))
    sample = np.sort(np.random.default_rng(7).choice(len(pop), nplain, replace=False))
    st_p = np.tile(np.repeat(np.arange(T, dtype=np.int32), runs), nplain)
    sp_p = np.repeat(np.arange(nplain, dtype=np.int32), T * runs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    counts_p = np.zeros(len(st_p), np.float64)
    for lo in range(0, len(st_p), chunk):
        hi = min(len(st_p), lo + chunk)
        b = Batch(params, tumors, [pop[i] for i in sample], st_p[lo:hi], sp_p[lo:hi],
                  seed=77 + lo)
        b.run(horizon)
        counts_p[lo:hi] = b.counts()
        del b
    plain_s = time.perf_counter() - t0
    clocks.stop()
    plain_mean = counts_p.reshape(nplain, T * runs).mean(1)
    plain_rel = np.abs(pred[sample] - plain_mean) / plain_mean
    sim_mean = counts.reshape(keep, T * runs).mean(1)
    pe = pred[elite]
    plain_rate = nplain / plain_s
    screened_rate = len(pop) / (score_s + sim_s)
    elite_rel = np.abs(pe - sim_mean) / sim_mean
    one_off = data_s + fit_s

    def amortised(gens):
        return gens * len(pop) / (one_off + gens * (score_s + sim_s))
    return {
        "metric": "GA protocols scored/s", "value": screened_rate,
        "unit": "protocols/s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": (score_s + sim_s) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (surrogate), f32 (simulation)",
        "data": "synthetic (seeded GA tumours and protocols); surrogate trained on simulator "
                "output only",
        "config": {"workload": f"surrogate-screened GA generation: {len(pop)} protocols x {T} "
                               f"tumours, top {keep} re-simulated with {T * runs} simulations "
                               f"each, {horizon}-step horizon",
                   "train_pairs": int(train.sum()), "train_reps": args.train_reps,
                   "ensemble": args.ensemble,
                   "best_epochs": [int(np.argmin(m.val_history)) for m in ens.nets],
                   "epochs": args.epochs, "batch": 4096},
        "plain_protocols_per_s": plain_rate, "speedup_vs_plain": screened_rate / plain_rate,
        "plain": {"measured": True, "protocols": nplain, "simulations_each": T * runs,
                  "seconds": plain_s, "protocols_per_s": plain_rate,
                  "surrogate_mean_rel_error": float(plain_rel.mean()),
                  "surrogate_within_5pct": float((plain_rel <= 0.05).mean()),
                  "spearman": _spearman(pred[sample], plain_mean)},
        "amortised": {"one_off_s": one_off,
                      "protocols_per_s": {str(g): amortised(g) for g in (1, 10, 100)},
                      "speedup_vs_plain": {str(g): amortised(g) / plain_rate
                                           for g in (1, 10, 100)}},
        "elites": {"spearman": _spearman(pe, sim_mean),
                   "mean_rel_error": float(elite_rel.mean()),
                   "max_rel_error": float(elite_rel.max()),
                   "within_5pct": float((elite_rel <= 0.05).mean()),
                   "rel_error_of_mean": float(abs(pe.mean() - sim_mean.mean()) / sim_mean.mean()),
                   "target_rel_error": 0.05,
                   "mean_target_met": bool(abs(pe.mean() - sim_mean.mean()) / sim_mean.mean()
                                           <= 0.05),
                   "per_protocol_target_met": bool(elite_rel.mean() <= 0.05),
                   "simulated_mean": float(sim_mean.mean()), "predicted_mean": float(pe.mean())},
        "held_out": held,
        "timings_s": {"training_data": data_s, "fit": fit_s, "surrogate_scoring": score_s,
                      "elite_simulation": sim_s, "plain_sample_simulation": plain_s},
        "train_step": {"ms": step_ms, "tflops": tflops,
                       "roofline": {"bound": "tensor", "achieved": tflops, "peak": bf16_peak,
                                    "unit": "TFLOP/s", "frac": tflops / bf16_peak,
                                    "traffic": None,
                                    "algorithmic": f"{flop_row} flop per row x 4096 rows "
                                                   "(forward, input-gradient and weight-"
                                                   "gradient GEMMs)"}},
        "clocks": clocks.summary(),
    }


def run_surrogate_train(args):
    """The surrogate's training step alone: Adam steps at batch 4096 on one
    resident batch of standardised synthetic rows, timed with CUDA events on
    the surrogate's stream; reports TFLOP/s against the measured BF16 peak."""
    import torch
    from emt6ro import _native as Nat
    from emt6ro.surrogate import Surrogate, N_FEATURES
    net = Surrogate(max_batch=4096, seed=0)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(4096, N_FEATURES)).astype(np.float32)
    t = rng.normal(size=4096).astype(np.float32)
    xd, td = net._to_dev(x), net._to_dev(t)
    L = Nat.lib()
    stream = net._stream()
    for _ in range(args.warmup):
        Nat.check(L.emt6_mlp_train_step(net._h, xd.data_ptr(), td.data_ptr(), 4096, 1e-4, None))
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        ev[k][0].record(stream)
        Nat.check(L.emt6_mlp_train_step(net._h, xd.data_ptr(), td.data_ptr(), 4096, 1e-4, None))
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    Nat.check(L.emt6_mlp_sync(net._h))
    ms = statistics.median(a.elapsed_time(b) for a, b in ev)
    tflops = SURROGATE_FLOP_ROW * 4096 / (ms * 1e-3) / 1e12
    peak = _measured_bf16()
    return {"metric": "surrogate training steps/s", "value": 1e3 / ms, "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic standardised rows",
            "config": {"workload": "surrogate MLP 100-512-512-512-1 training step, batch 4096"},
            "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": tflops / peak, "traffic": None,
                         "algorithmic": f"{SURROGATE_FLOP_ROW} flop per row x 4096 rows"}}


def _measured_bf16():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["bf16_tflops"])
        except (ValueError, KeyError):
            pass
    return 1900.0


def _window(protocols, k, sim_steps):
    """The (step, dose) pairs of each protocol falling in bench step k."""
    lo, hi = k * sim_steps, (k + 1) * sim_steps
    return [[(t, d) for t, d in prot if lo <= t < hi] for prot in protocols]


def _measured_hbm():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"])
        except (ValueError, KeyError):
            pass
    return 6800.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--sim-steps", type=int, default=600)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end API timing")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the reference-CUDA window and the 10-day horizon figures")
    ap.add_argument("--sims", type=int, default=0,
                    help="time a stratified subset of this many simulations (small "
                         "profiling case; implies --no-e2e)")
    ap.add_argument("--no-ref-cuda", action="store_true",
                    help="--impl reference: skip timing the reference's CUDA kernels")
    ap.add_argument("--workload", choices=["ga", "large", "ragged", "surrogate", "surrogate-train"],
                    default="ga",
                    help="ga: 40,000-simulation GA batch (default, the headline); "
                         "large: 4,864 simulations of radius >= 15 tumours (wide kernel); "
                         "ragged: 30,000 simulations with mixed sizes and horizons; "
                         "surrogate: surrogate training + a screened GA generation")
    ap.add_argument("--horizon", type=int, default=144_000,
                    help="surrogate: simulated steps per simulation")
    ap.add_argument("--train-pairs", type=int, default=96_000)
    ap.add_argument("--train-reps", type=int, default=1)
    ap.add_argument("--epochs", type=int, default=100)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--ensemble", type=int, default=5,
                    help="surrogate: members averaged for pre-screening")
    ap.add_argument("--population", type=int, default=10_000)
    ap.add_argument("--elite-frac", type=float, default=0.05)
    ap.add_argument("--elite-sims", type=int, default=100)
    ap.add_argument("--plain-sample", type=int, default=50,
                    help="surrogate: protocols simulated in full to measure plain scoring")
    ap.add_argument("--horizon-scale", type=float, default=1.0,
                    help="ragged: multiply the 72k/144k/288k-step horizons")
    args = ap.parse_args()
    if args.workload == "surrogate-train":
        print(json.dumps(run_surrogate_train(args)), flush=True)
        return
    if args.workload == "surrogate":
        print(json.dumps(run_surrogate(args)), flush=True)
        return
    if args.workload == "ragged":
        print(json.dumps(run_ragged(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        backend = "nccl" if args.impl == "ours" else "gloo"
        tdist.init_process_group(backend)
        dist = tdist
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_ours(args, rank, world, dist)
        if rank == 0 and not args.no_cpu_baseline:
            params, tumors, protocols, st, sp = (large_batch() if args.workload == "large"
                                                 else ga_batch())
            rates, threads, n = cpu_sample(params, tumors, protocols, st, sp, args.steps,
                                           args.warmup, args.sim_steps)
            lo, hi = args.warmup * args.sim_steps, (args.warmup + args.steps) * args.sim_steps
            line["cpu_baseline"] = {
                "value": statistics.median(rates), "unit": METRIC, "cores": threads,
                "kind": "port",
                "sample": f"{n} of the {len(st):,} simulations (stratified), steps "
                          f"{lo:,}-{hi:,} (the GPU's window); " + _cpu_kind()}
            if line.get("full_horizon"):
                v, nf = cpu_full_horizon(params, tumors, protocols, st, sp, threads)
                line["cpu_baseline"]["full_horizon"] = {
                    "value": v, "unit": METRIC,
                    "sample": f"{nf} simulations (stratified), steps 0-{HORIZON:,}"}
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
