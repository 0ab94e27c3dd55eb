"""Launch autotuner for the batch engine.

A CTA holds one simulation's lattice in shared memory, and the kernels pick
the register tiling (warps per field, rows per warp, one or two columns per
lane) per region themselves.  What is left to tune per workload is how the
step loop is launched: steps per launch (longer launches amortise the
per-launch load/store of every lattice; shorter ones let simulations that
finish or outgrow the narrow kernel be rescheduled sooner), the schedule (one
CTA per simulation vs persistent CTAs over a device work queue ordered by
horizon) and CUDA-graph replay of the launch sequence.  The tuner times each
candidate on a stratified sample of the batch, from identical initial states,
and returns the fastest.
"""
from __future__ import annotations

import itertools
import time

import numpy as np

from .batch import Batch

DEFAULT_CHUNKS = (300, 600, 1200, 2400)
DEFAULT_MODES = (0, 1, 2, 3)  # bit 0: work queue, bit 1: CUDA graph

_cache: dict = {}


def _sample(n: int, k: int) -> np.ndarray:
    return np.unique(np.linspace(0, n - 1, min(n, k)).astype(np.int64))


def tune(params, tumors, protocols, sim_tumor, sim_protocol, sim_horizon=None, *, device=0,
         sample=2432, trial_steps=600, warm_steps=64, chunks=DEFAULT_CHUNKS, modes=DEFAULT_MODES,
         seed=1, key=None):
    """Returns (mode, steps_per_launch, table) with table = [(mode, chunk, seconds)]."""
    if key is not None and key in _cache:
        return _cache[key]
    idx = _sample(len(sim_tumor), sample)
    st = np.asarray(sim_tumor)[idx]
    sp = np.asarray(sim_protocol)[idx]
    hz = None if sim_horizon is None else np.asarray(sim_horizon)[idx]
    table = []
    for mode, chunk in itertools.product(modes, chunks):
        b = Batch(params, tumors, protocols, st, sp, sim_horizon=hz, device=device, seed=seed)
        b.set_schedule(mode, min(chunk, warm_steps))
        b.run(warm_steps)
        b.sync()
        b.set_schedule(mode, chunk)
        t0 = time.perf_counter()
        b.run(trial_steps)
        b.sync()
        table.append((mode, chunk, time.perf_counter() - t0))
        del b
    mode, chunk, _ = min(table, key=lambda r: r[2])
    res = (mode, chunk, table)
    if key is not None:
        _cache[key] = res
    return res
