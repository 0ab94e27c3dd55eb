"""Launch and tile-shape autotuner for the batch engine.

A CTA holds one simulation's lattice in shared memory (52 KB: an SM holds
four whatever the grouping, so one simulation per CTA is fixed), and the
kernels pick a register tiling per region.  Tuned per workload, in two
stages on a stratified sample of the batch from identical initial states:

1. how the step loop is launched: steps per launch (longer launches amortise
   the per-launch load/store of every lattice; shorter ones let simulations
   that finish or outgrow the narrow kernel be rescheduled sooner), the
   schedule (one CTA per simulation vs persistent CTAs over a device work
   queue ordered by horizon) and CUDA-graph replay of the launch sequence;
2. with the fastest launch, which tile shapes the kernels may use
   (Batch.LAYOUT_* bits: eight-lane bands for small regions, three-column
   bands for 41-48-row wide regions, the 35 x 35 ring mapping).

Every candidate gives bit-identical results; only time differs.
"""
from __future__ import annotations

import itertools
import time

import numpy as np

from .batch import Batch

DEFAULT_CHUNKS = (300, 600, 1200, 2400)
DEFAULT_MODES = (0, 1, 2, 3)  # bit 0: work queue, bit 1: CUDA graph
DEFAULT_LAYOUTS = tuple(range(8))  # subsets of Batch.LAYOUT_* bits

_cache: dict = {}


def _sample(n: int, k: int) -> np.ndarray:
    return np.unique(np.linspace(0, n - 1, min(n, k)).astype(np.int64))


def tune(params, tumors, protocols, sim_tumor, sim_protocol, sim_horizon=None, *, device=0,
         sample=2432, trial_steps=600, warm_steps=64, chunks=DEFAULT_CHUNKS, modes=DEFAULT_MODES,
         layouts=DEFAULT_LAYOUTS, seed=1, key=None):
    """Returns (mode, steps_per_launch, layouts, table) with table rows
    (mode, chunk, layouts, seconds): stage 1 with all tile shapes allowed,
    stage 2 over `layouts` with the fastest (mode, chunk)."""
    if key is not None and key in _cache:
        return _cache[key]
    idx = _sample(len(sim_tumor), sample)
    st = np.asarray(sim_tumor)[idx]
    sp = np.asarray(sim_protocol)[idx]
    hz = None if sim_horizon is None else np.asarray(sim_horizon)[idx]

    def trial(mode, chunk, lay):
        b = Batch(params, tumors, protocols, st, sp, sim_horizon=hz, device=device, seed=seed)
        b.set_layouts(lay)
        b.set_schedule(mode, min(chunk, warm_steps))
        b.run(warm_steps)
        b.sync()
        b.set_schedule(mode, chunk)
        t0 = time.perf_counter()
        b.run(trial_steps)
        b.sync()
        dt = time.perf_counter() - t0
        del b
        return dt

    table = [(mode, chunk, Batch.LAYOUT_ALL, trial(mode, chunk, Batch.LAYOUT_ALL))
             for mode, chunk in itertools.product(modes, chunks)]
    mode, chunk, _, _ = min(table, key=lambda r: r[3])
    for lay in layouts:
        if lay != Batch.LAYOUT_ALL:
            table.append((mode, chunk, lay, trial(mode, chunk, lay)))
    mode, chunk, lay, _ = min(table, key=lambda r: r[3])
    res = (mode, chunk, lay, table)
    if key is not None:
        _cache[key] = res
    return res
