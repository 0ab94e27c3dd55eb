"""Replay a protocol file on the GPU: every protocol x every tumour x M runs,
one row of final living-cell counts per protocol (tumour-major, then run), the
layout of the reference's tools/run_protocols_gpu.py and its results files.

The reference's runner builds one Experiment per chunk of 10 protocols.  Here
the file is one index space: simulation (protocol p, tumour t, run r) is
g = p*T*M + t*M + r.  It is cut into contiguous ranges of about 200,000
simulations (`sims_per_batch`), each run as one persistent batch whose random
streams are keyed by the global index (emt6_batch_set_index_base), so the
counts for a seed do not depend on the cut and equal one Experiment over all
protocols with that seed.  With several devices the ranges run in waves, one
batch per device at a time; under torch.distributed each rank runs the
contiguous share of the index space of its rank and the counts are gathered
over the group.

    python -m emt6ro.replay --protocols protocols.txt --tumors tumor-*.txt \\
        --params default-parameters.json --reps 100 --steps 144000 --out results.txt
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

SIMS_PER_BATCH = 200_000


def replay(params, tumors, protocols, reps: int, steps: int, resolution: int = 300,
           seed: int | None = None, protocol_chunk: int | None = None, device: int = 0,
           log=None, devices=None, sims_per_batch: int | None = None,
           process_group=None) -> np.ndarray:
    """Final living counts, shape (protocols, tumours, reps), uint32.

    protocol_chunk: protocols per batch (the reference runner's knob; sets
    sims_per_batch to protocol_chunk * T * M).  devices: run batches on these
    devices concurrently (default [device], this process's GPU).
    process_group: a torch.distributed group; each rank runs its contiguous
    share with rank 0's seed and every rank returns the whole array."""
    from .batch import Batch
    n_t, n_p = len(tumors), len(protocols)
    per = n_t * reps
    total = n_p * per
    if sims_per_batch is None:
        sims_per_batch = protocol_chunk * per if protocol_chunk else SIMS_PER_BATCH
    sims_per_batch = max(1, int(sims_per_batch))
    if seed is None:
        seed = int.from_bytes(os.urandom(8), "little")
    lo, hi = 0, total
    if process_group is not None:
        import torch.distributed as dist
        from .ga_model.sharding import shard_range
        # every rank draws with rank 0's seed: one index space, one seed
        box = [seed]
        dist.broadcast_object_list(box, src=dist.get_global_rank(process_group, 0)
                                   if hasattr(dist, "get_global_rank") else 0,
                                   group=process_group)
        seed = box[0]
        lo, hi = shard_range(total, dist.get_rank(process_group),
                             dist.get_world_size(process_group))
    ranges = [(g0, min(g0 + sims_per_batch, hi)) for g0 in range(lo, hi, sims_per_batch)]
    devs = list(devices) if devices else [device]
    local = np.zeros(hi - lo, np.uint32)
    for w in range(0, len(ranges), len(devs)):
        live = []
        for dev, (g0, g1) in zip(devs, ranges[w:w + len(devs)]):
            g = np.arange(g0, g1)
            p_first = g0 // per
            part = protocols[p_first:(g1 - 1) // per + 1]
            b = Batch(params, tumors, part, ((g % per) // reps).astype(np.int32),
                      (g // per - p_first).astype(np.int32), protocol_resolution=resolution,
                      protocol_length=steps, device=dev, seed=seed)
            b.set_index_base(g0)
            b.run(steps)  # enqueues; the batches of a wave run concurrently
            live.append((g0, g1, b, time.time()))
        for g0, g1, b, t0 in live:
            local[g0 - lo:g1 - lo] = b.counts()
            if log:
                dt = time.time() - t0
                log(f"  simulations {g0}..{g1 - 1} of {total} (protocols {g0 // per}.."
                    f"{(g1 - 1) // per}) in {dt:.1f}s ({(g1 - g0) / max(dt, 1e-9):.0f} sims/sec)")
        live.clear()
        b = None  # free the wave's batches before the next one is made
    if process_group is not None:
        from .ga_model.sharding import gather_shards
        local = gather_shards(local, total, process_group)
    return local.reshape(n_p, n_t, reps)


def write_rows(counts: np.ndarray, path) -> None:
    """One line per protocol: its tumour-major, run-major counts."""
    with Path(path).open("w") as f:
        for row in counts.reshape(counts.shape[0], -1):
            f.write(" ".join(str(int(x)) for x in row) + "\n")


def main(argv=None) -> int:
    from . import protocols as P
    from .simulation import load_parameters, load_state
    ap = argparse.ArgumentParser(description="replay a protocol file on the GPU")
    ap.add_argument("--protocols", type=Path, required=True)
    ap.add_argument("--tumors", nargs="+", type=Path, required=True)
    ap.add_argument("--params", type=Path, required=True)
    ap.add_argument("--reps", type=int, default=100)
    ap.add_argument("--steps", type=int, default=144_000)
    ap.add_argument("--resolution", type=int, default=300)
    ap.add_argument("--out", type=Path, required=True)
    ap.add_argument("--meta-out", type=Path, default=None)
    ap.add_argument("--protocol-chunk", type=int, default=None,
                    help="protocols per batch (default: batches of about 200,000 simulations)")
    ap.add_argument("--limit-protocols", type=int, default=None)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--devices", type=int, nargs="+", default=None,
                    help="run batches on these devices concurrently")
    args = ap.parse_args(argv)
    args.out.parent.mkdir(parents=True, exist_ok=True)
    meta = args.meta_out or args.out.with_suffix(args.out.suffix + ".meta.json")

    params = load_parameters(str(args.params))
    tumors = [load_state(str(p), params) for p in args.tumors]
    protocols = P.to_experiment(P.read_protocols(args.protocols))
    if args.limit_protocols:
        protocols = protocols[:args.limit_protocols]
    print(f"{len(protocols)} protocols x {len(tumors)} tumors x {args.reps} reps, "
          f"{args.steps} steps")
    # a seed drawn here is recorded in the metadata, so the run can be repeated
    seed = args.seed if args.seed is not None else int.from_bytes(os.urandom(8), "little")
    t0 = time.time()
    counts = replay(params, tumors, protocols, args.reps, args.steps, args.resolution,
                    seed, args.protocol_chunk, args.device, log=print, devices=args.devices)
    wall = time.time() - t0
    write_rows(counts, args.out)
    meta.write_text(json.dumps({
        "n_protocols": len(protocols), "n_tumors": len(tumors), "reps_per_tumor": args.reps,
        "steps": args.steps, "resolution": args.resolution,
        "tumors": [str(p) for p in args.tumors], "protocols_file": str(args.protocols),
        "params_file": str(args.params), "wall_time_sec": wall, "seed": seed,
        "row_layout": "values per row are tumor-major then rep-major: "
                      "[t0r0, t0r1, ..., t0r{M-1}, t1r0, ...]"}, indent=2))
    print(f"Total: {len(protocols)} protocols in {wall:.1f}s; wrote {args.out} and {meta}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
