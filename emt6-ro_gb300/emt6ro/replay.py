"""Replay a protocol file on the GPU: every protocol x every tumour x M runs,
one row of final living-cell counts per protocol (tumour-major, then run), the
layout of the reference's tools/run_protocols_gpu.py and its results files.

The reference's runner builds one Experiment per chunk of 10 protocols.  Here
the protocols go through persistent batches as large as the device holds
(`--protocol-chunk` protocols each, by default as many as make about 200,000
simulations), one index space over the whole file: simulation
(protocol p, tumour t, run r) is p*T*M + t*M + r, and each batch keys its
random streams by that global index (emt6_batch_set_index_base), so the
counts for a seed do not depend on the chunking and equal one Experiment
over all protocols with that seed.

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
           log=None) -> np.ndarray:
    """Final living counts, shape (protocols, tumours, reps), uint32."""
    from .batch import Batch
    n_t, n_p = len(tumors), len(protocols)
    per = n_t * reps
    chunk = protocol_chunk or max(1, SIMS_PER_BATCH // max(per, 1))
    if seed is None:
        seed = int.from_bytes(os.urandom(8), "little")
    out = np.zeros((n_p, n_t, reps), np.uint32)
    for p0 in range(0, n_p, chunk):
        part = protocols[p0:p0 + chunk]
        n = len(part)
        t0 = time.time()
        sim_tumor = np.tile(np.repeat(np.arange(n_t, dtype=np.int32), reps), n)
        sim_protocol = np.repeat(np.arange(n, dtype=np.int32), per)
        b = Batch(params, tumors, part, sim_tumor, sim_protocol, protocol_resolution=resolution,
                  protocol_length=steps, device=device, seed=seed)
        b.set_index_base(p0 * per)
        b.run(steps)
        out[p0:p0 + n] = b.counts().reshape(n, n_t, reps)
        del b
        if log:
            dt = time.time() - t0
            log(f"  protocols {p0}..{p0 + n - 1} of {n_p}: {n} protocols x {n_t} tumors x "
                f"{reps} reps in {dt:.1f}s ({n * per / max(dt, 1e-9):.0f} sims/sec)")
    return out


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
                    help="protocols per batch (default: about 200,000 simulations)")
    ap.add_argument("--limit-protocols", type=int, default=None)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--device", type=int, default=0)
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
                    seed, args.protocol_chunk, args.device, log=print)
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
