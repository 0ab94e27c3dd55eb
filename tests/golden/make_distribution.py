"""Final living-cell distributions from the reference's CPU path.

The reference's own host-compiled cell model (Site::step, chooseNeighbour,
divideCell from src/emt6ro/...) with its own random engine (HostRandEngine,
std::mt19937, src/emt6ro/common/random-engine.cc) drives the oracle's
restatement of the occupied-list / ROI / diffusion kernels, diffusion in the
reference's own FP32 expression order (oracle/emt6_oracle.c built with
-DORC_REF_CELL).  Run where the reference checkout exists:

    python tests/golden/make_distribution.py

Writes tests/golden/dist_refcpu.npz: per case, 1000 replicate final counts.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "emt6-ro_gb300"))
from oracle import pyoracle as po  # noqa: E402

OUT = Path(__file__).resolve().parent / "dist_refcpu.npz"

# (name, disc radius, tumour seed, protocol [(step, Gy)], steps)
CASES = [
    ("r10_2x1.25Gy_36h", 10, 0, [(6 * 600, 1.25), (18 * 600, 1.25)], 36 * 600),
    ("r8_1x4Gy_24h", 8, 5, [(2 * 600, 4.0)], 24 * 600),
]
REPLICATES = 1000


def main():
    from emt6ro import workloads as wl
    ref = po.reference()
    if ref is None:
        raise SystemExit("reference checkout not available")
    params = wl.default_parameters()
    out = {}
    for name, radius, tseed, prot, steps in CASES:
        tumor = wl.disc_tumor(params, radius, seed=tseed)
        dose = wl.protocol_doses([prot], 480)[0]
        b = po.Batch(po.params_copy(params.native), REPLICATES, seed=7, lib=ref)
        for i in range(REPLICATES):
            b.set(i, tumor.sites, dose, resolution=300, length=144_000, sim_index=i)
        t = time.time()
        b.run(steps, nthreads=8)
        counts = b.counts()
        print(f"{name}: {time.time() - t:.0f}s mean {counts.mean():.2f} sd {counts.std():.2f}",
              flush=True)
        out[name] = counts
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
