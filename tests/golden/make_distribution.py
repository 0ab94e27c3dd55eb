"""Final living-cell distributions from the reference's CPU path.

The reference's own host-compiled cell model (Site::step, chooseNeighbour,
divideCell from src/emt6ro/...) with its own random engine (HostRandEngine,
std::mt19937, src/emt6ro/common/random-engine.cc) drives the oracle's
restatement of the occupied-list / ROI / diffusion kernels, diffusion in the
reference's own FP32 expression order (oracle/emt6_oracle.c built with
-DORC_REF_CELL).  Run where the reference checkout exists:

    python tests/golden/make_distribution.py            # 24-36 h cases
    python tests/golden/make_distribution.py --ten-day  # 10-day cases

Writes tests/golden/dist_refcpu.npz (CASES: per case, 1000 replicate final
counts) or tests/golden/dist_refcpu_10d.npz (CASES_10D, 144,000 steps; the
file is rewritten after every case, so an interrupted run keeps the cases
finished so far).
"""
from __future__ import annotations

import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "emt6-ro_gb300"))
from oracle import pyoracle as po  # noqa: E402

OUT = Path(__file__).resolve().parent / "dist_refcpu.npz"
OUT_10D = Path(__file__).resolve().parent / "dist_refcpu_10d.npz"

# (name, disc radius, tumour seed, protocol [(step, Gy)], steps)
CASES = [
    ("r10_2x1.25Gy_36h", 10, 0, [(6 * 600, 1.25), (18 * 600, 1.25)], 36 * 600),
    ("r8_1x4Gy_24h", 8, 5, [(2 * 600, 4.0)], 24 * 600),
]
REPLICATES = 1000

TEN_DAYS = 144_000
# 10-day cases.  "plain": the plain-simulation benchmark case (disc of radius
# 10 at the centre, 1.25 Gy at hours 12 and 36).  "ga_pP_tT": protocol P of
# the GA batch's 100 protocols (workloads.ga_protocols(100)) on tumour T of
# its 20 tumours (workloads.ga_tumors(params, 20)).
# (name, replicates, engine seed)
CASES_10D = [
    ("plain_r10_2x1.25Gy_10d", 1000, 101),
    ("ga_p0_t0_10d", 600, 102),
    ("ga_p1_t1_10d", 600, 103),
    ("ga_p2_t0_10d", 600, 104),
    ("ga_p3_t1_10d", 600, 105),
    ("ga_p6_t0_10d", 600, 106),
]


def case_inputs(name, params):
    """(tumour, protocol) of a 10-day case."""
    from emt6ro import workloads as wl
    if name.startswith("plain_"):
        return wl.disc_tumor(params, 10, seed=0), wl.protocol_2x125gy()
    _, p, t, _ = name.split("_")
    prot = wl.ga_protocols(100)[int(p[1:])]
    tumor = wl.ga_tumors(params, 20)[int(t[1:])]
    return tumor, prot


def _run(ref, params, tumor, prot, reps, steps, seed, threads):
    from emt6ro import workloads as wl
    dose = wl.protocol_doses([prot], 480)[0]
    b = po.Batch(po.params_copy(params.native), reps, seed=seed, lib=ref)
    for i in range(reps):
        b.set(i, tumor.sites, dose, resolution=300, length=144_000, sim_index=i)
    b.run(steps, nthreads=threads)
    return b.counts()


def main():
    from emt6ro import workloads as wl
    ref = po.reference()
    if ref is None:
        raise SystemExit("reference checkout not available")
    params = wl.default_parameters()
    threads = int(os.environ.get("THREADS", os.cpu_count() or 1))
    if "--ten-day" in sys.argv:
        out = dict(np.load(OUT_10D)) if OUT_10D.exists() else {}
        for name, reps, seed in CASES_10D:
            if name in out and len(out[name]) >= reps:
                continue
            tumor, prot = case_inputs(name, params)
            t = time.time()
            counts = _run(ref, params, tumor, prot, reps, TEN_DAYS, seed, threads)
            print(f"{name}: {time.time() - t:.0f}s mean {counts.mean():.2f} sd {counts.std():.2f}",
                  flush=True)
            out[name] = counts
            np.savez_compressed(OUT_10D, **out)
        print("wrote", OUT_10D)
        return
    out = {}
    for name, radius, tseed, prot, steps in CASES:
        tumor = wl.disc_tumor(params, radius, seed=tseed)
        t = time.time()
        counts = _run(ref, params, tumor, prot, REPLICATES, steps, 7, threads)
        print(f"{name}: {time.time() - t:.0f}s mean {counts.mean():.2f} sd {counts.std():.2f}",
              flush=True)
        out[name] = counts
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
