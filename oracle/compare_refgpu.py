"""Full-horizon distribution comparison with the reference's own CUDA build.

Test and measurement infrastructure: runs the reference's kernels
(oracle/pyrefgpu.py) and this project's simulator on the same initial state
and protocols, and prints a JSON report of per-protocol statistics.

Default case (the distribution check of the hot-path contract, at the
longest horizon the reference's kernels survive): the radius-10 disc tumour,
20 random 10-Gy protocols (1-8 doses, 0.25-Gy quanta, 30-min grid in the
first 48 h), 1,000 replicates each, 72,000 steps (5 days).

The reference's findOccupied gives each of its 32 threads a fixed array of
32 sites (simulation.cu:44-50: columns c and c + 32 of the lattice).  The
oracle's 160 replicates of this tumour (40 without irradiation, the rest
with these protocols) reach at most 27 per thread by 76,800 steps but 42 by
102,400 steps, when the tumour spans more than 32 columns: a 10-day run
would write past the reference's array.  Horizons above 72,000 steps are
refused here for that reason.

    python oracle/compare_refgpu.py [--reps 1000] [--steps 72000]
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
MAX_SAFE_STEPS = 72_000
for p in (ROOT / "emt6-ro_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=1000)
    ap.add_argument("--steps", type=int, default=MAX_SAFE_STEPS)
    ap.add_argument("--protocols", type=int, default=20)
    args = ap.parse_args()
    if args.steps > MAX_SAFE_STEPS:
        raise SystemExit(f"{args.steps} steps: beyond {MAX_SAFE_STEPS} the reference's kernels "
                         "overflow their per-thread occupied arrays for this tumour")
    from scipy import stats
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    from oracle import pyrefgpu
    if not pyrefgpu.available():
        raise SystemExit("reference cubin not built")
    params = wl.default_parameters()
    tumor = wl.disc_tumor(params, 10, seed=0)
    protocols = wl.ga_protocols(args.protocols, seed=606)
    P, R = len(protocols), args.reps
    doses = wl.protocol_doses(protocols, 480)
    sp = np.repeat(np.arange(P, dtype=np.int32), R)
    t0 = time.perf_counter()
    ref = pyrefgpu.RefGpuSimulation(params, [tumor], doses, np.zeros(len(sp), np.int32), sp,
                                    seed=20240)
    ref.run(args.steps)
    theirs = ref.counts().astype(np.float64).reshape(P, R)
    ref.close()
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    e = sim.Experiment(params, [tumor], R, P, 0, args.steps, seed=4321)
    e.add_irradiations(protocols)
    e.run(args.steps)
    ours = e.get_results().astype(np.float64).reshape(P, R)
    t_ours = time.perf_counter() - t0
    rows = []
    for k in range(P):
        a, b = ours[k], theirs[k]
        rows.append({
            "protocol": protocols[k],
            "mean": [round(a.mean(), 2), round(b.mean(), 2)],
            "sd": [round(a.std(), 2), round(b.std(), 2)],
            "q10_50_90": [np.quantile(a, [0.1, 0.5, 0.9]).tolist(),
                          np.quantile(b, [0.1, 0.5, 0.9]).tolist()],
            "rel_mean_diff": round((a.mean() - b.mean()) / b.mean(), 4),
            "ks_p": float(stats.ks_2samp(a, b).pvalue),
            "welch_p": float(stats.ttest_ind(a, b, equal_var=False).pvalue),
        })
    ks = np.array([r["ks_p"] for r in rows])
    rel = np.array([abs(r["rel_mean_diff"]) for r in rows])
    report = {
        "case": f"radius-10 disc, {P} protocols x {R} replicates, {args.steps} steps",
        "max_abs_rel_mean_diff": float(rel.max()),
        "mean_abs_rel_mean_diff": float(rel.mean()),
        "ks_p_below_0.01": int((ks < 0.01).sum()),
        "ks_p_min": float(ks.min()),
        "seconds": {"reference_cuda": round(t_ref, 1), "this_project": round(t_ours, 1)},
        "per_protocol": rows,
    }
    print(json.dumps(report))


if __name__ == "__main__":
    main()
