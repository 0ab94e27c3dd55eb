"""Generate golden vectors from the reference's own host-compiled code.

Run in a checkout where the reference is available (the oracle build script
compiles its sources into oracle/_ref/libemt6_ref.so):

    python tests/golden/make_golden.py

Outputs (committed, small):
  site_step.npz     Site::step with injected draws on randomised sites
                    (src/emt6ro/site/site.h:62-82 via ReplayRand)
  choose.npz        chooseNeighbour for a sweep of uniforms (cell-division.h:32-54)
  divide.npz        divideCell with injected standard normals (cell-division.h:10-30)
  kat.npz           the reference gtest known-answer cases, re-evaluated
  ref_params.npz    default/dummy parameters as the reference's JSON loader reads them
  ref_states.npz    data/tumor-lib states as the reference's text loader reads them
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import pyoracle as po  # noqa: E402
from oracle.build import REFERENCE_ROOT  # noqa: E402

OUT = Path(__file__).resolve().parent


def random_sites(rng, p, n):
    """Sites spanning every branch of the cell model: all modes/phases,
    substrate levels around each threshold, irradiated and repairing cells."""
    s = np.zeros(n, dtype=po.SITE_DTYPE)
    s["state"] = np.where(rng.random(n) < 0.9, po.OCCUPIED, po.VACANT)
    met = np.array([[p.metabolism[m][k] for k in range(3)] for m in range(4)], np.float32)
    pick = rng.integers(0, 4, n)
    jitter = rng.choice(np.array([-1, 0, 0, 1], np.float32), size=(n, 2)) * \
        rng.choice(np.array([0, 1e-6, 1e-3, 0.5, 5.0], np.float32), size=(n, 2))
    s["cho"] = np.maximum(met[pick, 0] + jitter[:, 0] * met[pick, 0], 0)
    s["ox"] = np.maximum(met[pick, 1] + jitter[:, 1] * np.maximum(met[pick, 1], 1), 0)
    wide = rng.random(n) < 0.2
    s["cho"][wide] = rng.uniform(0, 300, wide.sum()).astype(np.float32)
    s["ox"][wide] = rng.uniform(0, 15, wide.sum()).astype(np.float32)
    gi_choices = np.array([0.0, 0.0019, 0.0199, 0.01989, 0.0201, 0.049, 0.05, 0.051, 0.06],
                          np.float32)
    s["gi"] = rng.choice(gi_choices, n)
    t0 = rng.normal(6, 1, n).astype(np.float32)
    t1 = t0 + rng.normal(10, 2, n).astype(np.float32)
    t2 = t1 + np.float32(2)
    t3 = t2 + np.float32(2)
    t4 = t3 + np.float32(0.1)
    s["cycle_times"] = np.stack([t0, t1, t2, t3, t4], 1)
    s["phase"] = rng.integers(0, 5, n)
    tvals = np.stack([np.zeros(n, np.float32), t0, t1, t2, t3, t4], 1)
    ph = s["phase"].astype(int)
    lo, hi = tvals[np.arange(n), ph], tvals[np.arange(n), ph + 1]
    frac = rng.choice(np.array([0, 0.001, 0.5, 0.999, 1.0], np.float32), n)
    s["proliferation_time"] = (lo + (hi - lo) * frac).astype(np.float32)
    # exact-boundary cases for the death / G1-S tests
    b = rng.random(n) < 0.05
    s["proliferation_time"][b] = (t4 - np.float32(6 / 3600))[b]
    s["mode"] = rng.integers(0, 4, n)
    irr = rng.random(n) < 0.4
    s["irradiation"][irr] = rng.uniform(0, 12, irr.sum()).astype(np.float32)
    rep = irr & (rng.random(n) < 0.5)
    s["time_in_repair"][rep] = rng.uniform(0, 8, rep.sum()).astype(np.float32)
    s["repair_delay_time"][irr] = rng.uniform(0.5, 9, irr.sum()).astype(np.float32)
    edge = irr & (rng.random(n) < 0.2)
    s["time_in_repair"][edge] = s["repair_delay_time"][edge] - np.float32(6 / 3600)
    return s


def main():
    ref = po.reference()
    if ref is None:
        raise SystemExit("reference checkout not available")
    R = REFERENCE_ROOT
    p = po.params_from_json(R / "data" / "default-parameters.json")
    pd = po.params_from_json(R / "data" / "test" / "dummy-parameters.json")
    rng = np.random.default_rng(20240611)

    # -- Site::step with injected draws --------------------------------------
    n = 6000
    sites = random_sites(rng, p, n)
    vac = rng.integers(0, 9, n).astype(np.uint32)
    dose = np.where(rng.random(n) < 0.3, rng.choice(np.array([0.25, 1.25, 2.5, 5.0]), n),
                    0).astype(np.float32)
    draws = rng.random(n).astype(np.float32)
    draws[rng.random(n) < 0.05] = np.float32(1.0)
    out = sites.copy()
    ready = np.zeros(n, np.int32)
    used = np.zeros(n, np.int32)
    for i in range(n):
        u = ctypes.c_int()
        one = out[i:i + 1].copy()
        ready[i] = ref.L.ref_site_step_replay(one, ctypes.byref(p), int(vac[i]), float(dose[i]),
                                              draws[i:i + 1].copy(), 1, ctypes.byref(u))
        out[i] = one[0]
        used[i] = u.value
    np.savez_compressed(OUT / "site_step.npz", sites=sites, vac=vac, dose=dose, draws=draws,
                        out=out, ready=ready, used=used)

    # -- chooseNeighbour ------------------------------------------------------
    us = np.concatenate([np.linspace(0, 1, 4001, dtype=np.float32),
                         rng.random(6000).astype(np.float32),
                         np.array([1.0, np.nextafter(np.float32(1), np.float32(0))],
                                  np.float32)])
    rc = np.zeros((us.size, 2), np.int32)
    for i, u in enumerate(us):
        a, b = ctypes.c_int(), ctypes.c_int()
        ref.L.ref_choose_neighbour_replay(26, 26, float(u), ctypes.byref(a), ctypes.byref(b))
        rc[i] = (a.value, b.value)
    np.savez_compressed(OUT / "choose.npz", u=us, rc=rc)

    # -- divideCell ------------------------------------------------------------
    n = 2000
    parents = random_sites(rng, p, n)
    z = rng.normal(0, 1, (n, 5)).astype(np.float32)
    pa = parents.copy()
    ch = np.zeros(n, dtype=po.SITE_DTYPE)
    for i in range(n):
        a = pa[i:i + 1].copy()
        c = ch[i:i + 1].copy()
        ref.L.ref_divide_cell_replay(a, c, ctypes.byref(p), z[i].copy())
        pa[i] = a[0]
        ch[i] = c[0]
    np.savez_compressed(OUT / "divide.npz", parents=parents, z=z, parents_out=pa, children=ch)

    # -- known-answer cases of the reference gtests ------------------------------
    # cell-update-state-test.cc:20-89: params and 18 cases, evaluated by the reference
    pk = po.Params()
    pk.metabolism[0][:] = [21, 9, 0]
    pk.metabolism[1][:] = [54, 0, -3e-3]
    pk.metabolism[2][:] = [18, 8, 0]
    pk.metabolism[3][:] = [45, 0, -3e-5]
    pk.death_gi = 5e-2
    pk.quiescence_gi = 2e-2
    pk.time_step = 3600
    cases = [  # levels, vac, g1, phase, prolif, alive, mode
        ((17, 10, 0), 0, 100, 0, 50, False, 2), ((18, 10, 6e-2), 0, 100, 0, 50, False, 2),
        ((18, 10, 0), 0, 20, 3, 19, False, 2), ((44, 7, 0), 0, 20, 0, 19, False, 2),
        ((45, 7, 0), 0, 20, 2, 21, True, 3), ((18, 8, 0), 0, 20, 2, 21, True, 2),
        ((18, 10, 3e-2), 0, 20, 3, 15, False, 2), ((44, 7, 3e-2), 0, 20, 0, 15, False, 2),
        ((45, 7, 3e-2), 0, 20, 2, 15, True, 3), ((18, 8, 3e-2), 0, 20, 2, 15, True, 2),
        ((18, 8, 0), 0, 20, 3, 15, False, 2), ((44, 7, 0), 0, 20, 0, 15, False, 2),
        ((45, 7, 0), 0, 20, 2, 15, True, 3), ((18, 8, 0), 0, 20, 2, 15, True, 2),
        ((54, 7, 0), 0, 20, 0, 15, True, 1), ((21, 9, 0), 0, 20, 0, 15, True, 0),
        ((21, 8, 0), 0, 20, 0, 15, True, 2), ((21, 8, 0), 0, 20, 3, 15, False, 2),
    ]
    kat = np.zeros(len(cases), dtype=po.SITE_DTYPE)
    kat_alive = np.zeros(len(cases), np.int32)
    kat_vac = np.zeros(len(cases), np.uint32)
    for i, (lv, v, g1, ph, pt, alive, mode) in enumerate(cases):
        s = np.zeros(1, dtype=po.SITE_DTYPE)
        s["cho"], s["ox"], s["gi"] = lv
        s["cycle_times"][0, 0] = g1
        s["cycle_times"][0, 4] = 100
        s["phase"] = ph
        s["proliferation_time"] = pt
        s["mode"] = 2  # MOCK_MODE
        s["state"] = po.OCCUPIED
        kat[i] = s[0]
        kat_vac[i] = v
        r = ref.L.ref_update_state(s, ctypes.byref(pk), v)
        assert bool(r) == alive, (i, r, alive)
        if alive:
            assert s["mode"][0] == mode, (i, s["mode"][0], mode)
        kat_alive[i] = r
    np.savez_compressed(OUT / "kat.npz", update_sites=kat, update_vac=kat_vac,
                        update_alive=kat_alive,
                        update_params=np.frombuffer(bytes(pk), np.uint8))

    # -- file formats ---------------------------------------------------------------
    q1 = po.Params()
    q2 = po.Params()
    assert ref.L.ref_load_params(str(R / "data" / "default-parameters.json").encode(),
                                 ctypes.byref(q1)) == 0
    assert ref.L.ref_load_params(str(R / "data" / "test" / "dummy-parameters.json").encode(),
                                 ctypes.byref(q2)) == 0
    np.savez_compressed(OUT / "ref_params.npz",
                        default=np.frombuffer(bytes(q1), np.uint8),
                        dummy=np.frombuffer(bytes(q2), np.uint8))
    states = []
    for k in range(1, 11):
        buf = np.zeros(53 * 53, dtype=po.SITE_DTYPE)
        h, w = ctypes.c_int(), ctypes.c_int()
        assert ref.L.ref_load_state(str(R / "data" / "tumor-lib" / f"tumor-{k}.txt").encode(),
                                    ctypes.byref(q1), buf, buf.size, ctypes.byref(h),
                                    ctypes.byref(w)) == 53 * 53
        # state.cc:33-35 sets repair_delay_time only when irradiation > 0; the
        # HostGrid storage is otherwise uninitialised, so zero it here
        buf["repair_delay_time"][buf["irradiation"] <= 0] = 0
        states.append(buf.reshape(53, 53))
    np.savez_compressed(OUT / "ref_states.npz", states=np.stack(states))
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    main()
