"""The CPU oracle, pinned against the reference: golden vectors generated from
the reference's own host-compiled code (tests/golden/make_golden.py) and the
reference's gtest known-answer cases (src/emt6ro/cell/*-test.cc,
parameters/parameters-test.cc).  No GPU needed."""
import ctypes
import math

import numpy as np

from conftest import GOLDEN


def _site_mismatch(a, b):
    bad = {}
    for f in a.dtype.names:
        x = np.ascontiguousarray(a[f]).reshape(len(a), -1).view(np.uint8)
        y = np.ascontiguousarray(b[f]).reshape(len(b), -1).view(np.uint8)
        ne = (x != y).any(1)
        if ne.any():
            bad[f] = int(ne.sum())
    return bad


def test_philox_known_answers(oracle):
    L = oracle.oracle().L

    def ph(c, k):
        o = np.zeros(4, np.uint32)
        L.orc_philox4x32_10(np.array(c, np.uint32), np.array(k, np.uint32), o)
        return o.tolist()

    # Random123 kat_vectors, philox4x32 10 rounds
    assert ph([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert ph([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6,
                                                       0x6d5451fd]
    assert ph([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_double_math_accuracy(oracle):
    L = oracle.oracle().L
    xs = np.linspace(-25, 8, 20001, dtype=np.float32)
    mism = sum(L.orc_expf(float(x)) != np.float32(math.exp(float(x))) for x in xs)
    assert mism == 0  # rounds like a correctly rounded expf on this domain
    us = np.concatenate([np.linspace(2.0**-24, 1, 20001), [1.0]])
    err = max(abs(L.orc_log_core(float(u)) - math.log(u)) for u in us)
    assert err < 1e-15
    s, c = ctypes.c_double(), ctypes.c_double()
    err = 0.0
    for u in np.linspace(0, 1, 5001, endpoint=False):
        L.orc_sincos2pi(float(u), ctypes.byref(s), ctypes.byref(c))
        err = max(err, abs(s.value - math.sin(2 * math.pi * u)),
                  abs(c.value - math.cos(2 * math.pi * u)))
    assert err < 1e-15


def test_normals_distribution(oracle):
    L = oracle.oracle().L
    z = np.zeros((4000, 5), np.float32)
    for i in range(4000):
        L.orc_division_normals(11, i, i % 7, 0, z[i])
    zz = z.reshape(-1)
    assert abs(zz.mean()) < 0.03 and abs(zz.std() - 1) < 0.03
    from scipy import stats
    assert stats.kstest(zz, "norm").pvalue > 0.001


def test_site_step_bit_exact_vs_reference(params, oracle):
    """Site::step (site/site.h:62-82) with injected draws on 6000 sites spanning
    every branch; golden outputs from the reference's own compiled function."""
    L = oracle.oracle().L
    g = np.load(GOLDEN / "site_step.npz")
    out = g["sites"].copy()
    n = len(out)
    ready = np.zeros(n, np.int32)
    used = np.zeros(n, np.int32)
    for i in range(n):
        one = out[i:i + 1].copy()
        u = ctypes.c_int()
        ready[i] = L.orc_site_step(one, ctypes.byref(oracle.params_copy(params)), int(g["vac"][i]),
                                   float(g["dose"][i]), float(g["draws"][i]), ctypes.byref(u))
        out[i] = one[0]
        used[i] = u.value
    assert (ready == g["ready"]).all()
    assert (used == g["used"]).all()
    assert _site_mismatch(out, g["out"]) == {}
    # the vectors exercise deaths, divisions-ready, irradiation and repair draws
    assert g["ready"].sum() > 50 and g["used"].sum() > 50
    assert ((g["sites"]["state"] == 1) & (g["out"]["state"] == 0)).sum() > 500


def test_choose_neighbour_vs_reference(oracle):
    L = oracle.oracle().L
    g = np.load(GOLDEN / "choose.npz")
    a, b = ctypes.c_int(), ctypes.c_int()
    for u, rc in zip(g["u"], g["rc"]):
        L.orc_choose_neighbour(26, 26, float(u), ctypes.byref(a), ctypes.byref(b))
        assert (a.value, b.value) == tuple(rc)
    # u = 1 maps to orthogonal index 4 -> (r, c-1), cell-division.h:52
    L.orc_choose_neighbour(26, 26, 1.0, ctypes.byref(a), ctypes.byref(b))
    assert (a.value, b.value) == (26, 25)


def test_divide_cell_vs_reference(params, oracle):
    L = oracle.oracle().L
    L.orc_divide_cell.restype = None
    L.orc_divide_cell.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p]
    g = np.load(GOLDEN / "divide.npz")
    cell_dt = np.dtype([("tir", "<f4"), ("irr", "<f4"), ("delay", "<f4"), ("prolif", "<f4"),
                        ("t", "<f4", (5,)), ("mode", "u1"), ("phase", "u1"), ("pad", "u2")])
    for i in range(len(g["z"])):
        ps = g["parents"][i]
        pc = np.zeros(1, cell_dt)
        pc["tir"], pc["irr"], pc["delay"] = ps["time_in_repair"], ps["irradiation"], \
            ps["repair_delay_time"]
        pc["prolif"], pc["t"], pc["mode"], pc["phase"] = ps["proliferation_time"], \
            ps["cycle_times"], ps["mode"], ps["phase"]
        ch = np.zeros(1, cell_dt)
        z = np.ascontiguousarray(g["z"][i])
        L.orc_divide_cell(pc.ctypes.data, ch.ctypes.data, z.ctypes.data,
                          ctypes.addressof(oracle.params_copy(params)))
        ec = g["children"][i]
        ep = g["parents_out"][i]
        assert ch["t"][0].tobytes() == ec["cycle_times"].tobytes()
        assert ch["irr"][0] == ec["irradiation"] and ch["delay"][0] == ec["repair_delay_time"]
        assert pc["phase"][0] == ep["phase"] and pc["prolif"][0] == ep["proliferation_time"]


def test_update_state_known_answers(oracle):
    """cell-update-state-test.cc:52-89 (18 cases)."""
    L = oracle.oracle().L
    g = np.load(GOLDEN / "kat.npz")
    pk = oracle.Params.from_buffer_copy(g["update_params"].tobytes())
    expected = [(False, None), (False, None), (False, None), (False, None), (True, 3),
                (True, 2), (False, None), (False, None), (True, 3), (True, 2), (False, None),
                (False, None), (True, 3), (True, 2), (True, 1), (True, 0), (True, 2),
                (False, None)]
    for i, (alive, mode) in enumerate(expected):
        s = g["update_sites"][i:i + 1].copy()
        u = ctypes.c_int()
        # updateState alone: a cell with tir=0, irr=0 and no dose only passes
        # through updateState before metabolism; compare alive + mode
        c = np.zeros(1, np.dtype([("tir", "<f4"), ("irr", "<f4"), ("delay", "<f4"),
                                  ("prolif", "<f4"), ("t", "<f4", (5,)), ("mode", "u1"),
                                  ("phase", "u1"), ("pad", "u2")]))
        c["prolif"], c["t"], c["mode"], c["phase"] = s["proliferation_time"], \
            s["cycle_times"], s["mode"], s["phase"]
        lv = np.array([s["cho"][0], s["ox"][0], s["gi"][0]], np.float32)
        r = L.orc_update_state(c.ctypes.data, lv, ctypes.byref(pk), int(g["update_vac"][i]))
        assert bool(r) == alive == bool(g["update_alive"][i]), i
        if alive:
            assert c["mode"][0] == mode, i
        del u


def test_progress_clock_known_answers(oracle):
    """cell-progress-clock-test.cc:45-58 (time_step 360 s, cycle times 1..5)."""
    L = oracle.oracle().L
    dt = np.dtype([("tir", "<f4"), ("irr", "<f4"), ("delay", "<f4"), ("prolif", "<f4"),
                   ("t", "<f4", (5,)), ("mode", "u1"), ("phase", "u1"), ("pad", "u2")])
    cases = [(0, 0, 2, 0.95, False), (0, 0, 3, 0.95, False), (0, 1, 0, 0.95, True),
             (1, 1, 0, 1.85, False), (3, 4, 1, 3.95, False)]
    for cur, exp_phase, mode, t0, changed in cases:
        c = np.zeros(1, dt)
        c["phase"], c["mode"], c["prolif"], c["t"] = cur, mode, t0, [1, 2, 3, 4, 5]
        r = L.orc_progress_clock(c.ctypes.data, 360.0)
        assert bool(r) == changed
        assert c["phase"][0] == exp_phase
        if mode in (0, 1):
            assert c["prolif"][0] == np.float32(t0) + np.float32(360.0) / np.float32(3600)
        else:
            assert c["prolif"][0] == np.float32(t0)


def test_metabolise_known_answers(oracle):
    """cell-metabolise-test.cc:59-63: each mode subtracts its own row."""
    L = oracle.oracle().L
    L.orc_metabolise.restype = None
    L.orc_metabolise.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    p = oracle.Params()
    rows = [[0.11, 0.12, 0.13], [0.21, 0.22, 0.23], [0.31, 0.32, 0.33], [0.41, 0.42, 0.43]]
    for m in range(4):
        p.metabolism[m][:] = rows[m]
    dt = np.dtype([("tir", "<f4"), ("irr", "<f4"), ("delay", "<f4"), ("prolif", "<f4"),
                   ("t", "<f4", (5,)), ("mode", "u1"), ("phase", "u1"), ("pad", "u2")])
    for m in range(4):
        c = np.zeros(1, dt)
        c["mode"] = m
        lv = np.ones(3, np.float32)
        L.orc_metabolise(c.ctypes.data, lv.ctypes.data, ctypes.addressof(p))
        assert lv.tolist() == (np.float32(1) - np.array(rows[m], np.float32)).tolist()


def test_occupied_list_order(oracle):
    """simulation.cu:41-64: 32 column stripes; stripe k holds columns k, k+32
    (< W-1) row by row; stripes are concatenated in order."""
    L = oracle.oracle().L
    rng = np.random.default_rng(3)
    H = W = 53
    st = np.where(rng.random((H, W)) < 0.4, 1, 0).astype(np.uint8)
    st[0, :] = st[-1, :] = st[:, 0] = st[:, -1] = 2
    lst = np.zeros(H * W, np.uint16)
    n = L.orc_rebuild_list(np.ascontiguousarray(st.reshape(-1)), H, W, lst)
    expect = [r * W + c for k in range(32) for r in range(H - 1) for c in range(k, W - 1, 32)
              if st[r, c] == 1]
    assert lst[:n].tolist() == expect


def test_roi_properties(oracle):
    """diffusion.cu:65-100: the ROI covers every occupied site and for an
    unclipped ROI the mask ring around it is entirely fixed."""
    L = oracle.oracle().L
    rng = np.random.default_rng(4)
    H = W = 53
    for _ in range(40):
        st = np.zeros((H, W), np.uint8)
        st[0, :] = st[-1, :] = st[:, 0] = st[:, -1] = 2
        r0, c0, rad = rng.integers(5, 48), rng.integers(5, 48), rng.integers(0, 10)
        rr, cc = np.mgrid[0:H, 0:W]
        disc = ((rr - r0) ** 2 + (cc - c0) ** 2 <= rad * rad) & (st != 2)
        st[disc & (rng.random((H, W)) < 0.8)] = 1
        roi = np.zeros(5, np.int32)
        mask = np.zeros(H * W + 512, np.uint8)
        L.orc_find_roi(np.ascontiguousarray(st.reshape(-1)), H, W, roi, mask)
        occ = np.argwhere(st == 1)
        if len(occ) == 0:
            assert roi.tolist() == [0] * 5
            continue
        sr, sc, h, w, dist = roi
        assert (occ[:, 0] >= sr).all() and (occ[:, 0] < sr + h).all()
        assert (occ[:, 1] >= sc).all() and (occ[:, 1] < sc + w).all()
        m = mask[:(h + 2) * (w + 2)].reshape(h + 2, w + 2)
        if sr > 1 and sc > 1 and sr + h < H - 1 and sc + w < W - 1:
            assert m[0].all() and m[-1].all() and m[:, 0].all() and m[:, -1].all()


def test_diffusion_f32_within_1e5_of_f64(params, oracle):
    L = oracle.oracle().L
    rng = np.random.default_rng(5)
    H = W = 53
    # centred discs, and discs against the lattice edge (clipped ROIs whose
    # ring sites the mask can leave free, next to the zero ring of the tile)
    for rad, (cr, ccol) in ((4, (26, 26)), (10, (26, 26)), (14, (26, 26)), (20, (26, 26)),
                            (10, (26, 3)), (7, (3, 3)), (14, (45, 30)), (20, (8, 22))):
        st = np.zeros((H, W), np.uint8)
        st[0, :] = st[-1, :] = st[:, 0] = st[:, -1] = 2
        rr, cc = np.mgrid[0:H, 0:W]
        st[((rr - cr) ** 2 + (cc - ccol) ** 2 <= rad * rad) & (st != 2)] = 1
        roi = np.zeros(5, np.int32)
        mask = np.zeros(H * W + 512, np.uint8)
        L.orc_find_roi(np.ascontiguousarray(st.reshape(-1)), H, W, roi, mask)
        ext = np.array(params.native.external_levels[:], np.float32)
        fld = (ext[:, None, None] * (0.1 + 0.9 * rng.random((3, H, W)))).astype(np.float32)
        f32 = fld.reshape(-1).copy()
        f64 = np.ascontiguousarray(fld.reshape(-1).astype(np.float64))
        L.orc_diffuse_f32(f32, H, W, roi, mask, ctypes.byref(oracle.params_copy(params)))
        L.orc_diffuse_f64(f64, H, W, roi, mask, ctypes.byref(oracle.params_copy(params)))
        a = f32.reshape(3, H, W).astype(np.float64)
        b = f64.reshape(3, H, W)
        for f in range(3):
            rel = np.abs(a[f] - b[f]) / np.maximum(np.abs(b[f]), 1e-3 * ext[f])
            assert rel.max() <= 1e-5
        assert not np.array_equal(f32.reshape(3, H, W), fld)  # something diffused


def test_batch_deterministic_and_chunk_invariant(params, oracle):
    from emt6ro import workloads as wl
    tum = wl.disc_tumor(params, 9, seed=1)
    dose = wl.protocol_doses([[(200, 2.0), (900, 1.5)]], 480)[0]

    def run(chunks, threads):
        b = oracle.Batch(oracle.params_copy(params.native), 3, seed=42)
        for i in range(3):
            b.set(i, tum.sites, dose)
        for c in chunks:
            b.run(c, nthreads=threads)
        return [b.get(i).tobytes() for i in range(3)], b.counts()

    s1, c1 = run([1000], 1)
    s2, c2 = run([37, 91, 128, 744], 3)
    assert s1 == s2 and (c1 == c2).all()
    b = oracle.Batch(oracle.params_copy(params.native), 1, seed=43)
    b.set(0, tum.sites, dose)
    b.run(1000)
    assert b.get(0).tobytes() != s1[0]  # another seed, another trajectory


def test_instrumentation_counters(params, oracle):
    from emt6ro import workloads as wl
    tum = wl.disc_tumor(params, 10, seed=2)
    dose = wl.protocol_doses([[(0, 3.0)]], 480)[0]
    b = oracle.Batch(oracle.params_copy(params.native), 2, seed=1)
    for i in range(2):
        b.set(i, tum.sites, dose)
    b.run(6000, nthreads=2)
    ins, hist = b.instr()
    n0 = int((tum.occupancy() == 1).sum())
    assert ins.irradiation_events >= 2 * 0.9 * n0
    assert ins.repair_decisions > 0 and ins.repair_kills <= ins.repair_decisions
    assert hist[:300].sum() == ins.repair_decisions == hist[300:].sum()
    assert ins.divisions > 0
