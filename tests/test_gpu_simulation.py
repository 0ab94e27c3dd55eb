"""Whole-simulation parity: the fused CUDA step kernels vs the CPU oracle,
bit-exact on every lattice field and on the living counts, across the list
rebuild (128 steps) and ROI (32 steps) cadences, irradiation, chunked runs,
resets, regions that need the wide kernel, ragged horizons and the
work-queue schedule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_pair(params, oracle, tumors, protocols, sim_tumor, sim_protocol, steps, seed,
              horizon=None, chunks=None, schedule=0, epoch=0):
    from emt6ro.batch import Batch
    b = Batch(params, tumors, protocols, sim_tumor, sim_protocol, sim_horizon=horizon, seed=seed)
    if schedule:
        b.set_schedule(schedule, 0)
    for c in (chunks or [steps]):
        b.run(c)
    counts = b.counts()
    n = len(sim_tumor)
    ob = oracle.Batch(oracle.params_copy(params.native), n, seed)
    for i in range(n):
        hz = 0xFFFFFFFF if horizon is None else int(horizon[i])
        ob.set(i, tumors[sim_tumor[i]].sites, b.doses[sim_protocol[i]], resolution=300,
               length=144_000, epoch=epoch, horizon=hz)
    ob.run(steps, nthreads=8)
    return b, ob, counts, ob.counts()


def _assert_same(b, ob, n):
    for i in range(n):
        g = b.state(i).sites
        o = ob.get(i)
        if g.tobytes() != o.tobytes():
            bad = [f for f in g.dtype.names if np.ascontiguousarray(g[f]).tobytes()
                   != np.ascontiguousarray(o[f]).tobytes()]
            raise AssertionError(f"simulation {i}: fields {bad} differ from the oracle")


def test_small_batch_bit_exact(params, oracle):
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, r, seed=s) for r, s in ((5, 1), (9, 2), (12, 3))]
    protocols = [[], [(600, 1.25), (1500, 2.5)], [(0, 5.0)]]
    st = np.array([0, 1, 2, 0, 1, 2, 2, 1], np.int32)
    sp = np.array([0, 1, 2, 1, 2, 0, 1, 2], np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 2000, seed=77)
    assert (c == co).all(), (c, co)
    _assert_same(b, ob, len(st))


def test_tumours_against_the_lattice_edge_bit_exact(params, oracle):
    """Tumours in a corner and against the edges: clipped ROIs (even-sized
    regions, ring sites left free by the mask), divisions next to the mocked
    border, and regions that leave the narrow kernel for the wide one."""
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, 7, seed=11, center=(6, 6)),
              wl.disc_tumor(params, 10, seed=12, center=(26, 3)),
              wl.disc_tumor(params, 14, seed=13, center=(45, 30)),
              wl.disc_tumor(params, 18, seed=14, center=(26, 8))]
    protocols = [[], [(300, 2.0), (900, 1.5)]]
    st = np.array([0, 1, 2, 3, 0, 1, 2, 3], np.int32)
    sp = np.array([0, 0, 0, 0, 1, 1, 1, 1], np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 1500, seed=91)
    assert (c == co).all(), (c, co)
    _assert_same(b, ob, len(st))


@pytest.mark.parametrize("dims", [(40, 47), (54, 60)])
def test_other_lattice_sizes_bit_exact(oracle, dims):
    """Interiors other than 51 x 51, up to the largest the kernels hold
    (54 x 60): a non-square lattice, a tumour against its edge and one whose
    region needs the wide kernel."""
    from emt6ro import workloads as wl
    p = wl.default_parameters()
    p.native.lattice_height, p.native.lattice_width = dims
    H, W = dims[0] + 2, dims[1] + 2
    tumors = [wl.disc_tumor(p, 9, seed=21, center=(H // 2, W // 2)),
              wl.disc_tumor(p, 8, seed=22, center=(H // 2, 3)),
              wl.disc_tumor(p, 19, seed=23, center=(H // 2, W // 2))]
    protocols = [[], [(120, 2.5)]]
    st = np.array([0, 1, 2, 0, 1, 2], np.int32)
    sp = np.array([0, 0, 0, 1, 1, 1], np.int32)
    b, ob, c, co = _run_pair(p, oracle, tumors, protocols, st, sp, 600, seed=57)
    assert (c == co).all(), (c, co)
    _assert_same(b, ob, len(st))


def test_empty_and_single_cell_lattices_bit_exact(params, oracle):
    """No cell at all (empty list, 0 x 0 ROI from the first step) and a single
    cell in a corner and in the middle (3 x 3 regions), irradiated or not."""
    from emt6ro import workloads as wl
    import emt6ro.simulation as sim
    empty = wl.disc_tumor(params, 0, seed=41).sites.copy()
    empty["state"][1:-1, 1:-1] = 0
    corner = wl.disc_tumor(params, 0, seed=42, center=(1, 1))
    middle = wl.disc_tumor(params, 0, seed=43)
    tumors = [sim.TumorState(empty), corner, middle]
    protocols = [[], [(0, 3.0)]]
    st = np.array([0, 1, 2, 0, 1, 2], np.int32)
    sp = np.array([0, 0, 0, 1, 1, 1], np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 3000, seed=23)
    assert (c == co).all(), (c, co)
    assert c[0] == 0 and c[3] == 0
    _assert_same(b, ob, len(st))


def test_chunked_runs_equal_one_run(params, oracle):
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, 10, seed=9)]
    protocols = [[(300, 2.0), (1200, 2.0)]]
    st = np.zeros(4, np.int32)
    sp = np.zeros(4, np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 1500, seed=5,
                             chunks=[1, 31, 96, 100, 500, 772])
    assert (c == co).all()
    _assert_same(b, ob, 4)


def test_wide_regions_bit_exact(params, oracle):
    """Tumours whose region exceeds 32 x 31 run on the 384-thread kernel."""
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, 17, seed=11), wl.disc_tumor(params, 22, seed=12),
              wl.disc_tumor(params, 14, seed=13, center=(20, 30))]
    protocols = [[(0, 2.0), (600, 2.0)]]
    st = np.array([0, 1, 2, 1], np.int32)
    sp = np.zeros(4, np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 700, seed=21)
    assert (c == co).all()
    _assert_same(b, ob, 4)


def test_33_wide_regions_bit_exact(params, oracle):
    """Unclipped 31-wide ROIs (33 x 33 regions) run on the narrow kernel with
    the shifted mapping; a clipped one near the edge falls back to the wide
    kernel; both match the oracle bit for bit."""
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, r, seed=40 + r) for r in (13, 14, 15)]
    tumors.append(wl.disc_tumor(params, 14, seed=44, center=(15, 26)))
    protocols = [[(0, 1.5), (700, 2.0)]]
    st = np.array([0, 1, 2, 3, 1, 0], np.int32)
    sp = np.zeros(6, np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 1100, seed=31)
    assert (c == co).all()
    _assert_same(b, ob, 6)


def test_35_wide_regions_bit_exact(params, oracle):
    """Unclipped ROIs of distance 16 (35 x 35 regions, every free site in
    rows and columns 1..32) run on the narrow kernel with the ring mapping
    (the block in registers, the final substep of the ROI's last row and
    column as a separate pass); regions whose first row is fixed use the
    row-shifted half-warp bands (25, 29 rows); a tumour clipped by the
    lattice edge keeps the general layouts.  All match the oracle bit for
    bit over launches that cross ROI updates and list rebuilds."""
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, r, seed=50 + r) for r in (11, 15, 16)]
    tumors.append(wl.disc_tumor(params, 16, seed=57, center=(26, 16)))
    protocols = [[(0, 1.0)], [(300, 3.0), (900, 2.0)]]
    st = np.array([0, 1, 2, 3, 2, 1, 2], np.int32)
    sp = np.array([0, 0, 0, 0, 1, 1, 1], np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 1500, seed=35)
    assert (c == co).all()
    _assert_same(b, ob, 7)


def test_growing_and_shrinking_discs_bit_exact(params, oracle):
    """Unclipped tumours of radius 3 to 14 whose regions change size as they
    grow and die back after irradiation, crossing the narrow kernel's layouts
    (eight-lane and half-warp bands, row-shifted mappings): bit-exact against
    the oracle."""
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, r, seed=70 + r) for r in (3, 4, 7, 8, 10, 12, 14)]
    protocols = [[(0, 2.0)], [(600, 5.0)]]
    st = np.array([0, 1, 2, 3, 4, 5, 6, 3, 5, 6], np.int32)
    sp = np.array([0, 0, 0, 0, 0, 0, 0, 1, 1, 1], np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 2000, seed=41)
    assert (c == co).all()
    _assert_same(b, ob, 10)


def test_ragged_horizons_and_queue(params, oracle):
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, r, seed=30 + r) for r in (2, 7, 18)]
    protocols = [[], [(100, 3.0)], [(50, 1.0), (400, 1.0), (800, 1.0)]]
    st = np.array([0, 1, 2, 1, 2, 0], np.int32)
    sp = np.array([1, 2, 0, 0, 1, 2], np.int32)
    hz = np.array([100, 900, 450, 1000, 33, 700], np.uint32)
    for sched in (0, 1):
        b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 1000, seed=3,
                                 horizon=hz, schedule=sched)
        assert (c == co).all()
        _assert_same(b, ob, len(st))
        for i in range(len(st)):
            assert b.step(i) == min(1000, int(hz[i]))


def test_graph_replay_and_queue_bit_exact(params, oracle):
    """CUDA-graph replay of the launch sequence (schedule bit 1), with and
    without the work queue, gives the oracle's states; a reset and rerun
    replays a re-captured graph (new epoch)."""
    from emt6ro import workloads as wl
    from emt6ro.batch import Batch
    tumors = [wl.disc_tumor(params, r, seed=60 + r) for r in (6, 11, 16)]
    protocols = [[(0, 2.0)], [(300, 1.0), (600, 1.0)]]
    st = np.array([0, 1, 2, 2, 1, 0], np.int32)
    sp = np.array([0, 1, 0, 1, 0, 1], np.int32)
    hz = np.array([900, 500, 900, 700, 300, 900], np.uint32)
    for mode in (2, 3):
        b = Batch(params, tumors, protocols, st, sp, sim_horizon=hz, seed=12)
        b.set_schedule(mode, 256)
        b.run(900)
        ob = oracle.Batch(oracle.params_copy(params.native), 6, 12)
        for i in range(6):
            ob.set(i, tumors[st[i]].sites, b.doses[sp[i]], horizon=int(hz[i]))
        ob.run(900, nthreads=6)
        _assert_same(b, ob, 6)
        b.reset()
        b.set_doses(b.doses)
        b.run(900)
        ob2 = oracle.Batch(oracle.params_copy(params.native), 6, 12)
        for i in range(6):
            ob2.set(i, tumors[st[i]].sites, b.doses[sp[i]], horizon=int(hz[i]), epoch=1)
        ob2.run(900, nthreads=6)
        _assert_same(b, ob2, 6)
        assert b.launches() > 0


def test_reset_gives_fresh_epoch(params, oracle):
    from emt6ro import workloads as wl
    from emt6ro.batch import Batch
    tumors = [wl.disc_tumor(params, 9, seed=2)]
    protocols = [[(60, 2.5)]]
    st = np.zeros(3, np.int32)
    sp = np.zeros(3, np.int32)
    b = Batch(params, tumors, protocols, st, sp, seed=99)
    b.run(400)
    first = [b.state(i).sites.copy() for i in range(3)]
    b.reset()
    assert b.state(0).sites.tobytes() == tumors[0].sites.tobytes()
    b.set_doses(b.doses)
    b.run(400)
    ob = oracle.Batch(oracle.params_copy(params.native), 3, 99)
    for i in range(3):
        ob.set(i, tumors[0].sites, b.doses[0], epoch=1)
    ob.run(400, nthreads=3)
    _assert_same(b, ob, 3)
    assert any(first[i].tobytes() != b.state(i).sites.tobytes() for i in range(3))


def test_diffused_counter_matches_oracle(params, oracle):
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, 11, seed=4)]
    st = np.zeros(2, np.int32)
    sp = np.zeros(2, np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, [[]], st, sp, 300, seed=8)
    assert b.diffused() == ob.diffused()


def test_summary_and_timelapse_match_oracle_states(params, oracle):
    """Device-side summaries (centre substrates, living cells, cells per mode
    and per phase) equal the same quantities computed from the oracle's
    lattices at every recorded step."""
    from emt6ro import workloads as wl
    from emt6ro.batch import Batch
    tumors = [wl.disc_tumor(params, 9, seed=71), wl.disc_tumor(params, 12, seed=72)]
    protocols = [[(300, 2.0)], []]
    st = np.array([0, 1, 1], np.int32)
    sp = np.array([0, 0, 1], np.int32)
    b = Batch(params, tumors, protocols, st, sp, seed=17)
    rec = b.timelapse(900, every=300)
    assert rec.shape == (3, 3, 13)
    ob = oracle.Batch(oracle.params_copy(params.native), 3, 17)
    for i in range(3):
        ob.set(i, tumors[st[i]].sites, b.doses[sp[i]])
    for k in range(3):
        ob.run(300, nthreads=3)
        for i in range(3):
            s = ob.get(i).reshape(53, 53)
            occ = s["state"] == 1
            want = [s["cho"][26, 26], s["ox"][26, 26], s["gi"][26, 26], occ.sum()]
            want += [(s["mode"][occ] == m).sum() for m in range(4)]
            want += [(s["phase"][occ] == ph).sum() for ph in range(5)]
            assert np.array_equal(rec[k, i], np.array(want, np.float32)), (k, i)


def test_autotuner_picks_a_schedule_that_changes_nothing_but_time(params):
    """The autotuner times (schedule mode, steps per launch) candidates, then
    tile-shape sets with the fastest launch, on a sample, and returns the
    fastest; any schedule and tile-shape set it can pick gives the same
    lattices as the default one."""
    from emt6ro import autotune, workloads as wl
    from emt6ro.batch import Batch
    tumors = [wl.disc_tumor(params, r, seed=80 + r) for r in (5, 9, 13)]
    protocols = [[(60, 2.0)], [(0, 1.0), (120, 1.0)]]
    st = np.arange(24, dtype=np.int32) % 3
    sp = np.arange(24, dtype=np.int32) % 2
    hz = np.where(np.arange(24) % 4 == 0, 150, 300).astype(np.uint32)
    mode, chunk, lay, table = autotune.tune(params, tumors, protocols, st, sp, hz, sample=12,
                                            trial_steps=64, warm_steps=16, chunks=(32, 64),
                                            modes=(0, 1, 2, 3), layouts=(0, 3, 7))
    assert len(table) == 10 and (mode, chunk, lay) in [(m, c, y) for m, c, y, _ in table]
    ref = Batch(params, tumors, protocols, st, sp, sim_horizon=hz, seed=5)
    ref.run(300)
    tuned = Batch(params, tumors, protocols, st, sp, sim_horizon=hz, seed=5)
    tuned.set_schedule(mode, chunk)
    tuned.set_layouts(lay)
    tuned.run(300)
    for i in range(24):
        assert tuned.state(i).sites.tobytes() == ref.state(i).sites.tobytes()


@pytest.mark.parametrize("layouts", range(8))
def test_every_tile_shape_set_bit_exact(params, oracle, layouts):
    """Each subset of the optional tile shapes (eight-lane bands, wide
    three-column bands, the 35 x 35 ring mapping) gives the oracle's lattices
    bit for bit on tumours whose regions need each of them (small, 35 x 35,
    41-48-row and 49 x 49 regions)."""
    from emt6ro import workloads as wl
    from emt6ro.batch import Batch
    tumors = [wl.disc_tumor(params, r, seed=90 + r) for r in (6, 16, 20, 23)]
    protocols = [[(0, 1.5)]]
    st = np.array([0, 1, 2, 3], np.int32)
    sp = np.zeros(4, np.int32)
    b = Batch(params, tumors, protocols, st, sp, seed=17)
    b.set_layouts(layouts)
    b.run(700)
    ob = oracle.Batch(oracle.params_copy(params.native), 4, 17)
    for i in range(4):
        ob.set(i, tumors[st[i]].sites, b.doses[sp[i]], resolution=300, length=144_000)
    ob.run(700, nthreads=4)
    assert (b.counts() == ob.counts()).all()
    _assert_same(b, ob, 4)


def test_one_day_bit_exact(params, oracle):
    """A full simulated day (14,400 steps): tumours of radius 6, 10 and 14
    under GA-like protocols (doses from hour 2 to hour 20) and none, through
    growth, irradiation, repair, deaths and regrowth, across the narrow
    kernel's layouts and into the wide kernel: every site of every simulation
    bit-identical to the oracle."""
    from emt6ro import workloads as wl
    tumors = [wl.disc_tumor(params, r, seed=90 + r) for r in (6, 10, 14)]
    protocols = [[], [(1200, 2.5), (4800, 2.5), (9000, 2.5), (12000, 2.5)],
                 [(3000, 1.25), (6600, 1.25)]]
    st = np.array([0, 1, 2, 0, 1, 2], np.int32)
    sp = np.array([0, 0, 0, 1, 2, 1], np.int32)
    b, ob, c, co = _run_pair(params, oracle, tumors, protocols, st, sp, 14_400, seed=1440,
                             chunks=[600] * 24)
    assert (c == co).all(), (c, co)
    _assert_same(b, ob, len(st))
