"""Host logic of the protocol-file replay (emt6ro.replay) without a GPU: a
stand-in batch returns each simulation's global index as its count, so the
chunking, the index bases and the results layout (one row per protocol,
tumour-major then run-major) are checked exactly."""
import json

import numpy as np


class _IndexBatch:
    """Records its arguments; counts() gives base + local index."""
    made = []

    def __init__(self, params, tumors, protocols, sim_tumor, sim_protocol, **kw):
        self.n = len(sim_tumor)
        self.protocols, self.sim_tumor, self.sim_protocol, self.kw = (
            protocols, np.asarray(sim_tumor), np.asarray(sim_protocol), kw)
        self.base, self.steps = 0, 0
        _IndexBatch.made.append(self)

    def set_index_base(self, base):
        self.base = base

    def run(self, n):
        self.steps += n

    def counts(self):
        return (self.base + np.arange(self.n)).astype(np.uint32)


def test_chunks_cover_the_file_with_global_indices(monkeypatch):
    import emt6ro.batch
    from emt6ro import replay as R
    monkeypatch.setattr(emt6ro.batch, "Batch", _IndexBatch)
    _IndexBatch.made = []
    prots = [[(300 * k, 1.0)] for k in range(7)]
    out = R.replay(None, ["t0", "t1", "t2"], prots, reps=4, steps=3000, seed=5, protocol_chunk=3)
    assert out.shape == (7, 3, 4)
    assert np.array_equal(out.reshape(-1), np.arange(7 * 3 * 4))  # (p, t, r) -> p*T*M + t*M + r
    assert [b.base for b in _IndexBatch.made] == [0, 36, 72]
    assert [len(b.protocols) for b in _IndexBatch.made] == [3, 3, 1]
    b = _IndexBatch.made[1]
    assert b.protocols == prots[3:6] and b.steps == 3000 and b.kw["seed"] == 5
    assert b.kw["protocol_length"] == 3000 and b.kw["protocol_resolution"] == 300
    assert b.sim_tumor.tolist() == [0] * 4 + [1] * 4 + [2] * 4 + [0] * 4 + [1] * 4 + [2] * 4 + \
        [0] * 4 + [1] * 4 + [2] * 4
    assert b.sim_protocol.tolist() == [0] * 12 + [1] * 12 + [2] * 12
    # the default chunk holds about 200,000 simulations
    _IndexBatch.made = []
    R.replay(None, ["t"] * 10, [[]] * 450, reps=100, steps=10, seed=1)
    assert [len(b.protocols) for b in _IndexBatch.made] == [200, 200, 50]


def test_results_rows_and_metadata(monkeypatch, tmp_path, params):
    import emt6ro.batch
    import emt6ro.simulation as sim
    from emt6ro import protocols as P, replay as R, workloads as wl
    monkeypatch.setattr(emt6ro.batch, "Batch", _IndexBatch)
    paths = []
    for k in range(2):
        paths.append(tmp_path / f"tumor-{k}.txt")
        sim.save_state(wl.disc_tumor(params, 5 + k, seed=k), paths[-1])
    P.write_protocols([[(301, 1.0)], [(1, 2.0), (601, 1.0)], [(900, 3.0)]], tmp_path / "p.txt")
    pj = tmp_path / "params.json"
    subs = {"cho": 1, "ox": 1, "gi": 1}
    pj.write_text(json.dumps({
        "lattice_dims": {"height": 51, "width": 51}, "time_step": 6,
        "diffusion_params": {"coeffs": subs, "time_step": 0.25},
        "metabolism": {k: subs for k in ("aerobic_proliferation", "anaerobic_proliferation",
                                         "aerobic_quiescence", "anaerobic_quiescence")},
        "external_levels": subs, "death_gi": 1, "quiescence_gi": 1, "death_gi_production": 1,
        "cycle_times": {k: {"mean": 1, "stddev": 1} for k in ("g1", "s", "g2", "m", "d")},
        "cell_repair": {"delay_time": {"coeff": 1, "exp_coeff": 1},
                        "survival_prob": {"coeff": 1, "exp_coeff": 1}, "repair_half_time": 1}}))
    _IndexBatch.made = []
    assert R.main(["--protocols", str(tmp_path / "p.txt"), "--tumors", *map(str, paths),
                   "--params", str(pj), "--reps", "3", "--steps", "1200",
                   "--out", str(tmp_path / "out" / "r.txt"), "--limit-protocols", "2"]) == 0
    rows = (tmp_path / "out" / "r.txt").read_text().splitlines()
    assert rows == [" ".join(map(str, range(6 * p, 6 * p + 6))) for p in range(2)]
    # 1-indexed steps were shifted onto the grid before the batch saw them
    assert _IndexBatch.made[0].protocols == [[(300, 1.0)], [(0, 2.0), (600, 1.0)]]
    meta = json.loads((tmp_path / "out" / "r.txt.meta.json").read_text())
    assert meta["n_protocols"] == 2 and meta["n_tumors"] == 2 and meta["reps_per_tumor"] == 3
    assert isinstance(meta["seed"], int) and meta["seed"] == _IndexBatch.made[0].kw["seed"]


def test_ranges_that_split_protocols_and_device_waves(monkeypatch):
    import emt6ro.batch
    from emt6ro import replay as R
    monkeypatch.setattr(emt6ro.batch, "Batch", _IndexBatch)
    prots = [[(300 * k, 1.0)] for k in range(5)]
    for spb in (1, 7, 12, 13, 1000):
        for devices in (None, [0, 1], [3, 1, 2]):
            _IndexBatch.made = []
            out = R.replay(None, ["a", "b", "c"], prots, reps=4, steps=600, seed=2,
                           sims_per_batch=spb, devices=devices)
            assert np.array_equal(out.reshape(-1), np.arange(60)), (spb, devices)
            for b in _IndexBatch.made:
                g = b.base + np.arange(b.n)
                first = b.base // 12
                assert b.protocols == prots[first:(g[-1] // 12) + 1]
                assert np.array_equal(b.sim_protocol, g // 12 - first)
                assert np.array_equal(b.sim_tumor, (g % 12) // 4)
            devs = [b.kw["device"] for b in _IndexBatch.made]
            want = devices or [0]
            assert devs == [want[k % len(want)] for k in range(len(devs))]


def _gloo_worker(rank, world, port, q):
    import os
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import emt6ro.batch
    from emt6ro import replay as R
    emt6ro.batch.Batch = _IndexBatch
    prots = [[(300 * k, 1.0)] for k in range(5)]
    out = R.replay(None, ["a", "b", "c"], prots, reps=4, steps=600, sims_per_batch=7,
                   process_group=dist.group.WORLD)  # seed drawn on rank 0
    q.put((rank, out.reshape(-1).tolist(), [b.base for b in _IndexBatch.made],
           {b.kw["seed"] for b in _IndexBatch.made}))
    dist.barrier()
    dist.destroy_process_group()


def test_replay_over_a_process_group():
    """World size 2 over gloo: each rank runs its contiguous half of the 60
    simulations and both get the whole array back."""
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == list(range(60)) and res[1][1] == list(range(60))
    assert res[0][2] == [0, 7, 14, 21, 28] and res[1][2] == [30, 37, 44, 51, 58]
    assert len(res[0][3]) == 1 and res[0][3] == res[1][3]  # one seed on both ranks
