"""The multi-GPU host logic on CPU: world size 2 over gloo.  Each rank takes a
contiguous shard of the simulations (no data-path collective), the step time
is the max over ranks (bench.py), and the per-simulation counts are gathered
over the group (emt6ro.ga_model.sharding, used by EMT6RoModel under
torch.distributed).  The simulations of a shard run on the CPU oracle here,
keyed by their global index like the GPU batches (emt6_batch_set_index_base),
so the gathered counts must equal a single-rank run of the whole set."""
import os
import socket


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    lo, hi = bench.shard_range(40000, rank, world)
    t = torch.tensor([float(rank + 1) * 1.5])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([hi - lo])
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    q.put((rank, lo, hi, float(t.item()), int(n.item())))
    dist.barrier()
    dist.destroy_process_group()


def test_shards_cover_and_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1:3] == (0, 20000) and res[1][1:3] == (20000, 40000)
    assert all(r[3] == 3.0 for r in res)      # max over ranks
    assert all(r[4] == 40000 for r in res)    # every simulation once


def test_shard_range_partitions():
    import bench
    for total in (1, 7, 40000, 30001):
        for world in (1, 2, 3, 8):
            parts = [bench.shard_range(total, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))


def _simulations():
    """12 small simulations: 3 tumours x 2 protocols x 2 replicates."""
    from emt6ro import workloads as wl
    params = wl.default_parameters()
    tumors = [wl.disc_tumor(params, r, seed=r) for r in (3, 5, 7)]
    doses = wl.protocol_doses([[(0, 2.0)], [(150, 4.0), (300, 1.0)]], 480)
    sims = [(t, p) for p in range(2) for t in range(3) for _ in range(2)]
    return params, tumors, doses, sims


def _oracle_counts(lo, hi, steps=4000):
    from oracle import pyoracle as po
    params, tumors, doses, sims = _simulations()
    b = po.Batch(po.params_copy(params.native), hi - lo, seed=11)
    for k, i in enumerate(range(lo, hi)):
        t, p = sims[i]
        b.set(k, tumors[t].sites, doses[p], sim_index=i)
    b.run(steps, nthreads=2)
    return b.counts()


def _gather_worker(rank, world, port, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    for p in (root / "emt6-ro_gb300", root):
        if str(p) not in sys.path:
            sys.path.insert(0, str(p))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from emt6ro.ga_model.sharding import gather_shards, shard_range
    total = len(_simulations()[3])
    lo, hi = shard_range(total, rank, world)
    local = _oracle_counts(lo, hi)
    q.put((rank, lo, hi, gather_shards(local, total).tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_simulations_gather_to_the_single_rank_result():
    import multiprocessing as mp
    from oracle import pyoracle as po
    po.oracle()  # build before the workers start
    whole = _oracle_counts(0, 12)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gather_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1:3] for r in res] == [(0, 6), (6, 12)]
    for r in res:
        assert r[3] == whole.tolist()
    # the shards differ from each other (the gather is not trivially equal)
    assert whole[:6].tolist() != whole[6:].tolist()


def test_shard_range_matches_bench():
    import bench
    from emt6ro.ga_model.sharding import shard_range
    for total in (1, 7, 40000):
        for world in (1, 2, 3, 8):
            assert all(bench.shard_range(total, r, world) == shard_range(total, r, world)
                       for r in range(world))


class _FakeShard:
    """Stands in for a GPU batch: the count of global simulation g is g plus
    ten times its protocol's total dose; records the seed it was given."""

    def __init__(self, params, tumors, protocols, sim_tumor, sim_protocol, **kw):
        self.sim_protocol = list(sim_protocol)
        self.kw, self.base, self.doses = kw, 0, None

    def set_index_base(self, base):
        self.base = base

    def set_schedule(self, *a):
        pass

    def add_irradiations(self, protocols):
        self.doses = [sum(d for _, d in p) for p in protocols]

    def run(self, n):
        pass

    def counts(self):
        import numpy as np
        return np.array([self.base + i + int(10 * self.doses[p])
                         for i, p in enumerate(self.sim_protocol)], np.uint32)

    def reset(self):
        self.doses = None


_PROTOCOLS = [[(0, 1.0)], [(300, 2.5), (600, 0.5)], [], [(900, 4.0)]]


def _model_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import emt6ro.ga_model.model as M
    M.Batch = _FakeShard
    m = M.EMT6RoModel(None, ["t0", "t1"], num_protocols=4, num_tests=3,
                      process_group=dist.group.WORLD)  # seed drawn on rank 0
    fit = m.predict(_PROTOCOLS)
    q.put((rank, fit.tolist(), m.seed, [b.kw["seed"] for _, _, b in m.shards]))
    dist.barrier()
    dist.destroy_process_group()


def test_model_over_a_process_group_shares_one_seed_and_gathers():
    """EMT6RoModel under torch.distributed (world size 2, gloo): both ranks
    use rank 0's seed, each runs its contiguous shard, and the fitness equals
    one process holding both shards."""
    import multiprocessing as mp
    import emt6ro.ga_model.model as M
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_model_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == res[1][1]
    assert res[0][2] == res[1][2] and res[0][3] == [res[0][2]] and res[1][3] == [res[0][2]]
    orig = M.Batch
    try:
        M.Batch = _FakeShard
        one = M.EMT6RoModel(None, ["t0", "t1"], num_protocols=4, num_tests=3, devices=[0, 1],
                            seed=res[0][2])
        assert one.predict(_PROTOCOLS).tolist() == res[0][1]
    finally:
        M.Batch = orig
