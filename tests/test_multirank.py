"""The multi-GPU host logic of bench.py on CPU: world size 2 over gloo.  Each
rank takes a contiguous shard of the simulations (no data-path collective) and
the step time is the max over ranks."""
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
