"""Contiguous shards of a simulation index space and their host gather.

Every simulation is independent (no exchange step), so several GPUs split a
batch into contiguous slices and the only collective is a gather of the
per-simulation living counts, as the reference's multi-GPU fitness model
concatenates its per-GPU results (python/emt6ro/ga_model/model.py:48-50).
"""
from __future__ import annotations

import numpy as np


def shard_range(total: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous slice [lo, hi) of `total` units for `rank` of `world`: the
    first total % world ranks take one unit more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(int(total), world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def gather_shards(local: np.ndarray, total: int, group=None) -> np.ndarray:
    """Every rank's contiguous shard of a (total,) uint32 array, concatenated
    in rank order on every rank (torch.distributed all_gather; works on the
    gloo and nccl backends).  `local` holds this rank's shard_range slice."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = shard_range(total, rank, world)
    local = np.ascontiguousarray(local, np.uint32).reshape(-1)
    if local.size != hi - lo:
        raise ValueError(f"rank {rank} holds {local.size} values, its shard is {hi - lo}")
    cap = shard_range(total, 0, world)[1]  # the first shard is the largest
    buf = torch.zeros(cap, dtype=torch.int64)
    buf[:local.size] = torch.from_numpy(local.astype(np.int64))
    if dist.get_backend(group) == "nccl":
        buf = buf.cuda()
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    out = np.empty(total, np.uint32)
    for r, part in enumerate(parts):
        a, b = shard_range(total, r, world)
        out[a:b] = part[:b - a].cpu().numpy().astype(np.uint32)
    return out
