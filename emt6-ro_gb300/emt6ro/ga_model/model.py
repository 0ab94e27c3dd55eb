"""Fitness model of irradiation protocols, the reference's EMT6RoModel API
(python/emt6ro/ga_model/model.py:5-54) over persistent sharded batches.

fitness(protocol) = 1500 - mean final living-cell count over the tumours and
every replicate.

The reference keeps one Experiment per GPU, each running all protocols x
tumours x num_tests and reset after every generation.  Here a generation's
num_protocols x tumours x (num_tests x GPUs) simulations form one index
space, ordered (protocol, tumour, replicate), cut into contiguous shards, one
per GPU (emt6ro.ga_model.sharding).  Each shard is one Batch created once and
reused by every generation: predict uploads the population's doses, runs the
whole horizon as persistent CTAs taking simulations from the device work
queue, gathers the counts and resets the states for the next generation.
Random streams are keyed by the global simulation index
(emt6_batch_set_index_base), so for a given seed the fitness does not depend
on how the population is sharded, and on one GPU it equals that of an
Experiment with the same seed.  Under torch.distributed (process_group), each
process owns the shard of its rank and the counts are gathered over the
group.
"""
from __future__ import annotations

import os

import numpy as np

from ..batch import Batch
from .sharding import gather_shards, shard_range

# persistent CTAs over the device work queue, 2400 steps per launch (the
# schedule the launch autotuner picks for full-horizon batches)
DEFAULT_SCHEDULE = (1, 2400)


class EMT6RoModel:
    """
    params, tumors   as for simulation.Experiment
    num_protocols    population size evaluated by each predict call
    num_tests        replicates of each protocol x tumour per GPU (the
                     reference's meaning: total replicates = num_tests x GPUs)
    num_gpus         GPUs 0 .. num_gpus - 1, one shard each
    devices          explicit device per shard instead of range(num_gpus)
                     (the same device may hold several shards)
    process_group    torch.distributed group: this process holds the shard of
                     its rank on `devices[0]` (default: LOCAL_RANK), the
                     counts are gathered over the group
    seed             random-stream seed (default: drawn from the OS)
    """

    def __init__(self, params, tumors, num_protocols, num_tests, num_gpus=1, num_steps=144000,
                 protocol_resolution=300, seed=None, devices=None, process_group=None,
                 schedule=DEFAULT_SCHEDULE):
        self.params = params
        self.tumors = tumors
        self.num_protocols = int(num_protocols)
        self.num_tests = int(num_tests)
        self.num_steps = int(num_steps)
        self.protocol_resolution = int(protocol_resolution)
        self.group = process_group
        if process_group is not None:
            import torch.distributed as dist
            world, rank = dist.get_world_size(process_group), dist.get_rank(process_group)
            dev = devices[0] if devices else int(os.environ.get("LOCAL_RANK", 0))
            placement = [(rank, dev)]
        else:
            devs = list(devices) if devices is not None else list(range(int(num_gpus)))
            world = len(devs)
            placement = list(enumerate(devs))
        if world < 1:
            raise ValueError("at least one GPU is required")
        self.num_gpus = world
        self.replicates = self.num_tests * world
        T, R = len(tumors), self.replicates
        self.total = self.num_protocols * T * R
        idx = np.arange(self.total, dtype=np.int64)
        sim_protocol = (idx // (T * R)).astype(np.int32)
        sim_tumor = ((idx // R) % T).astype(np.int32)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        if process_group is not None:
            # every rank draws with rank 0's seed: one index space, one seed
            import torch.distributed as dist
            box = [int(seed)]
            dist.broadcast_object_list(box, src=dist.get_global_rank(process_group, 0)
                                       if hasattr(dist, "get_global_rank") else 0,
                                       group=process_group)
            seed = box[0]
        self.seed = int(seed)
        empty = [[] for _ in range(self.num_protocols)]
        self.shards = []
        for rank, dev in placement:
            lo, hi = shard_range(self.total, rank, world)
            if hi == lo:
                continue
            b = Batch(params, tumors, empty, sim_tumor[lo:hi], sim_protocol[lo:hi],
                      protocol_resolution=self.protocol_resolution, protocol_length=self.num_steps,
                      device=dev, seed=self.seed)
            b.set_index_base(lo)
            b.set_schedule(*schedule)
            self.shards.append((lo, hi, b))

    def predict(self, protocols):
        """
        Returns fitness of each protocol.

        protocols: list of lists of pairs (simulation step, irradiation dose)
        """
        assert len(protocols) == self.num_protocols
        # every shard is started before any count is read: the GPUs run together
        for _, _, b in self.shards:
            b.add_irradiations(protocols)
            b.run(self.num_steps)
        if self.group is None:
            counts = np.concatenate([b.counts() for _, _, b in self.shards])
        else:
            local = np.concatenate([b.counts() for _, _, b in self.shards]) if self.shards \
                else np.zeros(0, np.uint32)
            counts = gather_shards(local, self.total, self.group)
        for _, _, b in self.shards:
            b.reset()
        results = counts.reshape(self.num_protocols, -1).mean(1)
        return 1500 - results
