"""Batch engine: any mix of tumours x protocols x horizons on one GPU
(emt6_batch_* in include/emt6ro_gb300.h; replaces the reference's Simulation
class, src/emt6ro/simulation/simulation.h:13-114)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _native as N
from .simulation.backend import Parameters, TumorState, _stack_tumors
from .workloads import protocol_doses


class Batch:
    def __init__(self, params: Parameters, tumors, protocols, sim_tumor, sim_protocol,
                 sim_horizon=None, protocol_resolution: int = 300,
                 protocol_length: int = 144_000, device: int = 0, seed: int | None = None):
        stack, (H, W) = _stack_tumors(tumors)
        self.H, self.W = H, W
        self.params = params
        self.n = int(len(sim_tumor))
        self.resolution = int(protocol_resolution)
        self.length = int(protocol_length)
        self.bins = (self.length + self.resolution - 1) // self.resolution
        self.n_protocols = len(protocols)
        self.device = int(device)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        st = np.ascontiguousarray(sim_tumor, np.int32)
        sp = np.ascontiguousarray(sim_protocol, np.int32)
        hz = None if sim_horizon is None else np.ascontiguousarray(sim_horizon, np.uint32)
        self._h = ctypes.c_void_p()
        N.check(N.lib().emt6_batch_create(
            ctypes.byref(params.native), N.ptr(stack), len(tumors), H, W, self.n_protocols,
            self.bins, self.resolution, self.length, self.n, N.ptr(st), N.ptr(sp), N.ptr(hz),
            self.device, self.seed, ctypes.byref(self._h)))
        self.doses = protocol_doses(protocols, self.bins, self.resolution) if protocols and \
            not isinstance(protocols[0], (int, float)) else None
        if self.doses is not None and self.doses.any():
            self.set_doses(self.doses)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.lib().emt6_batch_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def add_irradiations(self, protocols):
        """protocols[i]: (step, dose) pairs of protocol i; doses accumulate into
        bin step // protocol_resolution (Protocol::closestDose,
        src/emt6ro/common/protocol.h:16-18)."""
        if len(protocols) != self.n_protocols:
            raise RuntimeError(f"Wrong number of protocols. Expected: {self.n_protocols}")
        idx = [i for i, prot in enumerate(protocols) for _ in prot]
        if not idx:
            return
        steps = np.asarray([int(t) for prot in protocols for t, _ in prot], np.uint32)
        doses = np.asarray([float(d) for prot in protocols for _, d in prot], np.float32)
        a = np.asarray(idx, np.int32)
        N.check(N.lib().emt6_batch_add_irradiations(self._h, N.ptr(a), N.ptr(steps), N.ptr(doses),
                                                    a.size))

    def set_doses(self, doses: np.ndarray):
        d = np.ascontiguousarray(doses, np.float32).reshape(self.n_protocols, self.bins)
        N.check(N.lib().emt6_batch_set_doses(self._h, N.ptr(d)))

    def reset(self):
        N.check(N.lib().emt6_batch_reset(self._h))

    def run(self, nsteps: int):
        N.check(N.lib().emt6_batch_run(self._h, int(nsteps)))

    def sync(self):
        N.check(N.lib().emt6_batch_sync(self._h))

    def counts(self) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        N.check(N.lib().emt6_batch_counts(self._h, N.ptr(out)))
        return out

    SUMMARY_FIELDS = ("cho", "ox", "gi", "living", "mode0", "mode1", "mode2", "mode3",
                      "g1", "s", "g2", "m", "d")

    def summary(self) -> np.ndarray:
        """(n, 13) float32 per simulation: centre-site cho, ox, gi, living
        cells, living cells per metabolic mode (4) and per phase (5)."""
        out = np.zeros((self.n, 13), np.float32)
        N.check(N.lib().emt6_batch_summary(self._h, N.ptr(out)))
        return out

    def timelapse(self, steps: int, every: int = 1) -> np.ndarray:
        """Run `steps` steps, recording `summary()` after every `every` steps
        (example/timelapse.cc:24-45 records every step on the host); returns
        (steps // every, n, 13)."""
        rec = []
        for _ in range(steps // every):
            self.run(every)
            rec.append(self.summary())
        return np.stack(rec) if rec else np.zeros((0, self.n, 13), np.float32)

    def state(self, sim: int) -> TumorState:
        buf = np.zeros((self.H, self.W), dtype=N.SITE_DTYPE)
        N.check(N.lib().emt6_batch_get_state(self._h, int(sim), N.ptr(buf)))
        return TumorState(buf)

    def step(self, sim: int) -> int:
        v = ctypes.c_uint32()
        N.check(N.lib().emt6_batch_step(self._h, int(sim), ctypes.byref(v)))
        return int(v.value)

    def diffused(self) -> int:
        v = ctypes.c_ulonglong()
        N.check(N.lib().emt6_batch_diffused(self._h, ctypes.byref(v)))
        return int(v.value)

    def launches(self) -> int:
        v = ctypes.c_ulonglong()
        N.check(N.lib().emt6_batch_launches(self._h, ctypes.byref(v)))
        return int(v.value)

    def stream(self) -> int:
        return int(N.lib().emt6_batch_stream(self._h) or 0)

    def set_schedule(self, mode: int, steps_per_launch: int = 0):
        N.check(N.lib().emt6_batch_set_schedule(self._h, int(mode), int(steps_per_launch)))

    LAYOUT_BANDS, LAYOUT_WIDE_BANDS, LAYOUT_RING, LAYOUT_ALL = 1, 2, 4, 7

    def set_layouts(self, layouts: int):
        """Tile shapes the step kernels may use (LAYOUT_* bits; results do not
        depend on it, only time)."""
        N.check(N.lib().emt6_batch_set_layouts(self._h, int(layouts)))

    def set_index_base(self, base: int):
        """Key simulation i's random stream by base + i: a batch holding the
        shard [base, base + n) of a larger set draws what the whole set would."""
        N.check(N.lib().emt6_batch_set_index_base(self._h, int(base)))
