"""Native layer of emt6ro.simulation (mirror of the reference's pybind11 module
python/emt6ro/simulation/backend.cc:181-232) over the C ABI of the CUDA library.
"""
from __future__ import annotations

import ctypes
import enum
import os

import numpy as np

from .. import _native as N

INSTR_HIST_N = 300      # src/emt6ro/common/instr.h:41
INSTR_HIST_DX = 0.1     # src/emt6ro/common/instr.h:42


class SiteState(enum.IntEnum):
    """backend.cc:185-189"""
    Vacant = 0
    Occupied = 1
    Mocked = 2


Vacant, Occupied, Mocked = SiteState.Vacant, SiteState.Occupied, SiteState.Mocked


class Coords:
    """backend.cc:191-196"""

    def __init__(self, r: int = 0, c: int = 0):
        self.r = int(r)
        self.c = int(c)

    def __repr__(self):
        return f"{{r: {self.r}, c: {self.c}}}"


class Parameters:
    """Model parameters (opaque in the reference, backend.cc:207); wraps emt6_params."""

    def __init__(self, native: N.Params):
        self._p = native

    @property
    def native(self) -> N.Params:
        return self._p

    @property
    def lattice_dims(self):
        return (self._p.lattice_height, self._p.lattice_width)

    def __getattr__(self, name):
        return getattr(object.__getattribute__(self, "_p"), name)


class TumorState:
    """Host copy of one lattice (the reference's HostGrid<Site>, backend.cc:198-205).
    Field accessors return (H, W) views into the state's own storage."""

    def __init__(self, sites: np.ndarray):
        self._sites = np.ascontiguousarray(sites, dtype=N.SITE_DTYPE)
        assert self._sites.ndim == 2

    @property
    def sites(self) -> np.ndarray:
        return self._sites

    @property
    def dims(self):
        return self._sites.shape

    def irradiation(self):
        return self._sites["irradiation"]

    def occupancy(self):
        return self._sites["state"]

    def cho(self):
        return self._sites["cho"]

    def ox(self):
        return self._sites["ox"]

    def gi(self):
        return self._sites["gi"]

    def mode(self):
        return self._sites["mode"]

    def phase(self):
        return self._sites["phase"]

    def copy(self) -> "TumorState":
        return TumorState(self._sites.copy())


def load_parameters(path) -> Parameters:
    """Parameters::loadFromJSONFile (src/emt6ro/parameters/parameters.cc:66-80)."""
    p = N.Params()
    N.check(N.lib().emt6_load_parameters(os.fsencode(str(path)), ctypes.byref(p)))
    return Parameters(p)


def load_state(path, params: Parameters) -> TumorState:
    """loadFromFile (src/emt6ro/state/state.cc:9-53): adds the MOCKED border ring."""
    L = N.lib()
    h = ctypes.c_int32()
    w = ctypes.c_int32()
    pn = params.native if isinstance(params, Parameters) else params
    N.check(L.emt6_load_state(os.fsencode(str(path)), ctypes.byref(pn), None, 0,
                              ctypes.byref(h), ctypes.byref(w)))
    out = np.zeros((h.value, w.value), dtype=N.SITE_DTYPE)
    N.check(L.emt6_load_state(os.fsencode(str(path)), ctypes.byref(pn), N.ptr(out), out.size,
                              ctypes.byref(h), ctypes.byref(w)))
    return TumorState(out)


def save_state(state: TumorState, path) -> None:
    """saveToFile (src/emt6ro/state/state.cc:55-82)."""
    s = np.ascontiguousarray(state.sites)
    N.check(N.lib().emt6_save_state(os.fsencode(str(path)), N.ptr(s), s.shape[0], s.shape[1]))


def _stack_tumors(tumors):
    arrs = [t.sites if isinstance(t, TumorState) else np.asarray(t, dtype=N.SITE_DTYPE)
            for t in tumors]
    if not arrs:
        raise RuntimeError("At least one tumor state is required.")
    shape = arrs[0].shape
    for a in arrs:
        if a.shape != shape:
            raise RuntimeError("All tumors must have the same dimensions.")
    return np.ascontiguousarray(np.stack(arrs)), shape


class _Experiment:
    """backend.cc:16-136: protocols x tumours x runs simulations on one GPU."""

    def __init__(self, params: Parameters, tumors, runs: int, protocols_num: int,
                 simulation_steps: int, protocol_resolution: int, gpu_id: int, seed=None):
        stack, (H, W) = _stack_tumors(tumors)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")  # std::random_device, backend.cc:31
        self.params = params
        self.shape = (int(protocols_num), len(tumors), int(runs))
        self.H, self.W = H, W
        self.protocols_num = int(protocols_num)
        self.simulation_steps = int(simulation_steps)
        self.protocol_resolution = int(protocol_resolution)
        self.gpu_id = int(gpu_id)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self._h = ctypes.c_void_p()
        L = N.lib()
        N.check(L.emt6_experiment_create(ctypes.byref(params.native), N.ptr(stack), len(tumors), H,
                                         W, int(runs), int(protocols_num), int(simulation_steps),
                                         int(protocol_resolution), int(gpu_id), self.seed,
                                         ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.lib().emt6_experiment_destroy(h)
            self._h = None

    @property
    def batch_handle(self):
        return N.lib().emt6_experiment_batch(self._h)

    def run(self, nsteps: int):
        N.check(N.lib().emt6_experiment_run(self._h, int(nsteps)))

    def results(self):
        out = np.zeros(int(np.prod(self.shape)), dtype=np.uint32)
        N.check(N.lib().emt6_experiment_results(self._h, N.ptr(out)))
        return out

    def add_irradiations(self, protocols):
        if len(protocols) != self.protocols_num:
            raise RuntimeError("Check failed: ps.size() == protocols_num; Wrong number of "
                               f"protocols. Expected: {self.protocols_num}")
        idx, steps, doses = [], [], []
        for i, prot in enumerate(protocols):
            for t, d in prot:
                idx.append(i)
                steps.append(int(t))
                doses.append(float(d))
        if not idx:
            return
        a = np.asarray(idx, np.int32)
        s = np.asarray(steps, np.uint32)
        d = np.asarray(doses, np.float32)
        N.check(N.lib().emt6_experiment_add_irradiations(self._h, N.ptr(a), N.ptr(s), N.ptr(d),
                                                         a.size))

    def reset(self):
        N.check(N.lib().emt6_experiment_reset(self._h))

    def state(self):
        n = int(np.prod(self.shape))
        out = []
        for i in range(n):
            buf = np.zeros((self.H, self.W), dtype=N.SITE_DTYPE)
            N.check(N.lib().emt6_experiment_state(self._h, i, N.ptr(buf)))
            out.append(TumorState(buf))
        return out


class InstrCounters:
    """backend.cc:221-226"""

    def __init__(self, c: N.InstrCountersC):
        self.repair_decisions = int(c.repair_decisions)
        self.repair_kills = int(c.repair_kills)
        self.irradiation_events = int(c.irradiation_events)
        self.divisions = int(c.divisions)
        self.sum_death_prob = float(c.sum_death_prob)

    def __repr__(self):
        return (f"InstrCounters(repair_decisions={self.repair_decisions}, "
                f"repair_kills={self.repair_kills}, irradiation_events={self.irradiation_events},"
                f" divisions={self.divisions}, sum_death_prob={self.sum_death_prob})")


def read_instr_counters(device: int = 0) -> InstrCounters:
    """instr.cu:6-18 (always collected here; the reference needs EMT6RO_INSTRUMENT)."""
    c = N.InstrCountersC()
    N.check(N.lib().emt6_read_instr_counters(device, ctypes.byref(c)))
    return InstrCounters(c)


def reset_instr_counters(device: int = 0) -> None:
    N.check(N.lib().emt6_reset_instr_counters(device))


def read_instr_histograms(device: int = 0):
    """Flat list of 2*INSTR_HIST_N counts: irradiation bins, then time-in-repair bins."""
    out = np.zeros(2 * INSTR_HIST_N, dtype=np.uint64)
    N.check(N.lib().emt6_read_instr_histograms(device, N.ptr(out)))
    return [int(x) for x in out]
