"""ctypes access to the CPU oracle (test infrastructure only).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg;
never by the product package.  See oracle/emt6_oracle.h for the semantics.
"""
from __future__ import annotations

import ctypes
import json
from pathlib import Path

import numpy as np

from . import build as _build

SITE_DTYPE = np.dtype([
    ("cho", "<f4"), ("ox", "<f4"), ("gi", "<f4"),
    ("time_in_repair", "<f4"), ("irradiation", "<f4"), ("repair_delay_time", "<f4"),
    ("proliferation_time", "<f4"), ("cycle_times", "<f4", (5,)),
    ("mode", "u1"), ("phase", "u1"), ("state", "u1"), ("pad", "u1"),
])
assert SITE_DTYPE.itemsize == 52

VACANT, OCCUPIED, MOCKED = 0, 1, 2


class Params(ctypes.Structure):
    _fields_ = [
        ("lattice_height", ctypes.c_int32), ("lattice_width", ctypes.c_int32),
        ("time_step", ctypes.c_float), ("diffusion_coeffs", ctypes.c_float * 3),
        ("diffusion_time_step", ctypes.c_float), ("metabolism", (ctypes.c_float * 3) * 4),
        ("external_levels", ctypes.c_float * 3), ("death_gi", ctypes.c_float),
        ("quiescence_gi", ctypes.c_float), ("death_gi_production", ctypes.c_float),
        ("cycle_times", (ctypes.c_float * 2) * 5), ("delay_time_coeff", ctypes.c_float),
        ("delay_time_exp_coeff", ctypes.c_float), ("survival_prob_coeff", ctypes.c_float),
        ("survival_prob_exp_coeff", ctypes.c_float), ("repair_half_time", ctypes.c_float),
    ]


class Instr(ctypes.Structure):
    _fields_ = [("repair_decisions", ctypes.c_ulonglong), ("repair_kills", ctypes.c_ulonglong),
                ("irradiation_events", ctypes.c_ulonglong), ("divisions", ctypes.c_ulonglong),
                ("sum_death_prob", ctypes.c_double)]


def params_from_json(path) -> Params:
    """The reference's JSON schema (data/default-parameters.json)."""
    o = json.loads(Path(path).read_text())
    p = Params()
    p.lattice_height = int(o["lattice_dims"]["height"])
    p.lattice_width = int(o["lattice_dims"]["width"])
    p.time_step = float(o["time_step"])
    dc = o["diffusion_params"]
    for i, k in enumerate(("cho", "ox", "gi")):
        p.diffusion_coeffs[i] = float(dc["coeffs"][k])
        p.external_levels[i] = float(o["external_levels"][k])
    p.diffusion_time_step = float(dc["time_step"])
    for m, name in enumerate(("aerobic_proliferation", "anaerobic_proliferation",
                              "aerobic_quiescence", "anaerobic_quiescence")):
        for i, k in enumerate(("cho", "ox", "gi")):
            p.metabolism[m][i] = float(o["metabolism"][name][k])
    p.death_gi = float(o["death_gi"])
    p.quiescence_gi = float(o["quiescence_gi"])
    p.death_gi_production = float(o["death_gi_production"])
    for i, k in enumerate(("g1", "s", "g2", "m", "d")):
        p.cycle_times[i][0] = float(o["cycle_times"][k]["mean"])
        p.cycle_times[i][1] = float(o["cycle_times"][k]["stddev"])
    cr = o["cell_repair"]
    p.delay_time_coeff = float(cr["delay_time"]["coeff"])
    p.delay_time_exp_coeff = float(cr["delay_time"]["exp_coeff"])
    p.survival_prob_coeff = float(cr["survival_prob"]["coeff"])
    p.survival_prob_exp_coeff = float(cr["survival_prob"]["exp_coeff"])
    p.repair_half_time = float(cr["repair_half_time"])
    return p


def params_copy(p) -> Params:
    """An oracle Params with the bytes of p (any ctypes struct of this layout)."""
    if hasattr(p, "native"):
        p = p.native
    assert ctypes.sizeof(p) == ctypes.sizeof(Params)
    q = Params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(Params))
    return q


_P = ctypes.POINTER
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_sitep = np.ctypeslib.ndpointer(SITE_DTYPE, flags="C_CONTIGUOUS")


def _declare(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


class _Lib:
    def __init__(self, path: Path, ref: bool = False):
        L = ctypes.CDLL(str(path))
        self.L = L
        c = ctypes
        _declare(L, "orc_philox4x32_10", None, [_u32p, _u32p, _u32p])
        _declare(L, "orc_expf", c.c_float, [c.c_float])
        _declare(L, "orc_log_core", c.c_double, [c.c_double])
        _declare(L, "orc_sincos2pi", None, [c.c_double, _P(c.c_double), _P(c.c_double)])
        _declare(L, "orc_division_normals", None,
                 [c.c_uint64, c.c_uint32, c.c_uint32, c.c_uint32, _f32p])
        _declare(L, "orc_uniform", c.c_float, [c.c_uint64] + [c.c_uint32] * 6)
        _declare(L, "orc_site_step", c.c_int,
                 [_sitep, _P(Params), c.c_uint32, c.c_float, c.c_float, _P(c.c_int)])
        _declare(L, "orc_choose_neighbour", None,
                 [c.c_int, c.c_int, c.c_float, _P(c.c_int), _P(c.c_int)])
        _declare(L, "orc_update_state", c.c_int, [c.c_void_p, _f32p, _P(Params), c.c_uint32])
        _declare(L, "orc_progress_clock", c.c_int, [c.c_void_p, c.c_float])
        _declare(L, "orc_batch_create", c.c_void_p, [_P(Params), c.c_int, c.c_uint64])
        _declare(L, "orc_batch_destroy", None, [c.c_void_p])
        _declare(L, "orc_batch_set", c.c_int,
                 [c.c_void_p, c.c_int, _sitep, _f32p, c.c_uint32, c.c_uint32, c.c_uint32,
                  c.c_uint32, c.c_uint32, c.c_uint32, c.c_uint32])
        _declare(L, "orc_batch_run", None, [c.c_void_p, c.c_uint32, c.c_int])
        _declare(L, "orc_batch_get", None, [c.c_void_p, c.c_int, _sitep])
        _declare(L, "orc_batch_counts", None, [c.c_void_p, _u32p])
        _declare(L, "orc_batch_list", None, [c.c_void_p, c.c_int, _u16p, _P(c.c_uint32)])
        _declare(L, "orc_batch_roi", None, [c.c_void_p, c.c_int, _i32p])
        _declare(L, "orc_batch_instr", None, [c.c_void_p, _P(Instr), c.c_void_p])
        _declare(L, "orc_batch_diffused", c.c_ulonglong, [c.c_void_p])
        _declare(L, "orc_rebuild_list", c.c_uint32, [_u8p, c.c_int, c.c_int, _u16p])
        _declare(L, "orc_find_roi", None, [_u8p, c.c_int, c.c_int, _i32p, _u8p])
        _declare(L, "orc_diffuse_f32", None,
                 [_f32p, c.c_int, c.c_int, _i32p, _u8p, _P(Params)])
        _declare(L, "orc_diffuse_f64", None,
                 [_f64p, c.c_int, c.c_int, _i32p, _u8p, _P(Params)])
        if ref:
            _declare(L, "ref_site_step_replay", c.c_int,
                     [_sitep, _P(Params), c.c_uint32, c.c_float, _f32p, c.c_int, _P(c.c_int)])
            _declare(L, "ref_update_state", c.c_int, [_sitep, _P(Params), c.c_uint32])
            _declare(L, "ref_progress_clock", c.c_int, [_sitep, c.c_float])
            _declare(L, "ref_metabolise", None, [_sitep, _P(Params)])
            _declare(L, "ref_irradiate", None, [_sitep, c.c_float, _P(Params)])
            _declare(L, "ref_try_repair", c.c_int,
                     [_sitep, _P(Params), c.c_int, c.c_float, _P(c.c_int)])
            _declare(L, "ref_choose_neighbour_replay", None,
                     [c.c_int, c.c_int, c.c_float, _P(c.c_int), _P(c.c_int)])
            _declare(L, "ref_divide_cell_replay", None, [_sitep, _sitep, _P(Params), _f32p])
            _declare(L, "ref_load_params", c.c_int, [c.c_char_p, _P(Params)])
            _declare(L, "ref_load_state", c.c_int,
                     [c.c_char_p, _P(Params), _sitep, c.c_int, _P(c.c_int), _P(c.c_int)])


_oracle = None
_ref = None


def oracle() -> _Lib:
    global _oracle
    if _oracle is None:
        _oracle = _Lib(_build.build_oracle())
    return _oracle


_fast = None


def oracle_fast() -> _Lib:
    """The timing-only build of the oracle (bench.py's CPU baseline): same
    source, -O3 with FP contraction and CPU tuning, results not checked."""
    global _fast
    if _fast is None:
        _fast = _Lib(_build.build_oracle_fast())
    return _fast


def reference():
    """The reference-host-code library, or None where the reference is absent."""
    global _ref
    if _ref is None:
        p = _build.build_ref()
        if p is None:
            return None
        _ref = _Lib(p, ref=True)
    return _ref


def load_state_txt(path, params: Params) -> np.ndarray:
    """Python restatement of the reference's text loader (src/emt6ro/state/state.cc:9-53).
    Returns an (H+2, W+2) SITE_DTYPE array with the MOCKED border ring."""
    toks = Path(path).read_text().split()
    h, w = int(toks[0]), int(toks[1])
    g = np.zeros((h + 2, w + 2), dtype=SITE_DTYPE)
    ext = np.array(params.external_levels[:], dtype=np.float32)
    g["state"] = MOCKED
    g["cho"], g["ox"], g["gi"] = ext
    L = oracle()
    i = 2
    for r in range(1, h + 1):
        for c in range(1, w + 1):
            s = int(toks[i])
            site = g[r, c]
            site["cho"], site["ox"], site["gi"] = (np.float32(toks[i + 1]), np.float32(toks[i + 2]),
                                                  np.float32(toks[i + 3]))
            i += 4
            if s:
                site["state"] = OCCUPIED
                tir, irr, pt = (np.float32(x) for x in toks[i:i + 3])
                site["time_in_repair"], site["irradiation"] = tir, irr
                if irr > 0:
                    site["repair_delay_time"] = np.float32(params.delay_time_coeff) * np.float32(
                        L.L.orc_expf(float(np.float32(params.delay_time_exp_coeff) * irr)))
                site["proliferation_time"] = pt
                site["cycle_times"] = np.array(toks[i + 3:i + 8], dtype=np.float32)
                site["mode"], site["phase"] = int(toks[i + 8]), int(toks[i + 9])
                i += 10
            else:
                site["state"] = VACANT
    return g


class Batch:
    """Batched CPU simulation (orc_batch_*)."""

    def __init__(self, params: Params, n_sims: int, seed: int, lib: _Lib | None = None):
        self.lib = lib or oracle()
        self.params = params_copy(params)
        self.H = params.lattice_height + 2
        self.W = params.lattice_width + 2
        self.n = n_sims
        self.h = self.lib.L.orc_batch_create(ctypes.byref(self.params), n_sims, seed)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.L.orc_batch_destroy(self.h)
            self.h = None

    def set(self, i, sites, protocol, resolution=300, length=144000, sim_index=None, epoch=0,
            step0=0, horizon=0xFFFFFFFF):
        sites = np.ascontiguousarray(sites, dtype=SITE_DTYPE).reshape(-1)
        assert sites.size == self.H * self.W
        prot = np.ascontiguousarray(protocol, dtype=np.float32)
        rc = self.lib.L.orc_batch_set(self.h, i, sites, prot, prot.size, resolution, length,
                                      i if sim_index is None else sim_index, epoch, step0,
                                      horizon)
        assert rc == 0

    def run(self, nsteps, nthreads=1):
        self.lib.L.orc_batch_run(self.h, nsteps, nthreads)

    def get(self, i) -> np.ndarray:
        out = np.zeros(self.H * self.W, dtype=SITE_DTYPE)
        self.lib.L.orc_batch_get(self.h, i, out)
        return out.reshape(self.H, self.W)

    def counts(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.uint32)
        self.lib.L.orc_batch_counts(self.h, out)
        return out

    def occupied_list(self, i) -> np.ndarray:
        buf = np.zeros(self.H * self.W + 512, dtype=np.uint16)
        n = ctypes.c_uint32()
        self.lib.L.orc_batch_list(self.h, i, buf, ctypes.byref(n))
        return buf[: n.value].copy()

    def roi(self, i) -> np.ndarray:
        out = np.zeros(5, dtype=np.int32)
        self.lib.L.orc_batch_roi(self.h, i, out)
        return out

    def instr(self):
        ins = Instr()
        hist = np.zeros(600, dtype=np.uint64)
        self.lib.L.orc_batch_instr(self.h, ctypes.byref(ins),
                                   hist.ctypes.data_as(ctypes.c_void_p))
        return ins, hist

    def diffused(self) -> int:
        return int(self.lib.L.orc_batch_diffused(self.h))
