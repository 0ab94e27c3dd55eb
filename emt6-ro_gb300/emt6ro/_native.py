"""ctypes binding of libemt6ro_gb300.so (the C ABI in include/emt6ro_gb300.h and
include/emt6ro_surrogate.h).

The CUDA library is the only implementation: if it is missing (and cannot be
built in place because nvcc is absent) importing this module raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB_PATH = _PKG / "_lib" / "libemt6ro_gb300.so"

EMT6_OK = 0
EMT6_ERR_INVALID = 1
EMT6_ERR_CUDA = 2
EMT6_ERR_STATE = 3
EMT6_ERR_IO = 4
EMT6_ERR_LIMIT = 5
EMT6_ERR_DEVICE = 6
MAX_INTERIOR_HEIGHT = 54
MAX_INTERIOR_WIDTH = 60
INSTR_HIST_N = 300

SITE_DTYPE = np.dtype([
    ("cho", "<f4"), ("ox", "<f4"), ("gi", "<f4"),
    ("time_in_repair", "<f4"), ("irradiation", "<f4"), ("repair_delay_time", "<f4"),
    ("proliferation_time", "<f4"), ("cycle_times", "<f4", (5,)),
    ("mode", "u1"), ("phase", "u1"), ("state", "u1"), ("pad", "u1"),
])
assert SITE_DTYPE.itemsize == 52


class Params(ctypes.Structure):
    """emt6_params (the reference's Parameters, parameters/parameters.h:10-70)."""
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


class InstrCountersC(ctypes.Structure):
    _fields_ = [("repair_decisions", ctypes.c_ulonglong), ("repair_kills", ctypes.c_ulonglong),
                ("irradiation_events", ctypes.c_ulonglong), ("divisions", ctypes.c_ulonglong),
                ("sum_death_prob", ctypes.c_double)]


class NativeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


_P = ctypes.POINTER
_c = ctypes
_VP = ctypes.c_void_p

# name -> (restype, argtypes)
_SIGNATURES = {
    "emt6_last_error": (_c.c_char_p, []),
    "emt6_version": (_c.c_int, []),
    "emt6_load_parameters": (_c.c_int, [_c.c_char_p, _P(Params)]),
    "emt6_load_state": (_c.c_int, [_c.c_char_p, _P(Params), _VP, _c.c_int32, _P(_c.c_int32),
                                   _P(_c.c_int32)]),
    "emt6_save_state": (_c.c_int, [_c.c_char_p, _VP, _c.c_int32, _c.c_int32]),
    "emt6_batch_create": (_c.c_int, [_P(Params), _VP, _c.c_int32, _c.c_int32, _c.c_int32,
                                     _c.c_int32, _c.c_uint32, _c.c_uint32, _c.c_uint32, _c.c_int64,
                                     _VP, _VP, _VP, _c.c_int32, _c.c_uint64, _P(_VP)]),
    "emt6_batch_destroy": (_c.c_int, [_VP]),
    "emt6_batch_reset": (_c.c_int, [_VP]),
    "emt6_batch_add_irradiations": (_c.c_int, [_VP, _VP, _VP, _VP, _c.c_int64]),
    "emt6_batch_set_doses": (_c.c_int, [_VP, _VP]),
    "emt6_batch_run": (_c.c_int, [_VP, _c.c_uint32]),
    "emt6_batch_sync": (_c.c_int, [_VP]),
    "emt6_batch_counts": (_c.c_int, [_VP, _VP]),
    "emt6_batch_get_state": (_c.c_int, [_VP, _c.c_int64, _VP]),
    "emt6_batch_summary": (_c.c_int, [_VP, _VP]),
    "emt6_batch_step": (_c.c_int, [_VP, _c.c_int64, _P(_c.c_uint32)]),
    "emt6_batch_stream": (_VP, [_VP]),
    "emt6_batch_diffused": (_c.c_int, [_VP, _P(_c.c_ulonglong)]),
    "emt6_batch_set_schedule": (_c.c_int, [_VP, _c.c_int32, _c.c_uint32]),
    "emt6_batch_set_index_base": (_c.c_int, [_VP, _c.c_uint32]),
    "emt6_batch_set_layouts": (_c.c_int, [_VP, _c.c_uint32]),
    "emt6_batch_launches": (_c.c_int, [_VP, _P(_c.c_ulonglong)]),
    "emt6_probe_fp32_peak": (_c.c_int, [_c.c_int32, _P(_c.c_double)]),
    "emt6_experiment_create": (_c.c_int, [_P(Params), _VP, _c.c_int32, _c.c_int32, _c.c_int32,
                                          _c.c_int32, _c.c_int32, _c.c_uint32, _c.c_uint32,
                                          _c.c_int32, _c.c_uint64, _P(_VP)]),
    "emt6_experiment_destroy": (_c.c_int, [_VP]),
    "emt6_experiment_add_irradiations": (_c.c_int, [_VP, _VP, _VP, _VP, _c.c_int64]),
    "emt6_experiment_run": (_c.c_int, [_VP, _c.c_uint32]),
    "emt6_experiment_results": (_c.c_int, [_VP, _VP]),
    "emt6_experiment_reset": (_c.c_int, [_VP]),
    "emt6_experiment_state": (_c.c_int, [_VP, _c.c_int64, _VP]),
    "emt6_experiment_batch": (_VP, [_VP]),
    "emt6_read_instr_counters": (_c.c_int, [_c.c_int32, _P(InstrCountersC)]),
    "emt6_reset_instr_counters": (_c.c_int, [_c.c_int32]),
    "emt6_read_instr_histograms": (_c.c_int, [_c.c_int32, _VP]),
    "emt6_test_philox": (_c.c_int, [_VP, _VP, _VP, _c.c_int64, _c.c_int32]),
    "emt6_test_math": (_c.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _c.c_int64, _c.c_int32]),
    "emt6_test_site_step": (_c.c_int, [_P(Params), _VP, _VP, _VP, _VP, _VP, _VP, _c.c_int64,
                                       _c.c_int32]),
    "emt6_test_choose": (_c.c_int, [_VP, _c.c_int32, _c.c_int32, _VP, _c.c_int64, _c.c_int32]),
    "emt6_test_divide": (_c.c_int, [_P(Params), _VP, _VP, _VP, _c.c_int64, _c.c_int32]),
    "emt6_test_normals": (_c.c_int, [_c.c_uint64, _VP, _VP, _c.c_uint32, _VP, _c.c_int64,
                                     _c.c_int32]),
    "emt6_test_roi": (_c.c_int, [_VP, _c.c_int32, _c.c_int32, _VP, _VP, _c.c_int32]),
    "emt6_test_list": (_c.c_int, [_VP, _c.c_int32, _c.c_int32, _VP, _P(_c.c_uint32), _c.c_int32]),
    "emt6_test_diffuse": (_c.c_int, [_P(Params), _VP, _c.c_int32, _c.c_int32, _VP, _c.c_int32,
                                     _c.c_int32]),
    "emt6_test_order": (_c.c_int, [_VP, _VP, _VP, _c.c_int64, _c.c_uint32, _VP, _c.c_int32]),
    "emt6_simulate_noalloc": (_c.c_int, [_P(Params), _VP, _c.c_int32, _c.c_int32, _VP, _VP,
                                         _c.c_int64, _VP, _c.c_uint32, _c.c_uint32, _c.c_uint32,
                                         _c.c_uint32, _c.c_uint64, _VP, _VP]),
    # surrogate MLP (include/emt6ro_surrogate.h)
    "emt6_mlp_create": (_c.c_int, [_c.c_int32, _c.c_uint64, _c.c_int32, _P(_VP)]),
    "emt6_mlp_destroy": (None, [_VP]),
    "emt6_mlp_stream": (_VP, [_VP]),
    "emt6_mlp_set_params": (_c.c_int, [_VP, _P(_VP)]),
    "emt6_mlp_get_params": (_c.c_int, [_VP, _P(_VP)]),
    "emt6_mlp_predict": (_c.c_int, [_VP, _VP, _c.c_int32, _VP]),
    "emt6_mlp_train_step": (_c.c_int, [_VP, _VP, _VP, _c.c_int32, _c.c_float,
                                       _P(_c.c_float)]),
    "emt6_mlp_gradients": (_c.c_int, [_VP, _VP, _VP, _c.c_int32, _P(_VP), _P(_c.c_float)]),
    "emt6_mlp_sync": (_c.c_int, [_VP]),
    "emt6_mlp_set_splitk": (_c.c_int, [_VP, _c.c_int32]),
    "emt6_test_mlp_gemm": (_c.c_int, [_VP, _VP, _VP, _c.c_int32, _c.c_int32, _c.c_int32, _VP]),
    "emt6_test_mlp_gemm_timeout": (_c.c_int, [_VP, _VP, _VP, _c.c_int32, _c.c_int32, _c.c_int32,
                                              _c.c_uint32, _VP]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> Path:
    return _LIB_PATH


def lib():
    """Load (building in place first if needed and possible) the CUDA library."""
    global _lib
    with _lock:
        if _lib is None:
            if not _LIB_PATH.exists():
                import importlib.util
                spec = importlib.util.spec_from_file_location(
                    "emt6_build_ext", _PKG.parent / "build_ext.py")
                if spec is None or spec.loader is None:
                    raise ImportError(f"{_LIB_PATH} is missing and its build script is absent")
                mod = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(mod)
                try:
                    mod.build()
                except Exception as e:  # noqa: BLE001
                    raise ImportError(f"{_LIB_PATH} is missing and could not be built: {e}")
            L = ctypes.CDLL(str(_LIB_PATH))
            for name, (res, args) in _SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def check(rc: int) -> None:
    if rc != EMT6_OK:
        msg = lib().emt6_last_error()
        raise NativeError(rc, msg.decode(errors="replace") if msg else f"error {rc}")


def ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)
