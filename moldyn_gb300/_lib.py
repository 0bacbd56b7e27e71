"""ctypes binding of libmdgb.so (the C ABI in include/mdgb.h).

The library is built in-tree (``python -m moldyn_gb300.build``) and loaded
from ``moldyn_gb300/_build/libmdgb.so``.  There is no fallback: if the library
is missing or cannot create an engine on a GPU, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

_lock = threading.Lock()
_LIB = None

MDGB_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "no state uploaded",
          4: "neighbour list overflow", 5: "fixed-point force overflow", 6: "unsupported",
          7: "device-side wait timed out", 8: "out of device memory", 9: "skin violation",
          10: "too many atoms for the allocation-free entry point"}

PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_FP32_NAIVE = 2
FLAG_REFERENCE_ORDER = 1
FLAG_PROFILE = 2
FLAG_PERSISTENT = 4
FLAG_TRACE = 8
FLAG_DIRECT_LIST = 16
TRACE_PHASES = ["coupling", "drift", "decide", "zero_cells", "bin", "scan_a", "scan_b", "scan_c", "scatter",
                "sort_cells", "gather", "verlet_list", "launches", "rebuild_launches"]
THERMOSTAT_BERENDSEN = 0
THERMOSTAT_NOSE_HOOVER = 1


class MdgbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"libmdgb: {STATUS.get(status, status)}: {message}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("precision", C.c_int), ("skin", C.c_double), ("rebuild_every", C.c_int),
                ("threads_per_atom", C.c_int), ("graph_steps", C.c_int),
                ("neighbor_capacity", C.c_int), ("device", C.c_int), ("flags", C.c_uint)]


class CThermostat(C.Structure):
    _fields_ = [("kind", C.c_int), ("tau", C.c_double), ("target_temperature", C.c_double),
                ("lambda_", C.c_double), ("psi", C.c_double)]


class CBarostat(C.Structure):
    _fields_ = [("beta", C.c_double), ("tau", C.c_double), ("target_pressure", C.c_double),
                ("myu", C.c_double)]


class CMacro(C.Structure):
    _fields_ = [("kinetic_energy", C.c_double), ("potential_energy", C.c_double),
                ("thermal_energy", C.c_double), ("temperature", C.c_double),
                ("pressure", C.c_double), ("com_velocity", C.c_double * 3),
                ("momentum", C.c_double * 3), ("count", C.c_int64)]


class CStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("rebuilds", C.c_int64), ("kernel_launches", C.c_int64),
                ("graph_launches", C.c_int64), ("neighbor_capacity", C.c_int),
                ("max_neighbors", C.c_int), ("threads_per_atom", C.c_int), ("retries", C.c_int),
                ("force_ms", C.c_double), ("force_launches", C.c_int64),
                ("integrate_ms", C.c_double), ("integrate_launches", C.c_int64),
                ("class_threads_per_atom", C.c_int * 3), ("class_replicas", C.c_int * 3),
                ("class_skin", C.c_double * 3), ("direct_list_builds", C.c_int64)]


class CSplatParams(C.Structure):
    _fields_ = [("view_pos", C.c_float * 4), ("view", C.c_float * 16), ("proj", C.c_float * 16),
                ("gradient_min", C.c_float * 4), ("gradient_mid", C.c_float * 4),
                ("gradient_max", C.c_float * 4), ("gradient_min_max", C.c_float * 4),
                ("mode", C.c_uint32), ("draw_box", C.c_int32), ("box", C.c_float * 4)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_opt_dp = C.POINTER(C.c_double)
_E = C.c_void_p

# name -> (restype, argtypes); every symbol declared in include/mdgb.h
SIGNATURES = {
    "mdgb_abi_version": (C.c_int, []),
    "mdgb_config_default": (C.c_int, [C.POINTER(Config)]),
    "mdgb_create": (C.c_int, [C.POINTER(Config), C.POINTER(_E)]),
    "mdgb_destroy": (C.c_int, [_E]),
    "mdgb_last_error": (C.c_char_p, [_E]),
    "mdgb_status_string": (C.c_char_p, [C.c_int]),
    "mdgb_stream": (C.c_void_p, [_E]),
    "mdgb_set_potential": (C.c_int, [_E, C.c_uint16, C.c_uint16, C.c_double, C.c_double]),
    "mdgb_set_potential_raw": (C.c_int, [_E, C.c_uint16, C.c_uint16, C.c_double, C.c_double,
                                         C.c_double, C.c_double]),
    "mdgb_upload_state": (C.c_int, [_E, C.c_int64, _u16p, _dp, _opt_dp, _dp, C.c_int, _dp]),
    "mdgb_upload_forces": (C.c_int, [_E, _opt_dp, _opt_dp, _opt_dp]),
    "mdgb_compute_forces": (C.c_int, [_E]),
    "mdgb_step": (C.c_int, [_E, C.c_int64, C.c_double, C.POINTER(CThermostat),
                            C.POINTER(CBarostat)]),
    "mdgb_prepare_step": (C.c_int, [_E, C.c_int64, C.c_double, C.POINTER(CThermostat), C.POINTER(CBarostat)]),
    "mdgb_ensemble_prepare": (C.c_int, [_E, C.c_int64, C.c_double]),
    "mdgb_test_barrier_timeout": (C.c_int, [_E, C.c_int, C.c_int64]),
    "mdgb_download_state": (C.c_int, [_E, _opt_dp, _opt_dp, _opt_dp, _opt_dp, _opt_dp, _opt_dp]),
    "mdgb_macro_parameters": (C.c_int, [_E, C.c_int, C.POINTER(CMacro)]),
    "mdgb_ensemble_upload": (C.c_int, [_E, C.c_int, _i64p, _u16p, _dp, _opt_dp, _dp, C.c_int, _dp]),
    "mdgb_ensemble_set_coupling": (C.c_int, [_E, C.POINTER(CThermostat), C.POINTER(CBarostat)]),
    "mdgb_ensemble_step": (C.c_int, [_E, C.c_int64, C.c_double]),
    "mdgb_ensemble_get_coupling": (C.c_int, [_E, C.POINTER(CThermostat), C.POINTER(CBarostat)]),
    "mdgb_ensemble_download": (C.c_int, [_E, _opt_dp, _opt_dp, _opt_dp, _opt_dp, _opt_dp, _opt_dp]),
    "mdgb_ensemble_macro": (C.c_int, [_E, C.c_int, C.POINTER(CMacro)]),
    "mdgb_interacting_pairs": (C.c_int, [_E, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int64)]),
    "mdgb_get_stats": (C.c_int, [_E, C.POINTER(CStats)]),
    "mdgb_reset_stats": (C.c_int, [_E]),
    "mdgb_trace_phases": (C.c_int, [_E, _dp, C.c_int]),
    "mdgb_synchronize": (C.c_int, [_E]),
    "mdgb_forces_noalloc": (C.c_int, [C.c_int64, C.c_void_p, _dp, C.c_double, C.c_double, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    "mdgb_splat": (C.c_int, [_fp, C.c_int64, C.POINTER(CSplatParams), C.c_int, C.c_int, _fp]),
    "mdgb_lj_new": (C.c_int, [C.c_double, C.c_double, _dp]),
    "mdgb_lj_eval": (C.c_int, [_dp, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mdgb_lattice": (C.c_int, [C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_double, _dp, _dp]),
    "mdgb_maxwell_boltzmann": (C.c_int, [C.c_int64, C.c_double, C.c_double, C.c_uint64, _dp]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libmdgb.so (building it first when it is missing or stale)."""
    global _LIB
    with _lock:
        if _LIB is None:
            path = _build.LIB
            if build_if_missing and not _build.up_to_date():
                _build.build()
            if not os.path.exists(path):
                raise MdgbError(2, f"{path} is not built; run python -m moldyn_gb300.build")
            L = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _LIB = L
    return _LIB


def as_ptr(a):
    """Optional float64 array -> POINTER(c_double) (None stays NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(_opt_dp)


def check(status: int, handle=None):
    if status != MDGB_OK:
        msg = ""
        if handle:
            m = load().mdgb_last_error(handle)
            msg = m.decode() if m else ""
        raise MdgbError(status, msg)
