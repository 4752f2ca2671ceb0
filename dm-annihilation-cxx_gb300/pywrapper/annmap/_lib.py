"""ctypes binding of libdmann.so (the C ABI declared in include/dmann.h).

The library is the only compute path: if it is missing or fails to load
this module raises, and there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG_DIR = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB_PATH = os.path.join(PKG_DIR, "libdmann.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_TIMEOUT, ERR_NODEVICE, ERR_TOO_LARGE = range(8)
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "STATE", 5: "TIMEOUT", 6: "NODEVICE",
                7: "TOO_LARGE"}
PLAIN_F64, COMP_F32 = 0, 1
(FLUX_ANN_NOSOM, FLUX_ANN_SOMV, FLUX_ANN_SOMV2, FLUX_ANN_PWAVE, FLUX_DECAY, FLUX_ANN_ADIABATIC,
 FLUX_ANN_CORE_NOSOM) = range(7)
FLUX_LAWS = {"ann_nosom": 0, "ann_somv": 1, "ann_somv2": 2, "ann_pwave": 3, "decay": 4, "ann_adiabatic": 5,
             "ann_core_nosom": 6}


class DmannError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"dmann status {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Stats(C.Structure):
    _fields_ = [("n_in", C.c_int64), ("n_kept", C.c_int64), ("n_invalid", C.c_int64),
                ("n_single", C.c_int64),
                ("n_disc", C.c_int64), ("n_disc_block", C.c_int64), ("deposits", C.c_int64),
                ("kernel_ms", C.c_double), ("disc_ms", C.c_double),
                ("disc_block_ms", C.c_double), ("disc_warp_ms", C.c_double),
                ("total_flux", C.c_double), ("launches", C.c_int64),
                ("pass1_ms", C.c_double), ("pass2_ms", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("warp_max_pixels", C.c_int64), ("block_threads", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("ring_chunk", C.c_int32),
                ("seg_min_deposits_log2", C.c_int32), ("reserved", C.c_int32 * 2)]


_LIB = None
_LOCK = threading.Lock()

# name -> (restype, argtypes)
_P = C.c_void_p
_D3 = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
SIGNATURES = {
    "dmann_abi_version": (C.c_int, []),
    "dmann_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "dmann_destroy": (None, [_P]),
    "dmann_last_error": (C.c_char_p, [_P]),
    "dmann_set_stream": (C.c_int, [_P, _P]),
    "dmann_synchronize": (C.c_int, [_P]),
    "dmann_set_observer": (C.c_int, [_P, _D3, _D3, _D3]),
    "dmann_set_frame": (C.c_int, [_P, _D3, _D3]),
    "dmann_set_units": (C.c_int, [_P, C.c_double, C.c_double, C.c_int]),
    "dmann_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "dmann_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "dmann_set_tuning_nside": (C.c_int, [_P, C.c_int, C.POINTER(Tuning)]),
    "dmann_get_tuning_nside": (C.c_int, [_P, C.c_int, C.POINTER(Tuning)]),
    "dmann_render": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.c_int64, C.c_int, C.c_int, _P, C.c_int]),
    "dmann_map_begin": (C.c_int, [_P, C.c_int, C.c_int]),
    "dmann_map_add": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.c_int64]),
    "dmann_map_end": (C.c_int, [_P, _P, C.c_int]),
    "dmann_map_abort": (C.c_int, [_P]),
    "dmann_map_add_v": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, C.c_int64]),
    "dmann_render_v": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, C.c_int64, C.c_int, C.c_int, _P, C.c_int]),
    "dmann_set_flux_params": (C.c_int, [_P, C.c_double, _D3]),
    "dmann_set_halo_cores": (C.c_int, [_P, _P, _P, _P, _P, C.c_int]),
    "dmann_flux_unit_factor": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, _D3]),
    "dmann_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "dmann_render_batch": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.c_int64, C.c_int, _D3, _D3,
                                     C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_void_p)]),
    "dmann_adjoint": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.c_int64, C.c_int, C.c_int, _P, _P, _D3]),
    "dmann_adjoint_v": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, C.c_int64, C.c_int, C.c_int, _P, _P,
                                  _D3]),
    "dmann_measure_l2_red": (C.c_int, [C.c_int, C.c_int, C.c_int64, C.c_int, _D3]),
    "dmann_observer_rotation": (C.c_int, [_D3, _D3, _D3, _D3, _D3]),
    "dmann_observer_rotation_jacobian": (C.c_int, [_D3, _D3, _D3, _D3]),
    "dmann_code_units": (C.c_int, [C.c_double, C.c_double, C.c_double, _D3]),
    "dmann_hires_threshold": (C.c_double, [_D3, C.c_int]),
    "dmann_render_noalloc": (C.c_int, [_P, _P, _P, _P, _P, _P, C.c_int64, C.c_int, _D3, _D3,
                                       C.c_double, C.c_double, _P, C.c_int, _P]),
}


def load(path: str = LIB_PATH):
    """Loads libdmann.so (building it in-tree first if it is absent)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        if not os.path.exists(path):
            import importlib.util
            spec = importlib.util.spec_from_file_location("_dmann_build", os.path.join(PKG_DIR, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def exported_symbols():
    return list(SIGNATURES)
