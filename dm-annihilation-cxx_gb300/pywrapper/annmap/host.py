"""ctypes access to the C++ host API (libannmap.so: Parameters, DataReader,
MapGenerator and the FITS writer in C++ over the C ABI) through its C hooks.
The C++ classes themselves are declared in dm-annihilation-cxx_gb300/host/annmap.hpp."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib

LIB_PATH = os.path.join(_lib.PKG_DIR, "libannmap.so")
_HOST = None


def load():
    global _HOST
    if _HOST is None:
        _lib.load()   # builds both libraries when absent
        L = C.CDLL(LIB_PATH)
        D = C.POINTER(C.c_double)
        L.annmap_parse_info.argtypes = [C.c_char_p, D, C.c_char_p, C.c_int]
        L.annmap_parse_info.restype = C.c_int
        L.annmap_read_native.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                                         C.POINTER(C.c_float), C.c_int64, C.c_char_p, C.c_int]
        L.annmap_read_native.restype = C.c_int64
        L.annmap_read_tipsy.argtypes = [C.c_char_p] * 5 + [C.c_int, C.c_int, C.c_int,
                                                           C.POINTER(C.c_float), C.c_int64, C.c_char_p, C.c_int]
        L.annmap_read_tipsy.restype = C.c_int64
        L.annmap_genmap.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_char_p, D, C.c_int64, D,
                                    C.c_char_p, C.c_int]
        L.annmap_genmap.restype = C.c_int
        L.annmap_write_fits.argtypes = [C.c_char_p, D, C.c_int64, C.c_char_p, C.c_int]
        L.annmap_write_fits.restype = C.c_int
        _HOST = L
    return _HOST


def _err():
    return C.create_string_buffer(512)


def parse_info(path: str) -> dict:
    out = (C.c_double * 24)()
    e = _err()
    if load().annmap_parse_info(path.encode(), out, e, 512) != 0:
        raise ValueError(e.value.decode())
    v = out[:]
    return {"nside": int(v[0]), "rotmatrix": np.array(v[1:10]).reshape(3, 3), "opos": v[10:13],
            "cpos": v[13:16], "unit_factor": v[16], "hires_threshold": v[17], "memParts": int(v[18]),
            "testNum": int(v[19]), "otheta": v[20], "ophi": v[21], "isMask": bool(v[22]),
            "isNative": bool(v[23])}


SOA = ("x", "y", "z", "m", "rho", "h", "sigmav")


def read_native(path: str, maskfile: str = "", test: int = -1, buf: int = 10000000, cap: int = None) -> dict:
    if cap is None:
        with open(path, "rb") as f:
            cap = max(1, int(np.fromfile(f, dtype="<i4", count=1)[0]))
    soa = np.zeros((7, cap), dtype=np.float32)
    e = _err()
    n = load().annmap_read_native(path.encode(), maskfile.encode(), int(test), int(buf),
                                  soa.ctypes.data_as(C.POINTER(C.c_float)), cap, e, 512)
    if n < 0:
        raise ValueError(e.value.decode())
    return {k: soa[i, :n].copy() for i, k in enumerate(SOA)}


def read_tipsy(part: str, dens: str, hsm: str, sigv: str, maskfile: str = "", single: bool = False,
               test: int = -1, buf: int = 10000000, cap: int = 1 << 20) -> dict:
    soa = np.zeros((7, cap), dtype=np.float32)
    e = _err()
    n = load().annmap_read_tipsy(part.encode(), dens.encode(), hsm.encode(), sigv.encode(),
                                 maskfile.encode(), int(single), int(test), int(buf),
                                 soa.ctypes.data_as(C.POINTER(C.c_float)), cap, e, 512)
    if n < 0:
        raise ValueError(e.value.decode())
    return {k: soa[i, :n].copy() for i, k in enumerate(SOA)}


def genmap(info_file: str, precision: int = 1, device: int = 0, nside: int = None,
           flux_model: int = 0, halo_file: str = "") -> tuple:
    """The reference's main flow in C++ (Parameters, DataReader, MapGenerator,
    saveToFits when the info file names an output map).  Returns (map, total flux)."""
    if nside is None:
        nside = parse_info(info_file)["nside"]
    mp = np.zeros(12 * nside * nside)
    tot = C.c_double()
    e = _err()
    if load().annmap_genmap(info_file.encode(), int(precision), int(device), int(flux_model),
                            halo_file.encode(), mp.ctypes.data_as(C.POINTER(C.c_double)), mp.size, C.byref(tot), e, 512) != 0:
        raise RuntimeError(e.value.decode())
    return mp, tot.value


def write_fits(path: str, m) -> None:
    m = np.ascontiguousarray(m, dtype=np.float64)
    e = _err()
    if load().annmap_write_fits(path.encode(), m.ctypes.data_as(C.POINTER(C.c_double)), m.size, e, 512) != 0:
        raise ValueError(e.value.decode())
