"""annmap -- the GB300 annihilation sky-map projection, Python entry point.

Stands where the reference's src/pywrapper module stands (which exposes only
the particle reader); this one also renders maps.  Every computation runs in
the native library libdmann.so (CUDA kernels for sm_103a behind the C ABI of
include/dmann.h); there is no CPU fallback.
"""
from ._lib import COMP_F32, PLAIN_F64, DmannError
from .mapgen import MapGenerator, Renderer
from .params import Parameters
from .reader import DataReader, write_native

__all__ = ["COMP_F32", "PLAIN_F64", "DmannError", "MapGenerator", "Renderer", "Parameters",
           "DataReader", "write_native"]
