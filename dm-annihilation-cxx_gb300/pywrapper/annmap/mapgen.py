"""Renderer (a handle on the native library) and MapGenerator (the reference's
map-generator API, src/mapgenerator.h:8-26, on top of it).

``MapGenerator(par, reader).start()`` streams the reader's chunks through
dmann_map_begin / dmann_map_add / dmann_map_end exactly where the reference's
start() loops over DataReader chunks (src/genmap.cpp:67-156); ``getMap()``
returns the FP64 RING map in flux per steradian (after the dOmega division,
genmap.cpp:168), ``getNside()`` and ``isFinished()`` as in the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import COMP_F32, PLAIN_F64, DmannError

FIELDS = ("x", "y", "z", "m", "rho", "h")


def _is_torch(a):
    return type(a).__module__.startswith("torch")


class Renderer:
    """One native context (its own CUDA stream and device workspace)."""

    def __init__(self, device: int = 0):
        self.L = _lib.load()
        self.ctx = C.c_void_p()
        st = self.L.dmann_create(C.byref(self.ctx), int(device))
        if st != _lib.OK:
            raise DmannError(st, "dmann_create failed (a GB300 / sm_103 device is required)")
        self.device = device
        self._keep = []
        self._nside = None

    # ------------------------------------------------------------ plumbing
    def _check(self, st):
        if st != _lib.OK:
            msg = self.L.dmann_last_error(self.ctx)
            raise DmannError(st, msg.decode() if msg else "")

    def close(self):
        if self.ctx:
            self.L.dmann_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ptr(self, a, dtype):
        """Raw pointer of a contiguous numpy array or torch tensor (kept alive)."""
        if _is_torch(a):
            import torch
            want = torch.float32 if dtype == np.float32 else torch.float64
            if a.dtype != want or not a.is_contiguous():
                a = a.to(want).contiguous()
            self._keep.append(a)
            return C.c_void_p(a.data_ptr())
        arr = np.ascontiguousarray(a, dtype=dtype)
        self._keep.append(arr)
        return C.c_void_p(arr.ctypes.data)

    CUDA_STREAM_LEGACY = 1   # cudaStreamLegacy: the legacy default ("NULL") stream

    def set_stream(self, stream=None):
        """Runs on a cudaStream_t: an int handle, or a torch.cuda.Stream (torch's
        default stream, handle 0, is the legacy default stream); None returns
        to the context's own stream."""
        if stream is None:
            h = None
        elif hasattr(stream, "cuda_stream"):
            h = stream.cuda_stream or self.CUDA_STREAM_LEGACY
        else:
            h = stream or None
        self._check(self.L.dmann_set_stream(self.ctx, C.c_void_p(h) if h else None))

    def _use_torch_stream(self, arrays):
        if any(_is_torch(a) and a.is_cuda for a in arrays):
            import torch
            self.set_stream(torch.cuda.current_stream(self.device))

    # ------------------------------------------------------------ frame / units
    def set_observer(self, opos, cpos, align):
        d3 = lambda v: (C.c_double * 3)(*[float(x) for x in v])
        self._check(self.L.dmann_set_observer(self.ctx, d3(opos), d3(cpos), d3(align)))

    def set_frame(self, rot, opos):
        r = np.asarray(rot, dtype=np.float64).reshape(9)
        self._check(self.L.dmann_set_frame(self.ctx, (C.c_double * 9)(*r.tolist()),
                                           (C.c_double * 3)(*[float(x) for x in opos])))

    def set_units(self, unit_factor: float, hires_threshold: float = float("inf"), flux_model: int = 0):
        self._check(self.L.dmann_set_units(self.ctx, float(unit_factor), float(hires_threshold),
                                           int(flux_model)))

    def set_flux_params(self, velocity_to_cgs: float, cpos=(0.0, 0.0, 0.0)):
        """Constants of the flux laws: code velocity unit, halo centre."""
        self._check(self.L.dmann_set_flux_params(self.ctx, float(velocity_to_cgs),
                                                 (C.c_double * 3)(*[float(v) for v in cpos])))

    def set_halo_cores(self, x, y, z, radius):
        """The ann_core_nosom law's halo table (annmap.halocore.read_halo_table)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, radius)]
        n = len(arrs[0])
        self._check(self.L.dmann_set_halo_cores(self.ctx, *[C.c_void_p(a.ctypes.data) for a in arrs], n))

    def set_params(self, par, flux_model: int = 0):
        """Frame, units and flux law from a Parameters object (flux_model is
        a dmann_flux value or a law name such as "ann_somv")."""
        if isinstance(flux_model, str):
            flux_model = _lib.FLUX_LAWS[flux_model]
        self.set_frame(par.rotmatrix, par.params.opos)
        self.set_units(par.flux_unit_factor(flux_model), par.hires_threshold, flux_model)
        self.set_flux_params(par.codeunits.velocity_to_cgs, par.params.cpos)

    def set_tuning(self, nside: int | None = None, **kw):
        """Default tuning, or the entry for maps of ``nside``
        (warp_max_pixels, block_threads, blocks_per_sm,
        seg_min_deposits_log2)."""
        t = _lib.Tuning()
        for k, v in kw.items():
            setattr(t, k, v)
        if nside is None:
            self._check(self.L.dmann_set_tuning(self.ctx, C.byref(t)))
        else:
            self._check(self.L.dmann_set_tuning_nside(self.ctx, int(nside), C.byref(t)))

    def clear_tuning(self, nside: int):
        self._check(self.L.dmann_set_tuning_nside(self.ctx, int(nside), None))

    def get_tuning(self, nside: int | None = None) -> dict:
        t = _lib.Tuning()
        if nside is None:
            self._check(self.L.dmann_get_tuning(self.ctx, C.byref(t)))
        else:
            self._check(self.L.dmann_get_tuning_nside(self.ctx, int(nside), C.byref(t)))
        return {k: getattr(t, k) for k, _ in _lib.Tuning._fields_ if k != "reserved"}

    # ------------------------------------------------------------ rendering
    def begin(self, nside: int, precision: int = COMP_F32):
        self._keep = []
        self._nside = int(nside)
        self._check(self.L.dmann_map_begin(self.ctx, int(nside), int(precision)))

    def add(self, parts: dict):
        """Deposits one chunk: float32 arrays x, y, z, m, rho, h and, for the
        flux laws that use it, the velocity dispersion "sigmav"."""
        arrays = [parts[k] for k in FIELDS]
        n = len(arrays[0])
        sv = parts.get("sigmav")
        if any(len(a) != n for a in arrays) or (sv is not None and len(sv) != n):
            raise ValueError("particle arrays differ in length")
        self._use_torch_stream(arrays + ([sv] if sv is not None else []))
        ptrs = [self._ptr(a, np.float32) for a in arrays]
        svp = self._ptr(sv, np.float32) if sv is not None else None
        self._check(self.L.dmann_map_add_v(self.ctx, *ptrs, svp, int(n)))

    def end(self, out=None, accumulate: bool = False):
        npix = 12 * self._nside * self._nside
        if out is None:
            out = np.zeros(npix, dtype=np.float64)
        if len(out) != npix:
            raise ValueError("output map has the wrong length")
        if _is_torch(out):
            if out.dtype.is_floating_point and out.dtype.itemsize != 8 or not out.is_contiguous():
                raise ValueError("output map must be a contiguous float64 tensor")
            if out.is_cuda:
                self._use_torch_stream([out])
            ptr = C.c_void_p(out.data_ptr())
        else:
            if out.dtype != np.float64 or not out.flags.c_contiguous:
                raise ValueError("output map must be a contiguous float64 array")
            ptr = C.c_void_p(out.ctypes.data)
        self._check(self.L.dmann_map_end(self.ctx, ptr, int(bool(accumulate))))
        if not (_is_torch(out) and out.is_cuda):
            self._keep = []
        return out

    def abort(self):
        """Closes an open streamed map without output (dmann_map_abort)."""
        self._check(self.L.dmann_map_abort(self.ctx))
        self._keep = []

    def render(self, parts: dict, nside: int, precision: int = COMP_F32, out=None,
               accumulate: bool = False):
        self.begin(nside, precision)
        try:
            self.add(parts)
        except BaseException:
            self.abort()
            raise
        return self.end(out, accumulate)

    def render_batch(self, parts: dict, frames, nsides, precision: int = COMP_F32, outs=None):
        """One map per observer: frames is a list of (rot 3x3, opos 3) pairs,
        nsides the Nside of each map.  outs (optional) are the output maps
        (float64 numpy arrays or CUDA tensors); host arrays are made if absent."""
        k = len(frames)
        if len(nsides) != k:
            raise ValueError("one Nside per observer")
        if outs is None:
            outs = [np.zeros(12 * int(ns) * int(ns), dtype=np.float64) for ns in nsides]
        arrays = [parts[f] for f in FIELDS]
        n = len(arrays[0])
        self._keep = []
        self._use_torch_stream(arrays + [o for o in outs if _is_torch(o)])
        ptrs = [self._ptr(a, np.float32) for a in arrays]
        rot = np.concatenate([np.asarray(r, dtype=np.float64).reshape(9) for r, _ in frames])
        opos = np.concatenate([np.asarray(o, dtype=np.float64).reshape(3) for _, o in frames])
        ns = (C.c_int * k)(*[int(v) for v in nsides])
        mp = (C.c_void_p * k)(*[o.data_ptr() if _is_torch(o) else o.ctypes.data for o in outs])
        self._check(self.L.dmann_render_batch(
            self.ctx, *ptrs, int(n), k, rot.ctypes.data_as(C.POINTER(C.c_double)),
            opos.ctypes.data_as(C.POINTER(C.c_double)), ns, int(precision), mp))
        self._keep = []
        return outs

    def adjoint(self, parts: dict, nside: int, grad_map, out=None, precision: int = PLAIN_F64):
        """Gradient of L = sum_p grad_map[p] * map[p] (the map of ``render``
        for this frame, these units and this flux law) with respect to the
        particle inputs and the observer position; precision PLAIN_F64
        recomputes the weights in FP64, COMP_F32 with the compensated form's
        FP32 weights (faster).  The velocity dispersion "sigmav" (the somv,
        somv2 and pwave laws) is an input, not differentiated.  Returns
        (grad, grad_opos): grad is [6, n] float64 (rows x, y, z, m, rho, h; a
        CUDA tensor when the inputs are CUDA tensors, else numpy), grad_opos a
        length-3 numpy array."""
        arrays = [parts[f] for f in FIELDS]
        n = len(arrays[0])
        sv = parts.get("sigmav")
        if any(len(a) != n for a in arrays) or (sv is not None and len(sv) != n):
            raise ValueError("particle arrays differ in length")
        npix = 12 * int(nside) * int(nside)
        if len(grad_map) != npix:
            raise ValueError("grad_map has the wrong length")
        self._keep = []
        on_gpu = any(_is_torch(a) and a.is_cuda for a in arrays)
        if out is None:
            if on_gpu:
                import torch
                out = torch.empty((6, n), dtype=torch.float64, device=arrays[0].device)
            else:
                out = np.zeros((6, n), dtype=np.float64)
        self._use_torch_stream(arrays + [grad_map, out] + ([sv] if sv is not None else []))
        ptrs = [self._ptr(a, np.float32) for a in arrays]
        svp = self._ptr(sv, np.float32) if sv is not None else None
        gm = self._ptr(grad_map, np.float64)
        optr = C.c_void_p(out.data_ptr() if _is_torch(out) else out.ctypes.data)
        go = (C.c_double * 3)()
        self._check(self.L.dmann_adjoint_v(self.ctx, *ptrs, svp, int(n), int(nside), int(precision),
                                           gm, optr, go))
        self._keep = []
        return out, np.array(go[:])

    def synchronize(self):
        self._check(self.L.dmann_synchronize(self.ctx))
        self._keep = []

    def stats(self) -> dict:
        s = _lib.Stats()
        self._check(self.L.dmann_get_stats(self.ctx, C.byref(s)))
        return {k: getattr(s, k) for k, _ in _lib.Stats._fields_}


class MapGenerator:
    """The reference's MapGenerator (src/mapgenerator.h:8-26) on the GPU."""

    def __init__(self, par, reader, precision: int = COMP_F32, device: int = 0, flux_model=0,
                 halo_file: str = "./halocore/VL2_Halos.data"):
        self.par_ = par
        self.reader_ = reader
        self.precision = precision
        self.device = device
        self.flux_model = flux_model   # the reference's link-time getflux plugin, chosen here
        self.halo_file = halo_file     # read by the ann_core_nosom law, as the reference does
        self.map_ = None
        self.isFinished_ = False
        self.total_flux = None

    def start(self):
        r = Renderer(self.device)
        try:
            r.set_params(self.par_, self.flux_model)
            if self.flux_model in (6, "ann_core_nosom"):
                from .halocore import read_halo_table
                r.set_halo_cores(*read_halo_table(self.halo_file))
            r.begin(self.par_.map.Nside, self.precision)
            try:
                while self.reader_.hasNext():
                    r.add(self.reader_.next_chunk())
            except BaseException:
                r.abort()
                raise
            self.map_ = r.end()
            st = r.stats()
            self.total_flux = st["total_flux"]  # the reference's "Total Conts"
            self.stats = st
        finally:
            r.close()
        self.isFinished_ = True

    def isFinished(self) -> bool:
        return self.isFinished_

    def getMap(self):
        return self.map_

    def getNside(self) -> int:
        return self.par_.map.Nside

    def saveToFits(self, fits_file: str, isVerbose: bool = False):
        from .fitsio import write_healpix_map
        if not self.isFinished():
            print("Map not generated yet")
            return
        write_healpix_map(fits_file or self.par_.outputFileName, self.map_)
