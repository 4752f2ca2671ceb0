"""vl2read: the reference's Python particle-reader module, kept by name.

The reference builds a SWIG module ``vl2read`` (src/pywrapper/vl2read.i,
src/pywrapper/setup.py:3) around one class, ``VL2Reader``
(src/pywrapper/vl2read.h:6-28, src/pywrapper/vl2read.cpp), that streams a
particle file through the reference's DataReader and keeps, for the particles
inside an axis-aligned box around (xc, yc, zc), their density and velocity
components.  This module keeps the same module name, class name,
constructors, getters and the ``INITMEMSIZE`` constant, so scripts that
``import vl2read`` run unchanged; it reads through ``annmap.DataReader``
(the same native / Tipsy XDR formats and byte-mask semantics).

Selection, as vl2read.cpp's loop does it: a particle is kept when
|pos_k - c_k| < boxsize / 2 for each axis k, the float position promoted to
double before the subtraction.  The mask does not remove particles; like the
reference's reader it sets the density of masked particles to -1.

The getters return float32 numpy arrays (the reference returns a reference
to its std::vector<float>): the same array on every call, so changes made
through one are seen by the next, as with the reference's proxy.
``fArray`` / ``dArray`` stand for the SWIG ``%array_class`` helpers of
vl2read.i (fixed-size float / double arrays with item access and ``cast``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from annmap.reader import DataReader

__all__ = ["VL2Reader", "fArray", "dArray"]


class VL2Reader:
    """Particles of a native or Tipsy file inside a box (vl2read.h:6-28).

    ``VL2Reader(filename, xc, yc, zc, boxsize, maskfile="")`` reads a native
    particle file (int32 count, 48-byte records).

    ``VL2Reader(basename, filename, xc, yc, zc, boxsize, maskfile="",
    isSingleFile=False)`` reads a Tipsy XDR snapshot ``basename/filename``
    and, unless ``isSingleFile``, the "smooth" side files
    ``basename/filename.den32``, ``.hsm32`` and ``.sigma32`` (the reference's
    directory/base-name DataReader constructor, src/datareader.cpp:73-93);
    with ``isSingleFile`` the densities are all zero.
    """

    INITMEMSIZE = 128 * 1024   # vl2read.cpp:14 (initial capacity of the vectors)

    def __init__(self, *args, **kw):
        if "basename" in kw or (len(args) >= 2 and isinstance(args[1], (str, bytes, os.PathLike))):
            names = ("basename", "filename", "xc", "yc", "zc", "boxsize", "maskfile", "isSingleFile")
            tipsy = True
        else:
            names = ("filename", "xc", "yc", "zc", "boxsize", "maskfile")
            tipsy = False
        if len(args) > len(names):
            raise TypeError(f"VL2Reader takes at most {len(names)} arguments")
        a = dict(zip(names, args))
        for k, v in kw.items():
            if k not in names or k in a:
                raise TypeError(f"unexpected or repeated argument {k!r}")
            a[k] = v
        missing = [k for k in names[: len(names) - (2 if tipsy else 1)] if k not in a]
        if missing:
            raise TypeError("missing arguments: " + ", ".join(missing))
        maskfile = str(a.get("maskfile", "") or "")
        single = bool(a.get("isSingleFile", False)) if tipsy else True
        self._load(str(a.get("basename", "")), str(a["filename"]), float(a["xc"]), float(a["yc"]),
                   float(a["zc"]), float(a["boxsize"]), maskfile, single, tipsy)

    def _load(self, basename, filename, xc, yc, zc, boxsize, maskfile, single, tipsy):
        is_mask = maskfile != ""
        if tipsy:
            part = basename + "/" + filename
            reader = DataReader.tipsy(part, part + ".den32", part + ".hsm32", part + ".sigma32",
                                      isMask=is_mask, maskfile=maskfile, isSingleFile=single)
        else:
            reader = DataReader(filename, is_mask, maskfile)
        reader.open()
        half = boxsize / 2
        dens, vx, vy, vz = [], [], [], []
        try:
            while reader.hasNext():
                c = reader.next_chunk(velocities=True)
                keep = ((np.abs(c["x"].astype(np.float64) - xc) < half) &
                        (np.abs(c["y"].astype(np.float64) - yc) < half) &
                        (np.abs(c["z"].astype(np.float64) - zc) < half))
                dens.append(c["rho"][keep])
                vx.append(c["vx"][keep])
                vy.append(c["vy"][keep])
                vz.append(c["vz"][keep])
        finally:
            reader.close()
        cat = lambda parts: np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros(0),
                                                 dtype=np.float32)
        self.density_ = cat(dens)
        self.velX_ = cat(vx)
        self.velY_ = cat(vy)
        self.velZ_ = cat(vz)

    def getDensity(self) -> np.ndarray:
        return self.density_

    def getVelocityX(self) -> np.ndarray:
        return self.velX_

    def getVelocityY(self) -> np.ndarray:
        return self.velY_

    def getVelocityZ(self) -> np.ndarray:
        return self.velZ_


class _CArray:
    """A fixed-size C array with item access (SWIG's %array_class)."""
    _ctype = C.c_float

    def __init__(self, nelements: int):
        self._buf = (self._ctype * int(nelements))()

    def __getitem__(self, i: int):
        return self._buf[i]

    def __setitem__(self, i: int, v):
        self._buf[i] = v

    def __len__(self):
        return len(self._buf)

    def cast(self):
        """A pointer to the first element."""
        return C.cast(self._buf, C.POINTER(self._ctype))

    @classmethod
    def frompointer(cls, ptr):
        """Item access to the elements at ptr (a ctypes pointer or an address)
        without a copy; as in C, nothing checks the index."""
        obj = cls.__new__(cls)
        addr = ptr if isinstance(ptr, int) else C.cast(ptr, C.c_void_p).value
        obj._buf = C.cast(C.c_void_p(addr), C.POINTER(cls._ctype))
        return obj


class fArray(_CArray):
    _ctype = C.c_float


class dArray(_CArray):
    _ctype = C.c_double
