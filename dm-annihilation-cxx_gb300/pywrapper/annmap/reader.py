"""DataReader: chunked reading of the reference's native particle file.

Native format (src/datareader.cpp:120,237; record layout src/datatypes.h:46-59):
an int32 particle count N, then N records of twelve float32 fields
(mass, dens, hsmooth, posx, posy, posz, velx, vely, velz, sigmav, eps, phi).
An optional mask file holds an int32 count and one byte per particle; a
zero byte marks the particle as masked by setting dens = -1
(src/datareader.cpp:263-271).  ``setTest(n)`` limits the stream to the first
n particles (src/datareader.cpp:202-206); ``setBuf(n)`` sets the chunk size.

The reader yields float32 SoA chunks (x, y, z, m, rho, h, and the velocity
dispersion sigmav some flux laws read) -- the layout the GPU kernels read --
instead of the 48-byte AoS records.
"""
from __future__ import annotations

import os

import numpy as np

RECORD = np.dtype([(n, "<f4") for n in ("mass", "dens", "hsmooth", "posx", "posy", "posz", "velx",
                                        "vely", "velz", "sigmav", "eps", "phi")])
assert RECORD.itemsize == 48


DARK = np.dtype([(n, ">f4") for n in ("mass", "posx", "posy", "posz", "velx", "vely", "velz", "eps",
                                      "phi")])   # a Tipsy XDR dark record (src/tipsy_io.c:174-192)


class DataReader:
    def __init__(self, path: str, isMask: bool = False, maskfile: str = ""):
        self.path = path
        self.isMask = bool(isMask)
        self.maskfile = maskfile
        self._tipsy = None
        self.memBuffer = 10000000
        self.testnum = -1
        self._n = 0
        self._cursor = 0
        self._mm = None
        self._mask = None
        self._open = False

    # reference API
    def setTest(self, tn: int):
        self.testnum = int(tn)

    def setBuf(self, mem: int):
        self.memBuffer = max(1, int(mem))

    def getPartNum(self) -> int:
        return self.testnum if self.testnum != -1 else self._n

    @classmethod
    def tipsy(cls, partfile: str, densfile: str, hsmfile: str, sigmafile: str, isMask: bool = False,
              maskfile: str = "", isSingleFile: bool = False) -> "DataReader":
        """The reference's XDR constructor (src/datareader.h:32-39): a Tipsy
        file (big-endian; only its dark particles are read, gas records are
        skipped) and the density / hsmooth / sigmav side files of "smooth"
        (int32 count of all bodies, one float per body, gas first)."""
        r = cls(partfile, isMask, maskfile)
        r._tipsy = (densfile, hsmfile, sigmafile, bool(isSingleFile))
        return r

    def _open_tipsy(self):
        dens, hsm, sig, single = self._tipsy
        with open(self.path, "rb") as f:
            h = f.read(32)
        if len(h) < 32:
            raise ValueError(f"Problem reading tipsy header: {self.path}")
        nbodies, _ndim, nsph, ndark, _nstar = np.frombuffer(h[8:28], dtype=">i4").tolist()
        self._mm = np.memmap(self.path, dtype=DARK, mode="r", offset=32 + 48 * nsph, shape=(ndark,))
        self._side = None
        if not single:
            self._side = []
            for path, what in ((dens, "density"), (hsm, "hsmooth"), (sig, "sigmav")):
                with open(path, "rb") as f:
                    np_ = int(np.fromfile(f, dtype="<i4", count=1)[0])
                if np_ != nbodies:
                    raise ValueError(f"Particle numbers in {what} not match.")
                self._side.append(np.memmap(path, dtype="<f4", mode="r", offset=4 + 4 * nsph,
                                            shape=(ndark,)))
        return ndark

    def open(self) -> bool:
        if not os.path.exists(self.path):
            raise FileNotFoundError(f"Datafile error: {self.path}")
        if self._tipsy is not None:
            n = self._open_tipsy()
        else:
            with open(self.path, "rb") as f:
                n = int(np.fromfile(f, dtype="<i4", count=1)[0])
            self._mm = np.memmap(self.path, dtype=RECORD, mode="r", offset=4, shape=(n,))
        self._n = n
        if self.isMask:
            with open(self.maskfile, "rb") as f:
                nm = int(np.fromfile(f, dtype="<i4", count=1)[0])
            if nm != n:
                raise ValueError("Particle numbers in mask file not match.")
            self._mask = np.memmap(self.maskfile, dtype=np.uint8, mode="r", offset=4, shape=(n,))
        if self.testnum != -1 and self._n > self.testnum:
            self._n = self.testnum
        self._cursor = 0
        self._open = True
        return True

    def hasNext(self) -> bool:
        return self._open and self._cursor < self._n

    def next_chunk(self, velocities: bool = False) -> dict:
        """The next chunk as float32 SoA arrays x, y, z, m, rho, h and sigmav;
        with ``velocities`` also the velocity components vx, vy, vz."""
        i0 = self._cursor
        i1 = min(self._n, i0 + self.memBuffer)
        rec = np.asarray(self._mm[i0:i1])
        if self._tipsy is not None:
            out = {"x": rec["posx"], "y": rec["posy"], "z": rec["posz"], "m": rec["mass"]}
            if velocities:
                out.update({"vx": rec["velx"], "vy": rec["vely"], "vz": rec["velz"]})
            out = {k: np.ascontiguousarray(v, dtype=np.float32) for k, v in out.items()}
            if self._side is None:
                z = np.zeros(i1 - i0, np.float32)
                dens, hs, sv = z, z.copy(), z.copy()
            else:
                dens, hs, sv = (np.array(a[i0:i1], dtype=np.float32) for a in self._side)
            if self._mask is not None:
                dens[np.asarray(self._mask[i0:i1]) == 0] = -1.0
            self._cursor = i1
            out.update({"rho": dens, "h": hs, "sigmav": sv})
            return out
        rho = np.ascontiguousarray(rec["dens"])
        if self._mask is not None:
            rho = rho.copy()
            rho[np.asarray(self._mask[i0:i1]) == 0] = -1.0
        self._cursor = i1
        out = {"x": np.ascontiguousarray(rec["posx"]), "y": np.ascontiguousarray(rec["posy"]),
               "z": np.ascontiguousarray(rec["posz"]), "m": np.ascontiguousarray(rec["mass"]),
               "rho": rho, "h": np.ascontiguousarray(rec["hsmooth"]),
               "sigmav": np.ascontiguousarray(rec["sigmav"])}
        if velocities:
            out.update({k: np.ascontiguousarray(rec["vel" + k[1]]) for k in ("vx", "vy", "vz")})
        return out

    def close(self):
        self._mm = None
        self._mask = None
        self._open = False


def write_native(path: str, parts: dict, extra: dict | None = None):
    """Writes float32 SoA arrays as a native particle file (the inverse of the reader)."""
    n = len(parts["x"])
    rec = np.zeros(n, dtype=RECORD)
    rec["mass"], rec["dens"], rec["hsmooth"] = parts["m"], parts["rho"], parts["h"]
    rec["posx"], rec["posy"], rec["posz"] = parts["x"], parts["y"], parts["z"]
    for k, v in (extra or {}).items():
        rec[k] = v
    with open(path, "wb") as f:
        np.array([n], dtype="<i4").tofile(f)
        rec.tofile(f)
