"""The halo table of the ann_core_nosom flux law (src/halocore/halocore.cpp:
16-45): one halo per line, ``x y z radius`` (centres in box units; the core
radius is radius / (0.73 * 40000) box units).  The reference reads it from
``./halocore/VL2_Halos.data``; the number of halos is the number of lines."""
from __future__ import annotations

import numpy as np

DEFAULT_HALO_FILE = "./halocore/VL2_Halos.data"


def read_halo_table(path: str = DEFAULT_HALO_FILE):
    """(x, y, z, radius) float32 arrays, in file order."""
    with open(path) as f:
        lines = f.read().splitlines()
    if not lines:
        raise ValueError(f"empty halo file: {path}")
    vals = np.array(" ".join(lines).split(), dtype=np.float64)
    if vals.size < 4 * len(lines):
        raise ValueError(f"halo file {path}: expected 4 values on each of {len(lines)} lines")
    t = vals[: 4 * len(lines)].reshape(len(lines), 4).astype(np.float32)
    return t[:, 0].copy(), t[:, 1].copy(), t[:, 2].copy(), t[:, 3].copy()


def write_halo_table(path: str, x, y, z, radius):
    with open(path, "w") as f:
        for row in zip(x, y, z, radius):
            f.write("\t".join(repr(float(np.float32(v))) for v in row) + "\n")
