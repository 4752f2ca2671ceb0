"""Writes a golden case as the reference's on-disk inputs (info file, native
particle file, mask file) for the C++ host-API tests."""
import os

import numpy as np

import golden_cases as G


def write_case(tmp_path, name="hires_mask_ns32", mem_buffer=333, output=None):
    case = G.load(name)
    z = np.load(os.path.join(G.GOLDEN, name + ".npz"))
    rec, mask = z["records"], z["mask"]
    data = os.path.join(str(tmp_path), "parts.bin")
    with open(data, "wb") as f:
        np.array([len(rec)], np.int32).tofile(f)
        rec.tofile(f)
    for k in ("tipsy", "dens", "hsm", "sigv"):   # a Tipsy case's XDR input and side files
        if "tipsy_" + k in z.files:
            with open(os.path.join(str(tmp_path), k + ".bin"), "wb") as f:
                f.write(z["tipsy_" + k].tobytes())
    mpath = os.path.join(str(tmp_path), "mask.bin")
    if mask.size:
        with open(mpath, "wb") as f:
            np.array([len(rec)], np.int32).tofile(f)
            mask.tofile(f)
    text = case["info_text"].replace("@DIR@/parts.bin", data).replace("@DIR@/mask.bin", mpath)
    text = text.replace("@DIR@", str(tmp_path))
    lines = [ln for ln in text.split("\n") if not ln.startswith("mem_buffer") and not ln.startswith("outputmap")]
    lines.append(f"mem_buffer = {mem_buffer}")
    if output:
        lines.append(f"outputmap = {output}")
    info = os.path.join(str(tmp_path), "info.ini")
    with open(info, "w") as f:
        f.write("\n".join(lines) + "\n")
    return case, info
