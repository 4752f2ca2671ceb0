"""Loads the golden fixtures of tests/golden (made by make_golden.py from the
reference's own CPU map path) back into particle arrays and info-file
values, applying the reference reader's semantics: the byte mask sets
dens = -1 where it is 0 (src/datareader.cpp:263-271) and ``test`` keeps the
first ``test`` particles (src/datareader.cpp:202-206)."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def parse_info(text):
    """Key/values with the reference's tokenisation: split on spaces, first
    token is the key, the second (``=``) is skipped (parameters.cpp:331-338)."""
    out = {}
    for line in text.splitlines():
        toks = [t for t in line.split(" ") if t]
        if not toks or toks[0].startswith("#") or len(toks) < 3:
            continue
        out[toks[0]] = toks[2:]
    return out


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    info = parse_info(str(z["info"]))
    rec = z["records"]
    parts = {"m": rec[:, 0].copy(), "rho": rec[:, 1].copy(), "h": rec[:, 2].copy(),
             "x": rec[:, 3].copy(), "y": rec[:, 4].copy(), "z": rec[:, 5].copy(),
             "sigmav": rec[:, 9].copy()}
    mask = z["mask"]
    if mask.size:
        parts["rho"][mask == 0] = -1.0
    if "test" in info and int(info["test"][0]) != -1:
        k = int(info["test"][0])
        parts = {k2: v[:k] for k2, v in parts.items()}
    par = {k[4:]: z[k] for k in z.files if k.startswith("par_")}
    law = str(z["flux_law"]) if "flux_law" in z.files else "ann_nosom"
    halos = z["halos"] if "halos" in z.files else np.zeros((0, 4), np.float32)
    return {"parts": parts, "info": info, "map": z["map"], "par": par, "info_text": str(z["info"]),
            "flux_law": law, "halos": halos}


FLUX_LAWS = {"ann_nosom": 0, "ann_somv": 1, "ann_somv2": 2, "ann_pwave": 3, "decay": 4,
             "ann_adiabatic": 5, "ann_core_nosom": 6}


def oracle_params(case):
    """orc_params for a golden case built from its info-file values."""
    import oracle as O
    info = case["info"]
    f = lambda k, d=None: [float(v) for v in info[k]] if k in info else d
    return O.make_params(
        nside=int(info["nside"][0]), obs_pos=f("obs_pos"), centerpos=f("centerpos"),
        align_vec=f("align_vec"), h100=f("h100")[0], Omega_M=f("Omega_M")[0],
        Lbox_in_Mpc=f("Lbox_in_Mpc")[0], mass_to_Msun=f("mass_to_Msun", [-1.0])[0],
        particle_masses=f("particle_masses"), flux_model=FLUX_LAWS[case["flux_law"]],
        halos=(tuple(case["halos"][:, k] for k in range(4)) if len(case["halos"]) else None))
