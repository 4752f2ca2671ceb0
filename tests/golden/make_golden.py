"""Generates the golden fixtures in tests/golden/ from the reference's own
CPU map path.

The reference's src/genmap.cpp, src/parameters.cpp, src/anglefuncs.cpp,
src/datatypes.cpp, src/datareader.cpp and src/flux/flux_ann_nosom.cpp are
compiled where they lie by oracle/ref_shim/Makefile (HEALPix and XDR replaced
by stand-ins; see that directory) into oracle/_ref/annmap_ref.  For each case
below this script writes the reference's own inputs -- an info file and a
native particle file (int32 N + N x 48-byte DMParticle records, plus an
optional byte mask file) -- runs the reference binary, and stores the inputs,
the info file text, the derived Parameters fields and the output map in
``<case>.npz``.

Run here (the reference sources are only present on this machine):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "dm-annihilation-cxx_gb300", "pywrapper"))
from annmap import synth  # noqa: E402

REF_BIN = os.path.join(REPO, "oracle", "_ref", "annmap_ref")


def build_ref():
    # the reference sources: DMANN_REF_SRC, else a `reference` checkout beside
    # this repository (the Makefile's default)
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref_shim")], check=True)


def write_native(path, P, extra_mass=None, sigmav=None):
    rec = np.zeros((len(P), 12), np.float32)
    if sigmav is not None:
        rec[:, 9] = sigmav
    rec[:, 0] = P.m if extra_mass is None else extra_mass
    rec[:, 1] = P.rho
    rec[:, 2] = P.h
    rec[:, 3] = P.x
    rec[:, 4] = P.y
    rec[:, 5] = P.z
    with open(path, "wb") as f:
        np.array([len(P)], np.int32).tofile(f)
        rec.tofile(f)
    return rec


def write_tipsy(d, P, rng):
    """The reference's XDR input (src/datareader.cpp:120-190, src/tipsy_io.c):
    a big-endian Tipsy file with 7 gas, the dark particles of P and 3 star
    particles, and the density / hsmooth / sigmav side files of "smooth"
    (native int32 count of all bodies, then one float per body, gas first).
    Returns the DMParticle records of the dark particles."""
    nsph, ndark, nstar = 7, len(P), 3
    nb = nsph + ndark + nstar
    dark = np.zeros((ndark, 9), np.float32)
    dark[:, 0] = P.m
    dark[:, 1], dark[:, 2], dark[:, 3] = P.x, P.y, P.z
    dark[:, 4:7] = rng.normal(0, 100, (ndark, 3))
    dark[:, 7] = 0.01
    dark[:, 8] = rng.normal(0, 1, ndark)
    paths = {k: os.path.join(d, k + ".bin") for k in ("tipsy", "dens", "hsm", "sigv")}
    with open(paths["tipsy"], "wb") as f:
        f.write(np.array([0.5], ">f8").tobytes())
        f.write(np.array([nb, 3, nsph, ndark, nstar, 0], ">i4").tobytes())
        f.write(rng.normal(size=(nsph, 12)).astype(">f4").tobytes())
        f.write(dark.astype(">f4").tobytes())
        f.write(rng.normal(size=(nstar, 11)).astype(">f4").tobytes())
    sv = rng.lognormal(np.log(3000.0), 1.0, ndark).astype(np.float32)
    side = {"dens": P.rho, "hsm": P.h, "sigv": sv}
    for k, v in side.items():
        with open(paths[k], "wb") as f:
            np.array([nb], np.int32).tofile(f)
            np.concatenate([rng.uniform(1, 2, nsph), v, rng.uniform(1, 2, nstar)]).astype(np.float32).tofile(f)
    rec = np.zeros((ndark, 12), np.float32)
    rec[:, 0], rec[:, 1], rec[:, 2] = P.m, P.rho, P.h
    rec[:, 3:6] = dark[:, 1:4]
    rec[:, 6:9] = dark[:, 4:7]
    rec[:, 9], rec[:, 10], rec[:, 11] = sv, dark[:, 7], dark[:, 8]
    files = {k: np.frombuffer(open(p_, "rb").read(), np.uint8) for k, p_ in paths.items()}
    return rec, paths, files


def parse_params(text):
    out = {}
    for line in text.strip().splitlines():
        k, *v = line.split()
        out[k] = np.array([float(x) for x in v])
    return out


def run_case(name, P, *, nside, info_extra="", mass=None, mask=None, particle_masses=None,
             obs=None, centre=(0.0, 0.0, 0.0), align=(0.0, 0.0, 1.0), units="kpc",
             mem_buffer=1000, test=None, law="ann_nosom", sigmav=None, halos=None, tipsy=False):
    d = tempfile.mkdtemp(prefix="golden_")
    if halos is not None:   # the core law reads ./halocore/VL2_Halos.data (x y z radius lines)
        os.makedirs(os.path.join(d, "halocore"))
        with open(os.path.join(d, "halocore", "VL2_Halos.data"), "w") as f:
            for row in np.stack(halos, axis=1):
                f.write("\t".join(repr(float(np.float32(v))) for v in row) + "\n")
    tipsy_files = {}
    if tipsy:
        rec, tpaths, tipsy_files = write_tipsy(d, P, np.random.Generator(np.random.PCG64(1113)))
    else:
        rec = write_native(os.path.join(d, "parts.bin"), P, extra_mass=mass, sigmav=sigmav)
    obs = P.obs_pos if obs is None else obs
    pm = particle_masses if particle_masses is not None else [P.particle_mass]
    lines = ["# golden case " + name, "Omega_M = 0.238", "h100 = 0.73", "n_s = 0.951",
             "sigma_8 = 0.74"]
    if units == "kpc":
        lines += ["Lbox_in_Mpc = 0.001", "mass_to_Msun = 1"]
    else:  # the reference's own Via Lactea II unit system: mass derived from rho_crit * L^3
        lines += ["Lbox_in_Mpc = 40.0"]
    lines += ["particle_masses = " + " ".join(repr(float(x)) for x in pm),
              "centerpos = " + " ".join(repr(float(x)) for x in centre),
              "align_vec = " + " ".join(repr(float(x)) for x in align),
              "obs_pos = " + " ".join(repr(float(x)) for x in obs),
              f"nside = {nside}", f"mem_buffer = {mem_buffer}"]
    if tipsy:
        lines += [f"partfile = {d}/tipsy.bin", f"densfile = {d}/dens.bin", f"hsmfile = {d}/hsm.bin",
                  f"vdspfile = {d}/sigv.bin"]
    else:
        lines += [f"datafile = {d}/parts.bin"]
    if test is not None:
        lines.append(f"test = {test}")
    if mask is not None:
        with open(os.path.join(d, "mask.bin"), "wb") as f:
            np.array([len(P)], np.int32).tofile(f)
            np.asarray(mask, np.uint8).tofile(f)
        lines.append(f"mask = {d}/mask.bin")
    lines.append("outputmap = unused.fits")
    ini = "\n".join(lines) + "\n" + info_extra
    with open(os.path.join(d, "info.ini"), "w") as f:
        f.write(ini)
    binary = REF_BIN if law == "ann_nosom" else REF_BIN + "_" + law
    r = subprocess.run([binary, os.path.join(d, "info.ini"), os.path.join(d, "map.bin"),
                        os.path.join(d, "par.txt")], capture_output=True, text=True, cwd=d)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: reference failed: {r.stderr[-500:]}")
    mp = np.fromfile(os.path.join(d, "map.bin"), np.float64)
    with open(os.path.join(d, "par.txt")) as f:
        par = parse_params(f.read())
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), map=mp, info=np.array(ini.replace(d, "@DIR@")),
        records=rec, mask=(np.asarray(mask, np.uint8) if mask is not None else np.zeros(0, np.uint8)),
        flux_law=np.array(law), **{"tipsy_" + k: v for k, v in tipsy_files.items()},
        halos=(np.stack(halos, axis=1).astype(np.float32) if halos is not None else np.zeros((0, 4), np.float32)),
        **{"par_" + k: v for k, v in par.items()})
    assert np.all(np.isfinite(mp)), name
    print(f"{name}: nside={nside} n={len(P)} sum(map*dOmega)={mp.sum() * par['dOmega'][0]:.6e}")


def main():
    build_ref()
    os.makedirs(HERE, exist_ok=True)
    # 1. small NFW host, generic observer, Nside 16
    run_case("nfw_ns16", synth.nfw_halo(400, seed=101), nside=16)
    # 2. host + subhalos, Nside 64, chunked reading (mem_buffer < N)
    run_case("nfw_sub_ns64", synth.nfw_halo(3000, seed=102, n_sub=8), nside=64, mem_buffer=700)
    # 3. near-observer particles (discs past pi: all-sky) + far tiny particles
    P = synth.nfw_halo(600, seed=103, near_observer=40, near_radius=0.5)
    run_case("near_observer_ns32", P, nside=32)
    # 4. observer on the z axis (polar frame) and on the x axis
    P = synth.nfw_halo(500, seed=104, obs_pos=(0.0, 0.0, 8.0))
    run_case("obs_zaxis_ns32", P, nside=32)
    P = synth.nfw_halo(500, seed=105, obs_pos=(8.0, 0.0, 0.0))
    run_case("obs_xaxis_ns32", P, nside=32, align=(0.3, -0.2, 0.93))
    # 5. two mass resolutions (the hires filter) and a mask (dens = -1)
    P = synth.nfw_halo(1500, seed=106)
    rng = np.random.Generator(np.random.PCG64(1106))
    mass = P.m.copy()
    heavy = rng.uniform(size=len(P)) < 0.3
    mass[heavy] = P.particle_mass * 8.0
    mask = (rng.uniform(size=len(P)) > 0.2).astype(np.uint8)
    run_case("hires_mask_ns32", P, nside=32, mass=mass, mask=mask,
             particle_masses=[P.particle_mass * 8.0, P.particle_mass])
    # 6. the reference's own unit system (Lbox 40 Mpc, mass from rho_crit L^3),
    #    positions in box units around a VL2-like centre, test limit
    P = synth.nfw_halo(800, seed=107)
    c = np.array([0.3612030, 0.2106580, 0.00687726])
    scale = 1.0 / 40000.0  # kpc -> box units of 40 Mpc
    Q = synth.Particles((P.x * scale + c[0]).astype(np.float32), (P.y * scale + c[1]).astype(np.float32),
                        (P.z * scale + c[2]).astype(np.float32), (P.m * 1e-12).astype(np.float32),
                        P.rho, (P.h * scale).astype(np.float32))
    obs = tuple((np.array(P.obs_pos) * scale + c).tolist())
    run_case("vl2units_ns16", Q, nside=16, units="vl2", particle_masses=[4.1e-9],
             obs=obs, centre=tuple(c.tolist()), align=(-0.025836, 0.133297, 0.990739), test=700)
    # 7. a non power of two Nside and high-resolution small discs (single-pixel branches)
    P = synth.nfw_halo(2000, seed=108, n_sub=4)
    run_case("nside24", P, nside=24)
    P = synth.nfw_halo(1200, seed=109, n_sub=30, sub_frac=0.6)
    run_case("subhalo_ns128", P, nside=128)
    # 8. the other flux laws (the reference links one getflux plugin per
    #    build): velocity dispersions log-normal around 30 km/s, some below
    #    the somv / somv2 saturation speeds of 1 and 5 km/s
    P = synth.nfw_halo(900, seed=110, n_sub=3)
    v_kms = np.exp(np.random.Generator(np.random.PCG64(1110)).normal(np.log(30.0), 1.6, len(P)))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    op = O.make_params(nside=8, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                       particle_masses=(P.particle_mass,))
    vel_to_cgs = op.velocity_to_cgs
    sigmav = (v_kms * 1.0e5 / vel_to_cgs).astype(np.float32)
    for law in ("ann_somv", "ann_somv2", "ann_pwave", "decay"):
        run_case("flux_" + law + "_ns32", P, nside=32, law=law, sigmav=sigmav, mem_buffer=400)
    # adiabatic contraction in the reference's own units (r in kpc/h there)
    Q = synth.nfw_halo(700, seed=111)
    c = np.array([0.3612030, 0.2106580, 0.00687726])
    scale = 1.0 / 40000.0
    R = synth.Particles((Q.x * scale + c[0]).astype(np.float32), (Q.y * scale + c[1]).astype(np.float32),
                        (Q.z * scale + c[2]).astype(np.float32), (Q.m * 1e-12).astype(np.float32),
                        Q.rho, (Q.h * scale).astype(np.float32))
    obs = tuple((np.array(Q.obs_pos) * scale + c).tolist())
    run_case("flux_ann_adiabatic_ns16", R, nside=16, units="vl2", particle_masses=[4.1e-9],
             obs=obs, centre=tuple(c.tolist()), align=(-0.025836, 0.133297, 0.990739),
             law="ann_adiabatic")
    # halo cores (VL2_Halos.data layout: x y z radius) on 300 synthetic halos
    # centred on particles, radius column 1..8 (core radius radius/29200 box units)
    rng = np.random.Generator(np.random.PCG64(1112))
    pick = rng.choice(len(R), 300, replace=False)
    jit = rng.normal(0.0, 5e-5, (300, 3))
    halos = ((R.x[pick] + jit[:, 0]).astype(np.float32), (R.y[pick] + jit[:, 1]).astype(np.float32),
             (R.z[pick] + jit[:, 2]).astype(np.float32), rng.uniform(1.0, 8.0, 300).astype(np.float32))
    run_case("flux_ann_core_nosom_ns16", R, nside=16, units="vl2", particle_masses=[4.1e-9],
             obs=obs, centre=tuple(c.tolist()), align=(-0.025836, 0.133297, 0.990739),
             law="ann_core_nosom", halos=halos)
    # 9. the Tipsy XDR input (gas and star particles skipped, side files of
    #    "smooth"), chunked and with a mask, under the somv law (reads sigmav)
    P = synth.nfw_halo(1100, seed=112, n_sub=2)
    mask = (np.random.Generator(np.random.PCG64(1114)).uniform(size=len(P)) > 0.1).astype(np.uint8)
    run_case("tipsy_somv_ns32", P, nside=32, tipsy=True, mask=mask, mem_buffer=300, law="ann_somv")


if __name__ == "__main__":
    main()
