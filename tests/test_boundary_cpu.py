"""The C-ABI library and the host-side layers, without a GPU: every symbol
include/*.h declares is exported; the host-only helpers reproduce the
reference's Parameters fields (golden fixtures); the Python Parameters mirror
parses info files like src/parameters.cpp; the native reader round-trips."""
import ctypes as C
import glob
import math
import os
import re

import numpy as np
import pytest

import golden_cases as G
import annmap
from annmap import _lib
from annmap.params import Parameters, atof, atoi
from annmap.reader import DataReader, write_native

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(dmann_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    decl = declared_symbols()
    assert decl, "no declarations found"
    for name in sorted(decl):
        assert hasattr(L, name), name
    # the ctypes table covers the header exactly
    assert set(_lib.SIGNATURES) == decl


def test_abi_version():
    assert _lib.load().dmann_abi_version() == 2


def test_no_gpu_fails_loudly():
    # This container has no GPU: creating a context must fail with a status,
    # never fall back to a CPU path.
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(annmap.DmannError) as e:
        annmap.Renderer()
    assert e.value.status == _lib.ERR_NODEVICE


def test_null_context_calls_are_rejected():
    L = _lib.load()
    assert L.dmann_render(None, None, None, None, None, None, None, 0, 16, 1, None, 0) == _lib.ERR_INVALID
    assert L.dmann_map_begin(None, 16, 1) == _lib.ERR_INVALID
    assert L.dmann_set_units(None, 1.0, 1.0, 0) == _lib.ERR_INVALID


@pytest.mark.parametrize("name", G.names())
def test_host_helpers_match_reference_parameters(name):
    case = G.load(name)
    par = case["par"]
    p = Parameters(text=case["info_text"].replace("@DIR@", "/nonexistent"))
    rot = np.array(p.rotmatrix)
    for i in range(3):
        assert np.array_equal(rot[i], par[f"rotmatrix{i}"]), (i, rot[i], par[f"rotmatrix{i}"])
    assert p.params.otheta == par["otheta"][0]
    assert p.params.ophi == par["ophi"][0]
    cu = p.codeunits
    for k in ("mass_to_cgs", "length_to_cgs", "density_to_cgs", "time_to_cgs", "velocity_to_cgs",
              "annihilation_flux_to_cgs"):
        assert getattr(cu, k) == par[k][0], k
    assert p.map.Nside == int(par["nside"][0]) and p.map.Npix == int(par["npix"][0])
    assert p.map.dOmega == par["dOmega"][0]
    assert p.memParts == int(par["memParts"][0])
    assert p.testNum == int(par["testNum"][0])
    assert p.isMask == bool(par["isMask"][0])
    assert p.params.particle_masses == list(par["particle_masses"])


def test_unit_factor_and_hires_match_oracle():
    import oracle as O
    case = G.load("nfw_sub_ns64")
    p = Parameters(text=case["info_text"].replace("@DIR@", "/x"))
    o = G.oracle_params(case)
    assert p.unit_factor == o.unit_factor
    assert p.hires_threshold == o.hires_threshold
    case = G.load("hires_mask_ns32")
    p = Parameters(text=case["info_text"].replace("@DIR@", "/x"))
    o = G.oracle_params(case)
    assert p.hires_threshold == o.hires_threshold


def test_observer_rotation_rejects_centre():
    L = _lib.load()
    d3 = lambda v: (C.c_double * 3)(*v)
    rot = (C.c_double * 9)()
    assert L.dmann_observer_rotation(d3([1, 2, 3]), d3([1, 2, 3]), d3([0, 0, 1]), rot, None) == _lib.ERR_INVALID
    assert L.dmann_observer_rotation(d3([8, 0, 0]), d3([0, 0, 0]), d3([0, 0, 1]), rot, None) == _lib.OK
    R = np.array(rot[:]).reshape(3, 3)
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-14)


def test_info_tokenisation():
    txt = "\n".join([
        "# comment line", "  # indented comment", "", "h100 = 0.73", "Lbox_in_Mpc = 0.001",
        "mass_to_Msun = 1", "particle_masses = 4100 0 8200", "centerpos = 1 2 3",
        "align_vec = 0 0 1", "obs_pos = 9 2 3", "nside = 64", "test = 123", "mem_buffer = 77",
        "unknown_key = 5", "datafile = /a/b.bin", "mask = /m.bin", "outputmap = out.fits",
        "h100\t= 0.5",  # a tab is not a separator: a different (unknown) key
    ])
    p = Parameters(text=txt)
    assert p.info["h100"] == 0.73
    assert p.map.Nside == 64 and p.testNum == 123 and p.memParts == 77
    assert p.nativeDatafile == "/a/b.bin" and p.isMask and p.maskFileName == "/m.bin"
    assert p.info["particle_masses"][:3] == [4100.0, 0.0, 8200.0]
    assert p.params.particle_masses[:2] == [4100.0, 8200.0]  # compacted (parameters.cpp:125-135)
    assert p.outputFileName == "out.fits"
    with pytest.raises(ValueError):
        Parameters(text="h100 =\n")
    with pytest.raises(ValueError):
        Parameters(text="h100 = 0.7\nLbox_in_Mpc = 1\nobs_pos = 0 0 0\ncenterpos = 0 0 0\nalign_vec = 0 0 1\n")


def test_atof_atoi_prefix_semantics():
    assert atof("1.5e3xyz") == 1500.0 and atof("abc") == 0.0 and atof("-.5\r") == -0.5
    assert atoi("42.7") == 42 and atoi("x") == 0 and atoi("-3") == -3


def test_native_reader_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    n = 1000
    parts = {k: rng.normal(size=n).astype(np.float32) for k in ("x", "y", "z", "m", "rho", "h")}
    path = str(tmp_path / "p.bin")
    write_native(path, parts)
    mask = (rng.uniform(size=n) > 0.3).astype(np.uint8)
    mpath = str(tmp_path / "m.bin")
    with open(mpath, "wb") as f:
        np.array([n], np.int32).tofile(f)
        mask.tofile(f)
    r = DataReader(path, True, mpath)
    r.setBuf(300)
    r.setTest(900)
    r.open()
    assert r.getPartNum() == 900
    got = {k: [] for k in parts}
    chunks = 0
    while r.hasNext():
        c = r.next_chunk()
        chunks += 1
        for k in parts:
            got[k].append(c[k])
    r.close()
    assert chunks == 3
    for k in parts:
        g = np.concatenate(got[k])
        exp = parts[k][:900].copy()
        if k == "rho":
            exp[mask[:900] == 0] = -1.0
        assert np.array_equal(g, exp), k


def test_reader_matches_golden_records():
    case = G.load("hires_mask_ns32")
    z = np.load(os.path.join(G.GOLDEN, "hires_mask_ns32.npz"))
    rec = z["records"]
    assert rec.shape[1] == 12 and rec.dtype == np.float32


def test_flux_unit_factors_match_oracle():
    import oracle as O
    case = G.load("flux_decay_ns32")
    p = O.make_params(nside=8, obs_pos=(1, 2, 3), centerpos=(0, 0, 0), align_vec=(0, 0, 1),
                      particle_masses=(4.1e3,))
    par = annmap.Parameters(text=case["info_text"].replace("@DIR@", "/x"))
    assert par.flux_unit_factor(4) == p.decay_unit_factor == par.flux_unit_factor("decay")
    assert par.flux_unit_factor("ann_nosom") == par.unit_factor
    for law in (0, 1, 2, 3, 5):
        assert par.flux_unit_factor(law) == p.unit_factor == par.unit_factor
    with pytest.raises(ValueError):
        par.flux_unit_factor(9)


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of dmann_stats and dmann_tuning have the header's
    field names, offsets and sizes (a C program compiled against dmann.h
    prints them)."""
    import subprocess
    mirrors = {"dmann_stats": _lib.Stats, "dmann_tuning": _lib.Tuning}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "dmann.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o", exe], check=True)
    got = {}
    for ln in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, field, val = ln.split()
        got[(cname, field)] = int(val)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
