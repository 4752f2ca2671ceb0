"""The C++ host API (libannmap.so) without a GPU: info-file parsing against
the Python mirror, the native reader (mask, test limit, chunking) against
the Python reader, the FITS writer byte for byte against the Python writer,
and a C++ program compiled against annmap.hpp."""
import json
import os
import subprocess

import numpy as np
import pytest

import annmap
import golden_cases as G
from annmap import host
from annmap.fitsio import read_healpix_map, write_healpix_map
from annmap.reader import DataReader, write_native
from host_cases import write_case

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "dm-annihilation-cxx_gb300")


@pytest.mark.parametrize("name", G.names())
def test_cpp_parameters_match_python(tmp_path, name):
    case, info = write_case(tmp_path, name)
    got = host.parse_info(info)
    par = annmap.Parameters(info)
    assert got["nside"] == par.map.Nside
    assert np.array_equal(got["rotmatrix"], np.array(par.rotmatrix))
    assert list(got["opos"]) == list(par.params.opos) and list(got["cpos"]) == list(par.params.cpos)
    assert got["unit_factor"] == par.unit_factor
    assert got["hires_threshold"] == par.hires_threshold
    assert got["memParts"] == par.memParts and got["testNum"] == par.testNum
    assert got["isMask"] == par.isMask
    assert (got["otheta"], got["ophi"]) == (par.params.otheta, par.params.ophi)


def test_cpp_parse_errors(tmp_path):
    p = tmp_path / "bad.ini"
    p.write_text("h100 = 0.73\nLbox_in_Mpc = 1\nobs_pos = 1 2\n")
    with pytest.raises(ValueError, match="lacks a value"):
        host.parse_info(str(p))
    p.write_text("h100 = 0.73\nLbox_in_Mpc = 1\nobs_pos = 0 0 0\ncenterpos = 0 0 0\nalign_vec = 0 0 1\n")
    with pytest.raises(ValueError, match="centre"):
        host.parse_info(str(p))
    with pytest.raises(ValueError, match="Info file"):
        host.parse_info(str(tmp_path / "missing.ini"))


@pytest.mark.parametrize("test,buf", [(-1, 10000000), (900, 300), (1000, 7), (0, 5)])
def test_cpp_reader_matches_python(tmp_path, test, buf):
    rng = np.random.default_rng(1)
    n = 1000
    parts = {k: rng.normal(size=n).astype(np.float32) for k in ("x", "y", "z", "m", "rho", "h")}
    path = str(tmp_path / "p.bin")
    write_native(path, parts)
    mask = (rng.uniform(size=n) > 0.3).astype(np.uint8)
    mpath = str(tmp_path / "m.bin")
    with open(mpath, "wb") as f:
        np.array([n], np.int32).tofile(f)
        mask.tofile(f)
    got = host.read_native(path, mpath, test=test, buf=buf)
    r = DataReader(path, True, mpath)
    r.setBuf(buf)
    r.setTest(test)
    r.open()
    exp = {k: [] for k in parts}
    while r.hasNext():
        c = r.next_chunk()
        for k in parts:
            exp[k].append(c[k])
    for k in parts:
        e = np.concatenate(exp[k]) if exp[k] else np.zeros(0, np.float32)
        assert np.array_equal(got[k], e), k


def test_cpp_reader_rejects_bad_mask(tmp_path):
    path = str(tmp_path / "p.bin")
    write_native(path, {k: np.zeros(10, np.float32) for k in ("x", "y", "z", "m", "rho", "h")})
    mpath = str(tmp_path / "m.bin")
    with open(mpath, "wb") as f:
        np.array([9], np.int32).tofile(f)
        np.ones(9, np.uint8).tofile(f)
    with pytest.raises(ValueError, match="mask"):
        host.read_native(path, mpath)
    with pytest.raises(ValueError, match="Datafile"):
        host.read_native(str(tmp_path / "none.bin"), "", cap=10)


@pytest.mark.parametrize("nside", [1, 16, 24])
def test_cpp_fits_equals_python_fits(tmp_path, nside):
    m = np.random.default_rng(nside).standard_normal(12 * nside * nside)
    a, b = str(tmp_path / "a.fits"), str(tmp_path / "b.fits")
    host.write_fits(a, m)
    write_healpix_map(b, m)
    assert open(a, "rb").read() == open(b, "rb").read()
    got, h = read_healpix_map(a)
    assert np.array_equal(got, m) and h["NSIDE"] == nside


def _compile_example(tmp_path):
    exe = str(tmp_path / "host_example")
    subprocess.run(["g++", "-O1", "-std=c++17", os.path.join(REPO, "tests", "cpp", "host_example.cpp"),
                    "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(PKG, "host"),
                    "-L" + PKG, "-lannmap", "-ldmann", "-Wl,-rpath," + PKG, "-o", exe], check=True)
    return exe


def test_cpp_example_program_reads_like_the_reference(tmp_path):
    host.load()
    case, info = write_case(tmp_path, "hires_mask_ns32", mem_buffer=333)
    exe = _compile_example(tmp_path)
    out = subprocess.run([exe, info], capture_output=True, text=True, check=True).stdout
    d = json.loads(out)
    parts = case["parts"]
    assert d["nside"] == 32 and d["particles"] == len(parts["x"])
    assert d["masked"] == int((parts["rho"] < 0).sum())
    assert d["chunks"] == -(-len(parts["x"]) // 333)
    assert d["mass_sum"] == pytest.approx(float(np.sum(parts["m"].astype(np.float64))), rel=1e-12)


def test_halo_table_roundtrip(tmp_path):
    from annmap.halocore import read_halo_table, write_halo_table
    rng = np.random.default_rng(4)
    h = [rng.normal(size=50).astype(np.float32) for _ in range(4)]
    p = str(tmp_path / "h.data")
    write_halo_table(p, *h)
    got = read_halo_table(p)
    for a, b in zip(got, h):
        assert np.array_equal(a, b)
    (tmp_path / "e.data").write_text("")
    with pytest.raises(ValueError):
        read_halo_table(str(tmp_path / "e.data"))


@pytest.mark.parametrize("buf,test", [(10000000, -1), (300, -1), (128, 1000)])
def test_tipsy_readers_match_the_reference_records(tmp_path, buf, test):
    """The Tipsy XDR input of the golden case (made through the reference's own
    XDR reader) through the C++ and the Python DataReader."""
    case, info = write_case(tmp_path, "tipsy_somv_ns32")
    d = str(tmp_path)
    files = [os.path.join(d, k + ".bin") for k in ("tipsy", "dens", "hsm", "sigv")]
    got = host.read_tipsy(*files, maskfile=os.path.join(d, "mask.bin"), test=test, buf=buf)
    r = DataReader.tipsy(*files, isMask=True, maskfile=os.path.join(d, "mask.bin"))
    r.setBuf(buf)
    r.setTest(test)
    r.open()
    py = {k: [] for k in got}
    while r.hasNext():
        c = r.next_chunk()
        for k in py:
            py[k].append(c[k])
    n = len(case["parts"]["x"]) if test == -1 else test
    for k in got:
        exp = case["parts"][k][:n]
        assert np.array_equal(got[k], exp), k
        assert np.array_equal(np.concatenate(py[k]), exp), k
    single = host.read_tipsy(*files, single=True, buf=buf)
    assert np.all(single["rho"] == 0) and np.array_equal(single["x"], case["parts"]["x"])
    assert host.parse_info(info)["isNative"] is False
