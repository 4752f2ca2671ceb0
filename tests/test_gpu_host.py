"""The C++ host API on the GPU: the reference's main flow (Parameters,
DataReader, MapGenerator::start with pinned double-buffered chunk streaming,
saveToFits) against the golden maps of the reference's own CPU build."""
import json
import math
import os
import subprocess

import numpy as np
import pytest

import annmap
from annmap import host
from annmap.fitsio import read_healpix_map
from host_cases import write_case
from test_gpu_parity import check

pytestmark = pytest.mark.gpu

PLAIN, COMP = annmap.PLAIN_F64, annmap.COMP_F32


@pytest.mark.parametrize("precision", [PLAIN, COMP])
@pytest.mark.parametrize("name,buf", [("hires_mask_ns32", 333), ("nfw_sub_ns64", 1000), ("vl2units_ns16", 7)])
def test_cpp_genmap_matches_golden(tmp_path, name, buf, precision):
    fits = str(tmp_path / "out.fits")
    case, info = write_case(tmp_path, name, mem_buffer=buf, output=fits)
    mp, total = host.genmap(info, precision)
    par = annmap.Parameters(info)
    ref = case["map"]
    check(mp, ref, precision, total=ref.sum() * par.map.dOmega, dOmega=par.map.dOmega)
    assert math.isclose(total, ref.sum() * par.map.dOmega, rel_tol=1e-12 if precision == PLAIN else 1e-9)
    got, h = read_healpix_map(fits)
    assert np.array_equal(got, mp) and h["NSIDE"] == par.map.Nside and h["ORDERING"] == "RING"


def test_cpp_genmap_chunking_is_linear(tmp_path):
    os.makedirs(tmp_path / "a")
    os.makedirs(tmp_path / "b")
    _, info_a = write_case(tmp_path / "a", "nfw_sub_ns64", mem_buffer=10000000)
    _, info_b = write_case(tmp_path / "b", "nfw_sub_ns64", mem_buffer=97)
    ma, ta = host.genmap(info_a, COMP)
    mb, tb = host.genmap(info_b, COMP)
    m = ma > 0
    assert np.array_equal(ma > 0, mb > 0)
    # FP64 sums in another order; a deposit's one FP32 rounding may flip
    # where the ring-claim order moved its particle's normalisation by ~1e-13
    assert np.max(np.abs(ma[m] - mb[m]) / ma[m]) < 1e-7
    assert math.isclose(ta, tb, rel_tol=1e-12)


def test_cpp_example_program_renders(tmp_path):
    from test_host_cpu import _compile_example
    fits = str(tmp_path / "ex.fits")
    case, info = write_case(tmp_path, "hires_mask_ns32", mem_buffer=500, output=fits)
    exe = _compile_example(tmp_path)
    out = subprocess.run([exe, info, "render"], capture_output=True, text=True, check=True).stdout
    d = json.loads(out)
    par = annmap.Parameters(info)
    ref = case["map"]
    assert math.isclose(d["total_flux"], ref.sum() * par.map.dOmega, rel_tol=1e-9)
    got, _ = read_healpix_map(fits)
    check(got, ref, COMP)


@pytest.mark.parametrize("name", ["flux_ann_somv_ns32", "flux_ann_somv2_ns32", "flux_ann_pwave_ns32",
                                  "flux_decay_ns32", "flux_ann_adiabatic_ns16", "flux_ann_core_nosom_ns16"])
def test_cpp_genmap_flux_laws(tmp_path, name):
    import golden_cases as G
    from annmap.halocore import write_halo_table
    case, info = write_case(tmp_path, name, mem_buffer=250)
    hfile = ""
    if len(case["halos"]):
        hfile = str(tmp_path / "halos.data")
        write_halo_table(hfile, *[case["halos"][:, k] for k in range(4)])
    mp, total = host.genmap(info, COMP, flux_model=G.FLUX_LAWS[case["flux_law"]], halo_file=hfile)
    par = annmap.Parameters(info)
    check(mp, case["map"], COMP, total=case["map"].sum() * par.map.dOmega, dOmega=par.map.dOmega)


@pytest.mark.parametrize("precision", [PLAIN, COMP])
def test_cpp_and_python_tipsy_input_match_golden(tmp_path, precision):
    """The Tipsy XDR input (through the reference's own XDR reader for the
    golden map) via the C++ and the Python MapGenerator, somv law."""
    case, info = write_case(tmp_path, "tipsy_somv_ns32", mem_buffer=300)
    par = annmap.Parameters(info)
    assert not par.isNative
    mp, total = host.genmap(info, precision, flux_model=annmap._lib.FLUX_ANN_SOMV)
    check(mp, case["map"], precision)
    reader = annmap.DataReader.tipsy(par.partFile, par.densFile, par.hsmFile, par.dspFile,
                                     par.isMask, par.maskFileName)
    reader.setTest(par.testNum)
    reader.setBuf(par.memParts)
    reader.open()
    gen = annmap.MapGenerator(par, reader, precision=precision, flux_model="ann_somv")
    gen.start()
    check(gen.getMap(), case["map"], precision)
