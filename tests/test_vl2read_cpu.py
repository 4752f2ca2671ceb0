"""The vl2read drop-in (src/pywrapper/vl2read.h:6-28, vl2read.cpp): both
constructors, the box selection and the getters, against the golden cases'
particle records (the reference reader's output) selected with the rule of
vl2read.cpp's loop: |float position - centre| < boxsize / 2 per axis, in
double, masked particles kept with density -1."""
import os
import shutil

import numpy as np
import pytest

import vl2read
from host_cases import write_case


def expected(case_records, mask, c, box):
    rec = case_records
    keep = np.ones(len(rec), bool)
    for k, ax in enumerate((3, 4, 5)):
        keep &= np.abs(rec[:, ax].astype(np.float64) - c[k]) < box / 2
    dens = rec[:, 1].copy()
    if mask is not None and mask.size:
        dens[mask == 0] = -1.0
    return keep, dens[keep], rec[keep, 6], rec[keep, 7], rec[keep, 8]


def check(r, exp):
    keep, d, vx, vy, vz = exp
    assert len(r.getDensity()) == int(keep.sum())
    for got, want in ((r.getDensity(), d), (r.getVelocityX(), vx), (r.getVelocityY(), vy),
                      (r.getVelocityZ(), vz)):
        assert got.dtype == np.float32
        assert np.array_equal(got, want)


def _records(name):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    return z["records"], z["mask"]


@pytest.mark.parametrize("name", ["hires_mask_ns32", "nfw_sub_ns64"])
def test_native_box_selection(tmp_path, name):
    rec, mask = _records(name)
    write_case(tmp_path, name)
    data = os.path.join(str(tmp_path), "parts.bin")
    mfile = os.path.join(str(tmp_path), "mask.bin") if mask.size else ""
    pos = rec[:, 3:6].astype(np.float64)
    c = np.median(pos, axis=0)
    box = float(np.percentile(np.abs(pos - c).max(axis=1), 40)) * 2
    r = vl2read.VL2Reader(data, c[0], c[1], c[2], box, mfile)
    exp = expected(rec, mask if mfile else None, c, box)
    assert 0 < exp[0].sum() < len(rec)
    check(r, exp)
    # keyword form and the whole box
    r2 = vl2read.VL2Reader(filename=data, xc=c[0], yc=c[1], zc=c[2], boxsize=1e9)
    assert len(r2.getDensity()) == len(rec)
    assert np.array_equal(r2.getVelocityZ(), rec[:, 8])
    # the getters hand out the same array (the reference returns a reference)
    r.getDensity()[:1] = 123.0
    assert r.getDensity()[0] == 123.0


def test_tipsy_box_selection(tmp_path):
    rec, mask = _records("tipsy_somv_ns32")
    write_case(tmp_path, "tipsy_somv_ns32")
    d = str(tmp_path)
    base = os.path.join(d, "snap")
    os.makedirs(base)
    shutil.copy(os.path.join(d, "tipsy.bin"), os.path.join(base, "run"))
    for k, ext in (("dens", "den32"), ("hsm", "hsm32"), ("sigv", "sigma32")):
        shutil.copy(os.path.join(d, k + ".bin"), os.path.join(base, "run." + ext))
    pos = rec[:, 3:6].astype(np.float64)
    c = pos[7]
    box = float(np.percentile(np.abs(pos - c).max(axis=1), 30)) * 2
    r = vl2read.VL2Reader(base, "run", c[0], c[1], c[2], box, os.path.join(d, "mask.bin"))
    exp = expected(rec, mask, c, box)
    assert 0 < exp[0].sum() < len(rec)
    check(r, exp)
    # isSingleFile: only the Tipsy file, densities zero (vl2read.h:12)
    s = vl2read.VL2Reader(base, "run", c[0], c[1], c[2], box, "", True)
    keep = exp[0]
    assert len(s.getDensity()) == int(keep.sum()) and np.all(s.getDensity() == 0)
    assert np.array_equal(s.getVelocityX(), rec[keep, 6])


def test_interface_and_arrays():
    assert vl2read.VL2Reader.INITMEMSIZE == 128 * 1024
    with pytest.raises(TypeError):
        vl2read.VL2Reader("x.bin", 0.0, 0.0)
    a = vl2read.fArray(4)
    for i in range(4):
        a[i] = i * 0.5
    assert [a[i] for i in range(4)] == [0.0, 0.5, 1.0, 1.5]
    b = vl2read.fArray.frompointer(a.cast())
    b[2] = 7.0
    assert a[2] == 7.0
    d = vl2read.dArray(2)
    d[1] = 1e300
    assert vl2read.dArray.frompointer(d.cast())[1] == 1e300
