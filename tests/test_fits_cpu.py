"""HEALPix FITS writer (the reference's saveToFits layout) round trip."""
import numpy as np
import pytest

from annmap.fitsio import BLOCK, healpix_repcount, read_healpix_map, write_healpix_map


@pytest.mark.parametrize("nside", [1, 8, 16, 24, 64])
def test_fits_roundtrip(tmp_path, nside):
    npix = 12 * nside * nside
    m = np.random.default_rng(nside).standard_normal(npix) * 1e-3
    p = str(tmp_path / "map.fits")
    write_healpix_map(p, m)
    raw = open(p, "rb").read()
    assert len(raw) % BLOCK == 0
    assert raw[:30] == b"SIMPLE  =                    T"
    got, h = read_healpix_map(p)
    assert np.array_equal(got, m)
    rep = healpix_repcount(npix)
    assert h["TFORM1"] == f"{rep}D" and h["NAXIS2"] * rep == npix
    assert (h["PIXTYPE"], h["ORDERING"], h["NSIDE"], h["FIRSTPIX"], h["LASTPIX"], h["INDXSCHM"]) == \
        ("HEALPIX", "RING", nside, 0, npix - 1, "IMPLICIT")
    assert h["TTYPE1"] == "signal"
    # the data are big-endian doubles right after the two headers
    hdr_len = raw.index(b"END".ljust(80), raw.index(b"XTENSION")) + 80
    hdr_len += -hdr_len % BLOCK
    assert np.array_equal(np.frombuffer(raw[hdr_len:hdr_len + 8 * npix], dtype=">f8"), m)


def test_repcount():
    assert healpix_repcount(768) == 1
    assert healpix_repcount(12 * 16 * 16) == 1024
    assert healpix_repcount(12 * 24 * 24) == 24


def test_fits_rejects_bad_length(tmp_path):
    with pytest.raises(ValueError):
        write_healpix_map(str(tmp_path / "x.fits"), np.zeros(13))


def test_mapgenerator_save_to_fits(tmp_path):
    from annmap.mapgen import MapGenerator

    class _Par:
        outputFileName = str(tmp_path / "out.fits")

        class map:
            Nside = 4

    g = MapGenerator(_Par(), None)
    g.map_ = np.arange(192, dtype=np.float64)
    g.isFinished_ = True
    g.saveToFits("")
    got, h = read_healpix_map(str(tmp_path / "out.fits"))
    assert np.array_equal(got, g.map_) and h["NSIDE"] == 4
