"""HEALPix FITS map files: a minimal writer and reader of the FITS standard
(version 4.0: 2880-byte records, 80-character header cards, big-endian
binary tables), laid out the way the reference's saveToFits leaves its maps
(src/mapgenerator.cpp:30-62, which calls HEALPix C++ write_Healpix_map_to_fits
with PLANCK_FLOAT64): an empty primary HDU, then one BINTABLE extension with
one FP64 column "signal" holding the RING map, ``repcount`` values per row,
and the HEALPix keywords PIXTYPE, ORDERING, NSIDE, FIRSTPIX, LASTPIX and
INDXSCHM.  cfitsio is not available, so this is written from the standard.
"""
from __future__ import annotations

import os

import numpy as np

BLOCK = 2880


def healpix_repcount(npix: int) -> int:
    """Values per table row: 1 for small maps, 1024 when it divides the
    pixel count, else sqrt(npix / 12) = nside."""
    if npix < 1024:
        return 1
    if npix % 1024 == 0:
        return 1024
    return int(round((npix // 12) ** 0.5))


def _card(key: str, value=None, comment: str = "") -> bytes:
    if value is None:
        s = key.ljust(80)
    else:
        if isinstance(value, bool):
            v = ("T" if value else "F").rjust(20)
        elif isinstance(value, (int, np.integer)):
            v = str(int(value)).rjust(20)
        elif isinstance(value, float):
            v = repr(value).upper().rjust(20)
        else:
            q = "'" + str(value).replace("'", "''").ljust(8) + "'"
            v = q.ljust(20)
        s = key.ljust(8)[:8] + "= " + v
        if comment:
            s += " / " + comment
        s = s[:80].ljust(80)
    return s.encode("ascii")


def _header(cards) -> bytes:
    h = b"".join(cards) + _card("END")
    return h + b" " * (-len(h) % BLOCK)


def write_healpix_map(path: str, m, *, ordering: str = "RING", column: str = "signal",
                      overwrite: bool = True) -> None:
    """Writes a full-sky HEALPix map (12 nside^2 values) as FP64."""
    m = np.asarray(m, dtype=np.float64).ravel()
    npix = m.size
    nside = int(round((npix / 12) ** 0.5))
    if 12 * nside * nside != npix or nside < 1:
        raise ValueError("map length is not 12 nside^2")
    if os.path.exists(path):
        if not overwrite:
            raise FileExistsError(path)
        os.remove(path)
    rep = healpix_repcount(npix)
    rows = npix // rep
    primary = _header([_card("SIMPLE", True, "file does conform to FITS standard"),
                       _card("BITPIX", 8, "number of bits per data pixel"),
                       _card("NAXIS", 0, "number of data axes"),
                       _card("EXTEND", True, "FITS dataset may contain extensions")])
    ext = _header([_card("XTENSION", "BINTABLE", "binary table extension"),
                   _card("BITPIX", 8, "8-bit bytes"),
                   _card("NAXIS", 2, "2-dimensional binary table"),
                   _card("NAXIS1", 8 * rep, "width of table in bytes"),
                   _card("NAXIS2", rows, "number of rows in table"),
                   _card("PCOUNT", 0, "size of special data area"),
                   _card("GCOUNT", 1, "one data group (required keyword)"),
                   _card("TFIELDS", 1, "number of fields in each row"),
                   _card("TTYPE1", column, "label for field   1"),
                   _card("TFORM1", f"{rep}D", "data format of field: 8-byte DOUBLE"),
                   _card("TUNIT1", "unknown", "physical unit of field"),
                   _card("EXTNAME", "xtension", "name of this binary table extension"),
                   _card("PIXTYPE", "HEALPIX", "HEALPIX pixelisation"),
                   _card("ORDERING", ordering, "Pixel ordering scheme, either RING or NESTED"),
                   _card("NSIDE", nside, "Resolution parameter for HEALPIX"),
                   _card("FIRSTPIX", 0, "First pixel # (0 based)"),
                   _card("LASTPIX", npix - 1, "Last pixel # (0 based)"),
                   _card("INDXSCHM", "IMPLICIT", "Indexing: IMPLICIT or EXPLICIT")])
    data = m.astype(">f8").tobytes()
    with open(path, "wb") as f:
        f.write(primary)
        f.write(ext)
        f.write(data)
        f.write(b"\0" * (-len(data) % BLOCK))


def _read_header(f):
    cards = {}
    while True:
        blk = f.read(BLOCK)
        if len(blk) < BLOCK:
            raise ValueError("truncated FITS header")
        for i in range(0, BLOCK, 80):
            c = blk[i:i + 80].decode("ascii")
            key = c[:8].strip()
            if key == "END":
                return cards
            if c[8:10] == "= ":
                v = c[10:].split(" /")[0].strip() if not c[10:].lstrip().startswith("'") else c[10:]
                if v.lstrip().startswith("'"):
                    s = v.lstrip()[1:]
                    v = s[:s.index("'")].rstrip() if "'" in s else s
                elif v in ("T", "F"):
                    v = v == "T"
                else:
                    try:
                        v = int(v)
                    except ValueError:
                        v = float(v)
                cards[key] = v


def read_healpix_map(path: str):
    """Reads a map written by write_healpix_map (or any single-column FP64
    or FP32 HEALPix binary table).  Returns (map, header dict)."""
    with open(path, "rb") as f:
        _read_header(f)
        h = _read_header(f)
        if h.get("XTENSION") != "BINTABLE":
            raise ValueError("no binary table extension")
        form = h["TFORM1"]
        rep = int(form[:-1] or 1)
        t = {"D": ">f8", "E": ">f4"}[form[-1]]
        n = rep * int(h["NAXIS2"])
        m = np.frombuffer(f.read(n * np.dtype(t).itemsize), dtype=t).astype(np.float64)
    return m, h
