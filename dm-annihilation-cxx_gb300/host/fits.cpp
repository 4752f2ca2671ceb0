// fits.cpp -- a minimal HEALPix FITS map writer, written from the FITS
// standard (2880-byte records, 80-character header cards, big-endian binary
// table data) with the layout of HEALPix C++ write_Healpix_map_to_fits as the
// reference calls it (src/mapgenerator.cpp:30-62, PLANCK_FLOAT64): an empty
// primary HDU, then one BINTABLE with a single FP64 column "signal" holding
// the map, `repcount` values per row, and the keywords PIXTYPE, ORDERING,
// NSIDE, FIRSTPIX, LASTPIX, INDXSCHM.  cfitsio is not used.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "annmap.hpp"

namespace annmap {

namespace {

constexpr size_t kBlock = 2880;

std::string card(const std::string &key, const std::string &value, const std::string &comment) {
    std::string s = key;
    s.resize(8, ' ');
    if (!value.empty()) {
        s += "= ";
        s += value;
        if (!comment.empty()) s += " / " + comment;
    }
    s.resize(80, ' ');
    return s;
}
std::string num(long long v) {
    std::string t = std::to_string(v);
    return std::string(t.size() < 20 ? 20 - t.size() : 0, ' ') + t;
}
std::string logical(bool v) { return std::string(19, ' ') + (v ? "T" : "F"); }
std::string str(const std::string &v) {
    std::string q = "'" + v;
    while (q.size() < 9) q += ' ';
    q += "'";
    while (q.size() < 20) q += ' ';
    return q;
}
void pad(std::string &h) {
    h += card("END", "", "");
    h.resize((h.size() + kBlock - 1) / kBlock * kBlock, ' ');
}

// values per table row (HEALPix's healpix_repcount)
int64_t repcount(int64_t npix) {
    if (npix < 1024) return 1;
    if (npix % 1024 == 0) return 1024;
    return (int64_t)std::llround(std::sqrt((double)(npix / 12)));
}

}  // namespace

void writeHealpixFits(const std::string &path, const double *map, int64_t npix,
                      const char *ordering) {
    const int64_t nside = (int64_t)std::llround(std::sqrt((double)npix / 12.0));
    if (nside < 1 || 12 * nside * nside != npix) throw std::runtime_error("map length is not 12 nside^2");
    const int64_t rep = repcount(npix);
    std::string h0 = card("SIMPLE", logical(true), "file does conform to FITS standard") +
                     card("BITPIX", num(8), "number of bits per data pixel") +
                     card("NAXIS", num(0), "number of data axes") +
                     card("EXTEND", logical(true), "FITS dataset may contain extensions");
    pad(h0);
    std::string h1 = card("XTENSION", str("BINTABLE"), "binary table extension") +
                     card("BITPIX", num(8), "8-bit bytes") +
                     card("NAXIS", num(2), "2-dimensional binary table") +
                     card("NAXIS1", num(8 * rep), "width of table in bytes") +
                     card("NAXIS2", num(npix / rep), "number of rows in table") +
                     card("PCOUNT", num(0), "size of special data area") +
                     card("GCOUNT", num(1), "one data group (required keyword)") +
                     card("TFIELDS", num(1), "number of fields in each row") +
                     card("TTYPE1", str("signal"), "label for field   1") +
                     card("TFORM1", str(std::to_string(rep) + "D"), "data format of field: 8-byte DOUBLE") +
                     card("TUNIT1", str("unknown"), "physical unit of field") +
                     card("EXTNAME", str("xtension"), "name of this binary table extension") +
                     card("PIXTYPE", str("HEALPIX"), "HEALPIX pixelisation") +
                     card("ORDERING", str(ordering), "Pixel ordering scheme, either RING or NESTED") +
                     card("NSIDE", num(nside), "Resolution parameter for HEALPIX") +
                     card("FIRSTPIX", num(0), "First pixel # (0 based)") +
                     card("LASTPIX", num(npix - 1), "Last pixel # (0 based)") +
                     card("INDXSCHM", str("IMPLICIT"), "Indexing: IMPLICIT or EXPLICIT");
    pad(h1);
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot create " + path);
    bool ok = std::fwrite(h0.data(), 1, h0.size(), f) == h0.size() &&
              std::fwrite(h1.data(), 1, h1.size(), f) == h1.size();
    // big-endian doubles, written in slices
    std::vector<unsigned char> buf;
    const int64_t slice = 1 << 16;
    for (int64_t i0 = 0; ok && i0 < npix; i0 += slice) {
        const int64_t k = std::min(slice, npix - i0);
        buf.resize((size_t)k * 8);
        for (int64_t i = 0; i < k; i++) {
            uint64_t u;
            std::memcpy(&u, map + i0 + i, 8);
            for (int b = 0; b < 8; b++) buf[(size_t)i * 8 + b] = (unsigned char)(u >> (56 - 8 * b));
        }
        ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    }
    const size_t data = (size_t)npix * 8, tail = (kBlock - data % kBlock) % kBlock;
    if (ok && tail) {
        std::vector<unsigned char> z(tail, 0);
        ok = std::fwrite(z.data(), 1, tail, f) == tail;
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) throw std::runtime_error("write error on " + path);
}

}  // namespace annmap
