// hooks.cpp -- C entry points into the C++ host API (libannmap.so), so that
// scripts can drive the reference-shaped flow -- Parameters from an info
// file, DataReader, MapGenerator::start, saveToFits -- without a C++
// compiler.  Each returns 0 (or a count) on success, else a negative code
// with the message copied into err.
#include <cstdio>
#include <cstring>
#include <exception>

#include "annmap.hpp"

namespace {

int fail(char *err, int errlen, const char *msg) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", msg);
    return -1;
}

// Reads every chunk of an unopened reader into float32 SoA planes
// (x, y, z, m, rho, h, sigmav; plane stride cap).  Returns the count or -1.
int64_t drain(annmap::DataReader &r, int test, int buf, float *soa, int64_t cap, char *err,
              int errlen) {
    r.setTest(test);
    r.setBuf((unsigned)buf);
    r.open();
    int64_t k = 0;
    while (r.hasNext()) {
        const annmap::DMParticle *p = r.getBuf();
        for (int i = 0; i < r.getMemparts(); i++, k++) {
            if (k >= cap) return fail(err, errlen, "output capacity exceeded");
            soa[k] = p[i].posx;
            soa[cap + k] = p[i].posy;
            soa[2 * cap + k] = p[i].posz;
            soa[3 * cap + k] = p[i].mass;
            soa[4 * cap + k] = p[i].dens;
            soa[5 * cap + k] = p[i].hsmooth;
            soa[6 * cap + k] = p[i].sigmav;
        }
        r.loadBuffer();
    }
    r.close();
    return k;
}

}  // namespace

extern "C" {

// Derived values of an info file: out[0] nside, [1..9] rotmatrix (row-major),
// [10..12] opos, [13..15] cpos, [16] unit_factor, [17] hires threshold,
// [18] memParts, [19] testNum, [20] otheta, [21] ophi, [22] isMask,
// [23] isNative.
int annmap_parse_info(const char *info_file, double out[24], char *err, int errlen) {
    try {
        annmap::Parameters p(info_file);
        out[0] = p.map.Nside;
        for (int i = 0; i < 9; i++) out[1 + i] = p.rotmatrix[i / 3][i % 3];
        for (int i = 0; i < 3; i++) {
            out[10 + i] = p.params.opos[i];
            out[13 + i] = p.params.cpos[i];
        }
        out[16] = p.unit_factor;
        out[17] = p.hiresThreshold();
        out[18] = p.memParts;
        out[19] = p.testNum;
        out[20] = p.params.otheta;
        out[21] = p.params.ophi;
        out[22] = p.isMask ? 1 : 0;
        out[23] = p.isNative ? 1 : 0;
        return 0;
    } catch (const std::exception &e) {
        return fail(err, errlen, e.what());
    }
}

// A native particle file (with optional mask) through DataReader, chunk by
// chunk, into float32 SoA (7 * cap floats).  Returns the particle count.
int64_t annmap_read_native(const char *path, const char *maskfile, int test, int buf,
                           float *soa, int64_t cap, char *err, int errlen) {
    try {
        annmap::DataReader r(path, maskfile && *maskfile, maskfile ? maskfile : "");
        return drain(r, test, buf, soa, cap, err, errlen);
    } catch (const std::exception &e) {
        return fail(err, errlen, e.what());
    }
}

// The same for a Tipsy XDR file and its side files (single != 0: no side files).
int64_t annmap_read_tipsy(const char *part, const char *dens, const char *hsm, const char *sigv,
                          const char *maskfile, int single, int test, int buf, float *soa,
                          int64_t cap, char *err, int errlen) {
    try {
        annmap::DataReader r(part, dens, hsm, sigv, maskfile && *maskfile,
                             maskfile ? maskfile : "", single != 0);
        return drain(r, test, buf, soa, cap, err, errlen);
    } catch (const std::exception &e) {
        return fail(err, errlen, e.what());
    }
}

// The reference's main flow (src/main.cpp:35-66) on the GPU: Parameters,
// DataReader (native or Tipsy input, test limit and buffer from the info
// file), MapGenerator::start, and saveToFits to the info file's outputmap
// when it names one, with the flux law flux_model (dmann_flux; halo_file for
// the core law, NULL or "" for the reference's default path).  map_out
// receives the 12 nside^2 map (npix must match); total_flux the "Total Conts".
int annmap_genmap(const char *info_file, int precision, int device, int flux_model,
                  const char *halo_file, double *map_out, int64_t npix, double *total_flux,
                  char *err, int errlen) {
    try {
        annmap::Parameters par(info_file);
        if (npix != par.map.Npix) return fail(err, errlen, "map length does not match nside");
        annmap::DataReader reader =
            par.isNative ? annmap::DataReader(par.nativeDatafile, par.isMask, par.maskFileName)
                         : annmap::DataReader(par.partFile, par.densFile, par.hsmFile, par.dspFile,
                                              par.isMask, par.maskFileName);
        reader.setTest(par.testNum);
        reader.setBuf((unsigned)par.memParts);
        reader.open();
        annmap::MapGenerator gen(&par, &reader, precision, device, flux_model);
        if (halo_file && *halo_file) gen.setHaloFile(halo_file);
        gen.start();
        reader.close();
        std::memcpy(map_out, gen.getMap(), sizeof(double) * (size_t)npix);
        if (total_flux) *total_flux = gen.totalFlux();
        if (!par.outputFileName.empty()) gen.saveToFits(par.outputFileName, false);
        return 0;
    } catch (const std::exception &e) {
        return fail(err, errlen, e.what());
    }
}

int annmap_write_fits(const char *path, const double *map, int64_t npix, char *err, int errlen) {
    try {
        annmap::writeHealpixFits(path, map, npix, "RING");
        return 0;
    } catch (const std::exception &e) {
        return fail(err, errlen, e.what());
    }
}

}  // extern "C"
