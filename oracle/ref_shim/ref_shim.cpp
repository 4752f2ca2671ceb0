/*
 * ref_shim.cpp -- the pieces the reference's CPU map path needs that live in
 * files this build does not compile, plus a driver that mirrors
 * src/main.cpp:16-73 without the FITS writer.
 *
 * TEST INFRASTRUCTURE ONLY.  Built from the reference sources where they lie
 * (see oracle/ref_shim/Makefile) into oracle/_ref/annmap_ref, which the
 * golden-fixture script runs to pin the oracle.  Nothing here is product code.
 *
 *   - MapGenerator's constructor/destructor/accessors: the reference defines
 *     them in src/mapgenerator.cpp:18-74 next to saveToFits(), which needs
 *     HEALPix FITS I/O; they are restated here with the same behaviour.
 *   - XDR / Tipsy entry points (src/tipsy_io.c, <rpc/xdr.h>): the decode
 *     side the reference's DataReader calls, reading big-endian values.
 *
 * Usage: annmap_ref <info.ini> <map.bin> <params.txt>
 *   writes Npix doubles (the map after the dOmega division) to map.bin and
 *   the derived Parameters fields to params.txt, one "key v..." per line.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <rpc/types.h>
#include <rpc/xdr.h>
#include "parameters.h"
#include "datareader.h"
#include "mapgenerator.h"

extern "C" {
void xdrstdio_create(XDR *x, FILE *f, enum xdr_op op) {
    x->x_op = op;
    x->fp = f;
}
void xdr_destroy(XDR *x) { x->fp = NULL; }
}

// XDR decoding of the Tipsy header and dark records (the layout of
// src/tipsy_io.c:159-192's xdr_header / xdr_dark): big-endian 4-byte ints and
// floats, 8-byte double.
static bool xdr_u32(XDR *x, unsigned int *v) {
    unsigned char b[4];
    if (fread(b, 1, 4, x->fp) != 4) return false;
    *v = ((unsigned int)b[0] << 24) | ((unsigned int)b[1] << 16) | ((unsigned int)b[2] << 8) | b[3];
    return true;
}
static bool xdr_f32(XDR *x, float *v) {
    unsigned int u;
    if (!xdr_u32(x, &u)) return false;
    memcpy(v, &u, 4);
    return true;
}
int xdr_header(XDR *x, tipsy_header *h) {
    unsigned int hi, lo, v[6];
    if (!xdr_u32(x, &hi) || !xdr_u32(x, &lo)) return 0;
    unsigned long long u = ((unsigned long long)hi << 32) | lo;
    memcpy(&h->time, &u, 8);
    for (int k = 0; k < 6; k++)
        if (!xdr_u32(x, &v[k])) return 0;
    h->nbodies = (int)v[0];
    h->ndim = (int)v[1];
    h->nsph = (int)v[2];
    h->ndark = (int)v[3];
    h->nstar = (int)v[4];
    return 1;
}
int xdr_dark(XDR *x, struct dark_particle *p) {
    float *f[9] = {&p->mass, &p->pos[0], &p->pos[1], &p->pos[2], &p->vel[0], &p->vel[1], &p->vel[2],
                   &p->eps, &p->phi};
    for (int k = 0; k < 9; k++)
        if (!xdr_f32(x, f[k])) return 0;
    return 1;
}

MapGenerator::MapGenerator(Parameters *par, DataReader *reader) {
    par_ = par;
    reader_ = reader;
    map_ = NULL;
    isFinished_ = false;
}
MapGenerator::~MapGenerator() {
    if (map_ != NULL) free(map_);
}
bool MapGenerator::isFinished() { return isFinished_; }
MAPTYPE *MapGenerator::getMap() { return map_; }
int MapGenerator::getNside() { return par_->map.Nside; }

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s info.ini map.bin params.txt\n", argv[0]);
        return 2;
    }
    Parameters par(argv[1]);
    DataReader *reader;
    if (par.isNative)
        reader = new DataReader(par.nativeDatafile, par.isMask, par.maskFileName);
    else   // src/main.cpp:46-53
        reader = new DataReader(par.partFile, par.densFile, par.hsmFile, par.dspFile, par.isMask,
                                par.maskFileName);
    reader->setTest(par.testNum);
    reader->setBuf(par.memParts);
    reader->open();
    MapGenerator generator(&par, reader);
    generator.start();
    reader->close();
    FILE *f = fopen(argv[2], "wb");
    if (!f) return 3;
    fwrite(generator.getMap(), sizeof(MAPTYPE), (size_t)par.map.Npix, f);
    fclose(f);
    FILE *g = fopen(argv[3], "w");
    if (!g) return 4;
    fprintf(g, "nside %d\nnpix %d\ndOmega %.17g\n", par.map.Nside, par.map.Npix, par.map.dOmega);
    fprintf(g, "opos %.17g %.17g %.17g\n", par.params.opos[0], par.params.opos[1], par.params.opos[2]);
    fprintf(g, "cpos %.17g %.17g %.17g\n", par.params.cpos[0], par.params.cpos[1], par.params.cpos[2]);
    fprintf(g, "otheta %.17g\nophi %.17g\n", par.params.otheta, par.params.ophi);
    for (int i = 0; i < 3; i++)
        fprintf(g, "rotmatrix%d %.17g %.17g %.17g\n", i, par.rotmatrix[i][0], par.rotmatrix[i][1], par.rotmatrix[i][2]);
    fprintf(g, "mass_to_cgs %.17g\nlength_to_cgs %.17g\ndensity_to_cgs %.17g\n",
            par.codeunits.mass_to_cgs, par.codeunits.length_to_cgs, par.codeunits.density_to_cgs);
    fprintf(g, "time_to_cgs %.17g\nvelocity_to_cgs %.17g\nannihilation_flux_to_cgs %.17g\n",
            par.codeunits.time_to_cgs, par.codeunits.velocity_to_cgs, par.codeunits.annihilation_flux_to_cgs);
    fprintf(g, "particle_masses");
    for (int i = 0; i < 10; i++) fprintf(g, " %.17g", par.params.particle_masses[i]);
    fprintf(g, "\nmemParts %d\ntestNum %d\nisMask %d\n", par.memParts, par.testNum, (int)par.isMask);
    fclose(g);
    delete reader;
    return 0;
}
