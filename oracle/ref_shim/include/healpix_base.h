/* Stand-in for HEALPix C++ 3.00 <healpix_base.h> (not vendored by the
 * reference, absent on this machine).  It declares only what the reference's
 * CPU map path uses -- pointing, vec3, dotprod and Healpix_Base's RING-scheme
 * constructor, ang2pix, pix2vec and the vector form of query_disc -- and
 * forwards them to the oracle's HEALPix restatement (oracle/healpix_ring.c),
 * so the reference's own genmap.cpp runs unchanged on top of it. */
#ifndef DMANN_SHIM_HEALPIX_BASE_H
#define DMANN_SHIM_HEALPIX_BASE_H
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>
#include "../../oracle.h"

enum Healpix_Ordering_Scheme { RING, NEST };
enum nside_dummy { SET_NSIDE };

struct pointing {
    double theta, phi;
    pointing() : theta(0), phi(0) {}
    pointing(double t, double p) : theta(t), phi(p) {}
};

struct vec3 {
    double x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(double a, double b, double c) : x(a), y(b), z(c) {}
};

inline double dotprod(const vec3 &a, const vec3 &b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

class Healpix_Base {
public:
    Healpix_Base(int nside, Healpix_Ordering_Scheme scheme, nside_dummy) {
        if (scheme != RING) { std::fprintf(stderr, "shim: RING only\n"); std::exit(1); }
        orc_hpx_init(&b_, nside);
    }
    int ang2pix(const pointing &p) const {
        return (int)orc_hpx_ang2pix(&b_, p.theta, p.phi);
    }
    vec3 pix2vec(int pix) const {
        double v[3];
        orc_hpx_pix2vec(&b_, pix, v);
        return vec3(v[0], v[1], v[2]);
    }
    void query_disc(pointing p, double radius, std::vector<int> &listpix) const {
        int64_t tot = 0;
        orc_hpx_query_disc(&b_, p.theta, p.phi, radius, 0, &tot);
        listpix.resize((size_t)tot);
        if (tot) orc_hpx_query_disc_list(&b_, p.theta, p.phi, radius, &listpix[0]);
    }
private:
    orc_hpx b_;
};
#endif
