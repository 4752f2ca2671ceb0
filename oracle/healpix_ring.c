/*
 * healpix_ring.c -- FP64 HEALPix RING-scheme functions for the oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * The reference calls HEALPix C++ 3.00 (Healpix_Base, RING scheme) at
 * src/genmap.cpp:40 (constructor), :106 (ang2pix), :119 (query_disc, the
 * non-inclusive vector form) and :135 (pix2vec).  HEALPix is not vendored by
 * the reference, so the functions are restated here from the published
 * scheme (Gorski et al. 2005, ApJ 622:759, sections 4-5):
 *   - 12*Nside^2 equal-area pixels on 4*Nside-1 iso-latitude rings;
 *   - polar-cap rings i < Nside hold 4i pixels with z = 1 - i^2/(3 Nside^2);
 *   - equatorial rings Nside <= i <= 3 Nside hold 4 Nside pixels with
 *     z = (2 Nside - i) * 2/(3 Nside), every other ring shifted by half a pixel;
 *   - query_disc walks the rings that cross the disc and keeps, per ring,
 *     the pixel centres whose azimuth lies inside the disc chord.
 * The choice of formulae near the poles (the sin(theta) form of the cap
 * index) and the half-open azimuth test of query_disc follow the library's
 * documented behaviour so that pixel sets agree with it.
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>
#include "oracle.h"

static const double k_pi = 3.141592653589793238462643383279502884197;
static const double k_halfpi = 1.570796326794896619231321691639751442099;
static const double k_inv_halfpi = 0.6366197723675813430755350534900574;
static const double k_twopi = 6.283185307179586476925286766559005768394;
static const double k_inv_twopi = 0.1591549430918953357688837633725143620345;
static const double k_twothird = 2.0 / 3.0;

static int64_t isqrt64(int64_t v) {
    int64_t r = (int64_t)sqrt((double)v + 0.5);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

/* v1 mod v2 into [0, v2) for floating point values (v2 > 0). */
static double fmodulo(double v1, double v2) {
    if (v1 >= 0) return (v1 < v2) ? v1 : fmod(v1, v2);
    double t = fmod(v1, v2) + v2;
    return (t == v2) ? 0.0 : t;
}

void orc_hpx_init(orc_hpx *b, int64_t nside) {
    b->nside = nside;
    b->npix = 12 * nside * nside;
    b->ncap = 2 * nside * (nside - 1);
    b->fact2 = 4.0 / (double)b->npix;
    b->fact1 = (double)(nside << 1) * b->fact2;
}

static int64_t loc2pix(const orc_hpx *b, double z, double phi, double sth,
                       int have_sth) {
    const int64_t ns = b->nside;
    double za = fabs(z);
    double tt = fmodulo(phi * k_inv_halfpi, 4.0); /* in [0,4) */
    if (za <= k_twothird) {                       /* equatorial belt */
        int64_t nl4 = 4 * ns;
        double temp1 = (double)ns * (0.5 + tt);
        double temp2 = (double)ns * z * 0.75;
        int64_t jp = (int64_t)(temp1 - temp2); /* ascending edge line */
        int64_t jm = (int64_t)(temp1 + temp2); /* descending edge line */
        int64_t ir = ns + 1 + jp - jm;         /* ring from z=2/3, 1..2ns+1 */
        int64_t kshift = 1 - (ir & 1);
        int64_t t1 = jp + jm - ns + kshift + 1 + nl4 + nl4;
        int64_t ip = (t1 >> 1) % nl4;
        return b->ncap + (ir - 1) * nl4 + ip;
    }
    /* polar caps */
    double tp = tt - (double)(int64_t)tt;
    double tmp = ((za < 0.99) || !have_sth)
                     ? (double)ns * sqrt(3.0 * (1.0 - za))
                     : (double)ns * sth / sqrt((1.0 + za) / 3.0);
    int64_t jp = (int64_t)(tp * tmp);
    int64_t jm = (int64_t)((1.0 - tp) * tmp);
    int64_t ir = jp + jm + 1;          /* ring counted from the nearest pole */
    int64_t ip = (int64_t)(tt * (double)ir);
    if (ip >= 4 * ir) ip = 4 * ir - 1; /* cannot happen for tt < 4 */
    return (z > 0) ? 2 * ir * (ir - 1) + ip : b->npix - 2 * ir * (ir + 1) + ip;
}

int64_t orc_hpx_ang2pix(const orc_hpx *b, double theta, double phi) {
    /* The library switches to the sin(theta) form within 0.01 rad of a pole. */
    if ((theta < 0.01) || (theta > 3.14159 - 0.01))
        return loc2pix(b, cos(theta), phi, sin(theta), 1);
    return loc2pix(b, cos(theta), phi, 0.0, 0);
}

static void pix2loc(const orc_hpx *b, int64_t pix, double *z, double *phi,
                    double *sth, int *have_sth) {
    const int64_t ns = b->nside;
    *have_sth = 0;
    *sth = 0.0;
    if (pix < b->ncap) { /* north polar cap */
        int64_t iring = (1 + isqrt64(1 + 2 * pix)) >> 1;
        int64_t iphi = (pix + 1) - 2 * iring * (iring - 1);
        double tmp = (double)(iring * iring) * b->fact2;
        *z = 1.0 - tmp;
        if (*z > 0.99) { *sth = sqrt(tmp * (2.0 - tmp)); *have_sth = 1; }
        *phi = ((double)iphi - 0.5) * k_halfpi / (double)iring;
    } else if (pix < (b->npix - b->ncap)) { /* equatorial belt */
        int64_t nl4 = 4 * ns;
        int64_t ip = pix - b->ncap;
        int64_t tmp = ip / nl4;
        int64_t iring = tmp + ns;
        int64_t iphi = ip - nl4 * tmp + 1;
        double fodd = ((iring + ns) & 1) ? 1.0 : 0.5;
        *z = (double)(2 * ns - iring) * b->fact1;
        *phi = ((double)iphi - fodd) * k_pi * 0.75 * b->fact1;
    } else { /* south polar cap */
        int64_t ip = b->npix - pix;
        int64_t iring = (1 + isqrt64(2 * ip - 1)) >> 1;
        int64_t iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
        double tmp = (double)(iring * iring) * b->fact2;
        *z = tmp - 1.0;
        if (*z < -0.99) { *sth = sqrt(tmp * (2.0 - tmp)); *have_sth = 1; }
        *phi = ((double)iphi - 0.5) * k_halfpi / (double)iring;
    }
}

void orc_hpx_pix2vec(const orc_hpx *b, int64_t pix, double v[3]) {
    double z, phi, sth;
    int have;
    pix2loc(b, pix, &z, &phi, &sth, &have);
    double st = have ? sth : sqrt((1.0 - z) * (1.0 + z));
    v[0] = st * cos(phi);
    v[1] = st * sin(phi);
    v[2] = z;
}

void orc_hpx_pix2ang(const orc_hpx *b, int64_t pix, double *theta, double *phi) {
    double z, sth;
    int have;
    pix2loc(b, pix, &z, phi, &sth, &have);
    *theta = have ? atan2(sth, z) : acos(z);
}

int64_t orc_hpx_ring_above(const orc_hpx *b, double z) {
    double az = fabs(z);
    if (az <= k_twothird) return (int64_t)((double)b->nside * (2.0 - 1.5 * z));
    int64_t iring = (int64_t)((double)b->nside * sqrt(3.0 * (1.0 - az)));
    return (z > 0) ? iring : 4 * b->nside - iring - 1;
}

double orc_hpx_ring2z(const orc_hpx *b, int64_t ring) {
    const int64_t ns = b->nside;
    if (ring < ns) return 1.0 - (double)(ring * ring) * b->fact2;
    if (ring <= 3 * ns) return (double)(2 * ns - ring) * b->fact1;
    ring = 4 * ns - ring;
    return (double)(ring * ring) * b->fact2 - 1.0;
}

void orc_hpx_ring_info(const orc_hpx *b, int64_t ring, int64_t *startpix,
                       int64_t *ringpix, int *shifted) {
    const int64_t ns = b->nside;
    if (ring < ns) {
        *shifted = 1;
        *ringpix = 4 * ring;
        *startpix = 2 * ring * (ring - 1);
    } else if (ring < 3 * ns) {
        *shifted = ((ring - ns) & 1) == 0;
        *ringpix = 4 * ns;
        *startpix = b->ncap + (ring - ns) * (*ringpix);
    } else {
        int64_t nr = 4 * ns - ring;
        *shifted = 1;
        *ringpix = 4 * nr;
        *startpix = b->npix - 2 * nr * (nr + 1);
    }
}

/* Range accumulator that merges a range adjacent to the previous one, as
 * the library's range set does; only the union matters for the callers. */
typedef struct {
    int64_t *r;
    int64_t n, total, last_hi;
} rangeacc;

static void racc_add(rangeacc *a, int64_t lo, int64_t hi) {
    if (hi <= lo) return;
    a->total += hi - lo;
    if (a->n > 0 && a->last_hi == lo) { /* adjacent: extend the last range */
        if (a->r) a->r[2 * a->n - 1] = hi;
        a->last_hi = hi;
        return;
    }
    if (a->r) {
        a->r[2 * a->n] = lo;
        a->r[2 * a->n + 1] = hi;
    }
    a->last_hi = hi;
    a->n++;
}

int64_t orc_hpx_query_disc(const orc_hpx *b, double theta, double phi,
                           double radius, int64_t *ranges, int64_t *npix_out) {
    rangeacc acc = {ranges, 0, 0, -1};
    const int64_t ns = b->nside;
    /* normalise the pointing: theta in [0,pi], phi in [0,2pi) */
    theta = fmodulo(theta, k_twopi);
    if (theta > k_pi) { phi += k_pi; theta = k_twopi - theta; }
    phi = fmodulo(phi, k_twopi);

    if (radius >= k_pi) {
        racc_add(&acc, 0, b->npix);
        if (npix_out) *npix_out = acc.total;
        return acc.n;
    }
    double cosrbig = cos(radius);
    double z0 = cos(theta);
    double xa = 1.0 / sqrt((1.0 - z0) * (1.0 + z0));

    double rlat1 = theta - radius;
    double zmax = cos(rlat1);
    int64_t irmin = orc_hpx_ring_above(b, zmax) + 1;
    if ((rlat1 <= 0) && (irmin > 1)) { /* north pole inside the disc */
        int64_t sp, rp;
        int sh;
        orc_hpx_ring_info(b, irmin - 1, &sp, &rp, &sh);
        racc_add(&acc, 0, sp + rp);
    }
    double rlat2 = theta + radius;
    double zmin = cos(rlat2);
    int64_t irmax = orc_hpx_ring_above(b, zmin);

    for (int64_t iz = irmin; iz <= irmax; ++iz) {
        double z = orc_hpx_ring2z(b, iz);
        double x = (cosrbig - z * z0) * xa;
        double ysq = 1.0 - z * z - x * x;
        double dphi = (ysq <= 0) ? 0.0 : atan2(sqrt(ysq), x);
        if (dphi > 0) {
            int64_t ipix1, nr;
            int shifted;
            orc_hpx_ring_info(b, iz, &ipix1, &nr, &shifted);
            double shift = shifted ? 0.5 : 0.0;
            int64_t ipix2 = ipix1 + nr - 1;
            int64_t ip_lo =
                (int64_t)floor((double)nr * k_inv_twopi * (phi - dphi) - shift) + 1;
            int64_t ip_hi =
                (int64_t)floor((double)nr * k_inv_twopi * (phi + dphi) - shift);
            if (ip_lo <= ip_hi) {
                if (ip_hi >= nr) { ip_lo -= nr; ip_hi -= nr; }
                if (ip_lo < 0) {
                    racc_add(&acc, ipix1, ipix1 + ip_hi + 1);
                    racc_add(&acc, ipix1 + ip_lo + nr, ipix2 + 1);
                } else {
                    racc_add(&acc, ipix1 + ip_lo, ipix1 + ip_hi + 1);
                }
            }
        }
    }
    if ((rlat2 >= k_pi) && (irmax + 1 < 4 * ns)) { /* south pole inside */
        int64_t sp, rp;
        int sh;
        orc_hpx_ring_info(b, irmax + 1, &sp, &rp, &sh);
        racc_add(&acc, sp, b->npix);
    }
    if (npix_out) *npix_out = acc.total;
    return acc.n;
}

int64_t orc_hpx_query_disc_list(const orc_hpx *b, double theta, double phi,
                                double radius, int32_t *out) {
    /* ranges: at most two per ring plus the two caps */
    int64_t maxr = 2 * (4 * b->nside) + 4;
    int64_t stackbuf[512];
    int64_t *r = stackbuf;
    int heap = 0;
    if (2 * maxr > 512) {
        r = (int64_t *)malloc(sizeof(int64_t) * 2 * maxr);
        heap = 1;
    }
    int64_t tot = 0;
    int64_t nr = orc_hpx_query_disc(b, theta, phi, radius, r, &tot);
    int64_t k = 0;
    for (int64_t i = 0; i < nr; i++)
        for (int64_t p = r[2 * i]; p < r[2 * i + 1]; p++) out[k++] = (int32_t)p;
    if (heap) {
        free(r);
    }
    return k;
}
