// plain_form.cuh -- the plain FP64 precision form of the disc engine: the
// reference CPU path's per-pixel arithmetic (pix2vec of each disc pixel,
// w = exp(-0.5 (acos(v_pix . v)/ar)^2 / 0.333), src/genmap.cpp:133-145,
// FP64 normalisation and FP64 atomic deposits, genmap.cpp:148-153).
// Shared by the plain render kernels (disc_plain.cu) and the adjoint
// kernels (adjoint.cu); both translation units are compiled with
// -fmad=false so the weights round exactly as the CPU path's do.
#pragma once
#include "disc_engine.cuh"

namespace dmann {

struct PlainForm {
    static constexpr bool kFastChord = false;  // the exact FP64 chord test
    static constexpr int kMinBlocks = 1;
    struct alignas(16) Seg {
        int start, nr, lo, off;
        double z, st, pf;
        int cap, ipole;
    };
    struct SegReg {
        int start, nr, lo;
        double z, st, pf;
        int cap, ipole;
    };
    struct Ext {
        double vx, vy, vz, ar, fact1;
    };
    struct NormAcc {
        double s = 0.0;
    };
    struct Dep {
        double S, flux;
    };

    // anglefuncs.cpp:55-71 ang2vec, from the un-normalised phi of calc_angles
    __device__ static void particle_setup(const DiscArgs &a, const DiscHdr &d, double phi_raw,
                                          Ext &e) {
        const double sz = sin(d.theta0);
        e.vx = sz * cos(phi_raw);
        e.vy = sz * sin(phi_raw);
        e.vz = cos(d.theta0);
        e.ar = d.ar;
        e.fact1 = a.g.fact1;
    }

    __device__ static void fill_seg(const DiscArgs &a, const DiscHdr &d, const Ext &e, int ring,
                                    int lo, int cnt, Seg &s) {
        (void)d;
        (void)e;
        (void)cnt;
        const int ns = a.g.nside;
        s.start = (int)ring_start(a.g, ring);
        s.nr = ring_npix(a.g, ring);
        s.lo = lo;
        s.z = a.rt.z[ring];
        s.st = a.rt.st[ring];
        s.cap = (ring < ns) || (ring > 3 * ns);
        s.ipole = (ring < ns) ? ring : 4 * ns - ring;
        s.pf = ((ring + ns) & 1) ? 1.0 : 0.5;
    }

    __device__ static void load_seg(const Seg &s, SegReg &r) {
        r.start = s.start;
        r.nr = s.nr;
        r.lo = s.lo;
        r.z = s.z;
        r.st = s.st;
        r.pf = s.pf;
        r.cap = s.cap;
        r.ipole = s.ipole;
    }

    // pix2vec of a pixel of the segment's ring, as the oracle restates it
    __device__ static void pixel_vec(const Ext &e, const SegReg &sr, int pix, double &px,
                                     double &py, double &pz) {
        const int k = pix - sr.start;
        const double iphi = (double)(k + 1);
        double phi;
        if (sr.cap) phi = (iphi - 0.5) * kHalfPi / (double)sr.ipole;
        else phi = (iphi - sr.pf) * kPi * 0.75 * e.fact1;
        double sp, cp;
        sincos(phi, &sp, &cp);
        px = sr.st * cp;
        py = sr.st * sp;
        pz = sr.z;
    }

    // src/genmap.cpp:135-143
    __device__ static double weight(const Ext &e, const SegReg &sr, int pix) {
        double px, py, pz;
        pixel_vec(e, sr, pix, px, py, pz);
        const double dot = px * e.vx + py * e.vy + pz * e.vz;
        const double dc = fmin(1.0, fmax(-1.0, dot));
        double d2 = acos(dc) / e.ar;
        d2 = d2 * d2;
        return exp(-0.5 * d2 / 0.333);
    }

    __device__ static void norm_add(const Ext &e, const SegReg &sr, int j, int pix, NormAcc &acc) {
        (void)j;
        acc.s += weight(e, sr, pix);
    }
    __device__ static double norm_value(const NormAcc &acc) { return acc.s; }

    __device__ static void deposit_setup(const DiscArgs &a, const DiscHdr &d, const Ext &e, double S,
                                         Dep &dep) {
        (void)a;
        (void)e;
        dep.S = S;
        dep.flux = d.flux;
    }
    __device__ static void deposit(const DiscArgs &a, const Ext &e, const Dep &dep, const SegReg &sr,
                                   int j, int pix) {
        (void)j;
        const double w = weight(e, sr, pix);
        red_add_f64(a.acc.acc64 + pix, (w / dep.S) * dep.flux);
    }
    __device__ static void single(const DiscArgs &a, const DiscHdr &d) {
        red_add_f64(a.acc.acc64 + d.cpix, d.flux);
    }
};

}  // namespace dmann
