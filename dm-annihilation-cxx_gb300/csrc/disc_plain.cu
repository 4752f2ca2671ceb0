// disc_plain.cu -- the plain FP64 form of the disc kernels.
//
// The reference CPU path's arithmetic on the GPU: each disc pixel's centre
// vector as pix2vec computes it (z and sin(theta) of its ring, phi from the
// in-ring index), w = exp(-0.5 (acos(v_pix . v)/ar)^2 / 0.333)
// (src/genmap.cpp:133-145), the FP64 normalisation and w/norm*flux added to
// an FP64 map with FP64 atomics (src/genmap.cpp:148-153).  Compiled with
// -fmad=false so every expression rounds as the CPU path's does; results
// differ from it only by the order of the additions.
#include "disc_engine.cuh"

namespace dmann {

namespace {

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

    // src/genmap.cpp:135-143 with pix2vec as the oracle restates it
    __device__ static double weight(const Ext &e, const SegReg &sr, int pix) {
        const int k = pix - sr.start;
        const double iphi = (double)(k + 1);
        double phi;
        if (sr.cap) phi = (iphi - 0.5) * kHalfPi / (double)sr.ipole;
        else phi = (iphi - sr.pf) * kPi * 0.75 * e.fact1;
        double sp, cp;
        sincos(phi, &sp, &cp);
        const double dot = sr.st * cp * e.vx + sr.st * sp * e.vy + sr.z * e.vz;
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

constexpr int kBT = 256, kRCH = 256;
constexpr int kWPB = 8, kRCHW = 64;

}  // namespace

cudaError_t launch_disc_plain(const DiscArgs &a, int num_sms, int blocks_per_sm, cudaStream_t s,
                              cudaEvent_t mid) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, k_disc_block<PlainForm, kBT, kRCH>, kBT, 0);
    if (e != cudaSuccess) return e;
    int bps = blocks_per_sm > 0 ? min(blocks_per_sm, occ) : occ;
    if (bps < 1) bps = 1;
    k_disc_block<PlainForm, kBT, kRCH><<<num_sms * bps, kBT, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (mid && (e = cudaEventRecord(mid, s)) != cudaSuccess) return e;
    int occw = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_disc_warp<PlainForm, kWPB, kRCHW>,
                                                      kWPB * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_disc_warp<PlainForm, kWPB, kRCHW><<<num_sms * occw, kWPB * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dmann
