// disc_comp.cu -- the compensated-FP32 form of the disc kernels.
//
// Per particle (FP64, once): direction, angular radius, disc rings and each
// ring's in-disc pixel run (the query_disc chord test, exactly the CPU
// path's arithmetic).  Per pixel (FP32): the angular distance to the particle
// from the haversine relation
//     hav(theta) = hav(theta_ring - theta0) + sin(theta_ring) sin(theta0) hav(dphi)
// (well conditioned at the small angles where acos(dot) is not), then
// theta^2 = 4 asin^2(sqrt(hav)) and w = 2^(-K theta^2) with
// K = log2(e) * 0.5 / (0.333 ar^2): the reference's exp(-0.5 (theta/ar)^2 /
// 0.333) (src/genmap.cpp:137-143).  The per-ring terms hav(theta_r - theta0)
// and sin(theta_r) sin(theta0), and the first pixel's azimuth offset, are
// formed in FP64 and rounded once, so the FP32 error does not grow with the
// absolute angles.  The normalisation is a Kahan-compensated FP32 sum per
// thread, reduced in FP64; deposits go to two FP32 planes (hi, lo) with an
// exact TwoSum on the value each atomic returns, plus the product's own
// rounding error.
//
// Polynomials (written from their Taylor series):
//   sin x = x - x^3/3! + x^5/5! - ... ; to x^7 for |x| < 0.35 (error
//   < 3e-10 relative), to x^15 for |x| <= pi/2 (error < 1e-11);
//   asin^2(sqrt h) = sum_n (4h)^n / (2 n^2 C(2n,n)) = h + h^2/3 + 8h^3/45 +
//   4h^4/35 + 128h^5/1575 + ... ; five terms for h < 0.02 (error < 3e-10
//   relative); otherwise asinf(sqrtf(h)) from the CUDA math library.
#include "disc_engine.cuh"

namespace dmann {

namespace {

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

struct CompForm {
    static constexpr bool kFastChord = true;
    static constexpr int kMinBlocks = 8;  // 8 x 256 threads per SM: full occupancy
    struct alignas(16) Seg {
        int start, nr, lo, off;
        float A, B, d0, step;
        float A2, pad0, pad1, pad2;
    };
    struct SegReg {
        int start, nr, lo;
        float A, B, d0, step, A2;
    };
    struct Ext {
        float K;
        int small_h, small_x;
    };
    struct NormAcc {
        float s = 0.0f, c = 0.0f;
    };
    struct Dep {
        float F, Flo;   // flux/norm as a two-float
    };

    __device__ static void particle_setup(const DiscArgs &a, const DiscHdr &d, double phi_raw,
                                          Ext &e) {
        (void)a;
        (void)phi_raw;
        e.K = (float)(4.0 * 1.4426950408889634 * 0.5 / (0.333 * d.ar * d.ar));
        double hmax = 1.0;
        if (!d.allsky) {
            double s = sin(0.5 * d.R);
            hmax = s * s;
        }
        e.small_h = hmax < 0.02;
        bool caps = d.allsky || d.r_first < d.irmin || d.r_last > d.irmax;
        int small_x = 0;
        if (!caps) {
            double sr = sin(d.R);
            if (sr < 0.999 * d.sth0) small_x = (0.5 * asin(sr / d.sth0)) < 0.33;
        }
        e.small_x = small_x;
    }

    __device__ static void fill_seg(const DiscArgs &a, const DiscHdr &d, const Ext &e, int ring,
                                    int lo, int cnt, Seg &s) {
        (void)e;
        (void)cnt;
        s.start = (int)ring_start(a.g, ring);
        s.nr = ring_npix(a.g, ring);
        s.lo = lo;
        const double shift = ring_shifted(a.g, ring) ? 0.5 : 0.0;
        const float dth = (float)(a.rt.theta[ring] - d.theta0);
        const float sa = sinf(0.5f * dth);
        s.A = sa * sa;
        s.B = (float)(a.rt.st[ring] * d.sth0);
        const double step = a.rt.step[ring];
        s.step = (float)step;
        // azimuth of the run's first pixel relative to the particle, in
        // [-pi, pi): runs that were shifted by -nr (disc across phi = 2 pi)
        // would otherwise start 2 pi low
        double d0 = ((double)lo + shift) * step - d.phi0;
        if (d0 < -kPi) d0 += kTwoPi;
        if (d0 >= kPi) d0 -= kTwoPi;
        s.d0 = (float)d0;
        // hav of the ring's colatitude distance to the particle's antipode
        const float dth2 = (float)(a.rt.theta[ring] + d.theta0 - kPi);
        const float sb = sinf(0.5f * dth2);
        s.A2 = sb * sb;
    }

    __device__ static void load_seg(const Seg &s, SegReg &r) {
        const int4 i4 = *reinterpret_cast<const int4 *>(&s.start);
        const float4 f4 = *reinterpret_cast<const float4 *>(&s.A);
        r.start = i4.x;
        r.nr = i4.y;
        r.lo = i4.z;
        r.A = f4.x;
        r.B = f4.y;
        r.d0 = f4.z;
        r.step = f4.w;
        r.A2 = s.A2;
    }

    // sin x for |x| <= pi/2 (Taylor to x^15) or |x| < 0.35 (to x^7)
    __device__ static float sin_poly(float x, bool small) {
        const float x2 = x * x;
        float p;
        if (small) {
            p = fmaf(x2, -1.0f / 5040.0f, 1.0f / 120.0f);
            p = fmaf(x2, p, -1.0f / 6.0f);
            p = fmaf(x2, p, 1.0f);
        } else {
            p = fmaf(x2, -1.0f / 1307674368000.0f, 1.0f / 6227020800.0f);
            p = fmaf(x2, p, -1.0f / 39916800.0f);
            p = fmaf(x2, p, 1.0f / 362880.0f);
            p = fmaf(x2, p, -1.0f / 5040.0f);
            p = fmaf(x2, p, 1.0f / 120.0f);
            p = fmaf(x2, p, -1.0f / 6.0f);
            p = fmaf(x2, p, 1.0f);
        }
        return x * p;
    }

    // theta^2 / 4 = asin^2(sqrt(hav theta)).  Beyond 90 degrees (hav > 1/2)
    // asin(sqrt(h)) loses precision as h -> 1, so the distance is taken to the
    // particle's antipode instead (same haversine form, ring term A2 and the
    // azimuth offset dphi -+ pi) and theta = pi - theta'.
    __device__ static float weight(const Ext &e, const SegReg &sr, int j) {
        const float dphi = fmaf((float)j, sr.step, sr.d0);
        const float sn = sin_poly(0.5f * dphi, e.small_x);
        const float h = fmaf(sr.B, sn * sn, sr.A);
        float g;
        if (e.small_h) {
            float q = fmaf(h, 128.0f / 1575.0f, 4.0f / 35.0f);
            q = fmaf(h, q, 8.0f / 45.0f);
            q = fmaf(h, q, 1.0f / 3.0f);
            q = fmaf(h, q, 1.0f);
            g = h * q;
        } else {
            float t;
            if (h <= 0.5f) {
                t = asinf(sqrtf(fmaxf(h, 0.0f)));
            } else {
                const float dpf = dphi - copysignf(3.14159265358979f, dphi);
                const float sf = sin_poly(0.5f * dpf, false);
                const float hf = fmaf(sr.B, sf * sf, sr.A2);
                t = 1.57079632679490f - asinf(sqrtf(fminf(fmaxf(hf, 0.0f), 1.0f)));
            }
            g = t * t;
        }
        return ex2_approx(-e.K * g);
    }

    __device__ static void norm_add(const Ext &e, const SegReg &sr, int j, int pix, NormAcc &acc) {
        (void)pix;
        const float w = weight(e, sr, j);
        const float y = __fsub_rn(w, acc.c);  // Kahan step
        const float t = __fadd_rn(acc.s, y);
        acc.c = __fsub_rn(__fsub_rn(t, acc.s), y);
        acc.s = t;
    }
    __device__ static double norm_value(const NormAcc &acc) { return (double)acc.s - (double)acc.c; }

    __device__ static void deposit_setup(const DiscArgs &a, const DiscHdr &d, const Ext &e, double S,
                                         Dep &dep) {
        (void)e;
        const double F = d.flux * a.f.inv_scale / S;
        dep.F = (float)F;
        dep.Flo = (float)(F - (double)dep.F);
    }
    // w * F as hi + lo: the product's rounding error (exact, from an FMA) and
    // w * Flo travel to the lo plane with the atomic's TwoSum error, so a
    // particle's deposits add up to its flux to ~1e-12, not to FP32 rounding.
    __device__ static void deposit(const DiscArgs &a, const Ext &e, const Dep &dep, const SegReg &sr,
                                   int j, int pix) {
        const float w = weight(e, sr, j);
        const float p = w * dep.F;
        const float pe = fmaf(w, dep.Flo, fmaf(w, dep.F, -p));
        deposit2f(a.acc.hi, a.acc.lo, pix, p, pe);
    }
    __device__ static void single(const DiscArgs &a, const DiscHdr &d) {
        const double vs = d.flux * a.f.inv_scale;
        const float vh = (float)vs;
        const float vl = (float)(vs - (double)vh);
        deposit2f(a.acc.hi, a.acc.lo, d.cpix, vh);
        if (vl != 0.0f) red_add_f32(a.acc.lo + d.cpix, vl);
    }
};

constexpr int kBT = 256, kRCH = 512;
constexpr int kWPB = 8, kRCHW = 64;

}  // namespace

cudaError_t launch_disc_comp(const DiscArgs &a, int num_sms, int blocks_per_sm, cudaStream_t s,
                             cudaEvent_t mid) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, k_disc_block<CompForm, kBT, kRCH>, kBT, 0);
    if (e != cudaSuccess) return e;
    int bps = blocks_per_sm > 0 ? min(blocks_per_sm, occ) : occ;
    if (bps < 1) bps = 1;
    k_disc_block<CompForm, kBT, kRCH><<<num_sms * bps, kBT, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (mid && (e = cudaEventRecord(mid, s)) != cudaSuccess) return e;
    int occw = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_disc_warp<CompForm, kWPB, kRCHW>,
                                                      kWPB * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_disc_warp<CompForm, kWPB, kRCHW><<<num_sms * occw, kWPB * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dmann
