// comp_engine.cuh -- device building blocks of the compensated-FP32 form
// (disc_comp.cu: the per-disc render kernels, the adjoint and the
// no-allocation path; disc_seg.cu: the segmented render).
//
// Per particle (FP64, once): direction, angular radius, disc rings and each
// ring's in-disc pixel run (the query_disc chord test; FP32 with an exact FP64
// fallback near ties, so the pixel sets equal the CPU path's).  Per pixel
// (FP32): the angular distance to the particle from the haversine relation
//     hav(theta) = hav(theta_ring - theta0) + sin(theta_ring) sin(theta0) hav(dphi)
// (well conditioned at the small angles where acos(dot) is not), then
// theta^2 = 4 asin^2(sqrt(hav)) and w = 2^(-K theta^2) with
// K = log2(e) * 0.5 / (0.333 ar^2): the reference's exp(-0.5 (theta/ar)^2 /
// 0.333) (src/genmap.cpp:137-143).  The per-ring terms hav(theta_r - theta0),
// sin(theta_r) sin(theta0) and the run's first azimuth offset are formed in
// FP64 and rounded once, so the FP32 error does not grow with the absolute
// angles.  Beyond 90 degrees (hav > 1/2) the distance is taken to the
// particle's antipode, where asin(sqrt(h)) would lose precision.
//
// Normalisation: a compensated FP32 sum per thread (offset so that Fast2Sum
// captures every rounding error exactly), reduced as two-floats; flux/norm
// as a two-float (F, Flo).
// Deposits: w (F + Flo) rounded once to FP32 (an FMA), converted exactly to
// FP64 and added with a non-returning red.global.add.f64 into the FP64 plane.
// Each deposit's only error is that one rounding (relative 2^-24, unbiased),
// so a particle's deposits add up to its flux to ~2^-24 / sqrt(#pixels) and a
// pixel's sum of many deposits is far more accurate than each weight.
//
// Work layout ("run engine"): the disc's rings are staged in shared memory
// as runs -- one ring's in-disc pixels, split where the ring wraps so that a
// run is contiguous in the map -- and each warp takes whole runs.  A lane
// evaluates two pixels of a run at once (j and j + 32) with the packed FP32x2
// instructions of sm_100+ (__ffma2_rn & co.), halving the issue slots of the
// polynomials, the compensated sums and the products.
//
// Polynomials (written from their Taylor series), the number of terms chosen
// per particle from the largest |x| and h its disc can reach:
//   sin x = x - x^3/3! + x^5/5! - ... ; to x^3 for |x| < 0.025 (error
//   < 3.3e-9 relative), to x^7 for |x| < 0.35 (< 3e-10), to x^15 for
//   |x| <= pi/2 (< 1e-11);
//   asin^2(sqrt h) = sum_n (4h)^n / (2 n^2 C(2n,n)) = h + h^2/3 + 8h^3/45 +
//   4h^4/35 + 128h^5/1575 + ... ; three terms for h < 4e-3 (error < 7.4e-9
//   relative), five for h < 0.02 (< 3e-10); otherwise, up to h = 1/2, a
//   fitted degree-9 polynomial (g_near2, 1.2e-8), and beyond 90 degrees
//   asinf(sqrtf()) of the antipode's haversine from the CUDA math library.
//   All truncation errors stay below FP32 rounding.
#pragma once
#include <type_traits>

#include "adjoint_common.cuh"
#include "kernels.cuh"

namespace dmann {

namespace {

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// packed FP32x2 arithmetic (round to nearest per element)
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {   // one packed subtract
    unsigned long long ua = *reinterpret_cast<unsigned long long *>(&a);
    unsigned long long ub = *reinterpret_cast<unsigned long long *>(&b);
    unsigned long long ud;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(ud) : "l"(ua), "l"(ub));
    return *reinterpret_cast<float2 *>(&ud);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// a + b = s + err exactly (Knuth's TwoSum)
__device__ __forceinline__ float two_sum(float a, float b, float &err) {
    const float s = a + b;
    const float bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}

// Two-float sum (s, c) over the warp; every lane ends with the total.
__device__ __forceinline__ void warp_sum_ff(float &s, float &c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
        float err;
        s = two_sum(s, s2, err);
        c = (c + c2) + err;
    }
}

// (ah + al) / (bh + bl) as a normalised two-float (Dekker): q1 = ah / bh,
// the remainder a - q1 b from an exact product (FMA) and an exact
// difference (q1 bh is within a few ulp of ah), then one correction.
__device__ inline float2 div_ff(float ah, float al, float bh, float bl) {
    const float b = bh + bl;
    const float b_lo = bl - (b - bh);
    const float q1 = __fdiv_rn(ah, b);
    const float p = q1 * b;
    const float pe = fmaf(q1, b, -p);
    const float r = (((ah - p) - pe) + al) - q1 * b_lo;
    const float q2 = __fdiv_rn(r, b);
    const float hi = q1 + q2;
    return make_float2(hi, q2 - (hi - q1));
}

constexpr float kHalfPiF = 1.57079632679490f;

// One run: pixels pix0 .. pix0+cnt-1 of one ring, in order of increasing
// azimuth; x(j) = d0h + j*steph is half the azimuth offset of pixel j from
// the particle.
struct alignas(16) Run {
    int pix0, cnt;
    float A, B;         // hav(theta_r - theta0), sin(theta_r) sin(theta0)
    float d0h, steph;   // half azimuth offset of pixel 0, half the pixel step
    float A2;           // hav(theta_r + theta0 - pi): distance to the antipode
    int more;           // the ring continues in the next run slot (it wrapped)
};

struct Ext {
    float nK;           // -K
    int tier_h, tier_x;  // polynomial lengths (0 shortest, 2 general)
    float fs_hi, fs_lo;  // flux * inv_scale as a two-float (render only)
    int rpi;            // rings per work item (segmented render; set by k_seg_count)
};

// Per-particle constants of the FP32 chord test (see chord_fast).
struct Chord {
    float hR;           // hav(R) = sin^2(R/2), R the disc radius
    float sth0;         // sin(theta0)
    int ci[2];          // c = nr/(2 pi) phi0 - shift for the equatorial rings
    float cf[2];        // (nr = 4 nside), shift 0 and 1/2: floor(c) and c - floor(c)
    int fast;           // the FP32 test may be used for this particle
};

}  // namespace

// Everything the disc kernels need of one particle besides its runs (the
// type that DiscArgs::chdr points to).
struct CompHdr {
    DiscHdr hdr;
    Ext ext;
    Chord ch;
};
static_assert(sizeof(CompHdr) % 8 == 0, "CompHdr is copied in 8-byte words");

namespace {

template <int RCH>
struct CompSmem {
    Run run[2 * RCH];   // two runs per ring (the second only where it wraps)
    CompHdr h;
    double red[32];
    float2 red2[32];    // per-warp two-float sums
    float2 fq;          // flux / S as a two-float
    int cnt_red[32];
    int next_run;       // runs claimed so far in the current pass (block groups)
};

__device__ inline void particle_setup(const Hpx &g, const DiscHdr &d, Ext &e, Chord &ch) {
    e.nK = -(float)(4.0 * 1.4426950408889634 * 0.5 / (0.333 * d.ar * d.ar));
    double hmax = 1.0;
    if (!d.allsky) {
        const double s = sin(0.5 * d.R);
        hmax = s * s;
    }
    e.tier_h = hmax < 4e-3 ? 0 : hmax < 0.02 ? 1 : 2;
    ch.hR = (float)hmax;
    ch.sth0 = (float)d.sth0;
    ch.fast = !d.allsky && d.sth0 > 1e-3;
    const double fnr = __dmul_rn((double)(4 * g.nside), kInvTwoPi);
    for (int k = 0; k < 2; k++) {
        const double c = __dsub_rn(__dmul_rn(fnr, d.phi0), k ? 0.5 : 0.0);
        const double fl = floor(c);
        ch.ci[k] = (int)fl;
        ch.cf[k] = (float)(c - fl);
    }
    const bool caps = d.allsky || d.r_first < d.irmin || d.r_last > d.irmax;
    int tier_x = 2;
    if (!caps) {
        const double sr = sin(d.R);
        if (sr < 0.999 * d.sth0) {
            const double xm = 0.5 * asin(sr / d.sth0);   // largest half azimuth offset
            tier_x = xm < 0.025 ? 0 : xm < 0.33 ? 1 : 2;
        }
    }
    e.tier_x = tier_x;
}

__device__ inline bool near_int_f(float a, float tau) {
    const float fr = a - floorf(a);
    return fr < tau || fr > 1.0f - tau;
}

// The chord of ring `ring` in FP32.  With q = sin^2(dphi/2), where dphi is
// the half-width of the in-disc azimuth interval,
//     q = (hav(R) - hav(theta_r - theta0)) / (sin theta_r sin theta0)
// (the haversine form of query_disc's x = (cos R - z z0) / sin theta0,
// ysq = 1 - z^2 - x^2 = 4 sin^2(theta_r) q (1 - q), dphi = atan2(sqrt(ysq), x)),
// which stays well conditioned for small discs, where ysq is a difference of
// numbers near 1.  The end points fnr (phi0 -+ dphi) - shift are formed as
// c -+ fnr dphi with c = fnr phi0 - shift split into floor(c) + frac (FP64,
// once per particle for the equatorial rings).  A running error bound covers
// the FP32 roundings (inputs, sinf, asinf, sqrtf: a few ulp each) and the
// rounding of the FP64 form this must reproduce; when an end point lies
// within the bound of an integer, or q is too close to 0 or 1 to decide, the
// caller takes the exact FP64 test instead.  So the pixel runs are those of
// the exact test.  Returns false for "undecided".
__device__ inline bool chord_fast(const Hpx &g, const DiscHdr &d, const Chord &ch, int ring, int nr,
                                  bool shifted, float A, float st32, int &ip_lo, int &ip_hi, int &ci,
                                  float &cf) {
    if (!(st32 > 0.01f)) return false;
    const float B = st32 * ch.sth0;
    const float num = ch.hR - A;
    const float dnum = 1.2e-7f * ch.hR + 8e-7f * A + 1.2e-7f * fabsf(num);
    if (num < -4.0f * dnum && -num > 1e-9f * B) {   // clearly outside: no pixel
        ip_lo = 1;
        ip_hi = 0;
        ci = 0;
        cf = 0.0f;
        return true;
    }
    if (!(num > 4.0f * dnum)) return false;
    const float q = __fdiv_rn(num, B);
    const float eq = __fdiv_rn(dnum, num) + 4.2e-7f;   // relative error of q
    if (!(q < 0.9999f) || eq > 1e-3f) return false;
    const float sq = sqrtf(q);
    const float dphi = 2.0f * asinf(sq);
    // FP32 error of dphi (d dphi / dq = 1 / sqrt(q (1 - q))), doubled, plus
    // the FP64 form's own rounding (ysq and x carry ~1e-16 absolute errors)
    const float ddphi = 2.0f * (eq * sq * rsqrtf(1.0f - q) + 6e-7f * dphi) +
                        1e-15f * (1.0f / (B * sq) + 1.0f / (st32 * st32 * sq)) + 1e-12f;
    if (ring >= g.nside && ring <= 3 * g.nside) {
        const int k = shifted ? 1 : 0;
        ci = ch.ci[k];
        cf = ch.cf[k];
    } else {
        const double fnr = __dmul_rn((double)nr, kInvTwoPi);
        const double c = __dsub_rn(__dmul_rn(fnr, d.phi0), shifted ? 0.5 : 0.0);
        const double fl = floor(c);
        ci = (int)fl;
        cf = (float)(c - fl);
    }
    const float fnr32 = (float)nr * 0.159154943091895336f;
    const float w = fnr32 * dphi;
    const float tau = fnr32 * ddphi + 2.4e-7f * w + 1.2e-7f * (1.0f + w) + 1e-6f;
    const float xlo = cf - w, xhi = cf + w;
    if (near_int_f(xlo, tau) || near_int_f(xhi, tau)) return false;
    ip_lo = ci + (int)floorf(xlo) + 1;
    ip_hi = ci + (int)floorf(xhi);
    return true;
}

// Stages ring `ring` as run(s) run[0], run[1]; returns its pixel count.
__device__ inline int make_runs(const DiscArgs &a, const DiscHdr &d, const Chord &ch, bool need_a2,
                                int ring, Run *run) {
    run[0].cnt = 0;
    run[1].cnt = 0;
    const int start = (int)ring_start(a.g, ring);
    const int nr = ring_npix(a.g, ring);
    const bool shifted = ring_shifted(a.g, ring);
    const double th = a.rt.theta[ring];
    const float sa = sinf(0.5f * (float)(th - d.theta0));
    const float A = sa * sa;
    float A2 = 0.0f;
    if (need_a2) {
        const float sb = sinf(0.5f * (float)(th + d.theta0 - kPi));
        A2 = sb * sb;
    }
    const float st32 = a.rt.st32[ring];
    const float B = st32 * ch.sth0;
    const float step32 = a.rt.step32[ring];
    const float steph = 0.5f * step32;
    int lo, cnt;
    float d0h;
    int ip_lo, ip_hi, ci;
    float cf;
    const bool chord = !(d.allsky || ring < d.irmin || ring > d.irmax);
    if (chord && ch.fast && chord_fast(a.g, d, ch, ring, nr, shifted, A, st32, ip_lo, ip_hi, ci, cf)) {
        if (ip_lo > ip_hi) return 0;
        // azimuth of pixel ip_lo relative to the particle: step (ip_lo - c),
        // in (-dphi, -dphi + step]
        d0h = 0.5f * fmaf(step32, (float)(ip_lo - ci), -step32 * cf);
        if (ip_hi >= nr) {
            ip_lo -= nr;
            ip_hi -= nr;
        }
        lo = ip_lo;
        cnt = ip_hi - ip_lo + 1;
        if (cnt > nr || lo < -nr || lo >= nr) return 0;  // cannot happen for finite input
    } else {
        ring_segment_t<true>(a.g, d, ring, lo, cnt);
        if (cnt <= 0) return 0;
        const double shift = shifted ? 0.5 : 0.0;
        // azimuth of the first pixel relative to the particle, in [-pi, pi)
        double d0 = ((double)lo + shift) * a.rt.step[ring] - d.phi0;
        if (d0 < -kPi) d0 += kTwoPi;
        if (d0 >= kPi) d0 -= kTwoPi;
        d0h = (float)(0.5 * d0);
    }
    // split where the in-ring index wraps (lo < 0 or lo + cnt > nr)
    int c0 = cnt, p0 = start + lo;
    if (lo < 0) {
        c0 = -lo;
        p0 = start + lo + nr;
    } else if (lo + cnt > nr) {
        c0 = nr - lo;
    }
    run[0] = Run{p0, c0, A, B, d0h, steph, A2, c0 < cnt};
    if (c0 < cnt) {
        // the rest continues at the ring's first pixel, azimuth continuing
        run[1] = Run{start, cnt - c0, A, B, fmaf((float)c0, steph, d0h), steph, A2, 0};
    }
    return cnt;
}

// sin x, |x| <= pi/2, Taylor to x^15 (scalar; the general path)
__device__ inline float sin_large(float x) {
    const float x2 = x * x;
    float p = fmaf(x2, -1.0f / 1307674368000.0f, 1.0f / 6227020800.0f);
    p = fmaf(x2, p, -1.0f / 39916800.0f);
    p = fmaf(x2, p, 1.0f / 362880.0f);
    p = fmaf(x2, p, -1.0f / 5040.0f);
    p = fmaf(x2, p, 1.0f / 120.0f);
    p = fmaf(x2, p, -1.0f / 6.0f);
    p = fmaf(x2, p, 1.0f);
    return x * p;
}

// theta^2 / 4 = asin^2(sqrt h) for pixels within 90 degrees of the particle
// (0 <= h <= 1/2), two at a time: h Q(h), Q a degree-8 polynomial fitted to
// asin^2(sqrt h) / h for relative error (least squares at 400 Chebyshev
// nodes of [0, 1/2] against a 40-digit asin, reweighted towards minimax):
// 1.2e-8 relative in exact arithmetic with the coefficients rounded to
// FP32, 1.2e-7 (two ulps) evaluated in FP32 (checked on a dense grid of
// [0, 1/2]) -- the accuracy of
// asinf(sqrtf(h)) squared, in nine packed FMAs instead of two scalar
// library calls per pixel.  Q(0) = 1 keeps g = h + h^2/3 + ... near 0.
__device__ __forceinline__ float2 g_near2(float2 h) {
    float2 q = fma2(h, f2(0.374805123f), f2(-0.423264921f));
    q = fma2(h, q, f2(0.331330061f));
    q = fma2(h, q, f2(-0.0322521478f));
    q = fma2(h, q, f2(0.0989379436f));
    q = fma2(h, q, f2(0.112454146f));
    q = fma2(h, q, f2(0.177871689f));
    q = fma2(h, q, f2(0.333331496f));
    q = fma2(h, q, f2(1.0f));
    return mul2(h, q);
}

// theta^2 / 4 beyond 90 degrees (h > 1/2), via the distance to the
// antipode (x -+ pi/2 is half the azimuth offset from it): asin(sqrt h)
// loses precision as h -> 1.
__device__ inline float g_far(float x, const Run &r) {
    const float sf = sin_large(x - copysignf(kHalfPiF, x));
    const float hf = fmaf(r.B, sf * sf, r.A2);
    const float t = kHalfPiF - asinf(sqrtf(fminf(fmaxf(hf, 0.0f), 1.0f)));
    return t * t;
}

// Weights of pixels jj = (j, j + 32) of run r; also sin(x) (x half the
// azimuth offset), the haversine h of the distance and g = theta^2 / 4.
// TX, TH >= 0 fix the polynomial tiers at compile time (the disc kernels
// dispatch on the particle's tiers once, outside the pixel loops); -1 reads
// them from e.
template <int TX = -1, int TH = -1>
__device__ __forceinline__ float2 weight2x(const Ext &e, const Run &r, float2 jj, float2 &sn_out,
                                          float2 &h_out, float2 &g_out) {
    const int tier_x = TX >= 0 ? TX : e.tier_x;
    const int tier_h = TH >= 0 ? TH : e.tier_h;
    const float2 x = fma2(jj, f2(r.steph), f2(r.d0h));
    const float2 x2 = mul2(x, x);
    float2 p;
    if (tier_x == 0) {
        p = fma2(x2, f2(-1.0f / 6.0f), f2(1.0f));
    } else if (tier_x == 1) {
        p = fma2(x2, f2(-1.0f / 5040.0f), f2(1.0f / 120.0f));
        p = fma2(x2, p, f2(-1.0f / 6.0f));
        p = fma2(x2, p, f2(1.0f));
    } else {
        p = fma2(x2, f2(-1.0f / 1307674368000.0f), f2(1.0f / 6227020800.0f));
        p = fma2(x2, p, f2(-1.0f / 39916800.0f));
        p = fma2(x2, p, f2(1.0f / 362880.0f));
        p = fma2(x2, p, f2(-1.0f / 5040.0f));
        p = fma2(x2, p, f2(1.0f / 120.0f));
        p = fma2(x2, p, f2(-1.0f / 6.0f));
        p = fma2(x2, p, f2(1.0f));
    }
    const float2 sn = mul2(x, p);
    const float2 h = fma2(f2(r.B), mul2(sn, sn), f2(r.A));
    float2 g;
    if (tier_h == 0) {
        float2 q = fma2(h, f2(8.0f / 45.0f), f2(1.0f / 3.0f));
        q = fma2(h, q, f2(1.0f));
        g = mul2(h, q);
    } else if (tier_h == 1) {
        float2 q = fma2(h, f2(128.0f / 1575.0f), f2(4.0f / 35.0f));
        q = fma2(h, q, f2(8.0f / 45.0f));
        q = fma2(h, q, f2(1.0f / 3.0f));
        q = fma2(h, q, f2(1.0f));
        g = mul2(h, q);
    } else {
        g = g_near2(make_float2(fmaxf(h.x, 0.0f), fmaxf(h.y, 0.0f)));
        if (h.x > 0.5f) g.x = g_far(x.x, r);
        if (h.y > 0.5f) g.y = g_far(x.y, r);
    }
    const float2 t = mul2(g, f2(e.nK));
    sn_out = sn;
    h_out = h;
    g_out = g;
    return make_float2(ex2_approx(t.x), ex2_approx(t.y));
}

// Weights only (the render passes).  For the small-disc tiers the
// haversine takes sin^2 x as one series in x^2 (sin^2 x = x^2 - x^4/3 +
// 2x^6/45 - x^8/315 + ..., from (1 - cos 2x)/2): to x^4 for tier 0 and to x^8
// for tier 1, truncation below 1.8e-8 resp. 2.1e-8 relative (|x| < 0.025, resp. 0.33), one
// operation fewer than sin x squared; and -K multiplies the asin^2 series'
// coefficients instead of its value.
template <int TX = -1, int TH = -1>
__device__ __forceinline__ float2 weight2(const Ext &e, const Run &r, float2 jj) {
    if constexpr (TX >= 0 && TH >= 0) {
        const float2 x = fma2(jj, f2(r.steph), f2(r.d0h));
        const float2 x2 = mul2(x, x);
        float2 q;
        if constexpr (TX == 0) {
            q = fma2(x2, f2(-1.0f / 3.0f), f2(1.0f));
        } else {
            q = fma2(x2, f2(-1.0f / 315.0f), f2(2.0f / 45.0f));
            q = fma2(x2, q, f2(-1.0f / 3.0f));
            q = fma2(x2, q, f2(1.0f));
        }
        const float2 h = fma2(f2(r.B), mul2(x2, q), f2(r.A));
        float2 t;
        if constexpr (TH == 0) {
            float2 u = fma2(h, f2(e.nK * (8.0f / 45.0f)), f2(e.nK * (1.0f / 3.0f)));
            u = fma2(h, u, f2(e.nK));
            t = mul2(h, u);
        } else {
            float2 u = fma2(h, f2(e.nK * (128.0f / 1575.0f)), f2(e.nK * (4.0f / 35.0f)));
            u = fma2(h, u, f2(e.nK * (8.0f / 45.0f)));
            u = fma2(h, u, f2(e.nK * (1.0f / 3.0f)));
            u = fma2(h, u, f2(e.nK));
            t = mul2(h, u);
        }
        return make_float2(ex2_approx(t.x), ex2_approx(t.y));
    } else {
        float2 sn, h, g;
        return weight2x<TX, TH>(e, r, jj, sn, h, g);
    }
}

// The double of a float f >= 0 from its bit pattern, with integer operations
// only (a cvt would run on the FP64 pipe, which GB300 has little of): the
// exponent is rebiased (127 -> 1023) and the mantissa shifted in.  Exact for
// normal f; a subnormal or zero f (below 2^-126) becomes a value in
// [2^-127, 2^-126), so callers do not pass zeros.  bias is f64_bias(sign):
// the exponent offset with the result's sign bit (u >> 3 stays below 2^28, so
// adding the bit sets it).
__host__ __device__ constexpr unsigned f64_bias(bool negative) {
    return (896u << 20) + (negative ? 0x80000000u : 0u);
}
__device__ __forceinline__ double f32_to_f64(float f, unsigned bias) {
    const unsigned u = __float_as_uint(f);
    return __hiloint2double((int)((u >> 3) + bias), (int)(u << 29));
}

// Calls f(integral_constant<TX>, integral_constant<TH>) with the particle's
// tiers as constants where both are below 2 (the common small discs), else
// with -1 (tiers read at run time): five instantiations of f instead of nine.
template <class F>
__device__ __forceinline__ void with_tiers(const Ext &e, F f) {
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using IR = std::integral_constant<int, -1>;
    if (e.tier_x < 2 && e.tier_h < 2) {
        if (e.tier_x == 0) {
            if (e.tier_h == 0) f(I0{}, I0{}); else f(I0{}, I1{});
        } else {
            if (e.tier_h == 0) f(I1{}, I0{}); else f(I1{}, I1{});
        }
    } else {
        f(IR{}, IR{});
    }
}

template <int G>
struct Grp {
    static constexpr int kWarps = G / 32;
    __device__ static void sync() {
        if (G == 32) __syncwarp(); else __syncthreads();
    }
    __device__ static int rank() { return G == 32 ? (threadIdx.x & 31) : (int)threadIdx.x; }
    __device__ static int warp() { return G == 32 ? 0 : (int)(threadIdx.x >> 5); }
};

// Stages rings r0 .. r0+n-1 as runs; returns the chunk's pixel count (all
// threads of the group).
// Per-ring terms of the adjoint's tangent vector (see adjc_particle).
struct AdjRing {
    float sr;    // sin(theta_r - theta0)
    float cr;    // 2 cos(theta0) sin(theta_r)
    float st2;   // 2 sin(theta_r)
};

template <int G, int RCH>
__device__ inline int build_runs(const DiscArgs &a, CompSmem<RCH> &sm, int r0, int n,
                                 AdjRing *aring = nullptr) {
    using Gp = Grp<G>;
    int c = 0;
    const bool need_a2 = sm.h.ext.tier_h == 2;
    for (int i = Gp::rank(); i < n; i += G) {
        c += make_runs(a, sm.h.hdr, sm.h.ch, need_a2, r0 + i, &sm.run[2 * i]);
        if (aring) {
            const float st = a.rt.st32[r0 + i];
            aring[i].sr = sinf((float)(a.rt.theta[r0 + i] - sm.h.hdr.theta0));
            aring[i].cr = 2.0f * (float)sm.h.hdr.z0 * st;
            aring[i].st2 = 2.0f * st;
        }
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if (G > 32) {
        if ((threadIdx.x & 31) == 0) sm.cnt_red[Gp::warp()] = c;
        Gp::sync();
        c = 0;
        for (int k = 0; k < Gp::kWarps; k++) c += sm.cnt_red[k];
    }
    Gp::sync();
    return c;
}

// Walks the staged rings; lane l handles pixels l and l + 32 of each
// 64-pixel stretch of a run.  body(run, ring, j, second) gets the ring's
// index in the chunk, the first pixel index j and whether j + 32 is inside
// the run.  In a block, warps claim whole
// rings (both run slots: the second only when the ring wrapped) from a shared
// counter reset by the caller; the next claim is issued before the current
// ring is walked, so its latency is hidden, and no warp waits at the next
// barrier for more than about one ring.
template <int G, int RCH, class Body>
__device__ inline void run_walk(CompSmem<RCH> &sm, int n, Body body) {
    const int lane = threadIdx.x & 31;
    auto ring = [&](int i) {
        const Run r = sm.run[2 * i];
        for (int j = lane; j < r.cnt; j += 64) body(r, i, j, j + 32 < r.cnt);
        if (r.more) {
            const Run r2 = sm.run[2 * i + 1];
            for (int j = lane; j < r2.cnt; j += 64) body(r2, i, j, j + 32 < r2.cnt);
        }
    };
    if (G == 32) {
        for (int i = 0; i < n; i++) ring(i);
        return;
    }
    int q = 0;
    if (lane == 0) q = atomicAdd(&sm.next_run, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    while (q < n) {
        int qn = 0;
        if (lane == 0) qn = atomicAdd(&sm.next_run, 1);
        ring(q);
        q = __shfl_sync(0xffffffffu, qn, 0);
    }
}

// The set-up of disc particle pidx: the FP64 geometry of query_disc and
// the run engine's per-particle constants.
__device__ inline void setup_hdr(const DiscArgs &a, int pidx, CompHdr &h) {
    disc_setup(a.g, a.theta[pidx], a.phi[pidx], a.ar[pidx], a.flux[pidx], a.cpix[pidx], pidx, h.hdr);
    particle_setup(a.g, h.hdr, h.ext, h.ch);
    const double fs = h.hdr.flux * a.f.inv_scale;
    h.ext.fs_hi = (float)fs;
    h.ext.fs_lo = (float)(fs - (double)h.ext.fs_hi);
    h.ext.rpi = 0;
}

// Stages the header of queue slot q in shared memory (all threads of the
// group call this, then synchronise): a copy of the precomputed header when
// the caller provided them (k_comp_hdr), else the set-up on one thread.
template <int G>
__device__ __forceinline__ void stage_hdr(const DiscArgs &a, long long q, CompHdr &dst) {
    constexpr int kWords = sizeof(CompHdr) / 8;
    static_assert(kWords <= G, "one word per thread");
    const int rk = Grp<G>::rank();
    if (a.chdr) {
        if (rk < kWords)
            reinterpret_cast<long long *>(&dst)[rk] =
                __ldg(reinterpret_cast<const long long *>(a.chdr + q) + rk);
    } else if (rk == 0) {
        setup_hdr(a, a.queue[q], dst);
    }
}

}  // namespace

}  // namespace dmann
