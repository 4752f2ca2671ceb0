// common.cuh -- device-side building blocks shared by the projection kernels.
//
// HEALPix RING geometry (FP64) restated from the published scheme (Gorski et
// al. 2005): the same formulas the reference reaches through HEALPix C++ at
// src/genmap.cpp:40,106,119,135.  Floating-point expressions that decide
// pixel membership are written with explicit round-to-nearest intrinsics so
// the compiler cannot contract them into FMAs: disc membership is then
// decided by exactly the arithmetic of the CPU path, whatever the fmad
// setting of the including translation unit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dmann {

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr double kHalfPi = 1.570796326794896619231321691639751442099;
constexpr double kInvHalfPi = 0.6366197723675813430755350534900574;
constexpr double kTwoPi = 6.283185307179586476925286766559005768394;
constexpr double kInvTwoPi = 0.1591549430918953357688837633725143620345;
constexpr double kTwoThird = 2.0 / 3.0;

// Observer frame and units of one render (src/parameters.h:17,
// src/datatypes.h:225, src/flux/flux_ann_nosom.cpp:13-16, genmap.cpp:52-58).
struct Frame {
    double rot[3][3];     // rotmatrix: v' = rot^T (pos - opos)
    double opos[3];
    double unit_factor;
    double hires_threshold;
    double inv_scale;     // power of two applied to fluxes deposited in FP32
    int flux_model;       // dmann_flux
    double vel_to_cgs;    // code velocity unit (somv, somv2, pwave laws)
    double fcpos[3];      // halo centre (adiabatic law)
};

// HEALPix constants of one Nside (src/datatypes.h:248-253 for dOmega).
struct Hpx {
    int nside, npix, ncap, nrings;  // nrings = 4*nside - 1
    double fact1, fact2;
    double dOmega, theta0;          // theta0 = acos(1 - dOmega/(2*3.141592))
};

// Per-ring tables (index 1..4*nside-1), built on the host with the same
// formulas as the oracle's pix2vec: z, the sin(theta) pix2vec uses, theta.
struct RingTab {
    const double *z;
    const double *st;
    const double *theta;
    const double *step;   // 2 pi / (pixels in the ring)
    const float *st32;    // st and step rounded to FP32 (the compensated form's
    const float *step32;  // per-ring set-up runs in FP32 where it can)
};

__host__ __device__ inline int64_t ring_start(const Hpx &g, int ring) {
    if (ring < g.nside) return 2LL * ring * (ring - 1);
    if (ring < 3 * g.nside) return (int64_t)g.ncap + (int64_t)(ring - g.nside) * 4 * g.nside;
    int64_t nr = 4LL * g.nside - ring;
    return (int64_t)g.npix - 2 * nr * (nr + 1);
}

__host__ __device__ inline int ring_npix(const Hpx &g, int ring) {
    if (ring < g.nside) return 4 * ring;
    if (ring < 3 * g.nside) return 4 * g.nside;
    return 4 * (4 * g.nside - ring);
}

__host__ __device__ inline bool ring_shifted(const Hpx &g, int ring) {
    if (ring < g.nside || ring >= 3 * g.nside) return true;
    return ((ring - g.nside) & 1) == 0;
}

// v1 mod v2 into [0, v2).
__device__ inline double fmodulo(double v1, double v2) {
    if (v1 >= 0) return (v1 < v2) ? v1 : fmod(v1, v2);
    double t = __dadd_rn(fmod(v1, v2), v2);
    return (t == v2) ? 0.0 : t;
}

__device__ inline double ring2z(const Hpx &g, int ring) {
    const int ns = g.nside;
    if (ring < ns) return __dsub_rn(1.0, __dmul_rn((double)((int64_t)ring * ring), g.fact2));
    if (ring <= 3 * ns) return __dmul_rn((double)(2 * ns - ring), g.fact1);
    int64_t r = 4 * ns - ring;
    return __dsub_rn(__dmul_rn((double)(r * r), g.fact2), 1.0);
}

__device__ inline int ring_above(const Hpx &g, double z) {
    double az = fabs(z);
    if (az <= kTwoThird)
        return (int)(int64_t)__dmul_rn((double)g.nside, __dsub_rn(2.0, __dmul_rn(1.5, z)));
    int iring = (int)(int64_t)__dmul_rn((double)g.nside,
                                        __dsqrt_rn(__dmul_rn(3.0, __dsub_rn(1.0, az))));
    return (z > 0) ? iring : 4 * g.nside - iring - 1;
}

// RING ang2pix; within 0.01 rad of a pole the cap index uses sin(theta)
// (the library's accurate form).
__device__ inline int ang2pix(const Hpx &g, double theta, double phi) {
    const int64_t ns = g.nside;
    bool have_sth = (theta < 0.01) || (theta > 3.14159 - 0.01);
    double z = cos(theta);
    double sth = have_sth ? sin(theta) : 0.0;
    double za = fabs(z);
    double tt = fmodulo(__dmul_rn(phi, kInvHalfPi), 4.0);
    if (za <= kTwoThird) {
        int64_t nl4 = 4 * ns;
        double temp1 = __dmul_rn((double)ns, __dadd_rn(0.5, tt));
        double temp2 = __dmul_rn(__dmul_rn((double)ns, z), 0.75);
        int64_t jp = (int64_t)__dsub_rn(temp1, temp2);
        int64_t jm = (int64_t)__dadd_rn(temp1, temp2);
        int64_t ir = ns + 1 + jp - jm;
        int64_t kshift = 1 - (ir & 1);
        int64_t t1 = jp + jm - ns + kshift + 1 + nl4 + nl4;
        int64_t ip = (t1 >> 1) % nl4;
        return (int)(g.ncap + (ir - 1) * nl4 + ip);
    }
    double tp = __dsub_rn(tt, (double)(int64_t)tt);
    double tmp = ((za < 0.99) || !have_sth)
                     ? __dmul_rn((double)ns, __dsqrt_rn(__dmul_rn(3.0, __dsub_rn(1.0, za))))
                     : __ddiv_rn(__dmul_rn((double)ns, sth),
                                 __dsqrt_rn(__ddiv_rn(__dadd_rn(1.0, za), 3.0)));
    int64_t jp = (int64_t)__dmul_rn(tp, tmp);
    int64_t jm = (int64_t)__dmul_rn(__dsub_rn(1.0, tp), tmp);
    int64_t ir = jp + jm + 1;
    int64_t ip = (int64_t)__dmul_rn(tt, (double)ir);
    if (ip >= 4 * ir) ip = 4 * ir - 1;
    return (int)((z > 0) ? 2 * ir * (ir - 1) + ip : (int64_t)g.npix - 2 * ir * (ir + 1) + ip);
}

// Per-particle disc description, computed once per particle and shared by
// the threads that render it.  Mirrors the set-up part of HEALPix
// query_disc (non-inclusive) called at src/genmap.cpp:119 with radius 2 ar.
struct DiscHdr {
    double theta0, phi0, ar, flux;
    double R, cosR, z0, xa, sth0;
    int cpix;
    int irmin, irmax;      // rings whose chord is computed
    int r_first, r_last;   // all rings touched (caps included)
    int allsky;
    int pidx;
};

__device__ inline void disc_setup(const Hpx &g, double theta, double phi, double ar,
                                  double flux, int cpix, int pidx, DiscHdr &d) {
    theta = fmodulo(theta, kTwoPi);  // pointing::normalize
    if (theta > kPi) { phi = __dadd_rn(phi, kPi); theta = __dsub_rn(kTwoPi, theta); }
    phi = fmodulo(phi, kTwoPi);
    d.theta0 = theta;
    d.phi0 = phi;
    d.ar = ar;
    d.flux = flux;
    d.cpix = cpix;
    d.pidx = pidx;
    d.R = __dmul_rn(2.0, ar);
    d.sth0 = sin(theta);
    d.z0 = cos(theta);
    d.allsky = d.R >= kPi;
    if (d.allsky) {
        d.cosR = -1.0;
        d.xa = 0.0;
        d.irmin = 1;
        d.irmax = 0;
        d.r_first = 1;
        d.r_last = g.nrings;
        return;
    }
    d.cosR = cos(d.R);
    d.xa = __ddiv_rn(1.0, __dsqrt_rn(__dmul_rn(__dsub_rn(1.0, d.z0), __dadd_rn(1.0, d.z0))));
    double rlat1 = __dsub_rn(theta, d.R);
    double zmax = cos(rlat1);
    d.irmin = ring_above(g, zmax) + 1;
    bool north = (rlat1 <= 0) && (d.irmin > 1);
    double rlat2 = __dadd_rn(theta, d.R);
    double zmin = cos(rlat2);
    d.irmax = ring_above(g, zmin);
    bool south = (rlat2 >= kPi) && (d.irmax + 1 < 4 * g.nside);
    d.r_first = max(1, north ? 1 : d.irmin);
    d.r_last = min(g.nrings, south ? g.nrings : d.irmax);
}

// Pixels of ring `ring` inside the disc: the half-open azimuth test of
// query_disc.  Returns cnt pixels starting at in-ring index lo (lo may be
// negative; indices wrap modulo nr).  Full rings (pole inside the disc, or
// the all-sky case) start at the pixel nearest phi0 - pi so that, walking
// forward, phi - phi0 stays in [-pi, pi).
// Fast variant of the chord test: the chord half-width dphi is computed in
// FP32 (atan2f on the FP64 x and y^2 the exact test forms).  Against the
// FP64 dphi it errs by at most 3.6e-7 dphi (atan2f, 3 ulp) + 3.8e-8 rad (x
// and sqrt(y^2) rounded to FP32) < 2e-6 rad, which moves the run's end
// points nr/2pi * (phi0 -+ dphi) - shift by less than tau = nr/2pi * 2e-6.
// Only when an end point lies within tau of an integer can its floor differ,
// and then the exact FP64 formula decides.  The pixel runs are therefore
// identical to the exact test's.
template <bool kFast>
__device__ inline void ring_segment_t(const Hpx &g, const DiscHdr &d, int ring, int &lo, int &cnt);

__device__ inline void ring_segment(const Hpx &g, const DiscHdr &d, int ring, int &lo,
                                    int &cnt) {
    ring_segment_t<false>(g, d, ring, lo, cnt);
}

__device__ inline bool near_integer(double a, double tau) {
    const double fr = a - floor(a);
    return fr < tau || fr > 1.0 - tau;
}

template <bool kFast>
__device__ inline void ring_segment_t(const Hpx &g, const DiscHdr &d, int ring, int &lo, int &cnt) {
    const int nr = ring_npix(g, ring);
    const double shift = ring_shifted(g, ring) ? 0.5 : 0.0;
    if (d.allsky || ring < d.irmin || ring > d.irmax) {
        double a = __dsub_rn(__dmul_rn(__dmul_rn((double)nr, kInvTwoPi), __dsub_rn(d.phi0, kPi)),
                             shift);
        lo = (int)ceil(a);
        cnt = nr;
        return;
    }
    double z = ring2z(g, ring);
    double x = __dmul_rn(__dsub_rn(d.cosR, __dmul_rn(z, d.z0)), d.xa);
    double ysq = __dsub_rn(__dsub_rn(1.0, __dmul_rn(z, z)), __dmul_rn(x, x));
    lo = 0;
    cnt = 0;
    if (ysq > 0) {
        const double fnr = __dmul_rn((double)nr, kInvTwoPi);
        double a_lo, a_hi;
        bool exact = !kFast;
        if (kFast) {
            const double dphif = (double)atan2f(sqrtf((float)ysq), (float)x);
            a_lo = __dsub_rn(__dmul_rn(fnr, __dsub_rn(d.phi0, dphif)), shift);
            a_hi = __dsub_rn(__dmul_rn(fnr, __dadd_rn(d.phi0, dphif)), shift);
            const double tau = fnr * 2.0e-6 + 1e-9;
            exact = near_integer(a_lo, tau) || near_integer(a_hi, tau);
        }
        if (exact) {
            const double dphi = atan2(__dsqrt_rn(ysq), x);
            a_lo = __dsub_rn(__dmul_rn(fnr, __dsub_rn(d.phi0, dphi)), shift);
            a_hi = __dsub_rn(__dmul_rn(fnr, __dadd_rn(d.phi0, dphi)), shift);
        }
        int ip_lo = (int)floor(a_lo) + 1;
        int ip_hi = (int)floor(a_hi);
        if (ip_lo <= ip_hi) {
            if (ip_hi >= nr) { ip_lo -= nr; ip_hi -= nr; }
            lo = ip_lo;
            cnt = ip_hi - ip_lo + 1;
        }
    }
    if (cnt < 0 || cnt > nr || lo < -nr || lo >= nr) {  // cannot happen for finite input
        lo = 0;
        cnt = 0;
    }
}

// Estimated number of disc pixels: cap area 4 pi sin^2(R/2) over dOmega.
__device__ inline double disc_npix_estimate(const Hpx &g, double ar) {
    if (2.0 * ar >= kPi) return (double)g.npix;
    double s = sin(ar);
    return (double)g.npix * s * s;
}

// ---------------------------------------------------------------- atomics
// The accumulation planes are only read after the kernel, so these carry no
// "memory" clobber: a clobber would make the compiler reload every loop-
// invariant value held in shared memory after each deposit.
__device__ inline void red_add_f64(double *addr, double v) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(addr), "d"(v));
}
__device__ inline void red_add_f32(float *addr, float v) {
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(v));
}
// Vector reductions (sm_90+): two or four consecutive floats, the address
// aligned to 8 or 16 bytes.
__device__ inline void red_add_v2_f32(float *addr, float a, float b) {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(a), "f"(b));
}
__device__ inline void red_add_v4_f32(float *addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c),
                 "f"(d));
}
__device__ inline float atom_add_f32(float *addr, float v) {
    float old;
    asm volatile("atom.global.add.f32 %0, [%1], %2;" : "=f"(old) : "l"(addr), "f"(v));
    return old;
}

// ---------------------------------------------------------------- reductions
__device__ inline double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ inline long long warp_sum_ll(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ inline int warp_excl_scan(int v, int &total) {
    const int lane = threadIdx.x & 31;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

}  // namespace dmann
