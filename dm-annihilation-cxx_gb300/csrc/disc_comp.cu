// disc_comp.cu -- the compensated-FP32 form of the disc kernels.
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
// captures every rounding error exactly), reduced in FP64.
// Deposits: two FP32 planes (hi, lo); the hi atomic returns the old value, so
// the exact TwoSum error of each addition -- plus the product's own rounding
// error and the low part of flux/norm -- goes to the lo plane.
//
// Work layout ("run engine"): the disc's rings are staged in shared memory
// as runs -- one ring's in-disc pixels, split where the ring wraps so that a
// run is contiguous in the map -- and each warp takes whole runs.  A lane
// evaluates two pixels of a run at once (j and j + 32) with the packed FP32x2
// instructions of sm_100+ (__ffma2_rn & co.), halving the issue slots of the
// polynomial, Kahan and TwoSum arithmetic.
//
// Polynomials (written from their Taylor series):
//   sin x = x - x^3/3! + x^5/5! - ... ; to x^7 for |x| < 0.35 (error
//   < 3e-10 relative), to x^15 for |x| <= pi/2 (error < 1e-11);
//   asin^2(sqrt h) = sum_n (4h)^n / (2 n^2 C(2n,n)) = h + h^2/3 + 8h^3/45 +
//   4h^4/35 + 128h^5/1575 + ... ; five terms for h < 0.02 (error < 3e-10
//   relative); otherwise asinf(sqrtf(h)) from the CUDA math library.
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
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

constexpr float kHalfPiF = 1.57079632679490f;

// One run: pixels pix0 .. pix0+cnt-1 of one ring, in order of increasing
// azimuth; x(j) = d0h + j*steph is half the azimuth offset of pixel j from
// the particle.
struct alignas(16) Run {
    int pix0, cnt;
    float A, B;         // hav(theta_r - theta0), sin(theta_r) sin(theta0)
    float d0h, steph;   // half azimuth offset of pixel 0, half the pixel step
    float A2, pad;      // hav(theta_r + theta0 - pi): distance to the antipode
};

struct Ext {
    float nK;           // -K
    int small_h, small_x;
};

template <int RCH>
struct CompSmem {
    Run run[2 * RCH];   // two runs per ring (the second only where it wraps)
    DiscHdr hdr;
    Ext ext;
    double red[32];
    int cnt_red[32];
    int next_run;       // runs claimed so far in the current pass (block groups)
};

__device__ inline void particle_setup(const DiscHdr &d, Ext &e) {
    e.nK = -(float)(4.0 * 1.4426950408889634 * 0.5 / (0.333 * d.ar * d.ar));
    double hmax = 1.0;
    if (!d.allsky) {
        const double s = sin(0.5 * d.R);
        hmax = s * s;
    }
    e.small_h = hmax < 0.02;
    const bool caps = d.allsky || d.r_first < d.irmin || d.r_last > d.irmax;
    int small_x = 0;
    if (!caps) {
        const double sr = sin(d.R);
        if (sr < 0.999 * d.sth0) small_x = (0.5 * asin(sr / d.sth0)) < 0.33;
    }
    e.small_x = small_x;
}

// Stages ring `ring` as run(s) run[0], run[1]; returns its pixel count.
__device__ inline int make_runs(const DiscArgs &a, const DiscHdr &d, int ring, Run *run) {
    int lo, cnt;
    ring_segment_t<true>(a.g, d, ring, lo, cnt);
    run[0].cnt = 0;
    run[1].cnt = 0;
    if (cnt <= 0) return 0;
    const int start = (int)ring_start(a.g, ring);
    const int nr = ring_npix(a.g, ring);
    const double shift = ring_shifted(a.g, ring) ? 0.5 : 0.0;
    const double step = a.rt.step[ring];
    const double th = a.rt.theta[ring];
    const float sa = sinf(0.5f * (float)(th - d.theta0));
    const float sb = sinf(0.5f * (float)(th + d.theta0 - kPi));
    const float A = sa * sa, A2 = sb * sb;
    const float B = (float)(a.rt.st[ring] * d.sth0);
    const float steph = (float)(0.5 * step);
    // azimuth of the first pixel relative to the particle, in [-pi, pi)
    double d0 = ((double)lo + shift) * step - d.phi0;
    if (d0 < -kPi) d0 += kTwoPi;
    if (d0 >= kPi) d0 -= kTwoPi;
    // split where the in-ring index wraps (lo < 0 or lo + cnt > nr)
    int c0 = cnt, p0 = start + lo;
    if (lo < 0) {
        c0 = -lo;
        p0 = start + lo + nr;
    } else if (lo + cnt > nr) {
        c0 = nr - lo;
    }
    run[0] = Run{p0, c0, A, B, (float)(0.5 * d0), steph, A2, 0.0f};
    if (c0 < cnt) {
        // the rest continues at the ring's first pixel, azimuth continuing
        run[1] = Run{start, cnt - c0, A, B, (float)(0.5 * (d0 + (double)c0 * step)), steph, A2, 0.0f};
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

// theta^2 / 4 for large discs: asin^2(sqrt h), or beyond 90 degrees via the
// distance to the antipode (x -+ pi/2 is half the azimuth offset from it).
__device__ inline float g_general(float h, float x, const Run &r) {
    float t;
    if (h <= 0.5f) {
        t = asinf(sqrtf(fmaxf(h, 0.0f)));
    } else {
        const float sf = sin_large(x - copysignf(kHalfPiF, x));
        const float hf = fmaf(r.B, sf * sf, r.A2);
        t = kHalfPiF - asinf(sqrtf(fminf(fmaxf(hf, 0.0f), 1.0f)));
    }
    return t * t;
}

// Weights of pixels jj = (j, j + 32) of run r.
__device__ __forceinline__ float2 weight2(const Ext &e, const Run &r, float2 jj) {
    const float2 x = fma2(jj, f2(r.steph), f2(r.d0h));
    const float2 x2 = mul2(x, x);
    float2 p;
    if (e.small_x) {
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
    if (e.small_h) {
        float2 q = fma2(h, f2(128.0f / 1575.0f), f2(4.0f / 35.0f));
        q = fma2(h, q, f2(8.0f / 45.0f));
        q = fma2(h, q, f2(1.0f / 3.0f));
        q = fma2(h, q, f2(1.0f));
        g = mul2(h, q);
    } else {
        g = make_float2(g_general(h.x, x.x, r), g_general(h.y, x.y, r));
    }
    const float2 t = mul2(g, f2(e.nK));
    return make_float2(ex2_approx(t.x), ex2_approx(t.y));
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
template <int G, int RCH>
__device__ inline int build_runs(const DiscArgs &a, CompSmem<RCH> &sm, int r0, int n) {
    using Gp = Grp<G>;
    int c = 0;
    for (int i = Gp::rank(); i < n; i += G) c += make_runs(a, sm.hdr, r0 + i, &sm.run[2 * i]);
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

// Walks the staged runs; lane l handles pixels l and l + 32 of each 64-pixel
// stretch of a run.  body(run, j, second) gets the first pixel index j and
// whether j + 32 is inside the run.  In a block, warps claim runs one at a
// time from a shared counter (reset by the caller), so no warp waits at the
// next barrier for more than about one run: ring runs differ a lot in length.
template <int G, int RCH, class Body>
__device__ inline void run_walk(CompSmem<RCH> &sm, int n, Body body) {
    const int lane = threadIdx.x & 31;
    if (G == 32) {
        for (int q = 0; q < 2 * n; q++) {
            const Run r = sm.run[q];
            for (int j = lane; j < r.cnt; j += 64) body(r, j, j + 32 < r.cnt);
        }
        return;
    }
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(&sm.next_run, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= 2 * n) break;
        const Run r = sm.run[q];
        for (int j = lane; j < r.cnt; j += 64) body(r, j, j + 32 < r.cnt);
    }
}

// Renders one particle with a group of G threads (a warp or a block).
template <int G, int RCH>
__device__ void render_particle(const DiscArgs &a, CompSmem<RCH> &sm, int pidx) {
    using Gp = Grp<G>;
    const int rk = Gp::rank();
    if (rk == 0) {
        disc_setup(a.g, a.theta[pidx], a.phi[pidx], a.ar[pidx], a.flux[pidx], a.cpix[pidx], pidx,
                   sm.hdr);
        particle_setup(sm.hdr, sm.ext);
    }
    Gp::sync();
    const Ext e = sm.ext;
    const int r_first = sm.hdr.r_first, r_last = sm.hdr.r_last;
    const int nring = r_last - r_first + 1;
    const int nchunk = nring > 0 ? (nring + RCH - 1) / RCH : 0;

    // pass 1: the normalisation, a compensated sum per lane (both halves).
    // The sums start at 1 and every weight is <= 1, so the running sum always
    // dominates the addend and Fast2Sum gives each step's rounding error
    // exactly; the errors are summed apart (not fed back into the next addend,
    // where Kahan's subtraction would round them away again).  The result is
    // independent of the order in which lanes meet the weights to ~1e-12.
    // The offset is removed in FP64.
    float2 ks = f2(1.0f), kc = f2(0.0f);
    long long total = 0;
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        total += build_runs<G, RCH>(a, sm, r0, n);
        if (G > 32) {
            if (rk == 0) sm.next_run = 0;
            Gp::sync();
        }
        run_walk<G, RCH>(sm, n, [&](const Run &r, int j, bool second) {
            const float jf = (float)j;
            float2 w = weight2(e, r, make_float2(jf, jf + 32.0f));
            if (!second) w.y = 0.0f;
            const float2 t = add2(ks, w);
            kc = add2(kc, sub2(w, sub2(t, ks)));
            ks = t;
        });
        Gp::sync();
    }
    double part = (((double)ks.x - 1.0) + (double)kc.x) + (((double)ks.y - 1.0) + (double)kc.y);
    part = warp_sum(part);
    double S = part;
    if (G > 32) {
        if ((rk & 31) == 0) sm.red[rk >> 5] = part;
        Gp::sync();
        S = 0.0;
        for (int k = 0; k < Gp::kWarps; k++) S += sm.red[k];
        Gp::sync();
    }
    if (total < 2) {  // genmap.cpp:125-128: the whole flux into the centre pixel
        if (rk == 0) {
            const double vs = sm.hdr.flux * a.f.inv_scale;
            const float vh = (float)vs;
            const float vl = (float)(vs - (double)vh);
            deposit2f(a.acc.hi, a.acc.lo, sm.hdr.cpix, vh);
            if (vl != 0.0f) red_add_f32(a.acc.lo + sm.hdr.cpix, vl);
            atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), 1ull);
        }
        Gp::sync();
        return;
    }
    if (rk == 0) atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), (unsigned long long)total);
    // flux / norm as a two-float
    const double Fd = sm.hdr.flux * a.f.inv_scale / S;
    const float F = (float)Fd, Flo = (float)(Fd - (double)F);
    float *const hi = a.acc.hi, *const lo = a.acc.lo;

    // pass 2: deposits.  w*F as hi + lo: the product's rounding error (exact,
    // from an FMA) and w*Flo go to the lo plane with the TwoSum error of the
    // hi atomic, so a particle's deposits add up to its flux to ~1e-12.
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        if (nchunk > 1) build_runs<G, RCH>(a, sm, r0, n);
        if (G > 32) {
            if (rk == 0) sm.next_run = 0;
            Gp::sync();
        }
        run_walk<G, RCH>(sm, n, [&](const Run &r, int j, bool second) {
            const float jf = (float)j;
            const float2 w = weight2(e, r, make_float2(jf, jf + 32.0f));
            const float2 p = mul2(w, f2(F));
            const float2 pe = fma2(w, f2(Flo), fma2(w, f2(F), make_float2(-p.x, -p.y)));
            const int pix = r.pix0 + j;
            const float a0 = atom_add_f32(hi + pix, p.x);
            const float a1 = second ? atom_add_f32(hi + pix + 32, p.y) : 0.0f;
            const float2 av = make_float2(a0, a1);
            const float2 pv = make_float2(p.x, second ? p.y : 0.0f);
            const float2 s = add2(av, pv);
            const float2 bb = sub2(s, av);
            float2 err = add2(sub2(av, sub2(s, bb)), sub2(pv, bb));
            err = add2(err, pe);
            red_add_f32(lo + pix, err.x);
            if (second) red_add_f32(lo + pix + 32, err.y);
        });
        Gp::sync();
    }
}

constexpr int kWPB = 8, kRCHW = 64;    // warp kernel

// One block per large disc, persistent over the block-class queue (largest
// discs first, claimed dynamically).  Block shapes: BT threads, runs of RCH
// rings staged per chunk, MINB resident blocks per SM -- every shape fills
// the SM with 2048 threads (the kernel is latency bound: returned atomics)
// and about 200 KB of staged runs.  The autotuner picks the shape.
template <int BT, int RCH, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_comp_block(DiscArgs a) {
    __shared__ CompSmem<RCH> sm;
    __shared__ int s_q;
    const long long nblk = a.ctr[C_ADD_BLOCK];
    for (;;) {
        if (threadIdx.x == 0) s_q = (int)atomicAdd((unsigned long long *)(a.ctr + C_QNEXT_BLOCK), 1ull);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= nblk) break;
        render_particle<BT, RCH>(a, sm, a.queue[q]);
    }
}

// One warp per small disc over the warp-class queue (after the block class).
__global__ void __launch_bounds__(kWPB * 32) k_comp_warp(DiscArgs a) {
    __shared__ CompSmem<kRCHW> sm[kWPB];
    const long long nblk = a.ctr[C_ADD_BLOCK];
    const long long ndisc = a.ctr[C_ADD_DISC];
    const int w = threadIdx.x >> 5;
    const long long gw = (long long)blockIdx.x * kWPB + w;
    const long long nw = (long long)gridDim.x * kWPB;
    for (long long q = nblk + gw; q < ndisc; q += nw) render_particle<32, kRCHW>(a, sm[w], a.queue[q]);
}

template <int BT, int RCH, int MINB>
cudaError_t launch_block(const DiscArgs &a, int num_sms, int blocks_per_sm, cudaStream_t s) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_comp_block<BT, RCH, MINB>, BT, 0);
    if (e != cudaSuccess) return e;
    int bps = blocks_per_sm > 0 ? min(blocks_per_sm, occ) : occ;
    if (bps < 1) bps = 1;
    k_comp_block<BT, RCH, MINB><<<num_sms * bps, BT, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_disc_comp(const DiscArgs &a, int num_sms, int blocks_per_sm, int block_threads,
                             cudaStream_t s, cudaEvent_t mid) {
    cudaError_t e;
    if (block_threads == 128) e = launch_block<128, 192, 16>(a, num_sms, blocks_per_sm, s);
    else if (block_threads == 512) e = launch_block<512, 640, 4>(a, num_sms, blocks_per_sm, s);
    else e = launch_block<256, 384, 8>(a, num_sms, blocks_per_sm, s);
    if (e != cudaSuccess) return e;
    if (mid && (e = cudaEventRecord(mid, s)) != cudaSuccess) return e;
    int occw = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_comp_warp, kWPB * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_comp_warp<<<num_sms * occw, kWPB * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dmann
