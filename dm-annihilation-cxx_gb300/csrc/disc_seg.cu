// disc_seg.cu -- the compensated-FP32 render of the block-class discs in
// work items and segments.
//
// Work items.  Each disc of the block class (queue slots [0, nblk), the
// largest discs) is cut into items of at most RCH rings (the block shape's
// staging capacity), fewer where its rings are long, so that an item holds
// about kItemPx pixels.  Items, not discs, are what the persistent blocks
// claim, so a disc of tens of millions of pixels is spread over many blocks
// instead of holding one block while the rest of the GPU idles.
//
// Pass 1 (k_seg_norm, all items) sums each item's weights; the sums of a
// disc's items meet in an FP64 total S per disc.  Pass 2 (k_seg_dep) reads
// S, forms F = flux / S and deposits w F for every pixel of the item.
// Because S is complete before any deposit, the two passes are two kernels
// and an item's runs are built twice.
//
// Per-pixel arithmetic.  For discs whose polynomial tiers are both below 2
// (the bulk: h < 0.02 and half azimuth offsets below 0.33 rad) the weight's
// exponent of 2 along a ring is one polynomial in y = x^2, x half the
// azimuth offset from the particle:
//     E(y) = nK G(A + B sin^2 x),  G(h) = asin^2(sqrt h) = sum_n a_n h^n,
// expanded in delta = B sin^2 x around the ring's A = hav(theta_r - theta0)
// with G_k = G^(k)(A)/k! and sin^2 x = y - y^2/3 + 2y^3/45 - y^4/315 + ...:
//     e0 = G0,  e1 = G1 B,  e2 = G2 B^2 - G1 B/3,
//     e3 = G3 B^3 - 2 G2 B^2/3 + 2 G1 B/45,
//     e4 = G4 B^4 - G3 B^3 + G2 B^2/5 - G1 B/315,
// truncated after y^4 (the next term of sin^2 x, 2y^5/14175, is below
// 1.4e-4 y^4 of the y term: under 2e-7 in E at the tier's bound x < 0.33).
// The builder of each ring computes nK e0..nK e4 once (FP32), and a pixel
// costs one FMA for x, one product for y, four FMAs of Horner and an ex2.
// The weights agree with the per-pixel series of comp_engine.cuh to FP32
// rounding (both take A and B rounded once to FP32).  Other discs take the
// general per-pixel path of comp_engine.cuh (weight2 with run-time tiers).
//
// Normalisation sums.  Each lane sums its pixels of a ring in plain FP32
// (at most kFoldPairs pixel pairs at a time for the large discs, whose
// rings can hold the whole ring of the map) and adds that partial into a
// two-float (s, c) with Knuth's TwoSum, so every rounding of the additions
// across partials is kept; the item's lanes are reduced as two-floats.
//
// Deposits and segments.  A deposit w (F + Flo) is rounded once to FP32 and
// added with red.global.add.f32 into an FP32 plane: half the L2 reduction
// bytes of an FP64 deposit.  The deposits of a chunk are made in segments;
// after each, k_seg_flush adds the FP32 plane into the FP64 plane and clears
// it.  Two bounds on a segment keep its FP32 sums accurate:
//   * Range.  The particles' deposit scales F span many decades, and a
//     round-to-nearest FP32 sum drops any addend below half an ulp of its
//     running total: small deposits landing on large totals would be lost,
//     a bias that is always downwards.  After pass 1 the items are sorted by
//     the octave of F (a counting sort, k_seg_class .. k_seg_sort); a segment
//     holds items of at most kClassSpan consecutive octaves, so its smallest
//     addend (w >= exp(-6) times its smallest F) stays above 2^-kClassSpan
//     e^-6 / n of a pixel total of n additions -- many ulps for n in the
//     hundreds, whatever order the concurrent blocks deposit in.
//   * Length.  A segment holds about kDepPerPix deposits per pixel (an
//     octave with more is dealt round robin into several segments), so a
//     pixel's FP32 partial sums stay short and their rounding errors random.
// The plan is made on the device from the per-octave histograms
// (k_seg_plan, running plan_segments of seg_plan.h), and every kernel of the
// sequence reads the chunk's mode
// (k_seg_decide) and returns at once when it has nothing to do, so the
// whole render is one stream of launches with no host synchronisation.
// Chunks too small for the L2 reduction rate to matter (a tunable threshold
// on the estimated deposits), or with more work items than the item buffers
// hold, take the per-disc kernels with FP64 deposits instead.
#include "comp_engine.cuh"

namespace dmann {

namespace {

constexpr int kItemPx = 32768;   // pixels per work item (from the disc's cap-area estimate)

// One staged run: a ring's pixels inside the disc, contiguous in the map.
struct alignas(16) SRun {
    int pix0, cnt;
    float d0h, steph;       // x(j) = d0h + j steph, half the azimuth offset of pixel j
    float c0, c1, c2, c3;   // polynomial path: E = c0 + y (c1 + y (c2 + y (c3 + y c4)));
    float c4;               // general path: c0 = A, c1 = B, c2 = A2 (see Run)
    int more;               // the ring continues in the next slot (it wrapped)
    float pad0, pad1;
};
static_assert(sizeof(SRun) == 48, "SRun is copied as three 16-byte words");

template <int RCH>
struct SegSmem {
    SRun run[2 * RCH];      // two slots per ring (the second only where it wraps)
    CompHdr h;
    float2 red2[32];        // per-warp two-float sums
    int cnt_red[32];
    double F;               // flux * inv_scale / S (pass 2)
    int next_run;           // rings claimed so far (dynamic claims of the walk)
    int item;               // the claimed item
};

// nK e0 .. nK e4 of the exponent polynomial for a ring (A, B) of a disc with
// tier_h th (three terms of G for th 0, five for th 1).
__device__ inline void poly_coeffs(float A, float B, float nK, int th, float c[5]) {
    const float a4 = th ? 4.0f / 35.0f : 0.0f, a5 = th ? 128.0f / 1575.0f : 0.0f;
    // G_k = sum_n C(n, k) a_n A^(n-k)
    const float G0 = fmaf(A, A * fmaf(A, fmaf(A, fmaf(A, a5, a4), 8.0f / 45.0f), 1.0f / 3.0f), A);
    const float G1 = fmaf(A, fmaf(A, fmaf(A, fmaf(A, 5.0f * a5, 4.0f * a4), 24.0f / 45.0f), 2.0f / 3.0f), 1.0f);
    const float G2 = fmaf(A, fmaf(A, fmaf(A, 10.0f * a5, 6.0f * a4), 24.0f / 45.0f), 1.0f / 3.0f);
    const float G3 = fmaf(A, fmaf(A, 10.0f * a5, 4.0f * a4), 8.0f / 45.0f);
    const float G4 = fmaf(A, 5.0f * a5, a4);
    const float B2 = B * B, B3 = B2 * B, B4 = B2 * B2;
    const float g1 = G1 * B, g2 = G2 * B2, g3 = G3 * B3;
    c[0] = nK * G0;
    c[1] = nK * g1;
    c[2] = nK * fmaf(g1, -1.0f / 3.0f, g2);
    c[3] = nK * fmaf(g2, -2.0f / 3.0f, fmaf(g1, 2.0f / 45.0f, g3));
    c[4] = nK * fmaf(G4, B4, fmaf(g2, 0.2f, fmaf(g1, -1.0f / 315.0f, -g3)));
}

template <int BT>
struct Blk {
    static constexpr int kWarps = BT / 32;
};

// Stages rings r0 .. r0+n-1 of the staged particle as runs (one thread per
// ring); returns the pixel count of those rings (all threads).
template <int BT, int RCH>
__device__ inline int seg_build(const DiscArgs &a, SegSmem<RCH> &sm, int r0, int n, bool poly) {
    int c = 0;
    const bool need_a2 = sm.h.ext.tier_h == 2;
    for (int i = threadIdx.x; i < n; i += BT) {
        Run r[2] = {};
        const int k = make_runs(a, sm.h.hdr, sm.h.ch, need_a2, r0 + i, r);
        c += k;
        float co[5] = {r[0].A, r[0].B, r[0].A2, 0.0f, 0.0f};
        if (poly && k > 0) poly_coeffs(r[0].A, r[0].B, sm.h.ext.nK, sm.h.ext.tier_h, co);
#pragma unroll
        for (int s = 0; s < 2; s++) {
            SRun o;
            o.pix0 = r[s].pix0;
            o.cnt = r[s].cnt;
            o.d0h = r[s].d0h;
            o.steph = r[s].steph;
            o.c0 = co[0];
            o.c1 = co[1];
            o.c2 = co[2];
            o.c3 = co[3];
            o.c4 = co[4];
            o.more = r[s].more;
            o.pad0 = o.pad1 = 0.0f;
            sm.run[2 * i + s] = o;
        }
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) sm.cnt_red[threadIdx.x >> 5] = c;
    if (threadIdx.x == 0) sm.next_run = 0;
    __syncthreads();
    c = 0;
    for (int k = 0; k < Blk<BT>::kWarps; k++) c += sm.cnt_red[k];
    return c;
}

// The weights of pixels jj = (j, j + S) of run r.
template <bool POLY>
__device__ __forceinline__ float2 seg_weight2(const Ext &e, const SRun &r, float2 jj) {
    if constexpr (POLY) {
        const float2 x = fma2(jj, f2(r.steph), f2(r.d0h));
        const float2 y = mul2(x, x);
        float2 t = fma2(y, f2(r.c4), f2(r.c3));
        t = fma2(y, t, f2(r.c2));
        t = fma2(y, t, f2(r.c1));
        t = fma2(y, t, f2(r.c0));
        return make_float2(ex2_approx(t.x), ex2_approx(t.y));
    } else {
        Run g;
        g.pix0 = r.pix0;
        g.cnt = r.cnt;
        g.A = r.c0;
        g.B = r.c1;
        g.d0h = r.d0h;
        g.steph = r.steph;
        g.A2 = r.c2;
        g.more = 0;
        return weight2<-1, -1>(e, g, jj);
    }
}

// Warps claim 32 / S consecutive rings (both slots of each) of the staged
// item at a time, one ring per group of S lanes, and call
// body(run, j, S, second) for pixels j and j + S of the ring (second: j + S
// is inside), so the per-ring work of the walk (the claim, the run's loads,
// the loop set-up, ring_done) is shared by the rings a warp walks together;
// neighbouring rings of a disc have similar lengths, so the groups finish
// together.  The S lanes of a group touch S consecutive pixels (S floats of
// the map per deposit instruction).  ring_done() runs on every lane after
// each claim.
template <int RCH, int S, class Body, class Done>
__device__ inline void seg_walk(SegSmem<RCH> &sm, int n, Body body, Done ring_done) {
    static_assert(S == 2 || S == 4 || S == 8 || S == 16 || S == 32, "lanes per ring");
    constexpr int G = 32 / S;
    const int lane = threadIdx.x & 31, sl = lane % S;
    int q0 = 0;
    if (lane == 0) q0 = atomicAdd(&sm.next_run, G);
    q0 = __shfl_sync(0xffffffffu, q0, 0);
    while (q0 < n) {
        int qn = 0;
        if (lane == 0) qn = atomicAdd(&sm.next_run, G);
        const int q = q0 + lane / S;
        if (q < n) {
            const SRun r = sm.run[2 * q];
            for (int j = sl; j < r.cnt; j += 2 * S) body(r, j, S, j + S < r.cnt);
            if (r.more) {
                const SRun r2 = sm.run[2 * q + 1];
                for (int j = sl; j < r2.cnt; j += 2 * S) body(r2, j, S, j + S < r2.cnt);
            }
        }
        ring_done();
        q0 = __shfl_sync(0xffffffffu, qn, 0);
    }
}

// The whole block on one ring at a time (items of a few long rings: the
// discs of hundreds of degrees): thread t takes pixels t, t + BT of every
// 2 BT; body(run, j, BT, second) as in seg_walk, ring_done() after each ring.
template <int BT, int RCH, class Body, class Done>
__device__ inline void seg_walk_block(SegSmem<RCH> &sm, int n, Body body, Done ring_done) {
    for (int q = 0; q < n; q++) {
        const SRun r = sm.run[2 * q];
        for (int j = threadIdx.x; j < r.cnt; j += 2 * BT) body(r, j, BT, j + BT < r.cnt);
        if (r.more) {
            const SRun r2 = sm.run[2 * q + 1];
            for (int j = threadIdx.x; j < r2.cnt; j += 2 * BT) body(r2, j, BT, j + BT < r2.cnt);
        }
        ring_done();
    }
}

// The walk for an item of n rings: S lanes per ring, the smallest of
// S0 .. 32 that keeps every lane group of the block on a ring (n >= BT / S),
// else the whole block on each ring in turn.
template <int BT, int RCH, int S0, class Body, class Done>
__device__ inline void seg_walk_any(SegSmem<RCH> &sm, int n, Body body, Done ring_done) {
    if (S0 <= 2 && n >= BT / 2) seg_walk<RCH, 2>(sm, n, body, ring_done);
    else if (S0 <= 4 && n >= BT / 4) seg_walk<RCH, 4>(sm, n, body, ring_done);
    else if (S0 <= 8 && n >= BT / 8) seg_walk<RCH, 8>(sm, n, body, ring_done);
    else if (S0 <= 16 && n >= BT / 16) seg_walk<RCH, 16>(sm, n, body, ring_done);
    else if (n >= BT / 32) seg_walk<RCH, 32>(sm, n, body, ring_done);
    else seg_walk_block<BT, RCH>(sm, n, body, ring_done);
}

// Lanes per ring.  Pass 1 (weights only) walks sixteen rings per warp:
// measured on the 16M workload at Nside 2048, 2 / 4 / 8 / 16 / 32 lanes per
// ring took 413 / 418 / 460 / 519 / 627 ms.  Pass 2 keeps whole warps on a ring, so a warp's
// reduction covers 32 consecutive floats: 16 lanes per ring, or eight lanes
// on aligned 32-byte sectors, measured slower (760 and 826 ms against 753).
constexpr int kNormLanes = 2;
constexpr int kDepLanes = 32;
constexpr int kFoldPairs = 8;    // pass 1, large discs: pixel pairs per plain FP32 partial

// Claims the next work item for the block (thread 0: first + t stride for
// the t-th claim, below end) and stages its disc's header; false when the
// item range is exhausted.  Callers return at once unless the chunk is
// segmented (sg.ctl[0]), so the item counts are within the buffers.
template <int BT, int RCH>
__device__ inline bool seg_claim(const DiscArgs &a, const SegArgs &sg, const int2 *items,
                                 SegSmem<RCH> &sm, unsigned long long *next, long long stride,
                                 long long first, long long end, int2 &it) {
    if (threadIdx.x == 0) {
        const long long t = (long long)atomicAdd(next, 1ull);
        const long long k = first + t * stride;
        sm.item = k < end ? (int)k : -1;
    }
    __syncthreads();
    const int k = sm.item;
    if (k < 0) return false;
    it = items[k];
    constexpr int kWords = sizeof(CompHdr) / 8;
    static_assert(kWords <= BT, "one header word per thread");
    if (threadIdx.x < kWords)
        reinterpret_cast<long long *>(&sm.h)[threadIdx.x] =
            __ldg(reinterpret_cast<const long long *>(a.chdr + it.x) + threadIdx.x);
    __syncthreads();
    return true;
}

// The item's ring range.
__device__ inline void item_rings(const CompHdr &h, int i, int &r0, int &n) {
    r0 = h.hdr.r_first + i * h.ext.rpi;
    n = min(h.ext.rpi, h.hdr.r_last - r0 + 1);
}

// Pass 1 of one item: the weight sum as a two-float (every thread of the
// block returns it) and the item's pixel count.
template <int BT, int RCH, bool POLY>
__device__ inline void norm_item(const DiscArgs &a, SegSmem<RCH> &sm, int r0, int n, float &S_hi,
                                 float &S_lo, int &total) {
    const Ext e = sm.h.ext;
    total = seg_build<BT, RCH>(a, sm, r0, n, POLY);
    float s = 0.0f, c = 0.0f;   // this lane's two-float sum of its partials
    float2 part = f2(0.0f);     // plain FP32 partial of at most kFoldPairs pixel pairs
    int np = 0;
    auto fold = [&]() {
        float err;
        s = two_sum(s, part.x + part.y, err);
        c += err;
        part = f2(0.0f);
        np = 0;
    };
    seg_walk_any<BT, RCH, kNormLanes>(
        sm, n,
        [&](const SRun &r, int j, int off, bool second) {
            const float jf = (float)j;
            float2 w = seg_weight2<POLY>(e, r, make_float2(jf, jf + (float)off));
            if (!second) w.y = 0.0f;
            part = add2(part, w);
            // the large discs' rings are long (up to the whole ring): keep the
            // plain partials short; the polynomial path's rings are short enough
            if constexpr (!POLY)
                if (++np == kFoldPairs) fold();
        },
        fold);
    warp_sum_ff(s, c);
    if ((threadIdx.x & 31) == 0) sm.red2[threadIdx.x >> 5] = make_float2(s, c);
    __syncthreads();
    S_hi = sm.red2[0].x;
    S_lo = sm.red2[0].y;
    for (int k = 1; k < Blk<BT>::kWarps; k++) {
        float err;
        S_hi = two_sum(S_hi, sm.red2[k].x, err);
        S_lo = (S_lo + sm.red2[k].y) + err;
    }
}

template <int BT, int RCH, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_seg_norm(DiscArgs a, SegArgs sg) {
    if (sg.ctl[0] == 0) return;
    __shared__ SegSmem<RCH> sm;
    int2 it;
    const long long n_items = a.ctr[C_SEG_ITEMS];
    while (seg_claim<BT, RCH>(a, sg, sg.items, sm, (unsigned long long *)(a.ctr + C_SEG_NEXT_NORM), 1, 0,
                              n_items, it)) {
        int r0, n;
        item_rings(sm.h, it.y, r0, n);
        const bool poly = sm.h.ext.tier_x < 2 && sm.h.ext.tier_h < 2;
        float S_hi, S_lo;
        int total;
        if (poly) norm_item<BT, RCH, true>(a, sm, r0, n, S_hi, S_lo, total);
        else norm_item<BT, RCH, false>(a, sm, r0, n, S_hi, S_lo, total);
        if (threadIdx.x == 0) {
            atomicAdd(sg.disc_S + it.x, (double)S_hi + (double)S_lo);
            atomicAdd((unsigned long long *)(sg.disc_px + it.x), (unsigned long long)total);
            atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), (unsigned long long)total);
        }
        __syncthreads();
    }
}

template <int BT, int RCH, bool POLY>
__device__ inline void dep_item(const DiscArgs &a, SegSmem<RCH> &sm, int r0, int n, float F, float Flo,
                                float *plane) {
    const Ext e = sm.h.ext;
    seg_build<BT, RCH>(a, sm, r0, n, POLY);
    seg_walk_any<BT, RCH, kDepLanes>(
        sm, n,
        [&](const SRun &r, int j, int off, bool second) {
            const float jf = (float)j;
            const float2 w = seg_weight2<POLY>(e, r, make_float2(jf, jf + (float)off));
            const float2 p = fma2(w, f2(F), mul2(w, f2(Flo)));   // w (F + Flo), rounded once
            float *const m = plane + (r.pix0 + j);
            red_add_f32(m, p.x);
            if (second) red_add_f32(m + off, p.y);
        },
        []() {});
    __syncthreads();
}

// Segment seg of the plan: its items of the sorted list (see SegSpan);
// returns at once when the plan has fewer segments.
template <int BT, int RCH, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_seg_dep(DiscArgs a, SegArgs sg, int seg) {
    if (sg.ctl[0] == 0 || seg >= sg.ctl[1]) return;
    __shared__ SegSmem<RCH> sm;
    const SegSpan sp = sg.spans[seg];
    int2 it;
    while (seg_claim<BT, RCH>(a, sg, sg.sorted, sm, sg.seg_next + seg, sp.stride, sp.lo + sp.offset,
                              sp.hi, it)) {
        const long long total = sg.disc_px[it.x];
        const double fs = sm.h.hdr.flux * a.f.inv_scale;
        if (total < 2) {   // genmap.cpp:125-128: the whole flux into the centre pixel
            if (threadIdx.x == 0 && it.y == 0) {
                red_add_f64(a.acc.acc64 + sm.h.hdr.cpix, fs);
                atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), (unsigned long long)(1 - total));
            }
            __syncthreads();
            continue;
        }
        if (threadIdx.x == 0) sm.F = fs / sg.disc_S[it.x];
        __syncthreads();
        const double Fd = sm.F;
        const float F = (float)Fd, Flo = (float)(Fd - (double)F);
        if (F == 0.0f) {   // zero flux deposits nothing (weights are >= exp(-6))
            __syncthreads();
            continue;
        }
        int r0, n;
        item_rings(sm.h, it.y, r0, n);
        if (sm.h.ext.tier_x < 2 && sm.h.ext.tier_h < 2) dep_item<BT, RCH, true>(a, sm, r0, n, F, Flo, sg.plane);
        else dep_item<BT, RCH, false>(a, sm, r0, n, F, Flo, sg.plane);
    }
}

// Items of each block-class disc: ring chunking from the cap-area estimate,
// the item count and its first item (claimed from C_SEG_ITEMS), and the
// estimated deposits (for the chunk's mode); clears the disc's pass-1 sums.
template <int RCH>
__global__ void __launch_bounds__(256) k_seg_count(DiscArgs a, SegArgs sg) {
    const long long nblk = a.ctr[C_ADD_BLOCK];
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    long long est_sum = 0;
    // warp-uniform trips: the warp claims its 32 discs' items with one atomic
    for (long long q0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); q0 < nblk; q0 += stride) {
        const long long q = q0 + lane;
        int nit = 0;
        if (q < nblk) {
            CompHdr &h = a.chdr[q];
            const int nring = max(1, h.hdr.r_last - h.hdr.r_first + 1);
            const double est = disc_npix_estimate(a.g, h.hdr.ar);
            const double per_ring = est / nring;
            int rpi = per_ring > 0.0 ? (int)min((double)RCH, (double)kItemPx / per_ring) : RCH;
            rpi = max(1, min(RCH, rpi));
            nit = (nring + rpi - 1) / rpi;
            h.ext.rpi = rpi;
            sg.disc_S[q] = 0.0;
            sg.disc_px[q] = 0;
            est_sum += (long long)est;
        }
        int tot;
        const int ex = warp_excl_scan(nit, tot);
        unsigned long long base = 0;
        if (lane == 0 && tot > 0)
            base = atomicAdd((unsigned long long *)(a.ctr + C_SEG_ITEMS), (unsigned long long)tot);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (q < nblk) {
            sg.disc_first[q] = (long long)base + ex;
            sg.disc_nitems[q] = nit;
        }
    }
    est_sum = warp_sum_ll(est_sum);
    if (lane == 0 && est_sum)
        atomicAdd((unsigned long long *)(a.ctr + C_SEG_EST), (unsigned long long)est_sum);
}

// The chunk's mode: segmented when its estimated deposits reach min_est and
// its items fit the item buffers (else the per-disc kernels deposit in FP64).
__global__ void k_seg_decide(DiscArgs a, SegArgs sg) {
    const long long items = a.ctr[C_SEG_ITEMS], est = a.ctr[C_SEG_EST];
    const int mode = (items > 0 && items <= sg.cap && est >= sg.min_est) ? 1 : 0;
    sg.ctl[0] = mode;
    a.ctr[C_SEG_MODE] = mode;
}

__global__ void __launch_bounds__(256) k_seg_fill(DiscArgs a, SegArgs sg) {
    if (sg.ctl[0] == 0) return;
    const long long nblk = a.ctr[C_ADD_BLOCK];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nblk; q += stride) {
        const long long f = sg.disc_first[q];
        const int nit = sg.disc_nitems[q];
        for (int i = 0; i < nit; i++) sg.items[f + i] = make_int2((int)q, i);
    }
}

// The item sort's key of block-class disc q: the octave of its deposit
// scale F = flux * inv_scale / S (class 0 for discs that deposit no
// weighted pixels: fewer than two pixels, or zero flux).
__device__ inline int seg_class(const DiscArgs &a, const SegArgs &sg, long long q) {
    const double S = sg.disc_S[q];
    const double F = a.chdr[q].hdr.flux * a.f.inv_scale / S;
    if (sg.disc_px[q] < 2 || !(F > 0.0) || !isfinite(F)) return 0;
    return min(kClasses - 1, max(1, ilogb(F) + kClasses / 2));
}

// Items and pixels per class (sg.cls[0 .. kClasses), sg.cls_px).
__global__ void __launch_bounds__(256) k_seg_class(DiscArgs a, SegArgs sg) {
    if (sg.ctl[0] == 0) return;
    __shared__ int hist[kClasses];
    __shared__ unsigned long long px[kClasses];
    for (int i = threadIdx.x; i < kClasses; i += blockDim.x) {
        hist[i] = 0;
        px[i] = 0;
    }
    __syncthreads();
    const long long nblk = a.ctr[C_ADD_BLOCK];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nblk; q += stride) {
        const int c = seg_class(a, sg, q);
        atomicAdd(&hist[c], sg.disc_nitems[q]);
        atomicAdd(&px[c], (unsigned long long)sg.disc_px[q]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kClasses; i += blockDim.x) {
        if (hist[i]) atomicAdd(sg.cls + i, hist[i]);
        if (px[i]) atomicAdd((unsigned long long *)sg.cls_px + i, px[i]);
    }
}

// Exclusive scan of the class histogram into the classes' first slots
// (sg.cls[kClasses .. 2 kClasses)); one block of kClasses threads.
__global__ void __launch_bounds__(kClasses) k_seg_cscan(SegArgs sg) {
    if (sg.ctl[0] == 0) return;
    int total;
    const int v = sg.cls[threadIdx.x];
    const int ex = warp_excl_scan(v, total);
    __shared__ int wsum[kClasses / 32];
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = total;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < (int)(threadIdx.x >> 5); w++) base += wsum[w];
    sg.cls[kClasses + threadIdx.x] = base + ex;
}

// Each disc's items into its class's range of the sorted list.
__global__ void __launch_bounds__(256) k_seg_sort(DiscArgs a, SegArgs sg) {
    if (sg.ctl[0] == 0) return;
    const long long nblk = a.ctr[C_ADD_BLOCK];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nblk; q += stride) {
        const int nit = sg.disc_nitems[q];
        const long long f = atomicAdd(sg.cls + kClasses + seg_class(a, sg, q), nit);
        for (int i = 0; i < nit; i++) sg.sorted[f + i] = make_int2((int)q, i);
    }
}

// The segment plan (plan_segments in seg_plan.h), one thread.
__global__ void k_seg_plan(SegArgs sg) {
    if (sg.ctl[0] == 0) return;
    sg.ctl[1] = plan_segments(sg.cls, sg.cls + kClasses, sg.cls_px, sg.budget, sg.spans);
}

// After segment seg: acc64 += plane, plane = 0 (four pixels per thread;
// npix is a multiple of 4); returns at once when the plan has no segment seg.
__global__ void __launch_bounds__(256) k_seg_flush(const int *ctl, int seg, float *plane, double *acc,
                                                   long long npix4) {
    if (ctl[0] == 0 || seg >= ctl[1]) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npix4; i += stride) {
        const float4 v = reinterpret_cast<float4 *>(plane)[i];
        if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f) {
            double2 *d = reinterpret_cast<double2 *>(acc) + 2 * i;
            double2 lo = d[0], hi = d[1];
            lo.x += v.x;
            lo.y += v.y;
            hi.x += v.z;
            hi.y += v.w;
            d[0] = lo;
            d[1] = hi;
            reinterpret_cast<float4 *>(plane)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

template <int BT, int RCH, int MINB>
int grid_of(int num_sms, int blocks_per_sm) {
    static const int occ = [] {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_seg_norm<BT, RCH, MINB>, BT, 0) != cudaSuccess) {
            cudaGetLastError();
            o = 1;
        }
        return o;
    }();
    const int bps = blocks_per_sm > 0 ? min(blocks_per_sm, occ) : occ;
    return num_sms * (bps < 1 ? 1 : bps);
}

template <int BT, int RCH, int MINB>
cudaError_t launch_norm(const DiscArgs &a, const SegArgs &sg, int num_sms, int blocks_per_sm, cudaStream_t s) {
    k_seg_fill<<<num_sms * 8, 256, 0, s>>>(a, sg);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_seg_norm<BT, RCH, MINB><<<grid_of<BT, RCH, MINB>(num_sms, blocks_per_sm), BT, 0, s>>>(a, sg);
    return cudaGetLastError();
}

template <int BT, int RCH, int MINB>
cudaError_t launch_deposits(const DiscArgs &a, const SegArgs &sg, int num_sms, int blocks_per_sm, int npix,
                            cudaStream_t s) {
    const int grid = grid_of<BT, RCH, MINB>(num_sms, blocks_per_sm);
    for (int k = 0; k < kSegSlots; k++) {
        k_seg_dep<BT, RCH, MINB><<<grid, BT, 0, s>>>(a, sg, k);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_seg_flush<<<num_sms * 8, 256, 0, s>>>(sg.ctl, k, sg.plane, a.acc.acc64, npix / 4);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_seg_count(const DiscArgs &a, const SegArgs &sg, int block_threads, int num_sms,
                             cudaStream_t s) {
    if (block_threads == 256) k_seg_count<256><<<num_sms * 8, 256, 0, s>>>(a, sg);
    else k_seg_count<128><<<num_sms * 8, 256, 0, s>>>(a, sg);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_seg_decide<<<1, 1, 0, s>>>(a, sg);
    return cudaGetLastError();
}

cudaError_t launch_seg_norm(const DiscArgs &a, const SegArgs &sg, int block_threads, int num_sms,
                            int blocks_per_sm, cudaStream_t s) {
    if (block_threads == 256) return launch_norm<256, 256, 8>(a, sg, num_sms, blocks_per_sm, s);
    return launch_norm<128, 128, 16>(a, sg, num_sms, blocks_per_sm, s);
}

cudaError_t launch_seg_sort(const DiscArgs &a, const SegArgs &sg, int num_sms, cudaStream_t s) {
    k_seg_class<<<num_sms * 4, 256, 0, s>>>(a, sg);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_seg_cscan<<<1, kClasses, 0, s>>>(sg);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_seg_sort<<<num_sms * 8, 256, 0, s>>>(a, sg);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_seg_plan<<<1, 1, 0, s>>>(sg);
    return cudaGetLastError();
}

cudaError_t launch_seg_deposits(const DiscArgs &a, const SegArgs &sg, int block_threads, int num_sms,
                                int blocks_per_sm, int npix, cudaStream_t s) {
    if (block_threads == 256) return launch_deposits<256, 256, 8>(a, sg, num_sms, blocks_per_sm, npix, s);
    return launch_deposits<128, 128, 16>(a, sg, num_sms, blocks_per_sm, npix, s);
}

}  // namespace dmann
