// disc_comp.cu -- the compensated-FP32 form's per-disc kernels: a block or
// a warp renders one disc in two passes (normalisation, then deposits as
// FP64 reductions), the compensated adjoint, and the disc headers.  The
// arithmetic (chord test, weights, two-float sums) is in comp_engine.cuh.
#include "comp_engine.cuh"

namespace dmann {

namespace {

// Both passes of one disc particle (tiers TX, TH; see weight2x), after
// render_particle has staged its header.
template <int G, int RCH, int TX, int TH>
__device__ void render_disc(const DiscArgs &a, CompSmem<RCH> &sm, const Ext &e) {
    using Gp = Grp<G>;
    const int rk = Gp::rank();
    const int r_first = sm.h.hdr.r_first, r_last = sm.h.hdr.r_last;
    const int nring = r_last - r_first + 1;
    const int nchunk = nring > 0 ? (nring + RCH - 1) / RCH : 0;

    // pass 1: the normalisation, a compensated sum per lane (both halves).
    // The sums start at 1 and every weight is <= 1, so the running sum always
    // dominates the addend and Fast2Sum gives each step's rounding error
    // exactly; the errors are summed apart (not fed back into the next addend,
    // where Kahan's subtraction would round them away again).  The result is
    // independent of the order in which lanes meet the weights to ~1e-12.
    // The offset is removed exactly after the pass.
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
        run_walk<G, RCH>(sm, n, [&](const Run &r, int, int j, bool second) {
            const float jf = (float)j;
            float2 w = weight2<TX, TH>(e, r, make_float2(jf, jf + 32.0f));
            if (!second) w.y = 0.0f;
            const float2 t = add2(ks, w);
            kc = add2(kc, sub2(w, sub2(t, ks)));
            ks = t;
        });
        Gp::sync();
    }
    if (total < 2) {  // genmap.cpp:125-128: the whole flux into the centre pixel
        if (rk == 0) {
            red_add_f64(a.acc.acc64 + sm.h.hdr.cpix, (double)e.fs_hi + (double)e.fs_lo);
            atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), 1ull);
        }
        Gp::sync();
        return;
    }
    if (rk == 0) atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), (unsigned long long)total);
    // S = sum of the lanes' (ks - 1) + kc, all in FP32 two-floats: ks - 1 is
    // exact (1 <= ks < 2^24: a multiple of ulp(ks) below ks), the lane and
    // warp sums are TwoSum trees, and F = flux inv_scale / S is Dekker's
    // two-float division (relative error ~2^-44).  Every lane of a warp ends
    // with the same sums (the xor tree adds the same pairs on each).
    float S_hi, S_lo;
    {
        float err;
        S_hi = two_sum(ks.x - 1.0f, ks.y - 1.0f, err);
        S_lo = (kc.x + kc.y) + err;
        warp_sum_ff(S_hi, S_lo);
    }
    float F, Flo;
    if (G > 32) {
        if ((rk & 31) == 0) sm.red2[rk >> 5] = make_float2(S_hi, S_lo);
        Gp::sync();
        if (rk == 0) {
            for (int k = 1; k < Gp::kWarps; k++) {
                float err;
                S_hi = two_sum(S_hi, sm.red2[k].x, err);
                S_lo = (S_lo + sm.red2[k].y) + err;
            }
            sm.fq = div_ff(e.fs_hi, e.fs_lo, S_hi, S_lo);
        }
        Gp::sync();
        F = sm.fq.x;
        Flo = sm.fq.y;
    } else {
        const float2 q = div_ff(e.fs_hi, e.fs_lo, S_hi, S_lo);
        F = q.x;
        Flo = q.y;
    }
    // |F| and the sign apart: the products are then >= 0 for the exact
    // conversion to FP64 (f32_to_f64), and the sign goes into its bit.  The
    // weights are >= exp(-6) (the disc edge), so a product is zero only when
    // the flux is: such a particle deposits nothing.
    if (F == 0.0f && Flo == 0.0f) return;
    const unsigned bias = f64_bias(F < 0.0f);
    const float Fa = fabsf(F), Floa = F < 0.0f ? -Flo : Flo;
    double *const acc = a.acc.acc64;

    // pass 2: deposits, one FP64 reduction per pixel (see the file header).
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        if (nchunk > 1) build_runs<G, RCH>(a, sm, r0, n);
        if (G > 32) {
            if (rk == 0) sm.next_run = 0;
            Gp::sync();
        }
        run_walk<G, RCH>(sm, n, [&](const Run &r, int, int j, bool second) {
            const float jf = (float)j;
            const float2 w = weight2<TX, TH>(e, r, make_float2(jf, jf + 32.0f));
            const float2 p = fma2(w, f2(Fa), mul2(w, f2(Floa)));   // w |F|, rounded once
            double *const m = acc + (r.pix0 + j);
            red_add_f64(m, f32_to_f64(p.x, bias));
            if (second) red_add_f64(m + 32, f32_to_f64(p.y, bias));
        });
        Gp::sync();
    }
}


// Renders the particle of queue slot q with a group of G threads (a warp or
// a block).
template <int G, int RCH>
__device__ void render_particle(const DiscArgs &a, CompSmem<RCH> &sm, long long q) {
    using Gp = Grp<G>;
    stage_hdr<G>(a, q, sm.h);
    Gp::sync();
    const Ext e = sm.h.ext;
    with_tiers(e, [&](auto tx, auto th) {
        render_disc<G, RCH, decltype(tx)::value, decltype(th)::value>(a, sm, e);
    });
}

constexpr int kWPB = 8, kRCHW = 64;    // warp kernel

// One block per large disc, persistent over the block-class queue (largest
// discs first, claimed dynamically).  Block shapes: BT threads, runs of RCH
// rings staged per chunk, MINB resident blocks per SM -- every shape fills
// the SM with 2048 threads (fewer, with more registers each, measured slower)
// and about 200 KB of staged runs.  The autotuner picks the shape.  Returns
// at once when the segmented render took the block class (*a.block_skip).
template <int BT, int RCH, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_comp_block(DiscArgs a) {
    if (a.block_skip && *a.block_skip) return;
    __shared__ CompSmem<RCH> sm;
    __shared__ int s_q;
    const long long nblk = a.ctr[C_ADD_BLOCK];
    for (;;) {
        if (threadIdx.x == 0) s_q = (int)atomicAdd((unsigned long long *)(a.ctr + C_QNEXT_BLOCK), 1ull);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= nblk) break;
        render_particle<BT, RCH>(a, sm, q);
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
    for (long long q = nblk + gw; q < ndisc; q += nw) render_particle<32, kRCHW>(a, sm[w], q);
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

// ------------------------------------------------------------------ adjoint
// The adjoint of the map (the formulas of adjoint.cu) with the compensated
// form's FP32 weights.  The tangent vector v_p - cos(alpha) n of each pixel is
// taken in the particle's local basis (e_theta, e_phi), where
//   v . e_theta = sin(theta_r - theta0) - 2 cos(theta0) sin(theta_r) sin^2(dphi/2),
//   v . e_phi   = sin(theta_r) sin(dphi) = 2 sin(theta_r) sin(x) cos(x),  x = dphi/2,
// both accurate to FP32 relative precision however small alpha is (the 3-D
// difference v - cos(alpha) n is not); alpha / sin(alpha) =
// sqrt(g / (h (1 - h))) with h = hav(alpha) and g = alpha^2 / 4 from the
// weight.  Sums: S with the offset Fast2Sum, the signed ones (sum G w, V_theta,
// V_phi, T) with Kahan's compensation per lane, all reduced in FP64; the
// epilogue turns V into the map frame and writes the gradient in FP64.
template <int RCH>
struct AdjcSmem {
    CompSmem<RCH> c;
    AdjRing aring[RCH];
    double red[3][32];
};

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

template <int G, int RCH>
__device__ void adjc_particle(const adj::AdjArgs &a, AdjcSmem<RCH> &sm, long long q, double acc[12]) {
    using Gp = Grp<G>;
    const DiscArgs &da = a.d;
    const int rk = Gp::rank();
    stage_hdr<G>(da, q, sm.c.h);
    Gp::sync();
    const int pidx = sm.c.h.hdr.pidx;
    const Ext e = sm.c.h.ext;
    const int r_first = sm.c.h.hdr.r_first, r_last = sm.c.h.hdr.r_last;
    const int nring = r_last - r_first + 1;
    const int nchunk = nring > 0 ? (nring + RCH - 1) / RCH : 0;
    const float *g32 = a.gmap32;

    // pass 1: S (offset Fast2Sum) and sum G w (Kahan)
    float2 ks = f2(1.0f), kc = f2(0.0f);
    float as = 0.0f, ac = 0.0f;
    long long total = 0;
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        total += build_runs<G, RCH>(da, sm.c, r0, n, sm.aring);
        if (G > 32) {
            if (rk == 0) sm.c.next_run = 0;
            Gp::sync();
        }
        run_walk<G, RCH>(sm.c, n, [&](const Run &r, int, int j, bool second) {
            const float jf = (float)j;
            float2 w = weight2(e, r, make_float2(jf, jf + 32.0f));
            if (!second) w.y = 0.0f;
            const int pix = r.pix0 + j;
            const float gw = g32[pix] * w.x + (second ? g32[pix + 32] * w.y : 0.0f);
            kahan(as, ac, gw);
            const float2 t = add2(ks, w);
            kc = add2(kc, sub2(w, sub2(t, ks)));
            ks = t;
        });
        Gp::sync();
    }
    double s1[3] = {(((double)ks.x - 1.0) + (double)kc.x) + (((double)ks.y - 1.0) + (double)kc.y),
                    (double)as - (double)ac, 0.0};
    adj::group_sum<G, 2>(s1, sm.red);
    if (total < 2) {  // genmap.cpp:125-128: the whole flux in the centre pixel
        if (rk == 0) {
            const double KV[3] = {0.0, 0.0, 0.0};
            adj::write_grad(a, pidx, a.gmap[sm.c.h.hdr.cpix] * a.inv_dOmega, 0.0, KV, false, acc);
            atomicAdd((unsigned long long *)(da.ctr + C_DEPOSITS), 1ull);
        }
        Gp::sync();
        return;
    }
    if (rk == 0) atomicAdd((unsigned long long *)(da.ctr + C_DEPOSITS), (unsigned long long)total);
    const double S = s1[0];
    const double Gm = s1[1] / S;
    const float gm = (float)Gm;

    // pass 2: V_theta, V_phi, T with q = (G - Gm) w
    float vts = 0.0f, vtc = 0.0f, vps = 0.0f, vpc = 0.0f, ts = 0.0f, tc = 0.0f;
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        if (nchunk > 1) build_runs<G, RCH>(da, sm.c, r0, n, sm.aring);
        if (G > 32) {
            if (rk == 0) sm.c.next_run = 0;
            Gp::sync();
        }
        run_walk<G, RCH>(sm.c, n, [&](const Run &r, int ring, int j, bool second) {
            const float jf = (float)j;
            float2 sn, h, g;
            const float2 w = weight2x(e, r, make_float2(jf, jf + 32.0f), sn, h, g);
            const AdjRing ar = sm.aring[ring];
            const int pix = r.pix0 + j;
            float vt = 0.0f, vp = 0.0f, tt = 0.0f;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (k == 1 && !second) break;
                const float wk = k ? w.y : w.x, snk = k ? sn.y : sn.x, hk = k ? h.y : h.x,
                            gk = k ? g.y : g.x;
                const float q = (g32[pix + 32 * k] - gm) * wk;
                // alpha / sin(alpha); 0 at the antipode, where the tangent is undefined
                const float om = 1.0f - hk;
                const float af = hk > 1e-30f ? (om > 1e-7f ? sqrtf(gk / (hk * om)) : 0.0f) : 1.0f;
                const float s2 = snk * snk;
                const float eth = fmaf(-ar.cr, s2, ar.sr);
                const float eph = ar.st2 * snk * sqrtf(fmaxf(1.0f - s2, 0.0f));
                const float qa = q * af;
                vt = fmaf(qa, eth, vt);
                vp = fmaf(qa, eph, vp);
                tt = fmaf(q, 4.0f * gk, tt);
            }
            kahan(vts, vtc, vt);
            kahan(vps, vpc, vp);
            kahan(ts, tc, tt);
        });
        Gp::sync();
    }
    double s2[3] = {(double)vts - (double)vtc, (double)vps - (double)vpc, (double)ts - (double)tc};
    adj::group_sum<G, 3>(s2, sm.red);
    if (rk == 0) {
        const DiscHdr &d = sm.c.h.hdr;
        const double ct = cos(d.theta0), st = sin(d.theta0), cp = cos(d.phi0), sp = sin(d.phi0);
        const double V[3] = {s2[0] * ct * cp - s2[1] * sp, s2[0] * ct * sp + s2[1] * cp, -s2[0] * st};
        const double K = adj::kInvC2 * d.flux / (S * d.ar * d.ar) * a.inv_dOmega;
        const double KV[3] = {K * V[0], K * V[1], K * V[2]};
        adj::write_grad(a, pidx, Gm * a.inv_dOmega, K * s2[2], KV, true, acc);
    }
    Gp::sync();
}

template <int BT, int RCH, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_adjc_block(adj::AdjArgs a) {
    __shared__ AdjcSmem<RCH> sm;
    __shared__ int s_q;
    double acc[12] = {0.0};
    const long long nblk = a.d.ctr[C_ADD_BLOCK];
    for (;;) {
        if (threadIdx.x == 0) s_q = (int)atomicAdd((unsigned long long *)(a.d.ctr + C_QNEXT_BLOCK), 1ull);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= nblk) break;
        adjc_particle<BT, RCH>(a, sm, q, acc);
    }
    if (threadIdx.x == 0) adj::flush_acc(a.oacc, acc);
}

constexpr int kWPBA = 4;   // warps per block of the adjoint's warp kernel (shared memory)

__global__ void __launch_bounds__(kWPBA * 32) k_adjc_warp(adj::AdjArgs a) {
    __shared__ AdjcSmem<kRCHW> sm[kWPBA];
    double acc[12] = {0.0};
    const long long nblk = a.d.ctr[C_ADD_BLOCK];
    const long long ndisc = a.d.ctr[C_ADD_DISC];
    const int w = threadIdx.x >> 5;
    const long long gw = (long long)blockIdx.x * kWPBA + w;
    const long long nw = (long long)gridDim.x * kWPBA;
    for (long long q = nblk + gw; q < ndisc; q += nw) adjc_particle<32, kRCHW>(a, sm[w], q, acc);
    if ((threadIdx.x & 31) == 0) adj::flush_acc(a.oacc, acc);
}

// The headers of every disc in the queue, one thread per particle (the
// FP64 set-up at full warp width instead of on one lane of a waiting block).
__global__ void __launch_bounds__(256) k_comp_hdr(DiscArgs a) {
    // each warp builds its 32 consecutive headers in shared memory and
    // stores them as one contiguous run of 16-byte words (a thread's own
    // 160-byte store would leave partial sectors for the L2 to merge)
    constexpr int kW16 = sizeof(CompHdr) / 16;
    static_assert(sizeof(CompHdr) % 16 == 0, "headers are stored in 16-byte words");
    __shared__ __align__(16) CompHdr stage[8][32];
    const long long ndisc = a.ctr[C_ADD_DISC];
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (long long q0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); q0 < ndisc; q0 += stride) {
        const long long q = q0 + lane;
        if (q < ndisc) setup_hdr(a, a.queue[q], stage[w][lane]);
        __syncwarp();
        const int nh = (int)min(32LL, ndisc - q0);
        const float4 *src = reinterpret_cast<const float4 *>(&stage[w][0]);
        float4 *dst = reinterpret_cast<float4 *>(a.chdr + q0);
        for (int k = lane; k < nh * kW16; k += 32) dst[k] = src[k];
        __syncwarp();
    }
}

}  // namespace

cudaError_t launch_hdr(const DiscArgs &a, int num_sms, cudaStream_t s) {
    if (!a.chdr) return cudaSuccess;
    k_comp_hdr<<<num_sms * 8, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_disc_comp_warp(const DiscArgs &a, int num_sms, cudaStream_t s) {
    int occw = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_comp_warp, kWPB * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_comp_warp<<<num_sms * occw, kWPB * 32, 0, s>>>(a);
    return cudaGetLastError();
}

size_t comp_hdr_bytes() { return sizeof(CompHdr); }

cudaError_t launch_disc_comp_block(const DiscArgs &a, int num_sms, int blocks_per_sm, int block_threads,
                                   cudaStream_t s) {
    if (block_threads == 128) return launch_block<128, 192, 16>(a, num_sms, blocks_per_sm, s);
    if (block_threads == 512) return launch_block<512, 640, 4>(a, num_sms, blocks_per_sm, s);
    return launch_block<256, 384, 8>(a, num_sms, blocks_per_sm, s);
}

cudaError_t launch_disc_comp(const DiscArgs &a, int num_sms, int blocks_per_sm, int block_threads,
                             cudaStream_t s, cudaEvent_t mid, bool headers) {
    cudaError_t e = headers ? launch_hdr(a, num_sms, s) : cudaSuccess;
    if (e != cudaSuccess) return e;
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

// The compensated adjoint's disc kernels (block class, then warp class).
cudaError_t launch_adjoint_comp_discs(const adj::AdjArgs &a, int num_sms, cudaStream_t s) {
    cudaError_t e = launch_hdr(a.d, num_sms, s);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_adjc_block<256, 256, 4>, 256, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
    k_adjc_block<256, 256, 4><<<num_sms * occ, 256, 0, s>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int occw = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_adjc_warp, kWPBA * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_adjc_warp<<<num_sms * occw, kWPBA * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dmann
