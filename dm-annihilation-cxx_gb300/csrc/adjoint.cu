// adjoint.cu -- the adjoint (reverse-mode derivative) of the plain-form
// projection: for a pixelwise loss with gradient G[p] = dL/dmap[p] (map in
// flux per steradian, i.e. the per-pixel sums divided by dOmega), the
// derivatives of L with respect to every particle's x, y, z, m, rho, h and,
// summed over particles, the terms of dL/d(observer position).
//
// Forward model of one kept particle (src/genmap.cpp:82-153 with
// src/flux/flux_ann_nosom.cpp:18):
//   u = pos - opos,  d = |u|,  F = unit_factor rho m / (4 pi d^2),
//   n = D R^T u / d  (D = diag(-1, -1, 1): the pi shift of phi),  ar = h / d,
//   alpha_p = acos(v_p . n),  w_p = exp(-c alpha_p^2 / ar^2),  c = 0.5/0.333,
//   map[p] += F w_p / S / dOmega over the disc pixels p,  S = sum_p w_p,
// or map[cpix] += F / dOmega for a single-pixel deposit.  With g_p =
// G[p] / dOmega, Gb = sum_p g_p w_p / S, q_p = (g_p - Gb) w_p and
//   V = sum_p q_p (alpha_p / sin alpha_p) (v_p - cos(alpha_p) n),
//   T = sum_p q_p alpha_p^2,   K = 2 c F / (S ar^2):
//   dL/dF = Gb, dL/dm = Gb F/m, dL/drho = Gb F/rho, dL/dh = K T / h,
//   dL/du = -(2 Gb F + K T)/d * u/d + (K/d) R D V,
//   dL/dR[j][a] = K (D V)_a u_j / d  (through n only).
// The pixel sets are held fixed (the derivative of the map where disc
// membership does not change); the single-pixel case has V = T = 0.
// The weights are recomputed (two passes over the disc: S and sum g w, then
// V and T), not stored.  Compiled with -fmad=false like the plain form, so
// the weights and S are bit for bit those of the plain forward kernels.
// With precision DMANN_COMP_F32 the disc particles go to the compensated
// form's kernels instead (disc_comp.cu), with FP32 weights.
#include "../../include/dmann.h"
#include "adjoint_common.cuh"
#include "plain_form.cuh"

namespace dmann {

namespace {

using namespace adj;

template <int RCH>
struct AdjSmem {
    GroupSmem<PlainForm, RCH> g;
    double red[4][32];
};

// Gradient of one disc particle with a group of G threads.  The group's
// rank 0 adds the observer terms into acc.
template <int G, int RCH>
__device__ inline void adjoint_particle(const AdjArgs &a, AdjSmem<RCH> &sm, int pidx,
                                        double acc[12]) {
    using Grp = Group<G>;
    const DiscArgs &da = a.d;
    const int r = Grp::rank();
    if (r == 0) {
        disc_setup(da.g, da.theta[pidx], da.phi[pidx], da.ar[pidx], da.flux[pidx], da.cpix[pidx],
                   pidx, sm.g.hdr);
        PlainForm::particle_setup(da, sm.g.hdr, da.phi[pidx], sm.g.ext);
    }
    Grp::sync();
    const PlainForm::Ext ext = sm.g.ext;
    const int r_first = sm.g.hdr.r_first, r_last = sm.g.hdr.r_last;
    const int nring = r_last - r_first + 1;
    const int nchunk = nring > 0 ? (nring + RCH - 1) / RCH : 0;
    const double *gmap = a.gmap;

    // pass 1: S = sum w, A = sum G w
    double s1[2] = {0.0, 0.0};
    long long total = 0;
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int nr = min(RCH, r_last - r0 + 1);
        build_chunk<PlainForm, G, RCH>(da, sm.g, r0, nr);
        const int ct = (int)sm.g.chunk_total;
        total += ct;
        pixel_walk<PlainForm, G, RCH>(sm.g, nr, ct, [&](const PlainForm::SegReg &sr, int j, int pix) {
            (void)j;
            const double w = PlainForm::weight(ext, sr, pix);
            s1[0] += w;
            s1[1] += gmap[pix] * w;
        });
        Grp::sync();
    }
    group_sum<G, 2>(s1, sm.red);
    if (total < 2) {  // genmap.cpp:125-128: the whole flux in the centre pixel
        if (r == 0) {
            const double KV[3] = {0.0, 0.0, 0.0};
            write_grad(a, pidx, gmap[sm.g.hdr.cpix] * a.inv_dOmega, 0.0, KV, false, acc);
            atomicAdd((unsigned long long *)(da.ctr + C_DEPOSITS), 1ull);
        }
        Grp::sync();
        return;
    }
    if (r == 0) atomicAdd((unsigned long long *)(da.ctr + C_DEPOSITS), (unsigned long long)total);
    const double S = s1[0];
    const double Gm = s1[1] / S;   // the w-weighted mean of G over the disc

    // pass 2: V and T with q = (G - Gm) w (the staged chunk is reused when
    // there is only one)
    double s2[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int nr = min(RCH, r_last - r0 + 1);
        if (nchunk > 1) build_chunk<PlainForm, G, RCH>(da, sm.g, r0, nr);
        const int ct = (int)sm.g.chunk_total;
        pixel_walk<PlainForm, G, RCH>(sm.g, nr, ct, [&](const PlainForm::SegReg &sr, int j, int pix) {
            (void)j;
            double px, py, pz;
            PlainForm::pixel_vec(ext, sr, pix, px, py, pz);
            const double dot = px * ext.vx + py * ext.vy + pz * ext.vz;
            const double dc = fmin(1.0, fmax(-1.0, dot));
            const double alpha = acos(dc);
            double d2 = alpha / ext.ar;
            d2 = d2 * d2;
            const double w = exp(-0.5 * d2 / 0.333);
            const double q = (gmap[pix] - Gm) * w;
            // tangent of the great circle from n towards the pixel, length sin(alpha)
            const double ex = px - dc * ext.vx, ey = py - dc * ext.vy, ez = pz - dc * ext.vz;
            const double sa = sqrt(ex * ex + ey * ey + ez * ez);
            const double f = sa > 0.0 ? q * alpha / sa : 0.0;
            s2[0] += f * ex;
            s2[1] += f * ey;
            s2[2] += f * ez;
            s2[3] += q * alpha * alpha;
        });
        Grp::sync();
    }
    group_sum<G, 4>(s2, sm.red);
    if (r == 0) {
        const double ar = ext.ar;
        const double K = kInvC2 * da.flux[pidx] / (S * ar * ar) * a.inv_dOmega;
        const double KV[3] = {K * s2[0], K * s2[1], K * s2[2]};
        write_grad(a, pidx, Gm * a.inv_dOmega, K * s2[3], KV, true, acc);
    }
    Grp::sync();
}

template <int BT, int RCH>
__global__ void __launch_bounds__(BT, 1) k_adj_block(AdjArgs a) {
    __shared__ AdjSmem<RCH> sm;
    __shared__ int s_q;
    double acc[12] = {0.0};
    const long long nblk = a.d.ctr[C_ADD_BLOCK];
    for (;;) {
        if (threadIdx.x == 0) s_q = (int)atomicAdd((unsigned long long *)(a.d.ctr + C_QNEXT_BLOCK), 1ull);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= nblk) break;
        adjoint_particle<BT, RCH>(a, sm, a.d.queue[q], acc);
    }
    if (threadIdx.x == 0) flush_acc(a.oacc, acc);
}

template <int WPB, int RCH>
__global__ void __launch_bounds__(WPB * 32) k_adj_warp(AdjArgs a) {
    __shared__ AdjSmem<RCH> sm[WPB];
    double acc[12] = {0.0};
    const long long nblk = a.d.ctr[C_ADD_BLOCK];
    const long long ndisc = a.d.ctr[C_ADD_DISC];
    const int w = threadIdx.x >> 5;
    const long long gw = (long long)blockIdx.x * WPB + w;
    const long long nw = (long long)gridDim.x * WPB;
    for (long long q = nblk + gw; q < ndisc; q += nw) adjoint_particle<32, RCH>(a, sm[w], a.d.queue[q], acc);
    if ((threadIdx.x & 31) == 0) flush_acc(a.oacc, acc);
}

// Every particle that is not a disc: zero gradient for skipped and invalid
// particles, the flux terms for single-pixel deposits.
__global__ void __launch_bounds__(256) k_adj_point(AdjArgs a) {
    __shared__ double red[3][32];
    double acc[12] = {0.0};
    const int n = a.p.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = a.cls[i];
        if (c == PC_DISC) continue;
        if (c == PC_SINGLE) {
            const double KV[3] = {0.0, 0.0, 0.0};
            write_grad(a, i, a.gmap[a.d.cpix[i]] * a.inv_dOmega, 0.0, KV, false, acc);
        } else {
#pragma unroll
            for (int k = 0; k < 6; k++) a.grad[(size_t)k * n + i] = 0.0;
        }
    }
    group_sum<256, 3>(acc, red);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; k++)
            if (acc[k] != 0.0) atomicAdd(a.oacc + k, acc[k]);
}

// dL/dmap rounded to FP32 for the compensated adjoint's per-pixel loads.
__global__ void k_to_f32(const double *in, float *out, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

constexpr int kBT = 256, kRCH = 256;
constexpr int kWPB = 8, kRCHW = 64;

}  // namespace

cudaError_t launch_adjoint(const DiscArgs &d, const Particles &p, const signed char *cls,
                           const double *gmap, float *gmap32, double *grad, double *oacc,
                           int precision, int num_sms, cudaStream_t s, const double *core_corr,
                           const double *core_gln) {
    AdjArgs a;
    a.d = d;
    a.p = p;
    a.core_corr = core_corr;
    a.core_gln = core_gln;
    a.cls = cls;
    a.gmap = gmap;
    a.gmap32 = gmap32;
    a.inv_dOmega = 1.0 / d.g.dOmega;
    a.grad = grad;
    a.oacc = oacc;
    if (p.n <= 0) return cudaSuccess;
    k_adj_point<<<num_sms * 8, 256, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (precision == DMANN_COMP_F32) {
        int blocks = (d.g.npix + 255) / 256;
        if (blocks > num_sms * 16) blocks = num_sms * 16;
        k_to_f32<<<blocks, 256, 0, s>>>(gmap, gmap32, d.g.npix);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        return launch_adjoint_comp_discs(a, num_sms, s);
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_adj_block<kBT, kRCH>, kBT, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
    k_adj_block<kBT, kRCH><<<num_sms * occ, kBT, 0, s>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int occw = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_adj_warp<kWPB, kRCHW>, kWPB * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_adj_warp<kWPB, kRCHW><<<num_sms * occw, kWPB * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dmann
