// disc_engine.cuh -- renders one particle's disc with a group of threads
// (one warp, or one thread block), parameterised by a precision form.
//
// For a particle with angular radius ar the disc is every RING pixel whose
// centre lies within 2 ar of the particle direction (non-inclusive HEALPix
// query_disc, src/genmap.cpp:119).  Its pixels get Gaussian weights
// w = exp(-0.5 (theta/ar)^2 / 0.333) (genmap.cpp:137-143), normalised so the
// particle deposits exactly its flux (genmap.cpp:148-153).
//
// Work layout: the rings the disc touches are processed in chunks of RCH
// rings.  For each chunk the group first computes, one thread per ring, the
// in-disc pixel run of every ring (the query_disc chord test in FP64) and
// stages it in shared memory with an exclusive prefix of run lengths; the
// group then walks the chunk's pixels as one flattened index space, each
// warp taking a contiguous stretch with lanes on consecutive pixels, so
// lanes of a warp touch consecutive map addresses.  Pass 1 sums the weights
// (the per-particle normalisation); pass 2 recomputes them and deposits
// w * flux / norm.  A disc with fewer than 2 pixels puts its whole flux into
// the centre pixel (genmap.cpp:125-128).
#pragma once
#include "kernels.cuh"

namespace dmann {

template <int G>
struct Group {
    static constexpr int kWarps = G / 32;
    __device__ static void sync() {
        if (G == 32) __syncwarp(); else __syncthreads();
    }
    __device__ static int rank() { return G == 32 ? (threadIdx.x & 31) : (int)threadIdx.x; }
    __device__ static int warp() { return G == 32 ? 0 : (int)(threadIdx.x >> 5); }
};

// Shared state of one group for one particle.
template <class Form, int RCH>
struct GroupSmem {
    typename Form::Seg seg[RCH + 1];   // +1: sentinel holding the chunk total in .off
    DiscHdr hdr;
    typename Form::Ext ext;
    double red[32];
    long long chunk_total;
    int scan_tmp[32];
};

// Exclusive scan of seg[0..n).cnt (held in .off on entry) into .off; the
// sentinel seg[n].off receives the total.  Every thread of the group calls.
template <class Form, int G, int RCH>
__device__ inline void group_scan(GroupSmem<Form, RCH> &sm, int n) {
    using Grp = Group<G>;
    constexpr int PER = (RCH + G - 1) / G;
    const int r = Grp::rank();
    int v[PER];
    int s = 0;
#pragma unroll
    for (int k = 0; k < PER; k++) {
        int idx = r * PER + k;
        v[k] = (idx < n) ? sm.seg[idx].off : 0;
        s += v[k];
    }
    int wtot;
    int ex = warp_excl_scan(s, wtot);
    if (G > 32) {
        if ((r & 31) == 0) sm.scan_tmp[r >> 5] = wtot;
        Grp::sync();
        if (r < 32) {
            int x = (r < Grp::kWarps) ? sm.scan_tmp[r] : 0;
            int t2;
            int e2 = warp_excl_scan(x, t2);
            if (r < Grp::kWarps) sm.scan_tmp[r] = e2;
            if (r == 0) sm.chunk_total = t2;
        }
        Grp::sync();
        ex += sm.scan_tmp[r >> 5];
    } else {
        if (r == 0) sm.chunk_total = wtot;
    }
#pragma unroll
    for (int k = 0; k < PER; k++) {
        int idx = r * PER + k;
        if (idx < n) sm.seg[idx].off = ex;
        ex += v[k];
    }
    Grp::sync();
    if (r == 0) sm.seg[n].off = (int)sm.chunk_total;
    Grp::sync();
}

template <class Form, int G, int RCH>
__device__ inline void build_chunk(const DiscArgs &a, GroupSmem<Form, RCH> &sm, int r0, int n) {
    using Grp = Group<G>;
    for (int i = Grp::rank(); i < n; i += G) {
        const int ring = r0 + i;
        int lo, cnt;
        ring_segment_t<Form::kFastChord>(a.g, sm.hdr, ring, lo, cnt);
        Form::fill_seg(a, sm.hdr, sm.ext, ring, lo, cnt, sm.seg[i]);
        sm.seg[i].off = cnt;
    }
    Grp::sync();
    group_scan<Form, G, RCH>(sm, n);
}

// Largest s in [0, n) with seg[s].off <= f (f < total).
template <class Seg>
__device__ inline int find_seg(const Seg *seg, int n, int f) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (seg[mid].off <= f) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Walks the chunk's flattened pixels; `body(seg_cache, j, pix)` per pixel.
template <class Form, int G, int RCH, class Body>
__device__ inline void pixel_walk(const GroupSmem<Form, RCH> &sm, int n, int total, Body body) {
    using Grp = Group<G>;
    if (total <= 0) return;
    const int lane = threadIdx.x & 31;
    const int w = Grp::warp();
    // contiguous stretch per warp, a multiple of 32 pixels
    int per = (total + Grp::kWarps - 1) / Grp::kWarps;
    per = (per + 31) & ~31;
    const int f0 = w * per;
    const int f1 = min(total, f0 + per);
    int f = f0 + lane;
    if (f >= f1) return;
    int s = find_seg(sm.seg, n, f);
    typename Form::SegReg cur;
    Form::load_seg(sm.seg[s], cur);
    int seg_off = sm.seg[s].off;
    int seg_end = sm.seg[s + 1].off;
    while (f < f1) {
        const int j = f - seg_off;
        int k = cur.lo + j;
        k += (k < 0) ? cur.nr : 0;
        k -= (k >= cur.nr) ? cur.nr : 0;
        body(cur, j, cur.start + k);
        f += 32;
        if (f >= seg_end && f < f1) {
            do {
                ++s;
                seg_off = seg_end;
                seg_end = sm.seg[s + 1].off;
            } while (f >= seg_end);
            Form::load_seg(sm.seg[s], cur);
        }
    }
}

template <class Form, int G, int RCH>
__device__ inline void render_particle(const DiscArgs &a, GroupSmem<Form, RCH> &sm, int pidx) {
    using Grp = Group<G>;
    const int r = Grp::rank();
    if (r == 0) {
        disc_setup(a.g, a.theta[pidx], a.phi[pidx], a.ar[pidx], a.flux[pidx], a.cpix[pidx], pidx,
                   sm.hdr);
        Form::particle_setup(a, sm.hdr, a.phi[pidx], sm.ext);
    }
    Grp::sync();
    const typename Form::Ext ext = sm.ext;  // per-particle constants, in registers
    const int r_first = sm.hdr.r_first, r_last = sm.hdr.r_last;
    const int nring = r_last - r_first + 1;
    const int nchunk = nring > 0 ? (nring + RCH - 1) / RCH : 0;

    // pass 1: normalisation
    typename Form::NormAcc nacc;
    long long total = 0;
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        build_chunk<Form, G, RCH>(a, sm, r0, n);
        const int ct = (int)sm.chunk_total;
        total += ct;
        pixel_walk<Form, G, RCH>(sm, n, ct, [&](const typename Form::SegReg &sr, int j, int pix) {
            Form::norm_add(ext, sr, j, pix, nacc);
        });
        Grp::sync();
    }
    double part = Form::norm_value(nacc);
    part = warp_sum(part);
    double S = part;
    if (G > 32) {
        if ((r & 31) == 0) sm.red[r >> 5] = part;
        Grp::sync();
        S = 0.0;
        for (int k = 0; k < Grp::kWarps; k++) S += sm.red[k];
        Grp::sync();
    }
    if (total < 2) {  // genmap.cpp:125-128
        if (r == 0) {
            Form::single(a, sm.hdr);
            atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), 1ull);
        }
        Grp::sync();
        return;
    }
    if (r == 0) atomicAdd((unsigned long long *)(a.ctr + C_DEPOSITS), (unsigned long long)total);
    typename Form::Dep dep;
    Form::deposit_setup(a, sm.hdr, ext, S, dep);

    // pass 2: deposits (the staged chunk is reused when there is only one)
    for (int c = 0; c < nchunk; c++) {
        const int r0 = r_first + c * RCH;
        const int n = min(RCH, r_last - r0 + 1);
        if (nchunk > 1) build_chunk<Form, G, RCH>(a, sm, r0, n);
        const int ct = (int)sm.chunk_total;
        pixel_walk<Form, G, RCH>(sm, n, ct, [&](const typename Form::SegReg &sr, int j, int pix) {
            Form::deposit(a, ext, dep, sr, j, pix);
        });
        Grp::sync();
    }
}

// One thread block per particle, persistent over the block-class queue
// (largest discs first, claimed dynamically).  Form::kMinBlocks resident
// blocks per SM are asked of the compiler: the compensated kernel is latency
// bound (returned atomics), and full occupancy measured fastest even with
// some register spilling.
template <class Form, int BT, int RCH>
__global__ void __launch_bounds__(BT, Form::kMinBlocks) k_disc_block(DiscArgs a) {
    __shared__ GroupSmem<Form, RCH> sm;
    __shared__ int s_q;
    const long long nblk = a.ctr[C_ADD_BLOCK];
    for (;;) {
        if (threadIdx.x == 0) s_q = (int)atomicAdd((unsigned long long *)(a.ctr + C_QNEXT_BLOCK), 1ull);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= nblk) break;
        render_particle<Form, BT, RCH>(a, sm, a.queue[q]);
    }
}

// One warp per particle over the warp-class queue (after the block class).
template <class Form, int WPB, int RCH>
__global__ void __launch_bounds__(WPB * 32) k_disc_warp(DiscArgs a) {
    __shared__ GroupSmem<Form, RCH> sm[WPB];
    const long long nblk = a.ctr[C_ADD_BLOCK];
    const long long ndisc = a.ctr[C_ADD_DISC];
    const int w = threadIdx.x >> 5;
    const long long gw = (long long)blockIdx.x * WPB + w;
    const long long nw = (long long)gridDim.x * WPB;
    for (long long q = nblk + gw; q < ndisc; q += nw) {
        render_particle<Form, 32, RCH>(a, sm[w], a.queue[q]);
    }
}

}  // namespace dmann
