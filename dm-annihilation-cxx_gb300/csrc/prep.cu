// prep.cu -- per-particle preparation, single-pixel deposits, the disc work
// queue (counting sort by size bucket and sky cell) and the final map pass.
//
// Compiled with -fmad=false: the per-particle FP64 geometry below repeats
// the reference CPU path's operations in the same order, unfused, so d, the
// flux, theta, phi, the angular radius and the centre pixel are those of
// src/genmap.cpp:82-106 (with src/anglefuncs.cpp:15-52 and
// src/flux/flux_ann_nosom.cpp:12-23).
#include "kernels.cuh"

namespace dmann {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ inline int morton_cell(double theta, double phi) {
    // 64 x 64 cells in (theta, phi), bits interleaved (Z order), with the
    // top 4 bits (16 coarse sky regions) rotated to the bottom: consecutive
    // cells of the queue take turns among the 16 regions and keep Z order
    // within each.  The discs rendered at the same time then spread over 16
    // regions -- fewer reductions to the same pixel queue up in L2 -- while
    // each region's discs still share L2 lines (16M particles at Nside 2048:
    // 4.8 % faster than plain Z order; rotating 2, 3, 5 or 6 bits: 3.5, 4.2,
    // 4.2, 3.2 %).
    int it = min(63, max(0, (int)(theta * (64.0 / kPi))));
    int ip = min(63, max(0, (int)(phi * (64.0 / kTwoPi))));
    int c = 0;
#pragma unroll
    for (int b = 0; b < 6; b++) c |= (((it >> b) & 1) << (2 * b + 1)) | (((ip >> b) & 1) << (2 * b));
    return ((c << 4) | (c >> (kCellBits - 4))) & (kCells - 1);
}

// Adds `v` at `pix` once per group of lanes that share `pix` (warp
// aggregation: one atomic per distinct pixel of the warp).
template <class DepositFn>
__device__ inline void aggregated_add(bool active, int pix, double v, DepositFn dep) {
    unsigned act = __ballot_sync(kFull, active);
    if (!active) return;
    unsigned peers = __match_any_sync(act, pix);
    int lane = threadIdx.x & 31;
    double sum = 0.0;
    unsigned mm = peers;
    while (mm) {
        int src = __ffs(mm) - 1;
        sum += __shfl_sync(peers, v, src);
        mm &= mm - 1;
    }
    if (lane == __ffs(peers) - 1) dep(pix, sum);
}

__device__ inline void count_warp(long long *ctr, bool pred) {
    unsigned b = __ballot_sync(kFull, pred);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd((unsigned long long *)ctr, (unsigned long long)__popc(b));
}

constexpr double kCinCgs = 2.99792458e10;   // src/datatypes.cpp:5-10

// getflux of the context's flux law (the reference's link-time plugins in
// src/flux), each in its plugin's operation order.
__device__ inline double particle_flux(const PrepArgs &a, int i, float mass, float dens, double d) {
    const double uf = a.f.unit_factor;
    switch (a.f.flux_model) {
    case 1: {  // flux_ann_somv.cpp:16-43: <sigma v> ~ 1/v, saturated at 1 km/s, / 1e4
        double v = (double)a.p.sigmav[i] * a.f.vel_to_cgs;
        v /= 1.0e5;
        if (v < 1) v = 1;
        const double somer_v = kCinCgs / v / 1.0e4;
        return uf * somer_v * (double)dens * (double)mass / (4.0 * kPi * d * d);
    }
    case 2: {  // flux_ann_somv2.cpp:16-44: ~ 1/v^2, saturated at 5 km/s, / 1e8
        double v = (double)a.p.sigmav[i] * a.f.vel_to_cgs;
        v /= 1.0e5;
        if (v < 5) v = 5;
        double somer_v = kCinCgs / v;
        somer_v *= (somer_v / 1.0e8);
        return uf * somer_v * (double)dens * (double)mass / (4.0 * kPi * d * d);
    }
    case 3: {  // flux_ann_pwave.cpp:13-31: ~ v^2
        double somer_v = ((double)a.p.sigmav[i] * a.f.vel_to_cgs) / kCinCgs;
        somer_v = somer_v * somer_v;
        return uf * somer_v * (double)dens * (double)mass / (4.0 * kPi * d * d);
    }
    case 4:    // flux_decay.cpp:9-16 (unit_factor is the decay law's own)
        return uf * (double)mass / (4.0 * kPi * d * d);
    case 5: {  // flux_ann_adiabatic.cpp:10-33: adiabatic-contraction boost of the host
        const double dx = (double)a.p.x[i] - a.f.fcpos[0];
        const double dy = (double)a.p.y[i] - a.f.fcpos[1];
        const double dz = (double)a.p.z[i] - a.f.fcpos[2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz) * 40000.0;
        const double factor = (14.6534 * pow(1 + 0.0355872 * r, 1.76)) /
                               (pow(1 + 0.10888 * pow(r, 0.76), 3.34211) * pow(r, 0.13));
        double fluxes = uf * (double)dens * (double)mass / (4.0 * kPi * d * d);
        fluxes *= (factor * factor);
        return fluxes;
    }
    case 6: {  // flux_ann_core_nosom.cpp:9-17: the halo-core factor squared
        const double r = a.core_corr[i];
        return r * r * uf * (double)dens * (double)mass / (4.0 * kPi * d * d);
    }
    default:   // flux_ann_nosom.cpp:18
        return uf * (double)dens * (double)mass / (4.0 * kPi * d * d);
    }
}

__global__ void __launch_bounds__(256) k_prep(PrepArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < a.p.n;
    bool kept = false, single = false, disc = false, invalid = false;
    double flux = 0.0;
    int cpix = 0;
    if (in) {
        const float mass = a.p.m[i], dens = a.p.rho[i];
        // genmap.cpp:82-85: low-resolution and masked particles are skipped
        kept = !((double)mass >= a.f.hires_threshold || dens < 0);
        if (kept) {
            const float px = a.p.x[i], py = a.p.y[i], pz = a.p.z[i], hs = a.p.h[i];
            const double dx = (double)px - a.f.opos[0];
            const double dy = (double)py - a.f.opos[1];
            const double dz = (double)pz - a.f.opos[2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);  // genmap.cpp:87-89
            flux = particle_flux(a, i, mass, dens, d);
            // anglefuncs.cpp:15-52: v' = rot^T v, cos(theta) = v'_z/d, phi shifted by pi
            double t[3];
            const double v[3] = {dx, dy, dz};
#pragma unroll
            for (int k = 0; k < 3; k++) {
                t[k] = 0.0;
#pragma unroll
                for (int j = 0; j < 3; j++) t[k] += a.f.rot[j][k] * v[j];
            }
            double costheta = t[2] / d;
            double phi = atan2(t[1], t[0]);
            if (phi < 0) phi += 2.0 * kPi;
            phi -= kPi;
            if (phi < 0) phi = 2.0 * kPi + phi;
            if (phi > 2 * kPi) phi = phi - 2.0 * kPi;
            if (costheta > 1.0) costheta = 1.0;  // acos guard (NaN in the reference)
            if (costheta < -1.0) costheta = -1.0;
            const double theta = acos(costheta);       // genmap.cpp:98
            const double ar = (double)hs / d;           // genmap.cpp:99
            // Particles the reference cannot place (at the observer, non-finite
            // inputs, negative smoothing length) would give NaN pixel and ring
            // indices; they are skipped and counted instead.
            invalid = !(d > 0.0 && isfinite(flux) && isfinite(theta) && isfinite(phi) &&
                        isfinite(ar) && ar >= 0.0);
            if (invalid) {
                kept = false;
                flux = 0.0;
            } else {
                cpix = ang2pix(a.g, theta, phi);        // genmap.cpp:106
                cpix = min(max(cpix, 0), a.g.npix - 1);
                single = (2.0 * ar < a.g.theta0);       // genmap.cpp:107
                disc = !single;
            }
            a.out.theta[i] = theta;
            a.out.phi[i] = phi;
            a.out.ar[i] = ar;
            a.out.flux[i] = flux;
            a.out.cpix[i] = cpix;
            int key = -1;
            if (disc) {
                double est = disc_npix_estimate(a.g, ar);
                int bucket = est < 1.0 ? 0 : min(kBuckets - 1, ilogb(est));
                key = (kBuckets - 1 - bucket) * kCells + morton_cell(theta, fmodulo(phi, kTwoPi));
                atomicAdd(a.hist + key, 1);
            }
            a.out.key[i] = key;
        } else {
            a.out.key[i] = -1;
        }
        if (a.out.cls)
            a.out.cls[i] = disc ? PC_DISC : single ? PC_SINGLE : invalid ? PC_INVALID : PC_SKIPPED;
    }
    count_warp(a.ctr + C_KEPT, kept);
    count_warp(a.ctr + C_SINGLE, single);
    count_warp(a.ctr + C_DISC, disc);
    count_warp(a.ctr + C_INVALID, invalid);
    // total kept flux (the reference's "Total Conts", genmap.cpp:161-172)
    double fs = warp_sum(kept ? flux : 0.0);
    if ((threadIdx.x & 31) == 0 && fs != 0.0) atomicAdd(a.flux_sum, fs);
    // single-pixel particles: all their flux into the centre pixel
    if (!a.deposit_singles) {
        // classification only
    } else if (a.precision == 0) {
        double *acc = a.acc.acc64;
        aggregated_add(single, cpix, flux, [acc](int p, double v) { red_add_f64(acc + p, v); });
    } else {
        double *acc = a.acc.acc64;
        const double sc = a.f.inv_scale;
        aggregated_add(single, cpix, flux, [acc, sc](int p, double v) { red_add_f64(acc + p, v * sc); });
    }
    count_warp(a.ctr + C_DEPOSITS, single);
}

// Exclusive scan of the key histogram (one block); also publishes the
// number of disc particles in the block-per-particle class.
__global__ void __launch_bounds__(1024) k_scan(int *hist, long long *ctr, int block_bucket_min) {
    constexpr int T = 1024, PER = kKeys / T;
    __shared__ int wsum[32];
    const int tid = threadIdx.x;
    int local[PER];
    int s = 0;
#pragma unroll 8
    for (int k = 0; k < PER; k++) {
        local[k] = hist[tid * PER + k];
        s += local[k];
    }
    int tot;
    int ex = warp_excl_scan(s, tot);
    if ((tid & 31) == 0) wsum[tid >> 5] = tot;
    __syncthreads();
    if (tid < 32) {
        int t2;
        int e2 = warp_excl_scan(wsum[tid], t2);
        wsum[tid] = e2;
    }
    __syncthreads();
    int base = wsum[tid >> 5] + ex;
    const int boundary_key = (kBuckets - block_bucket_min) * kCells;
#pragma unroll 8
    for (int k = 0; k < PER; k++) {
        int key = tid * PER + k;
        if (key == boundary_key) {
            ctr[C_ADD_BLOCK] = base;
            ctr[C_DISC_BLOCK] += base;
        }
        hist[key] = base;
        base += local[k];
    }
    if (tid == T - 1) {
        ctr[C_ADD_DISC] = base;
        if (boundary_key >= kKeys) {
            ctr[C_ADD_BLOCK] = base;
            ctr[C_DISC_BLOCK] += base;
        }
    }
}

__global__ void __launch_bounds__(256) k_scatter(const int *key, int n, int *offsets, int *queue) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = (i < n) ? key[i] : -1;
    const bool act = k >= 0;
    unsigned am = __ballot_sync(kFull, act);
    if (!act) return;
    unsigned peers = __match_any_sync(am, k);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(offsets + k, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    queue[base + __popc(peers & ((1u << lane) - 1))] = i;
}

// map_out = (accumulate ? map_out : 0) + acc / dOmega   (genmap.cpp:168)
__global__ void k_finalize(Accum acc, int precision, int npix, double dOmega, double scale,
                           double *out, int accumulate) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        double v;
        if (precision == 0) {
            v = acc.acc64[p] / dOmega;
        } else {
            v = acc.acc64[p] * scale / dOmega;
        }
        out[p] = accumulate ? out[p] + v : v;
    }
}

}  // namespace

cudaError_t launch_prep(const PrepArgs &a, cudaStream_t s) {
    if (a.p.n <= 0) return cudaSuccess;
    k_prep<<<(a.p.n + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_scan(int *hist, long long *ctr, int block_bucket_min, cudaStream_t s) {
    k_scan<<<1, 1024, 0, s>>>(hist, ctr, block_bucket_min);
    return cudaGetLastError();
}

cudaError_t launch_scatter(const PrepArgs &a, int *queue, cudaStream_t s) {
    if (a.p.n <= 0) return cudaSuccess;
    k_scatter<<<(a.p.n + 255) / 256, 256, 0, s>>>(a.out.key, a.p.n, a.hist, queue);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const Accum &acc, int precision, int npix, double dOmega, double scale,
                            double *out, int accumulate, cudaStream_t s) {
    int blocks = (npix + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_finalize<<<blocks, 256, 0, s>>>(acc, precision, npix, dOmega, scale, out, accumulate);
    return cudaGetLastError();
}

}  // namespace dmann
