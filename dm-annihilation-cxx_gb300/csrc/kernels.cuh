// kernels.cuh -- argument blocks and launch entry points of the projection
// kernels (prep.cu, disc_plain.cu, disc_comp.cu).  Host-callable wrappers
// only take plain pointers and PODs.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"
#include "seg_plan.h"

namespace dmann {

// Sort keys of disc particles: (31 - log2 size bucket) * kCells + sky cell,
// so the queue runs from the largest discs to the smallest (longest jobs
// first) and, within a size bucket, in sky order taking turns among 16
// coarse regions (discs rendered together share L2 lines of the map but
// spread over 16 places; see morton_cell in prep.cu).
constexpr int kCellBits = 12;
constexpr int kCells = 1 << kCellBits;
constexpr int kBuckets = 32;
constexpr int kKeys = kBuckets * kCells;

// Segmented render (disc_seg.cu; its constants and segment plan are in
// seg_plan.h).  The plan is made on the device; each chunk launches
// kSegSlots deposit/flush pairs, the unused ones return at once.  Chunks
// whose estimated deposits are below 2^seg_min_deposits_log2 (a tunable), or
// whose work items exceed the item buffers, deposit in FP64 with the per-disc
// kernels.
// The segment buffer, zeroed per chunk: cls, cls_px, seg_next, spans, ctl.
constexpr size_t kSegClsBytes = 2 * 4 * kClasses;
constexpr size_t kSegClsPxBytes = 8 * kClasses;
constexpr size_t kSegNextBytes = 8 * kSegSlots;
constexpr size_t kSegSpanBytes = 24 * kSegSlots;
constexpr size_t kSegBufBytes = kSegClsBytes + kSegClsPxBytes + kSegNextBytes + kSegSpanBytes + 16;

// Device counters (int64).  The first six accumulate over every chunk of
// a map; the ones from C_ADD_DISC on describe the chunk being added and are
// reset for each chunk.
enum Ctr {
    C_KEPT = 0, C_SINGLE, C_DISC, C_DISC_BLOCK, C_DEPOSITS, C_INVALID,
    C_ADD_DISC, C_ADD_BLOCK, C_QNEXT_BLOCK, C_QNEXT_WARP,
    C_SEG_ITEMS,       // work items of the chunk's block-class discs
    C_SEG_EST,         // their estimated pixels (cap areas)
    C_SEG_NEXT_NORM,   // items claimed by pass 1
    C_SEG_MODE,        // 1: the chunk took the segmented render
    C_COUNT
};
constexpr int kCtrChunkFirst = C_ADD_DISC;

struct Particles {
    const float *x, *y, *z, *m, *rho, *h;
    int n;
    const float *sigmav;   // velocity dispersion; only the laws that use it read it
};

// Per-particle geometry written by the prep kernel (FP64).
struct PrepOut {
    double *theta, *phi, *ar, *flux;
    int *cpix;
    int *key;     // sort key, -1 for skipped / single-pixel particles
    signed char *cls;  // optional (may be null): a PClass per particle
};

// Particle classes written to PrepOut::cls.
enum PClass : signed char { PC_SKIPPED = 0, PC_INVALID = 1, PC_SINGLE = 2, PC_DISC = 3 };

// The accumulation plane: per pixel an FP64 sum.  The plain form adds the
// flux itself; the compensated form adds flux * inv_scale (its FP32
// products stay normal), which the final pass multiplies back.
struct Accum {
    double *acc64;
};

// Halo cores of the ann_core_nosom law, bucketed into a uniform grid whose
// cell is at least the largest core radius (halocore.cu).
struct HaloGrid {
    const float *hx, *hy, *hz, *hr;   // centres and radii (box units), sorted by cell
    const int *cell_start;            // [nx*ny*nz + 1], x fastest
    float ox, oy, oz, inv_cell;       // grid origin and 1 / cell size
    int nx, ny, nz, n_halos;
};

struct PrepArgs {
    Particles p;
    Frame f;
    Hpx g;
    PrepOut out;
    int *hist;                  // [kKeys]
    long long *ctr;             // [C_COUNT]
    double *flux_sum;           // [1] total kept flux
    Accum acc;
    int precision;
    int block_bucket_min;       // discs whose size bucket >= this go block-per-particle
    int deposit_singles;        // 0: classify only (the adjoint), no map deposits
    const double *core_corr;    // per-particle halo-core factor r (ann_core_nosom law)
};

struct CompHdr;   // the compensated form's per-particle disc header (disc_comp.cu)

struct DiscArgs {
    Hpx g;
    Frame f;
    RingTab rt;
    const double *theta, *phi, *ar, *flux;
    const int *cpix;
    const int *queue;           // disc particles, largest first
    long long *ctr;
    Accum acc;
    // compensated form: comp_hdr_bytes() per queue slot, filled by the disc
    // launch; null computes each header inside the disc kernels instead
    CompHdr *chdr = nullptr;
    // compensated block kernel: returns at once when *block_skip != 0 (the
    // segmented render took the chunk's block class); null = never
    const int *block_skip = nullptr;
};



// Segmented render of the block-class discs (disc_seg.cu).
struct SegArgs {
    int2 *items;              // (queue slot, item index within its disc), queue order
    int2 *sorted;             // the same items in ascending octave of the disc's F
    long long cap;            // capacity of items and sorted
    int *cls;                 // [2 kClasses]: items per octave, then each octave's first slot
    long long *cls_px;        // [kClasses]: pixels (deposits) per octave
    unsigned long long *seg_next;   // [kSegSlots]: items claimed by each segment
    SegSpan *spans;           // [kSegSlots]: the segment plan
    int *ctl;                 // [0] mode (1 segmented, 0 per-disc kernels), [1] segments
    long long min_est;        // estimated deposits from which the chunk is segmented
    long long budget;         // deposits per segment before the plan splits an octave
    long long *disc_first;    // per block-class disc: its first item
    int *disc_nitems;         //   its item count
    double *disc_S;           //   the sum of its weights (pass 1)
    long long *disc_px;       //   its pixel count (pass 1)
    float *plane;             // FP32 deposit plane, npix floats, zero between segments
};

// prep.cu
cudaError_t launch_prep(const PrepArgs &a, cudaStream_t s);
cudaError_t launch_scan(int *hist, long long *ctr, int block_bucket_min, cudaStream_t s);
cudaError_t launch_scatter(const PrepArgs &a, int *queue, cudaStream_t s);
cudaError_t launch_finalize(const Accum &acc, int precision, int npix, double dOmega,
                            double scale, double *out, int accumulate, cudaStream_t s);
// halocore.cu: corr[i] = the halo-core factor r of particle i; grad_ln
// (optional, [3][n]) = d ln r / d pos
cudaError_t launch_halo_core(const HaloGrid &g, const Particles &p, double *corr, double *grad_ln,
                             cudaStream_t s);
// disc_plain.cu / disc_comp.cu
// Launch the block-per-particle kernel, record `mid` (if not null), then the
// warp-per-particle kernel.
cudaError_t launch_disc_plain(const DiscArgs &a, int num_sms, int blocks_per_sm, cudaStream_t s,
                              cudaEvent_t mid);
// block_threads: 128, 256 or 512 (the compensated block kernel's shape;
// anything else means 256).
// headers = false: the disc headers were already built (launch_hdr).
cudaError_t launch_disc_comp(const DiscArgs &a, int num_sms, int blocks_per_sm, int block_threads,
                             cudaStream_t s, cudaEvent_t mid, bool headers = true);
size_t comp_hdr_bytes();
// the headers of every queued disc (k_comp_hdr; nothing when a.chdr is null)
cudaError_t launch_hdr(const DiscArgs &a, int num_sms, cudaStream_t s);
// the warp-per-particle compensated kernel alone (the warp class)
cudaError_t launch_disc_comp_warp(const DiscArgs &a, int num_sms, cudaStream_t s);
// disc_seg.cu, in stream order (nothing synchronises with the host, so
// the sequence can be captured in a graph): the item count of every
// block-class disc (needs the headers) and the chunk's mode; the item list
// and pass 1; the items sorted by octave and the segment plan; the
// kSegSlots deposit segments with their flushes.  block_threads 128 or 256
// picks the block shape.
cudaError_t launch_seg_count(const DiscArgs &a, const SegArgs &sg, int block_threads, int num_sms,
                             cudaStream_t s);
cudaError_t launch_seg_norm(const DiscArgs &a, const SegArgs &sg, int block_threads, int num_sms,
                            int blocks_per_sm, cudaStream_t s);
cudaError_t launch_seg_sort(const DiscArgs &a, const SegArgs &sg, int num_sms, cudaStream_t s);
cudaError_t launch_seg_deposits(const DiscArgs &a, const SegArgs &sg, int block_threads, int num_sms,
                                int blocks_per_sm, int npix, cudaStream_t s);
// disc_comp.cu: the compensated block kernel alone (headers built)
cudaError_t launch_disc_comp_block(const DiscArgs &a, int num_sms, int blocks_per_sm, int block_threads,
                                   cudaStream_t s);
// adjoint.cu: gradients of the plain-form map for dL/dmap = gmap; grad is
// [6][n] (x, y, z, m, rho, h); oacc[12] (zeroed by the caller) receives
// sum_i dL/du_i and dL/drot (row-major).  Needs the prep outputs (with cls)
// and the disc queue of the same particles and frame.
// precision: DMANN_PLAIN_F64 (FP64 weights) or DMANN_COMP_F32 (the
// compensated form's FP32 weights; gmap32 receives gmap rounded, npix floats).
cudaError_t launch_adjoint(const DiscArgs &d, const Particles &p, const signed char *cls,
                           const double *gmap, float *gmap32, double *grad, double *oacc,
                           int precision, int num_sms, cudaStream_t s,
                           const double *core_corr = nullptr, const double *core_gln = nullptr);

}  // namespace dmann
