// capi.cu -- the C ABI (include/dmann.h): contexts, device workspace, ring
// tables and the render pipeline
//   prep (geometry, filter, single-pixel deposits, size/sky keys)
//   -> key scan -> queue scatter (largest discs first)
//   -> disc kernels (block per large disc, warp per small disc)
//   -> final map pass (divide by dOmega, optional accumulate).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/dmann.h"
#include "frame.h"
#include "kernels.cuh"

using namespace dmann;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct RingTables {
    double *z = nullptr, *st = nullptr, *theta = nullptr, *step = nullptr;
    float *st32 = nullptr, *step32 = nullptr;
};

}  // namespace

// One map's device work: the prep outputs, the queue, the counters and
// accumulation planes, the disc headers and the segmented render's buffers.
// A context renders with work[0]; a batch of device maps uses both, one
// observer on each at a time.
struct Work {
    DevBuf theta, phi, ar, flux, cpix, key, queue, hist, ctr, fsum, acc;
    DevBuf chdr;              // the compensated form's disc headers, one per queue slot
    // segmented render (disc_seg.cu): work items, per-disc item ranges,
    // weight sums and pixel counts, and the FP32 deposit plane
    DevBuf seg_items, seg_sorted, seg_cls, seg_first, seg_nit, seg_S, seg_px, plane32;
    bool seg_plane = false;   // plane32 holds a zeroed plane for the open map
};

struct dmann_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evd0 = nullptr, evdm = nullptr, evd1 = nullptr;
    cudaEvent_t evp1 = nullptr;   // end of the segmented render's pass 1
    bool disc_timed = false, seg_timed = false;
    bool have_frame = false, have_units = false;
    double rot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    double opos[3] = {0, 0, 0};
    // halo centre and alignment of the last dmann_set_observer (the adjoint
    // differentiates the rotation through them); unset after dmann_set_frame
    bool have_geom = false;
    double cpos[3] = {0, 0, 0}, align[3] = {0, 0, 0};
    double unit_factor = 1.0, hires = INFINITY;
    int flux_model = DMANN_FLUX_ANN_NOSOM;
    double vel_to_cgs = 0.0, fcpos[3] = {0, 0, 0};   // dmann_set_flux_params
    dmann_tuning tune{};
    std::map<int, dmann_tuning> tune_ns;   // per-Nside overrides (the autotuner's table)
    std::map<int, RingTables> rings;
    // workspace: the staged inputs and map, the adjoint's buffers, and the
    // per-map work (w: work[0], or a batch lane's)
    DevBuf in[7], map;
    DevBuf cls, oacc, grad;   // the adjoint's class array, observer sums, staged gradient
    DevBuf core_gln;          // the adjoint's d ln(halo-core factor) / d pos, [3][n]
    Work work[2];
    Work *w = &work[0];
    cudaStream_t lane_stream = nullptr;   // the batch's second lane
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // dmann_render_batch: the instantiated graph of the last batch of device
    // maps and the parameters it was captured with (relaunched when a batch
    // repeats them), and the batch's counters summed over its observers
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<char> batch_key;
    long long batch_launches = 0;
    DevBuf bstats;
    // halo cores of the ann_core_nosom law (dmann_set_halo_cores)
    DevBuf halo_f, halo_cells, corr;
    HaloGrid halo{};
    bool have_halos = false;
    dmann_stats stats{};
    bool stats_pending = false;
    long long *h_ctr = nullptr;   // pinned: C_COUNT counters, the flux sum, 12 adjoint sums
    double *h_fsum = nullptr;
    double *h_oacc = nullptr;
    // the map being accumulated (dmann_map_begin .. dmann_map_end)
    Hpx g{};
    RingTables rt;
    int precision = DMANN_COMP_F32;
    bool in_map = false;
    int64_t launches = 0;   // kernels launched for the current / last map
    std::string err;
};

namespace {

dmann_status fail(dmann_ctx *c, dmann_status s, const std::string &msg) {
    if (c) c->err = msg;
    return s;
}

// The tuning in force for maps of `nside`: its per-Nside entry, else the
// context's default.
const dmann_tuning &tuning_for(const dmann_ctx *ctx, int nside) {
    auto it = ctx->tune_ns.find(nside);
    return it != ctx->tune_ns.end() ? it->second : ctx->tune;
}

int block_bucket_min(const dmann_tuning &t) {
    int bmin = 0;
    while (bmin < kBuckets && (1LL << bmin) <= t.warp_max_pixels) bmin++;
    return bmin;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(ctx, DMANN_ERR_CUDA,                                                      \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

// The compensated kernels' disc headers for n particles (comp_hdr_bytes()
// each, with headroom for slowly growing chunks).  Optional: without them
// the kernels compute each header themselves -- slower, the same results --
// so a failed allocation is not an error.
// Incremented by every (re)allocation of a context buffer: a captured batch
// graph holds buffer addresses, so a batch is recaptured after any.
std::atomic<unsigned long long> g_alloc_gen{0};

void reserve_headers(dmann_ctx *ctx, size_t n) {
    const size_t bytes = comp_hdr_bytes() * (n > 0 ? n : 1);
    if (ctx->w->chdr.bytes >= bytes) return;
    if (ctx->w->chdr.p) cudaFree(ctx->w->chdr.p);
    ctx->w->chdr.p = nullptr;
    ctx->w->chdr.bytes = 0;
    ++g_alloc_gen;
    for (size_t want : {bytes + bytes / 8, bytes}) {
        if (cudaMalloc(&ctx->w->chdr.p, want) == cudaSuccess) {
            ctx->w->chdr.bytes = want;
            return;
        }
        cudaGetLastError();
        ctx->w->chdr.p = nullptr;
    }
}

// An optional buffer: grows like ensure() but a failed allocation is not an
// error (the caller takes a path that does without it).
bool ensure_opt(DevBuf &b, size_t bytes) {
    if (b.bytes >= bytes) return true;
    ++g_alloc_gen;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    for (size_t want : {bytes + bytes / 8, bytes}) {
        if (cudaMalloc(&b.p, want) == cudaSuccess) {
            b.bytes = want;
            return true;
        }
        cudaGetLastError();
        b.p = nullptr;
    }
    return false;
}

CompHdr *headers_for(const dmann_ctx *ctx, size_t n) {
    const bool fits = ctx->w->chdr.p && ctx->w->chdr.bytes >= comp_hdr_bytes() * (n > 0 ? n : 1);
    return fits ? (CompHdr *)ctx->w->chdr.p : nullptr;
}

dmann_status ensure(dmann_ctx *ctx, DevBuf &b, size_t bytes) {
    if (b.bytes >= bytes) return DMANN_OK;
    ++g_alloc_gen;
    if (b.p) {
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = bytes + bytes / 8;  // headroom for slowly growing chunks
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&b.p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            b.p = nullptr;
            return fail(ctx, DMANN_ERR_NOMEM,
                        "device allocation of " + std::to_string(bytes) + " bytes failed");
        }
        want = bytes;
    }
    b.bytes = want;
    return DMANN_OK;
}

bool is_device_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

Hpx make_hpx(int nside) {
    Hpx g;
    g.nside = nside;
    g.npix = 12 * nside * nside;
    g.ncap = 2 * nside * (nside - 1);
    g.nrings = 4 * nside - 1;
    g.fact2 = 4.0 / (double)g.npix;
    g.fact1 = (double)(nside << 1) * g.fact2;
    g.dOmega = 4 * 3.14159265358979323846 / (double)g.npix;  // datatypes.h:251
    g.theta0 = std::acos(1.0 - g.dOmega / (2.0 * 3.141592));   // genmap.cpp:38
    return g;
}

// z, sin(theta) and theta of every ring, as pix2vec computes them for the
// ring's pixels (sin(theta) from 1 - z near the poles).
dmann_status ring_tables(dmann_ctx *ctx, int nside, RingTables &out) {
    auto it = ctx->rings.find(nside);
    if (it != ctx->rings.end()) {
        out = it->second;
        return DMANN_OK;
    }
    const Hpx g = make_hpx(nside);
    const int n = 4 * nside;
    std::vector<double> z(n, 0.0), st(n, 0.0), th(n, 0.0), stp(n, 0.0);
    for (int r = 1; r < n; r++) {
        bool have = false;
        double tmp = 0.0;
        if (r < nside) {
            tmp = (double)((long long)r * r) * g.fact2;
            z[r] = 1.0 - tmp;
            have = z[r] > 0.99;
        } else if (r <= 3 * nside) {
            z[r] = (double)(2 * nside - r) * g.fact1;
        } else {
            long long ir = 4LL * nside - r;
            tmp = (double)(ir * ir) * g.fact2;
            z[r] = tmp - 1.0;
            have = z[r] < -0.99;
        }
        st[r] = have ? std::sqrt(tmp * (2.0 - tmp)) : std::sqrt((1.0 - z[r]) * (1.0 + z[r]));
        th[r] = have ? std::atan2(st[r], z[r]) : std::acos(z[r]);
        const int nr = r < nside ? 4 * r : (r < 3 * nside ? 4 * nside : 4 * (4 * nside - r));
        stp[r] = 6.283185307179586476925286766559005768394 / (double)nr;
    }
    RingTables t;
    CK(cudaMalloc(&t.z, sizeof(double) * n));
    CK(cudaMalloc(&t.st, sizeof(double) * n));
    CK(cudaMalloc(&t.theta, sizeof(double) * n));
    CK(cudaMemcpy(t.z, z.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t.st, st.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t.theta, th.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&t.step, sizeof(double) * n));
    CK(cudaMemcpy(t.step, stp.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    std::vector<float> st32(n), stp32(n);
    for (int r = 0; r < n; r++) {
        st32[r] = (float)st[r];
        stp32[r] = (float)stp[r];
    }
    CK(cudaMalloc(&t.st32, sizeof(float) * n));
    CK(cudaMemcpy(t.st32, st32.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&t.step32, sizeof(float) * n));
    CK(cudaMemcpy(t.step32, stp32.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    ctx->rings[nside] = t;
    out = t;
    return DMANN_OK;
}

dmann_status collect_stats(dmann_ctx *ctx) {
    if (!ctx->stats_pending) return DMANN_OK;
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.kernel_ms = ms;
    ctx->stats.disc_ms = 0.0;
    if (ctx->disc_timed) {
        CK(cudaEventElapsedTime(&ms, ctx->evd0, ctx->evd1));
        ctx->stats.disc_ms = ms;
        CK(cudaEventElapsedTime(&ms, ctx->evd0, ctx->evdm));
        ctx->stats.disc_block_ms = ms;
        ctx->stats.disc_warp_ms = ctx->stats.disc_ms - ms;
    }
    ctx->stats.pass1_ms = ctx->stats.pass2_ms = 0.0;
    if (ctx->seg_timed && ctx->h_ctr[C_SEG_MODE] == 1) {   // the last chunk was segmented
        CK(cudaEventElapsedTime(&ms, ctx->evd0, ctx->evp1));
        ctx->stats.pass1_ms = ms;
        CK(cudaEventElapsedTime(&ms, ctx->evp1, ctx->evdm));
        ctx->stats.pass2_ms = ms;
    }
    ctx->stats.n_kept = ctx->h_ctr[C_KEPT];
    ctx->stats.n_invalid = ctx->h_ctr[C_INVALID];
    ctx->stats.n_single = ctx->h_ctr[C_SINGLE];
    ctx->stats.n_disc = ctx->h_ctr[C_DISC];
    ctx->stats.n_disc_block = ctx->h_ctr[C_DISC_BLOCK];
    ctx->stats.deposits = ctx->h_ctr[C_DEPOSITS];
    ctx->stats.total_flux = *ctx->h_fsum;
    ctx->stats.launches = ctx->launches;
    ctx->stats_pending = false;
    return DMANN_OK;
}

}  // namespace

extern "C" {

int dmann_abi_version(void) { return DMANN_ABI_VERSION; }

dmann_status dmann_create(dmann_ctx **out, int device) {
    if (!out) return DMANN_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return DMANN_ERR_NODEVICE;
    }
    if (device < 0 || device >= ndev) return DMANN_ERR_INVALID;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return DMANN_ERR_CUDA;
    if (!(prop.major == 10 && prop.minor == 3)) return DMANN_ERR_NODEVICE;  // built for sm_103a only
    dmann_ctx *ctx = new dmann_ctx();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        cudaEventCreate(&ctx->evd0) != cudaSuccess || cudaEventCreate(&ctx->evd1) != cudaSuccess ||
        cudaEventCreate(&ctx->evdm) != cudaSuccess || cudaEventCreate(&ctx->evp1) != cudaSuccess ||
        cudaHostAlloc((void **)&ctx->h_ctr, 8 * (C_COUNT + 1 + 12), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return DMANN_ERR_CUDA;
    }
    ctx->h_fsum = (double *)(ctx->h_ctr + C_COUNT);
    ctx->h_oacc = (double *)(ctx->h_ctr + C_COUNT + 1);
    ctx->stream = ctx->own;
    ctx->tune.warp_max_pixels = 1024;
    ctx->tune.block_threads = 256;
    ctx->tune.blocks_per_sm = 0;
    ctx->tune.ring_chunk = 384;
    ctx->tune.seg_min_deposits_log2 = 28;
    *out = ctx;
    return DMANN_OK;
}

void dmann_destroy(dmann_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    DevBuf *bufs[] = {&ctx->in[0], &ctx->in[1], &ctx->in[2], &ctx->in[3], &ctx->in[4], &ctx->in[5],
                      &ctx->in[6], &ctx->map, &ctx->cls, &ctx->oacc, &ctx->grad, &ctx->halo_f,
                      &ctx->halo_cells, &ctx->corr, &ctx->core_gln, &ctx->bstats};
    for (Work &wk : ctx->work) {
        DevBuf *wb[] = {&wk.theta, &wk.phi, &wk.ar, &wk.flux, &wk.cpix, &wk.key, &wk.queue, &wk.hist,
                        &wk.ctr, &wk.fsum, &wk.acc, &wk.chdr, &wk.seg_items, &wk.seg_sorted,
                        &wk.seg_cls, &wk.seg_first, &wk.seg_nit, &wk.seg_S, &wk.seg_px, &wk.plane32};
        for (DevBuf *b : wb)
            if (b->p) cudaFree(b->p);
    }
    if (ctx->lane_stream) cudaStreamDestroy(ctx->lane_stream);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
    for (DevBuf *b : bufs)
        if (b->p) cudaFree(b->p);
    for (auto &kv : ctx->rings) {
        cudaFree(kv.second.z);
        cudaFree(kv.second.st);
        cudaFree(kv.second.theta);
        cudaFree(kv.second.step);
        cudaFree(kv.second.st32);
        cudaFree(kv.second.step32);
    }
    if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->evd0) cudaEventDestroy(ctx->evd0);
    if (ctx->evd1) cudaEventDestroy(ctx->evd1);
    if (ctx->evdm) cudaEventDestroy(ctx->evdm);
    if (ctx->evp1) cudaEventDestroy(ctx->evp1);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}

const char *dmann_last_error(const dmann_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

dmann_status dmann_set_stream(dmann_ctx *ctx, void *stream) {
    if (!ctx) return DMANN_ERR_INVALID;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return DMANN_OK;
}

dmann_status dmann_synchronize(dmann_ctx *ctx) {
    if (!ctx) return DMANN_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    return DMANN_OK;
}

dmann_status dmann_set_observer(dmann_ctx *ctx, const double opos[3], const double cpos[3],
                                const double align[3]) {
    if (!ctx || !opos || !cpos || !align) return fail(ctx, DMANN_ERR_INVALID, "null argument");
    double rot[9];
    if (!observer_rotation(opos, cpos, align, rot, nullptr, nullptr))
        return fail(ctx, DMANN_ERR_INVALID, "observer position equals the halo centre");
    std::memcpy(ctx->rot, rot, sizeof rot);
    std::memcpy(ctx->opos, opos, sizeof(double) * 3);
    std::memcpy(ctx->cpos, cpos, sizeof(double) * 3);
    std::memcpy(ctx->align, align, sizeof(double) * 3);
    ctx->have_geom = true;
    ctx->have_frame = true;
    return DMANN_OK;
}

dmann_status dmann_set_frame(dmann_ctx *ctx, const double rot[9], const double opos[3]) {
    if (!ctx || !rot || !opos) return fail(ctx, DMANN_ERR_INVALID, "null argument");
    for (int i = 0; i < 9; i++)
        if (!std::isfinite(rot[i])) return fail(ctx, DMANN_ERR_INVALID, "non-finite rotation");
    std::memcpy(ctx->rot, rot, sizeof(double) * 9);
    std::memcpy(ctx->opos, opos, sizeof(double) * 3);
    ctx->have_geom = false;
    ctx->have_frame = true;
    return DMANN_OK;
}

dmann_status dmann_set_units(dmann_ctx *ctx, double unit_factor, double hires_threshold,
                             int flux_model) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (!(std::isfinite(unit_factor) && unit_factor > 0))
        return fail(ctx, DMANN_ERR_INVALID, "unit_factor must be finite and positive");
    if (flux_model < DMANN_FLUX_ANN_NOSOM || flux_model > DMANN_FLUX_ANN_CORE_NOSOM)
        return fail(ctx, DMANN_ERR_INVALID, "unknown flux model");
    ctx->unit_factor = unit_factor;
    ctx->hires = hires_threshold;
    ctx->flux_model = flux_model;
    ctx->have_units = true;
    return DMANN_OK;
}

namespace {
dmann_status merge_tuning(dmann_ctx *ctx, const dmann_tuning &t, dmann_tuning &dst) {
    if (t.block_threads != 0 && t.block_threads != 128 && t.block_threads != 256 &&
        t.block_threads != 512)
        return fail(ctx, DMANN_ERR_INVALID, "block_threads must be 128, 256 or 512");
    if (t.warp_max_pixels < 0 || t.blocks_per_sm < 0)
        return fail(ctx, DMANN_ERR_INVALID, "negative tuning value");
    if (t.seg_min_deposits_log2 < 0 || t.seg_min_deposits_log2 > 62)
        return fail(ctx, DMANN_ERR_INVALID, "seg_min_deposits_log2 must be in [1, 62]");
    if (t.seg_min_deposits_log2 > 0) dst.seg_min_deposits_log2 = t.seg_min_deposits_log2;
    if (t.warp_max_pixels > 0) dst.warp_max_pixels = t.warp_max_pixels;
    if (t.blocks_per_sm > 0) dst.blocks_per_sm = t.blocks_per_sm;
    if (t.block_threads > 0) dst.block_threads = t.block_threads;
    dst.ring_chunk = dst.block_threads == 128 ? 192 : dst.block_threads == 512 ? 640 : 384;
    return DMANN_OK;
}
}  // namespace

dmann_status dmann_set_flux_params(dmann_ctx *ctx, double velocity_to_cgs, const double cpos[3]) {
    if (!ctx || !cpos) return DMANN_ERR_INVALID;
    if (!std::isfinite(velocity_to_cgs) || !std::isfinite(cpos[0]) || !std::isfinite(cpos[1]) ||
        !std::isfinite(cpos[2]))
        return fail(ctx, DMANN_ERR_INVALID, "non-finite flux parameter");
    ctx->vel_to_cgs = velocity_to_cgs;
    std::memcpy(ctx->fcpos, cpos, sizeof(double) * 3);
    return DMANN_OK;
}

dmann_status dmann_set_halo_cores(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                                  const float *radius, int n_halos) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (n_halos < 0 || (n_halos > 0 && (!x || !y || !z || !radius)))
        return fail(ctx, DMANN_ERR_INVALID, "bad halo arrays");
    CK(cudaSetDevice(ctx->device));
    const int n = n_halos;
    // core radius in box units, held in a float as the reference passes it
    // (halocore.cpp:62-66: radius / (0.73 * 40000.0) into a float parameter)
    std::vector<float> r(n);
    float rmax = 0.0f;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const float *c[3] = {x, y, z};
    for (int i = 0; i < n; i++) {
        r[i] = (float)((double)radius[i] / (0.73 * 40000.0));
        if (!std::isfinite(r[i]) || !std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(z[i]))
            return fail(ctx, DMANN_ERR_INVALID, "non-finite halo");
        rmax = std::max(rmax, r[i]);
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], c[k][i]);
            hi[k] = std::max(hi[k], c[k][i]);
        }
    }
    HaloGrid gr{};
    gr.n_halos = n;
    if (n == 0 || !(rmax > 0.0f)) {   // no halo can contain a particle
        gr.nx = gr.ny = gr.nz = 1;
        gr.ox = gr.oy = gr.oz = 0.0f;
        gr.inv_cell = 0.0f;
        std::vector<int> cs(2, 0);
        dmann_status st = ensure(ctx, ctx->halo_cells, sizeof(int) * 2);
        if (st != DMANN_OK) return st;
        CK(cudaMemcpy(ctx->halo_cells.p, cs.data(), sizeof(int) * 2, cudaMemcpyHostToDevice));
        gr.cell_start = (const int *)ctx->halo_cells.p;
        gr.nx = 0;   // every particle falls outside
        ctx->halo = gr;
        ctx->have_halos = true;
        return DMANN_OK;
    }
    // cells of at least the largest radius (with a margin for the rounding
    // of a particle's cell index), at most 256 per axis
    float cell = rmax * 1.001f + 1e-30f;
    int dims[3];
    for (;;) {
        bool ok = true;
        for (int k = 0; k < 3; k++) {
            const double ext = (double)hi[k] - lo[k] + 2.0 * cell;
            dims[k] = (int)std::ceil(ext / cell) + 1;
            if (dims[k] > 256) ok = false;
        }
        if (ok) break;
        cell *= 1.5f;
    }
    gr.ox = lo[0] - cell;
    gr.oy = lo[1] - cell;
    gr.oz = lo[2] - cell;
    gr.inv_cell = 1.0f / cell;
    gr.nx = dims[0];
    gr.ny = dims[1];
    gr.nz = dims[2];
    const size_t ncell = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<int> cid(n), cs(ncell + 1, 0);
    for (int i = 0; i < n; i++) {
        int k3[3];
        const float o[3] = {gr.ox, gr.oy, gr.oz};
        for (int k = 0; k < 3; k++)
            k3[k] = std::min(dims[k] - 1, std::max(0, (int)((c[k][i] - o[k]) * gr.inv_cell)));
        cid[i] = (k3[2] * dims[1] + k3[1]) * dims[0] + k3[0];
        cs[cid[i] + 1]++;
    }
    for (size_t k = 0; k < ncell; k++) cs[k + 1] += cs[k];
    std::vector<float> hf(4 * (size_t)n);
    std::vector<int> fill(cs.begin(), cs.end() - 1);
    for (int i = 0; i < n; i++) {   // halos of a cell keep the table's order
        const int at = fill[cid[i]]++;
        hf[at] = x[i];
        hf[n + at] = y[i];
        hf[2 * (size_t)n + at] = z[i];
        hf[3 * (size_t)n + at] = r[i];
    }
    dmann_status st;
    if ((st = ensure(ctx, ctx->halo_f, sizeof(float) * hf.size())) ||
        (st = ensure(ctx, ctx->halo_cells, sizeof(int) * cs.size())))
        return st;
    CK(cudaMemcpy(ctx->halo_f.p, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->halo_cells.p, cs.data(), sizeof(int) * cs.size(), cudaMemcpyHostToDevice));
    const float *f = (const float *)ctx->halo_f.p;
    gr.hx = f;
    gr.hy = f + n;
    gr.hz = f + 2 * (size_t)n;
    gr.hr = f + 3 * (size_t)n;
    gr.cell_start = (const int *)ctx->halo_cells.p;
    ctx->halo = gr;
    ctx->have_halos = true;
    return DMANN_OK;
}

dmann_status dmann_set_tuning(dmann_ctx *ctx, const dmann_tuning *t) {
    if (!ctx || !t) return DMANN_ERR_INVALID;
    return merge_tuning(ctx, *t, ctx->tune);
}

dmann_status dmann_get_tuning(const dmann_ctx *ctx, dmann_tuning *t) {
    if (!ctx || !t) return DMANN_ERR_INVALID;
    *t = ctx->tune;
    return DMANN_OK;
}

dmann_status dmann_set_tuning_nside(dmann_ctx *ctx, int nside, const dmann_tuning *t) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (nside < 1 || nside > 8192) return fail(ctx, DMANN_ERR_INVALID, "nside must be in [1, 8192]");
    if (!t) {
        ctx->tune_ns.erase(nside);
        return DMANN_OK;
    }
    dmann_tuning merged = ctx->tune;
    dmann_status st = merge_tuning(ctx, *t, merged);
    if (st != DMANN_OK) return st;
    ctx->tune_ns[nside] = merged;
    return DMANN_OK;
}

dmann_status dmann_get_tuning_nside(const dmann_ctx *ctx, int nside, dmann_tuning *t) {
    if (!ctx || !t) return DMANN_ERR_INVALID;
    *t = tuning_for(ctx, nside);
    return DMANN_OK;
}

dmann_status dmann_get_stats(const dmann_ctx *ctx_c, dmann_stats *out) {
    dmann_ctx *ctx = const_cast<dmann_ctx *>(ctx_c);
    if (!ctx || !out) return DMANN_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    dmann_status s = collect_stats(ctx);
    if (s != DMANN_OK) return s;
    *out = ctx->stats;
    return DMANN_OK;
}

namespace {

dmann_status check_particles(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                             const float *m, const float *rho, const float *h, int64_t n) {
    if (n < 0 || n > (int64_t)0x7fffffff)
        return fail(ctx, DMANN_ERR_INVALID, "particle count out of range [0, 2^31)");
    if (n > 0 && (!x || !y || !z || !m || !rho || !h))
        return fail(ctx, DMANN_ERR_INVALID, "null particle array");
    return DMANN_OK;
}

Frame make_frame(const dmann_ctx *ctx, double *scale) {
    Frame f{};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) f.rot[i][j] = ctx->rot[3 * i + j];
    for (int i = 0; i < 3; i++) f.opos[i] = ctx->opos[i];
    f.unit_factor = ctx->unit_factor;
    f.hires_threshold = ctx->hires;
    int e2 = 0;
    std::frexp(ctx->unit_factor, &e2);
    f.inv_scale = std::ldexp(1.0, -e2);  // FP32 deposits hold flux / 2^e2 (exact scaling)
    *scale = std::ldexp(1.0, e2);
    f.flux_model = ctx->flux_model;
    f.vel_to_cgs = ctx->vel_to_cgs;
    for (int i = 0; i < 3; i++) f.fcpos[i] = ctx->fcpos[i];
    return f;
}

bool law_needs_sigmav(int model) {
    return model == DMANN_FLUX_ANN_SOMV || model == DMANN_FLUX_ANN_SOMV2 || model == DMANN_FLUX_ANN_PWAVE;
}

Accum make_accum(dmann_ctx *ctx) {
    Accum acc;
    acc.acc64 = (double *)ctx->w->acc.p;
    return acc;
}

// The compensated form's block-class discs in work items and segments
// (disc_seg.cu), then the warp class with the per-disc kernel.  The item
// list holds up to 4 N + 2^20 items; the device decides per chunk whether
// the segmented render or the per-disc block kernel (FP64 deposits) takes
// the block class, and both are launched -- the one not chosen returns at
// once -- so nothing here waits for the device and the sequence can be
// captured in a graph.  Needs the disc headers, the FP32 plane and the item
// buffers; without them `used` stays false and the caller renders with the
// per-disc kernels alone.
// Item slots of the segmented render: 4 n + 2^20 (items are indexed as int).
size_t seg_capacity(size_t n) {
    return std::min<size_t>(4 * (n > 0 ? n : 1) + ((size_t)1 << 20), (size_t)0x7fffffff);
}

// The segmented render's buffers for chunks of n particles (optional: false
// when an allocation fails; nothing is allocated when they are big enough).
bool reserve_seg(dmann_ctx *ctx, size_t n) {
    const size_t n1 = n > 0 ? n : 1, cap = seg_capacity(n);
    return ensure_opt(ctx->w->seg_first, 8 * n1) && ensure_opt(ctx->w->seg_nit, 4 * n1) &&
           ensure_opt(ctx->w->seg_S, 8 * n1) && ensure_opt(ctx->w->seg_px, 8 * n1) &&
           ensure_opt(ctx->w->seg_cls, kSegBufBytes) && ensure_opt(ctx->w->seg_items, 8 * cap) &&
           ensure_opt(ctx->w->seg_sorted, 8 * cap);
}

dmann_status render_segmented(dmann_ctx *ctx, const DiscArgs &da, const dmann_tuning &tu, size_t N,
                              bool &used, bool timed = true) {
    used = false;
    if (!da.chdr || !ctx->w->seg_plane || !reserve_seg(ctx, N)) return DMANN_OK;
    const size_t cap = seg_capacity(N);
    cudaStream_t s = ctx->stream;
    const int bt = tu.block_threads == 128 ? 128 : 256;
    const int lg = tu.seg_min_deposits_log2 > 0 ? tu.seg_min_deposits_log2 : 28;
    char *buf = (char *)ctx->w->seg_cls.p;
    SegArgs sg{};
    sg.items = (int2 *)ctx->w->seg_items.p;
    sg.sorted = (int2 *)ctx->w->seg_sorted.p;
    sg.cap = (long long)cap;
    sg.cls = (int *)buf;
    sg.cls_px = (long long *)(buf + kSegClsBytes);
    sg.seg_next = (unsigned long long *)(buf + kSegClsBytes + kSegClsPxBytes);
    sg.spans = (SegSpan *)(buf + kSegClsBytes + kSegClsPxBytes + kSegNextBytes);
    sg.ctl = (int *)(buf + kSegClsBytes + kSegClsPxBytes + kSegNextBytes + kSegSpanBytes);
    sg.min_est = 1LL << lg;
    sg.budget = (long long)ctx->g.npix * kDepPerPix;
    sg.disc_first = (long long *)ctx->w->seg_first.p;
    sg.disc_nitems = (int *)ctx->w->seg_nit.p;
    sg.disc_S = (double *)ctx->w->seg_S.p;
    sg.disc_px = (long long *)ctx->w->seg_px.p;
    sg.plane = (float *)ctx->w->plane32.p;
    CK(cudaMemsetAsync(buf, 0, kSegBufBytes, s));
    CK(launch_hdr(da, ctx->num_sms, s));
    CK(launch_seg_count(da, sg, bt, ctx->num_sms, s));
    CK(launch_seg_norm(da, sg, bt, ctx->num_sms, tu.blocks_per_sm, s));
    if (timed) CK(cudaEventRecord(ctx->evp1, s));
    CK(launch_seg_sort(da, sg, ctx->num_sms, s));
    CK(launch_seg_deposits(da, sg, bt, ctx->num_sms, tu.blocks_per_sm, ctx->g.npix, s));
    DiscArgs db = da;
    db.block_skip = sg.ctl;
    CK(launch_disc_comp_block(db, ctx->num_sms, tu.blocks_per_sm, tu.block_threads, s));
    if (timed) CK(cudaEventRecord(ctx->evdm, s));
    CK(launch_disc_comp_warp(da, ctx->num_sms, s));
    if (timed) ctx->seg_timed = true;
    // prep, scan, scatter, headers, item count, mode, item fill, pass 1,
    // octave histogram, scan, sort, plan, kSegSlots x (deposits, flush),
    // per-disc block kernel, warp class
    ctx->launches += 14 + 2 * kSegSlots;
    used = true;
    return DMANN_OK;
}

}  // namespace

// Every context call that uses the accumulation planes, the queue or the
// counters refuses to run while a streamed map is open: it would zero or
// reuse the buffers the open map is accumulating into.
const char *const map_open_msg =
    "a streamed map is in progress: dmann_map_end or dmann_map_abort it first";

dmann_status dmann_map_begin(dmann_ctx *ctx, int nside, int precision) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (nside < 1 || nside > 8192) return fail(ctx, DMANN_ERR_INVALID, "nside must be in [1, 8192]");
    if (precision != DMANN_PLAIN_F64 && precision != DMANN_COMP_F32)
        return fail(ctx, DMANN_ERR_INVALID, "unknown precision form");
    if (!ctx->have_frame) return fail(ctx, DMANN_ERR_STATE, "observer frame not set");
    if (!ctx->have_units) return fail(ctx, DMANN_ERR_STATE, "units not set");
    if (ctx->in_map) return fail(ctx, DMANN_ERR_STATE, map_open_msg);
    CK(cudaSetDevice(ctx->device));
    dmann_status st = collect_stats(ctx);
    if (st != DMANN_OK) return st;
    ctx->g = make_hpx(nside);
    ctx->precision = precision;
    if ((st = ring_tables(ctx, nside, ctx->rt)) != DMANN_OK) return st;
    const size_t P = (size_t)ctx->g.npix;
    if ((st = ensure(ctx, ctx->w->acc, 8 * P)) || (st = ensure(ctx, ctx->w->hist, 4 * (size_t)kKeys)) ||
        (st = ensure(ctx, ctx->w->ctr, 8 * C_COUNT)) || (st = ensure(ctx, ctx->w->fsum, 8)))
        return st;
    cudaStream_t s = ctx->stream;
    CK(cudaEventRecord(ctx->ev0, s));
    CK(cudaMemsetAsync(ctx->w->acc.p, 0, 8 * P, s));
    CK(cudaMemsetAsync(ctx->w->ctr.p, 0, 8 * C_COUNT, s));
    CK(cudaMemsetAsync(ctx->w->fsum.p, 0, 8, s));
    // the segmented render's FP32 plane: zero at the start of a map, and
    // every segment's flush leaves it zero
    ctx->w->seg_plane = precision == DMANN_COMP_F32 && ensure_opt(ctx->w->plane32, 4 * P);
    if (ctx->w->seg_plane) CK(cudaMemsetAsync(ctx->w->plane32.p, 0, 4 * P, s));
    ctx->stats = dmann_stats{};
    ctx->launches = 0;
    ctx->disc_timed = false;
    ctx->seg_timed = false;
    ctx->in_map = true;
    return DMANN_OK;
}

dmann_status dmann_map_add(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                           const float *m, const float *rho, const float *h, int64_t n) {
    return dmann_map_add_v(ctx, x, y, z, m, rho, h, nullptr, n);
}

dmann_status dmann_map_add_v(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                             const float *m, const float *rho, const float *h,
                             const float *sigmav, int64_t n) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (!ctx->in_map) return fail(ctx, DMANN_ERR_STATE, "dmann_map_add outside begin/end");
    dmann_status st = check_particles(ctx, x, y, z, m, rho, h, n);
    if (st != DMANN_OK) return st;
    if (n > 0 && !sigmav && law_needs_sigmav(ctx->flux_model))
        return fail(ctx, DMANN_ERR_INVALID, "this flux law needs the velocity dispersion (dmann_map_add_v)");
    ctx->stats.n_in += n;
    if (n == 0) return DMANN_OK;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t N = (size_t)n;
    if ((st = ensure(ctx, ctx->w->theta, 8 * N)) || (st = ensure(ctx, ctx->w->phi, 8 * N)) ||
        (st = ensure(ctx, ctx->w->ar, 8 * N)) || (st = ensure(ctx, ctx->w->flux, 8 * N)) ||
        (st = ensure(ctx, ctx->w->cpix, 4 * N)) || (st = ensure(ctx, ctx->w->key, 4 * N)) ||
        (st = ensure(ctx, ctx->w->queue, 4 * N)))
        return st;
    if (ctx->precision == DMANN_COMP_F32) reserve_headers(ctx, N);
    // inputs: device pointers are used in place, host arrays are copied
    const float *src[7] = {x, y, z, m, rho, h, law_needs_sigmav(ctx->flux_model) ? sigmav : nullptr};
    const float *dev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < 7; k++) {
        if (!src[k]) continue;
        if (is_device_ptr(src[k])) {
            dev[k] = src[k];
        } else {
            if ((st = ensure(ctx, ctx->in[k], 4 * N)) != DMANN_OK) return st;
            CK(cudaMemcpyAsync(ctx->in[k].p, src[k], 4 * N, cudaMemcpyHostToDevice, s));
            dev[k] = (const float *)ctx->in[k].p;
        }
    }
    double scale;
    const Frame f = make_frame(ctx, &scale);
    const Accum acc = make_accum(ctx);
    const dmann_tuning &tu = tuning_for(ctx, ctx->g.nside);
    const int bmin = block_bucket_min(tu);

    CK(cudaMemsetAsync(ctx->w->hist.p, 0, 4 * (size_t)kKeys, s));
    CK(cudaMemsetAsync((long long *)ctx->w->ctr.p + kCtrChunkFirst, 0, 8 * (C_COUNT - kCtrChunkFirst), s));
    PrepArgs pa;
    pa.p = {dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], (int)N, dev[6]};
    pa.core_corr = nullptr;
    if (ctx->flux_model == DMANN_FLUX_ANN_CORE_NOSOM) {
        if (!ctx->have_halos) return fail(ctx, DMANN_ERR_STATE, "halo cores not set (dmann_set_halo_cores)");
        if ((st = ensure(ctx, ctx->corr, 8 * N)) != DMANN_OK) return st;
        CK(launch_halo_core(ctx->halo, pa.p, (double *)ctx->corr.p, nullptr, s));
        pa.core_corr = (const double *)ctx->corr.p;
        ctx->launches++;
    }
    pa.f = f;
    pa.g = ctx->g;
    pa.out = {(double *)ctx->w->theta.p, (double *)ctx->w->phi.p, (double *)ctx->w->ar.p,
              (double *)ctx->w->flux.p, (int *)ctx->w->cpix.p, (int *)ctx->w->key.p};
    pa.hist = (int *)ctx->w->hist.p;
    pa.ctr = (long long *)ctx->w->ctr.p;
    pa.flux_sum = (double *)ctx->w->fsum.p;
    pa.acc = acc;
    pa.precision = ctx->precision;
    pa.block_bucket_min = bmin;
    pa.deposit_singles = 1;
    CK(launch_prep(pa, s));
    CK(launch_scan(pa.hist, pa.ctr, bmin, s));
    CK(launch_scatter(pa, (int *)ctx->w->queue.p, s));

    DiscArgs da;
    da.g = ctx->g;
    da.f = f;
    da.rt = {ctx->rt.z, ctx->rt.st, ctx->rt.theta, ctx->rt.step, ctx->rt.st32, ctx->rt.step32};
    da.theta = pa.out.theta;
    da.phi = pa.out.phi;
    da.ar = pa.out.ar;
    da.flux = pa.out.flux;
    da.cpix = pa.out.cpix;
    da.queue = (const int *)ctx->w->queue.p;
    da.ctr = pa.ctr;
    da.acc = acc;
    if (ctx->precision == DMANN_COMP_F32) da.chdr = headers_for(ctx, N);
    CK(cudaEventRecord(ctx->evd0, s));
    if (ctx->precision == DMANN_PLAIN_F64) {
        CK(launch_disc_plain(da, ctx->num_sms, tu.blocks_per_sm, s, ctx->evdm));
        ctx->launches += 5;   // prep, scan, scatter, disc block, disc warp
    } else {
        bool seg = false;
        if ((st = render_segmented(ctx, da, tu, N, seg)) != DMANN_OK) return st;
        if (!seg) {
            CK(launch_disc_comp(da, ctx->num_sms, tu.blocks_per_sm, tu.block_threads, s, ctx->evdm));
            ctx->launches += 5 + (da.chdr ? 1 : 0);   // prep, scan, scatter, headers, block, warp
        }
    }
    CK(cudaEventRecord(ctx->evd1, s));
    ctx->disc_timed = true;
    return DMANN_OK;
}

dmann_status dmann_map_end(dmann_ctx *ctx, double *map_out, int accumulate) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (!ctx->in_map) return fail(ctx, DMANN_ERR_STATE, "dmann_map_end without dmann_map_begin");
    if (!map_out) return fail(ctx, DMANN_ERR_INVALID, "map_out is null");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t P = (size_t)ctx->g.npix;
    dmann_status st;
    const bool map_dev = is_device_ptr(map_out);
    double *dmap = map_out;
    if (!map_dev) {
        if ((st = ensure(ctx, ctx->map, 8 * P)) != DMANN_OK) return st;
        dmap = (double *)ctx->map.p;
        if (accumulate) CK(cudaMemcpyAsync(dmap, map_out, 8 * P, cudaMemcpyHostToDevice, s));
    }
    double scale;
    (void)make_frame(ctx, &scale);
    CK(launch_finalize(make_accum(ctx), ctx->precision, ctx->g.npix, ctx->g.dOmega, scale, dmap,
                       accumulate, s));
    ctx->launches++;
    CK(cudaEventRecord(ctx->ev1, s));
    CK(cudaMemcpyAsync(ctx->h_ctr, ctx->w->ctr.p, 8 * C_COUNT, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctx->h_fsum, ctx->w->fsum.p, 8, cudaMemcpyDeviceToHost, s));
    ctx->stats_pending = true;
    ctx->in_map = false;
    if (!map_dev) {
        CK(cudaMemcpyAsync(map_out, dmap, 8 * P, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    return DMANN_OK;
}

dmann_status dmann_map_abort(dmann_ctx *ctx) {
    if (!ctx) return DMANN_ERR_INVALID;
    ctx->in_map = false;
    return DMANN_OK;
}

dmann_status dmann_render(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                          const float *m, const float *rho, const float *h, int64_t n, int nside,
                          int precision, double *map_out, int accumulate) {
    return dmann_render_v(ctx, x, y, z, m, rho, h, nullptr, n, nside, precision, map_out, accumulate);
}

dmann_status dmann_render_v(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                            const float *m, const float *rho, const float *h, const float *sigmav,
                            int64_t n, int nside, int precision, double *map_out, int accumulate) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (!map_out) return fail(ctx, DMANN_ERR_INVALID, "map_out is null");
    dmann_status st = check_particles(ctx, x, y, z, m, rho, h, n);
    if (st != DMANN_OK) return st;
    if ((st = dmann_map_begin(ctx, nside, precision)) != DMANN_OK) return st;
    if ((st = dmann_map_add_v(ctx, x, y, z, m, rho, h, sigmav, n)) != DMANN_OK) {
        ctx->in_map = false;
        return st;
    }
    return dmann_map_end(ctx, map_out, accumulate);
}

}  // extern "C"

namespace {

// Issues one observer's map into dmap (device) on the context's stream:
// zero the planes, prep, key scan, queue scatter, disc kernels, finalize.
// The workspace and the ring table must already exist: nothing here
// allocates or synchronises, so the sequence can be captured in a graph.
// Adds one observer's counters into the batch's sums (ctx->bstats: kept,
// invalid, single, disc, block-class, deposits, then the kept flux).
__global__ void k_batch_stats(const long long *ctr, const double *fsum, long long *out) {
    // atomics: the two lanes of a batch add concurrently
    const int idx[6] = {C_KEPT, C_INVALID, C_SINGLE, C_DISC, C_DISC_BLOCK, C_DEPOSITS};
    for (int i = 0; i < 6; i++)
        atomicAdd(reinterpret_cast<unsigned long long *>(out) + i, (unsigned long long)ctr[idx[i]]);
    atomicAdd(reinterpret_cast<double *>(out) + 6, *fsum);
}

constexpr int kBatchStats = 7;

dmann_status issue_observer(dmann_ctx *ctx, const float *const dev[6], int n, int nside,
                            const RingTables &rt, int precision, double *dmap) {
    cudaStream_t s = ctx->stream;
    ctx->g = make_hpx(nside);
    ctx->precision = precision;
    const size_t P = (size_t)ctx->g.npix;
    CK(cudaMemsetAsync(ctx->w->acc.p, 0, 8 * P, s));
    CK(cudaMemsetAsync(ctx->w->ctr.p, 0, 8 * C_COUNT, s));
    CK(cudaMemsetAsync(ctx->w->fsum.p, 0, 8, s));
    double scale;
    const Frame f = make_frame(ctx, &scale);
    const Accum acc = make_accum(ctx);
    if (n > 0) {
        const dmann_tuning &tu = tuning_for(ctx, nside);
        const int bmin = block_bucket_min(tu);
        CK(cudaMemsetAsync(ctx->w->hist.p, 0, 4 * (size_t)kKeys, s));
        PrepArgs pa;
        pa.p = {dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], n};
        pa.core_corr = (const double *)ctx->corr.p;   // filled once per batch (core law)
        pa.f = f;
        pa.g = ctx->g;
        pa.out = {(double *)ctx->w->theta.p, (double *)ctx->w->phi.p, (double *)ctx->w->ar.p,
                  (double *)ctx->w->flux.p, (int *)ctx->w->cpix.p, (int *)ctx->w->key.p};
        pa.hist = (int *)ctx->w->hist.p;
        pa.ctr = (long long *)ctx->w->ctr.p;
        pa.flux_sum = (double *)ctx->w->fsum.p;
        pa.acc = acc;
        pa.precision = precision;
        pa.block_bucket_min = bmin;
        pa.deposit_singles = 1;
        CK(launch_prep(pa, s));
        CK(launch_scan(pa.hist, pa.ctr, bmin, s));
        CK(launch_scatter(pa, (int *)ctx->w->queue.p, s));
        DiscArgs da;
        da.g = ctx->g;
        da.f = f;
        da.rt = {rt.z, rt.st, rt.theta, rt.step, rt.st32, rt.step32};
        da.theta = pa.out.theta;
        da.phi = pa.out.phi;
        da.ar = pa.out.ar;
        da.flux = pa.out.flux;
        da.cpix = pa.out.cpix;
        da.queue = (const int *)ctx->w->queue.p;
        da.ctr = pa.ctr;
        da.acc = acc;
        if (precision == DMANN_PLAIN_F64) {
            CK(launch_disc_plain(da, ctx->num_sms, tu.blocks_per_sm, s, nullptr));
        } else {
            da.chdr = headers_for(ctx, (size_t)n);
            bool seg = false;
            dmann_status st = render_segmented(ctx, da, tu, (size_t)n, seg, false);
            if (st != DMANN_OK) return st;
            if (!seg) CK(launch_disc_comp(da, ctx->num_sms, tu.blocks_per_sm, tu.block_threads, s, nullptr));
        }
    }
    CK(launch_finalize(acc, precision, ctx->g.npix, ctx->g.dOmega, scale, dmap, 0, s));
    k_batch_stats<<<1, 1, 0, s>>>((const long long *)ctx->w->ctr.p, (const double *)ctx->w->fsum.p,
                                  (long long *)ctx->bstats.p);
    CK(cudaGetLastError());
    return DMANN_OK;
}

}  // namespace

extern "C" {

dmann_status dmann_render_batch(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                                const float *m, const float *rho, const float *h, int64_t n,
                                int n_obs, const double *rot, const double *opos,
                                const int *nside, int precision, double *const *maps) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (n_obs < 1 || !rot || !opos || !nside || !maps)
        return fail(ctx, DMANN_ERR_INVALID, "batch needs n_obs >= 1 and rot/opos/nside/maps");
    if (precision != DMANN_PLAIN_F64 && precision != DMANN_COMP_F32)
        return fail(ctx, DMANN_ERR_INVALID, "unknown precision form");
    if (!ctx->have_units) return fail(ctx, DMANN_ERR_STATE, "units not set");
    if (ctx->in_map) return fail(ctx, DMANN_ERR_STATE, map_open_msg);
    if (law_needs_sigmav(ctx->flux_model))
        return fail(ctx, DMANN_ERR_INVALID, "the batch takes no velocity dispersion: render this flux law per observer");
    dmann_status st = check_particles(ctx, x, y, z, m, rho, h, n);
    if (st != DMANN_OK) return st;
    int maxns = 0;
    for (int k = 0; k < n_obs; k++) {
        if (nside[k] < 1 || nside[k] > 8192) return fail(ctx, DMANN_ERR_INVALID, "nside must be in [1, 8192]");
        if (!maps[k]) return fail(ctx, DMANN_ERR_INVALID, "null output map");
        for (int i = 0; i < 9; i++)
            if (!std::isfinite(rot[9 * k + i])) return fail(ctx, DMANN_ERR_INVALID, "non-finite rotation");
        maxns = std::max(maxns, nside[k]);
    }
    CK(cudaSetDevice(ctx->device));
    if ((st = collect_stats(ctx)) != DMANN_OK) return st;
    cudaStream_t s = ctx->stream;
    const size_t N = (size_t)n, n1 = N > 0 ? N : 1, Pmax = 12 * (size_t)maxns * (size_t)maxns;
    // device maps: the observers alternate between two workspaces (lanes),
    // each on its own stream in the captured graph, so one observer's prep and
    // the tails of its passes overlap the other's work
    std::vector<char> on_dev(n_obs);
    bool all_dev = true;
    for (int k = 0; k < n_obs; k++) all_dev &= (on_dev[k] = is_device_ptr(maps[k])) != 0;
    int lanes = (all_dev && n_obs > 1) ? 2 : 1;
    if (lanes == 2 && !ctx->lane_stream &&
        (cudaStreamCreateWithFlags(&ctx->lane_stream, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess)) {
        cudaGetLastError();
        lanes = 1;
    }
    // everything is sized and uploaded before the observers are issued
    if ((st = ensure(ctx, ctx->map, 8 * Pmax)) || (st = ensure(ctx, ctx->bstats, 8 * kBatchStats))) return st;
    for (int L = 0; L < lanes; L++) {
        ctx->w = &ctx->work[L];
        st = DMANN_OK;
        if ((st = ensure(ctx, ctx->w->theta, 8 * n1)) || (st = ensure(ctx, ctx->w->phi, 8 * n1)) ||
            (st = ensure(ctx, ctx->w->ar, 8 * n1)) || (st = ensure(ctx, ctx->w->flux, 8 * n1)) ||
            (st = ensure(ctx, ctx->w->cpix, 4 * n1)) || (st = ensure(ctx, ctx->w->key, 4 * n1)) ||
            (st = ensure(ctx, ctx->w->queue, 4 * n1)) || (st = ensure(ctx, ctx->w->hist, 4 * (size_t)kKeys)) ||
            (st = ensure(ctx, ctx->w->ctr, 8 * C_COUNT)) || (st = ensure(ctx, ctx->w->fsum, 8)) ||
            (st = ensure(ctx, ctx->w->acc, 8 * Pmax))) {
            ctx->w = &ctx->work[0];
            if (L == 0) return st;
            lanes = 1;   // no room for a second workspace: one lane
            break;
        }
        // before any capture: the disc headers and the segmented render's
        // buffers (the render checks them again and allocates nothing when
        // they fit)
        ctx->w->seg_plane = false;
        if (precision == DMANN_COMP_F32) {
            reserve_headers(ctx, n1);
            ctx->w->seg_plane = ensure_opt(ctx->w->plane32, 4 * Pmax) && reserve_seg(ctx, N);
            if (ctx->w->seg_plane) CK(cudaMemsetAsync(ctx->w->plane32.p, 0, 4 * Pmax, s));
        }
    }
    ctx->w = &ctx->work[0];
    std::vector<RingTables> rts(n_obs);
    for (int k = 0; k < n_obs; k++)
        if ((st = ring_tables(ctx, nside[k], rts[k])) != DMANN_OK) return st;
    const float *src[6] = {x, y, z, m, rho, h};
    const float *dev[6];
    for (int k = 0; k < 6; k++) {
        if (N == 0 || is_device_ptr(src[k])) {
            dev[k] = src[k];
        } else {
            if ((st = ensure(ctx, ctx->in[k], 4 * N)) != DMANN_OK) return st;
            CK(cudaMemcpyAsync(ctx->in[k].p, src[k], 4 * N, cudaMemcpyHostToDevice, s));
            dev[k] = (const float *)ctx->in[k].p;
        }
    }
    if (ctx->flux_model == DMANN_FLUX_ANN_CORE_NOSOM) {   // observer-independent: once
        if (!ctx->have_halos) return fail(ctx, DMANN_ERR_STATE, "halo cores not set (dmann_set_halo_cores)");
        if ((st = ensure(ctx, ctx->corr, 8 * n1)) != DMANN_OK) return st;
        Particles pp = {dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], (int)N};
        CK(launch_halo_core(ctx->halo, pp, (double *)ctx->corr.p, nullptr, s));
    }
    // the parameters a captured graph depends on: a batch that repeats them
    // relaunches the cached graph instead of capturing again
    std::vector<char> key;
    auto put = [&key](const void *p, size_t nb) {
        key.insert(key.end(), (const char *)p, (const char *)p + nb);
    };
    const unsigned long long gen = g_alloc_gen.load();
    put(&gen, sizeof gen);
    put(&n, sizeof n);
    put(&n_obs, sizeof n_obs);
    put(&precision, sizeof precision);
    put(dev, sizeof dev);
    put(nside, sizeof(int) * n_obs);
    put(rot, sizeof(double) * 9 * n_obs);
    put(opos, sizeof(double) * 3 * n_obs);
    put(maps, sizeof(double *) * n_obs);
    put(&ctx->unit_factor, sizeof ctx->unit_factor);
    put(&ctx->hires, sizeof ctx->hires);
    put(&ctx->flux_model, sizeof ctx->flux_model);
    put(&ctx->vel_to_cgs, sizeof ctx->vel_to_cgs);
    put(ctx->fcpos, sizeof ctx->fcpos);
    put(&lanes, sizeof lanes);
    for (int L = 0; L < lanes; L++) put(&ctx->work[L].seg_plane, sizeof(bool));
    for (int k = 0; k < n_obs; k++) put(&tuning_for(ctx, nside[k]), sizeof(dmann_tuning));
    double rot0[9], opos0[3];
    std::memcpy(rot0, ctx->rot, sizeof rot0);
    std::memcpy(opos0, ctx->opos, sizeof opos0);
    const bool had_frame = ctx->have_frame, had_geom = ctx->have_geom;
    // device maps: the whole batch is captured into one CUDA graph (kept and
    // relaunched while the batch's parameters repeat); host maps go through
    // the context's staging map.  The graph runs on the context's own stream
    // (a caller's stream may be the legacy default stream, which cannot be
    // captured), fenced to the caller's stream with events on both sides.
    const cudaStream_t caller = s;
    const long long launches0 = ctx->launches;
    ctx->launches = 0;
    if (all_dev) {
        if (s != ctx->own) {
            CK(cudaEventRecord(ctx->evdm, s));
            CK(cudaStreamWaitEvent(ctx->own, ctx->evdm, 0));
        }
        s = ctx->own;
    }
    const bool cached = all_dev && ctx->batch_exec && key == ctx->batch_key;
    cudaGraph_t graph = nullptr;
    if (!cached) {
        if (all_dev) {
            ctx->stream = s;
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        }
        cudaError_t e = cudaMemsetAsync(ctx->bstats.p, 0, 8 * kBatchStats, s);
        if (e != cudaSuccess) st = fail(ctx, DMANN_ERR_CUDA, std::string("batch: ") + cudaGetErrorString(e));
        if (st == DMANN_OK && lanes == 2) {   // the second lane joins the capture
            e = cudaEventRecord(ctx->ev_fork, s);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->lane_stream, ctx->ev_fork, 0);
            if (e != cudaSuccess) st = fail(ctx, DMANN_ERR_CUDA, std::string("batch fork: ") + cudaGetErrorString(e));
        }
        for (int k = 0; k < n_obs && st == DMANN_OK; k++) {
            std::memcpy(ctx->rot, rot + 9 * k, sizeof(double) * 9);
            std::memcpy(ctx->opos, opos + 3 * k, sizeof(double) * 3);
            double *dmap = on_dev[k] ? maps[k] : (double *)ctx->map.p;
            const int L = k % lanes;
            ctx->w = &ctx->work[L];
            ctx->stream = L == 0 ? s : ctx->lane_stream;
            st = issue_observer(ctx, dev, (int)N, nside[k], rts[k], precision, dmap);
            ctx->w = &ctx->work[0];
            ctx->stream = s;
            if (st == DMANN_OK && !on_dev[k]) {
                const size_t P = 12 * (size_t)nside[k] * (size_t)nside[k];
                e = cudaMemcpyAsync(maps[k], dmap, 8 * P, cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) st = fail(ctx, DMANN_ERR_CUDA, std::string("batch copy: ") + cudaGetErrorString(e));
            }
        }
        std::memcpy(ctx->rot, rot0, sizeof rot0);
        std::memcpy(ctx->opos, opos0, sizeof opos0);
        ctx->have_frame = had_frame;
        ctx->have_geom = had_geom;
        if (lanes == 2) {   // join the second lane before the capture ends
            cudaError_t ej = cudaEventRecord(ctx->ev_join, ctx->lane_stream);
            if (ej == cudaSuccess) ej = cudaStreamWaitEvent(s, ctx->ev_join, 0);
            if (ej != cudaSuccess && st == DMANN_OK)
                st = fail(ctx, DMANN_ERR_CUDA, std::string("batch join: ") + cudaGetErrorString(ej));
        }
        if (all_dev) {
            e = cudaStreamEndCapture(s, &graph);
            ctx->stream = caller;
            if (st != DMANN_OK) {
                if (graph) cudaGraphDestroy(graph);
                ctx->launches = launches0;
                return st;
            }
            if (e != cudaSuccess) return fail(ctx, DMANN_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
            // same topology (new frames, maps or units): update the kept
            // graph in place; else instantiate afresh
            bool updated = false;
            if (ctx->batch_exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(ctx->batch_exec, graph, &info) == cudaSuccess;
                if (!updated) {
                    cudaGetLastError();
                    cudaGraphExecDestroy(ctx->batch_exec);
                    ctx->batch_exec = nullptr;
                }
            }
            if (!updated) e = cudaGraphInstantiate(&ctx->batch_exec, graph, 0);
            cudaGraphDestroy(graph);
            ctx->batch_key.clear();
            if (e != cudaSuccess) {
                ctx->batch_exec = nullptr;
                return fail(ctx, DMANN_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
            }
            ctx->batch_key = key;
            ctx->batch_launches = ctx->launches;
        }
    }
    if (st != DMANN_OK) return st;
    if (all_dev) {
        cudaError_t e = cudaEventRecord(ctx->ev0, s);
        if (e == cudaSuccess) e = cudaGraphLaunch(ctx->batch_exec, s);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(ctx, DMANN_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
        ctx->launches = ctx->batch_launches;
    } else {
        CK(cudaStreamSynchronize(s));
    }
    // the batch's counters: summed over its observers
    long long hb[kBatchStats];
    CK(cudaMemcpy(hb, ctx->bstats.p, sizeof hb, cudaMemcpyDeviceToHost));
    ctx->stats = dmann_stats{};
    ctx->stats.n_in = n * n_obs;
    ctx->stats.n_kept = hb[0];
    ctx->stats.n_invalid = hb[1];
    ctx->stats.n_single = hb[2];
    ctx->stats.n_disc = hb[3];
    ctx->stats.n_disc_block = hb[4];
    ctx->stats.deposits = hb[5];
    std::memcpy(&ctx->stats.total_flux, &hb[6], sizeof(double));
    if (all_dev) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        ctx->stats.kernel_ms = ms;
    }
    ctx->stats.launches = ctx->launches;
    return DMANN_OK;
}

dmann_status dmann_adjoint(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                           const float *m, const float *rho, const float *h, int64_t n, int nside,
                           int precision, const double *grad_map, double *grad,
                           double grad_opos[3]) {
    return dmann_adjoint_v(ctx, x, y, z, m, rho, h, nullptr, n, nside, precision, grad_map, grad,
                           grad_opos);
}

dmann_status dmann_adjoint_v(dmann_ctx *ctx, const float *x, const float *y, const float *z,
                             const float *m, const float *rho, const float *h, const float *sigmav,
                             int64_t n, int nside, int precision, const double *grad_map,
                             double *grad, double grad_opos[3]) {
    if (!ctx) return DMANN_ERR_INVALID;
    if (precision != DMANN_PLAIN_F64 && precision != DMANN_COMP_F32)
        return fail(ctx, DMANN_ERR_INVALID, "unknown precision form");
    if (!grad_map || !grad || !grad_opos)
        return fail(ctx, DMANN_ERR_INVALID, "grad_map, grad and grad_opos are required");
    if (nside < 1 || nside > 8192) return fail(ctx, DMANN_ERR_INVALID, "nside must be in [1, 8192]");
    if (!ctx->have_frame) return fail(ctx, DMANN_ERR_STATE, "observer frame not set");
    if (!ctx->have_units) return fail(ctx, DMANN_ERR_STATE, "units not set");
    if (ctx->in_map) return fail(ctx, DMANN_ERR_STATE, map_open_msg);
    dmann_status st = check_particles(ctx, x, y, z, m, rho, h, n);
    if (st != DMANN_OK) return st;
    if (n > 0 && !sigmav && law_needs_sigmav(ctx->flux_model))
        return fail(ctx, DMANN_ERR_INVALID, "this flux law needs the velocity dispersion (dmann_adjoint_v)");
    const bool core = ctx->flux_model == DMANN_FLUX_ANN_CORE_NOSOM;
    if (core && !ctx->have_halos) return fail(ctx, DMANN_ERR_STATE, "halo cores not set (dmann_set_halo_cores)");
    CK(cudaSetDevice(ctx->device));
    if ((st = collect_stats(ctx)) != DMANN_OK) return st;
    cudaStream_t s = ctx->stream;
    const Hpx g = make_hpx(nside);
    const size_t N = (size_t)n, n1 = N > 0 ? N : 1, P = (size_t)g.npix;
    RingTables rt;
    if ((st = ring_tables(ctx, nside, rt)) != DMANN_OK) return st;
    if ((st = ensure(ctx, ctx->w->theta, 8 * n1)) || (st = ensure(ctx, ctx->w->phi, 8 * n1)) ||
        (st = ensure(ctx, ctx->w->ar, 8 * n1)) || (st = ensure(ctx, ctx->w->flux, 8 * n1)) ||
        (st = ensure(ctx, ctx->w->cpix, 4 * n1)) || (st = ensure(ctx, ctx->w->key, 4 * n1)) ||
        (st = ensure(ctx, ctx->w->queue, 4 * n1)) || (st = ensure(ctx, ctx->cls, n1)) ||
        (st = ensure(ctx, ctx->w->hist, 4 * (size_t)kKeys)) || (st = ensure(ctx, ctx->w->ctr, 8 * C_COUNT)) ||
        (st = ensure(ctx, ctx->w->fsum, 8)) || (st = ensure(ctx, ctx->oacc, 8 * 12)))
        return st;
    if (core && ((st = ensure(ctx, ctx->corr, 8 * n1)) || (st = ensure(ctx, ctx->core_gln, 24 * n1))))
        return st;
    if (precision == DMANN_COMP_F32) {
        if ((st = ensure(ctx, ctx->w->acc, 4 * P)) != DMANN_OK) return st;
        reserve_headers(ctx, n1);
    }
    const float *src[7] = {x, y, z, m, rho, h, law_needs_sigmav(ctx->flux_model) ? sigmav : nullptr};
    const float *dev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < 7; k++) {
        if (!src[k]) continue;
        if (N == 0 || is_device_ptr(src[k])) {
            dev[k] = src[k];
        } else {
            if ((st = ensure(ctx, ctx->in[k], 4 * N)) != DMANN_OK) return st;
            CK(cudaMemcpyAsync(ctx->in[k].p, src[k], 4 * N, cudaMemcpyHostToDevice, s));
            dev[k] = (const float *)ctx->in[k].p;
        }
    }
    const double *dgmap = grad_map;
    if (!is_device_ptr(grad_map)) {
        if ((st = ensure(ctx, ctx->map, 8 * P)) != DMANN_OK) return st;
        CK(cudaMemcpyAsync(ctx->map.p, grad_map, 8 * P, cudaMemcpyHostToDevice, s));
        dgmap = (const double *)ctx->map.p;
    }
    const bool grad_dev = is_device_ptr(grad);
    double *dgrad = grad;
    if (!grad_dev) {
        if ((st = ensure(ctx, ctx->grad, 48 * n1)) != DMANN_OK) return st;
        dgrad = (double *)ctx->grad.p;
    }
    double scale;
    const Frame f = make_frame(ctx, &scale);
    const int bmin = block_bucket_min(ctx->tune);
    CK(cudaEventRecord(ctx->ev0, s));
    CK(cudaMemsetAsync(ctx->w->ctr.p, 0, 8 * C_COUNT, s));
    CK(cudaMemsetAsync(ctx->w->fsum.p, 0, 8, s));
    CK(cudaMemsetAsync(ctx->oacc.p, 0, 8 * 12, s));
    CK(cudaMemsetAsync(ctx->w->hist.p, 0, 4 * (size_t)kKeys, s));
    PrepArgs pa;
    pa.p = {dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], (int)N, dev[6]};
    pa.f = f;
    pa.g = g;
    pa.out = {(double *)ctx->w->theta.p, (double *)ctx->w->phi.p, (double *)ctx->w->ar.p,
              (double *)ctx->w->flux.p, (int *)ctx->w->cpix.p, (int *)ctx->w->key.p,
              (signed char *)ctx->cls.p};
    pa.hist = (int *)ctx->w->hist.p;
    pa.ctr = (long long *)ctx->w->ctr.p;
    pa.flux_sum = (double *)ctx->w->fsum.p;
    pa.acc = Accum{nullptr};
    pa.precision = DMANN_PLAIN_F64;
    pa.block_bucket_min = bmin;
    pa.deposit_singles = 0;
    pa.core_corr = nullptr;
    if (core) {   // the law's factor and its position gradient
        CK(launch_halo_core(ctx->halo, pa.p, (double *)ctx->corr.p, (double *)ctx->core_gln.p, s));
        pa.core_corr = (const double *)ctx->corr.p;
    }
    CK(launch_prep(pa, s));
    CK(launch_scan(pa.hist, pa.ctr, bmin, s));
    CK(launch_scatter(pa, (int *)ctx->w->queue.p, s));
    DiscArgs da;
    da.g = g;
    da.f = f;
    da.rt = {rt.z, rt.st, rt.theta, rt.step, rt.st32, rt.step32};
    da.theta = pa.out.theta;
    da.phi = pa.out.phi;
    da.ar = pa.out.ar;
    da.flux = pa.out.flux;
    da.cpix = pa.out.cpix;
    da.queue = (const int *)ctx->w->queue.p;
    da.ctr = pa.ctr;
    da.acc = pa.acc;
    if (precision == DMANN_COMP_F32) da.chdr = headers_for(ctx, n1);
    CK(cudaEventRecord(ctx->evd0, s));
    CK(launch_adjoint(da, pa.p, pa.out.cls, dgmap, (float *)ctx->w->acc.p, dgrad, (double *)ctx->oacc.p,
                      precision, ctx->num_sms, s, core ? (const double *)ctx->corr.p : nullptr,
                      core ? (const double *)ctx->core_gln.p : nullptr));
    CK(cudaEventRecord(ctx->evd1, s));
    CK(cudaEventRecord(ctx->evdm, s));
    CK(cudaEventRecord(ctx->ev1, s));
    if (!grad_dev && N > 0) CK(cudaMemcpyAsync(grad, dgrad, 48 * N, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctx->h_ctr, ctx->w->ctr.p, 8 * C_COUNT, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctx->h_fsum, ctx->w->fsum.p, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctx->h_oacc, ctx->oacc.p, 8 * 12, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ctx->stats = dmann_stats{};
    ctx->stats.n_in = n;
    ctx->disc_timed = true;
    ctx->stats_pending = true;
    // observer: u = pos - opos gives -sum_i dL/du_i; the rotation adds
    // sum_e dL/drot[e] * drot[e]/dopos when the frame came from
    // dmann_set_observer (with dmann_set_frame the rotation is held fixed)
    double jac[27] = {0};
    const bool rot_terms =
        ctx->have_geom && observer_rotation_jacobian(ctx->opos, ctx->cpos, ctx->align, jac);
    for (int k = 0; k < 3; k++) {
        double v = -ctx->h_oacc[k];
        if (rot_terms)
            for (int e = 0; e < 9; e++) v += ctx->h_oacc[3 + e] * jac[3 * e + k];
        grad_opos[k] = v;
    }
    return collect_stats(ctx);
}

dmann_status dmann_observer_rotation(const double opos[3], const double cpos[3],
                                     const double align[3], double rot[9], double angles[2]) {
    if (!opos || !cpos || !align || !rot) return DMANN_ERR_INVALID;
    double th = 0, ph = 0;
    if (!observer_rotation(opos, cpos, align, rot, &th, &ph)) return DMANN_ERR_INVALID;
    if (angles) {
        angles[0] = th;
        angles[1] = ph;
    }
    return DMANN_OK;
}

dmann_status dmann_observer_rotation_jacobian(const double opos[3], const double cpos[3],
                                              const double align[3], double jac[27]) {
    if (!opos || !cpos || !align || !jac) return DMANN_ERR_INVALID;
    return observer_rotation_jacobian(opos, cpos, align, jac) ? DMANN_OK : DMANN_ERR_INVALID;
}

dmann_status dmann_code_units(double h100, double Lbox_in_Mpc, double mass_to_Msun, double out[9]) {
    if (!out) return DMANN_ERR_INVALID;
    CodeUnits u;
    setup_units(h100, Lbox_in_Mpc, mass_to_Msun, &u);
    out[0] = u.rho_crit_in_cgs;
    out[1] = u.length_to_cgs;
    out[2] = u.time_to_cgs;
    out[3] = u.density_to_cgs;
    out[4] = u.mass_to_cgs;
    out[5] = u.mass_to_Msun;
    out[6] = u.velocity_to_cgs;
    out[7] = u.annihilation_flux_to_cgs;
    out[8] = nosom_unit_factor(u);
    return DMANN_OK;
}

dmann_status dmann_flux_unit_factor(int flux_model, double h100, double Lbox_in_Mpc,
                                    double mass_to_Msun, double *unit_factor) {
    if (!unit_factor || flux_model < DMANN_FLUX_ANN_NOSOM || flux_model > DMANN_FLUX_ANN_CORE_NOSOM)
        return DMANN_ERR_INVALID;
    CodeUnits u;
    setup_units(h100, Lbox_in_Mpc, mass_to_Msun, &u);
    *unit_factor = flux_model == DMANN_FLUX_DECAY ? decay_unit_factor(u) : nosom_unit_factor(u);
    return DMANN_OK;
}

double dmann_hires_threshold(const double *masses, int n) {
    return hires_threshold(masses, masses ? n : 0);
}

}  // extern "C"
