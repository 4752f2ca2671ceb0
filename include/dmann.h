/*
 * dmann.h -- C ABI of the GB300 annihilation sky-map projection library
 * (libdmann.so).
 *
 * Plain C types only: no C++ or torch types cross this boundary.  Every entry
 * point returns a status code (never exits, never throws); the message of the
 * last failure on a context is available from dmann_last_error().  Buffers
 * are owned by the caller; a context owns only its stream and its device
 * workspace.  One context per host thread / stream: calls on one context are
 * serialised on its stream, different contexts are independent (reentrant).
 *
 * What each entry point replaces in the reference (paths relative to the
 * reference project):
 *   dmann_create / dmann_destroy      initializeCUDA / cudaCleaingUp
 *                                     (src/chealpixrender.h:60-64,
 *                                     src/kernel.h:10-11), which keep module-
 *                                     global device state; here it is a handle.
 *   dmann_set_observer                Parameters::setupParams / setupRotation
 *                                     (src/parameters.cpp:111-152,183-289)
 *   dmann_set_frame                   the rotmatrix/opos fields those set
 *                                     (src/parameters.h:17, datatypes.h:225)
 *   dmann_set_units                   getflux's unit factor and the hires-mass
 *                                     filter (src/flux/flux_ann_nosom.cpp:13-16,
 *                                     src/genmap.cpp:52-58,82-85)
 *   dmann_render                      MapGenerator::start's per-chunk work:
 *                                     the host prep loop plus
 *                                     calculateMapByGPU / getCUDAMap
 *                                     (src/genmap_cuda_render.cpp:102-196,
 *                                     src/chealpixrender.h:61-63) and
 *                                     calulateMapWithCUDA (src/kernel.h:11),
 *                                     with the CPU semantics of
 *                                     src/genmap.cpp:67-169.
 *   dmann_render_batch                no reference counterpart (many
 *                                     observers / Nside values in one call)
 *   dmann_adjoint                     no reference counterpart (gradients of
 *                                     a pixelwise loss of the map)
 */
#ifndef DMANN_H
#define DMANN_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DMANN_ABI_VERSION 2

typedef struct dmann_ctx dmann_ctx;

typedef enum {
    DMANN_OK = 0,
    DMANN_ERR_INVALID = 1,   /* bad argument (null pointer, bad Nside, ...) */
    DMANN_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    DMANN_ERR_NOMEM = 3,     /* device or host allocation failed */
    DMANN_ERR_STATE = 4,     /* call order (e.g. render before an observer) */
    DMANN_ERR_TIMEOUT = 5,   /* a bounded device wait gave up */
    DMANN_ERR_NODEVICE = 6,  /* no CUDA device / wrong architecture */
    DMANN_ERR_TOO_LARGE = 7  /* dmann_render_noalloc: problem exceeds its fixed scratch */
} dmann_status;

/* Precision forms of the projection. */
typedef enum {
    /* FP64 throughout: geometry, weights exp(-0.5 (acos(v_p.v)/ar)^2/0.333),
     * normalisation and FP64 atomic accumulation -- the reference CPU path's
     * arithmetic on the GPU. */
    DMANN_PLAIN_F64 = 0,
    /* FP64 per-particle geometry and disc bounds; FP32 weights (haversine
     * distance, Gaussian); per-particle normalisation as compensated
     * two-float sums; each deposit w * flux / norm rounded once to FP32 and
     * accumulated per pixel in FP64.  The fast form. */
    DMANN_COMP_F32 = 1
} dmann_precision;

/* Flux laws: the reference's link-time getflux plugins (the files of src/flux,
 * src/flux.h:6), selected per context at run time.  unit_factor is the
 * law's factor (dmann_flux_unit_factor); v = sigmav * velocity_to_cgs / 1e5 is
 * the velocity dispersion in km/s, c the speed of light in cm/s.  Each law
 * keeps its plugin's operation order. */
typedef enum {
    DMANN_FLUX_ANN_NOSOM = 0,     /* unit_factor rho m / (4 pi d^2)   flux_ann_nosom.cpp */
    DMANN_FLUX_ANN_SOMV = 1,      /* x c / max(v, 1) / 1e4           flux_ann_somv.cpp */
    DMANN_FLUX_ANN_SOMV2 = 2,     /* x (c / max(v, 5))^2 / 1e8       flux_ann_somv2.cpp */
    DMANN_FLUX_ANN_PWAVE = 3,     /* x (sigmav velocity_to_cgs / c)^2 flux_ann_pwave.cpp */
    DMANN_FLUX_DECAY = 4,         /* unit_factor m / (4 pi d^2)      flux_decay.cpp */
    DMANN_FLUX_ANN_ADIABATIC = 5, /* nosom x f(r)^2, r = |pos - cpos| * 40000
                                     (kpc/h in the reference's units) flux_ann_adiabatic.cpp */
    DMANN_FLUX_ANN_CORE_NOSOM = 6 /* nosom x r^2, r the halo-core factor of the
                                     halos set by dmann_set_halo_cores
                                     flux_ann_core_nosom.cpp, halocore/halocore.cpp */
} dmann_flux;

/* Counters of the last dmann_render call on a context. */
typedef struct {
    int64_t n_in;          /* particles passed in */
    int64_t n_kept;        /* passed the hires-mass and mask filter */
    int64_t n_invalid;     /* skipped: at the observer or non-finite geometry */
    int64_t n_single;      /* deposited into one pixel (2 ar < theta0) */
    int64_t n_disc;        /* rendered as discs (incl. < 2 pixel discs) */
    int64_t n_disc_block;  /* of which in the block-per-particle class */
    int64_t deposits;      /* algorithmic deposits: sum of disc sizes + singles */
    double kernel_ms;      /* device time from map_begin to map_end (events) */
    double disc_ms;        /* device time of the disc kernels of the last chunk */
    double disc_block_ms;  /* of which the block-per-particle kernel */
    double disc_warp_ms;   /* of which the warp-per-particle kernel */
    double total_flux;     /* sum of kept flux (before the dOmega division) */
    int64_t launches;      /* kernels launched for the last map (all chunks) */
    double pass1_ms;       /* compensated form, block class of the last chunk: from the
                              disc kernels' start to the end of the weight sums (headers,
                              work items, pass 1) */
    double pass2_ms;       /* the item sort, the deposit segments and their flushes
                              (both 0 when the chunk deposited in FP64) */
} dmann_stats;

/* Tunables (set by the annmap autotuner; zero fields keep the current
 * values).  Defaults: warp_max_pixels 1024, block_threads 256, blocks_per_sm
 * 0 (as many as fit), seg_min_deposits_log2 28. */
typedef struct {
    int64_t warp_max_pixels;   /* footprint-class bin edge: discs estimated up
                                  to this many pixels go warp-per-particle,
                                  larger ones block-per-particle */
    int32_t block_threads;     /* compensated block kernel shape: 128, 256 or
                                  512 threads (the plain form always uses 256) */
    int32_t blocks_per_sm;     /* resident blocks per SM of the persistent
                                  block kernel, capped by occupancy; 0 = max */
    int32_t ring_chunk;        /* read only: rings staged per pass for the
                                  block shape (192, 384, 640) */
    int32_t seg_min_deposits_log2;  /* compensated form: a chunk whose block-
                                  class discs are estimated to make at least
                                  2^this many deposits takes the segmented
                                  render (FP32 deposits flushed into the FP64
                                  plane per segment, 128 or 256 threads);
                                  smaller chunks deposit in FP64.  1 .. 62 */
    int32_t reserved[2];
} dmann_tuning;

/* ---- lifetime ---- */
dmann_status dmann_create(dmann_ctx **ctx, int device);
void dmann_destroy(dmann_ctx *ctx);
const char *dmann_last_error(const dmann_ctx *ctx);
int dmann_abi_version(void);

/* Runs subsequent work on `stream` (a cudaStream_t; NULL = the context's
 * own stream; the legacy default stream is cudaStreamLegacy).  Lets a caller
 * such as PyTorch share its current stream. */
dmann_status dmann_set_stream(dmann_ctx *ctx, void *stream);
dmann_status dmann_synchronize(dmann_ctx *ctx);

/* ---- observer frame and units ---- */
/* Observer at opos, halo centre cpos, alignment vector align: computes the
 * rotation matrix exactly as Parameters::setupRotation does.  Fails with
 * DMANN_ERR_INVALID when opos == cpos (the reference's angles are NaN). */
dmann_status dmann_set_observer(dmann_ctx *ctx, const double opos[3],
                                const double cpos[3], const double align[3]);
/* Sets the frame directly: rot is rotmatrix[3][3] row-major, as used by
 * calc_angles (v' = rot^T (pos - opos)). */
dmann_status dmann_set_frame(dmann_ctx *ctx, const double rot[9],
                             const double opos[3]);
/* unit_factor multiplies the flux law (dmann_flux); hires_threshold is the
 * mass at or above which a particle is skipped ((double)(float)min_mass * 1.1
 * in the reference; pass INFINITY to keep every particle). */
dmann_status dmann_set_units(dmann_ctx *ctx, double unit_factor,
                             double hires_threshold, int flux_model);
/* The constants some flux laws read besides unit_factor: the code velocity
 * unit (somv, somv2, pwave; Parameters' codeunits.velocity_to_cgs) and the
 * halo centre (adiabatic; params.cpos).  Default 0 and the origin. */
dmann_status dmann_set_flux_params(dmann_ctx *ctx, double velocity_to_cgs,
                                   const double cpos[3]);
/* The context's default tuning (DMANN_ERR_INVALID for a block shape other
 * than 128/256/512 or negative values). */
dmann_status dmann_set_tuning(dmann_ctx *ctx, const dmann_tuning *t);
dmann_status dmann_get_tuning(const dmann_ctx *ctx, dmann_tuning *t);
/* Per-Nside tuning: maps of this nside (dmann_render, the streaming calls
 * and each observer of dmann_render_batch) use this entry instead of the
 * default; zero fields take the default's current values.  t = NULL removes
 * the entry.  dmann_get_tuning_nside returns the tuning in force for nside. */
dmann_status dmann_set_tuning_nside(dmann_ctx *ctx, int nside, const dmann_tuning *t);
dmann_status dmann_get_tuning_nside(const dmann_ctx *ctx, int nside, dmann_tuning *t);

/* The halo table of the ann_core_nosom law (src/halocore/halocore.cpp:
 * the VL2_Halos.data columns x y z radius, one halo per line): centres in
 * box units, radius in the table's units (the core radius is
 * radius / (0.73 * 40000) box units).  Each particle's factor is the product
 * over the halos whose core contains it of 0.55 (d / R)^-0.9.  Copied to the
 * device; n_halos = 0 makes every factor 1. */
dmann_status dmann_set_halo_cores(dmann_ctx *ctx, const float *x, const float *y,
                                  const float *z, const float *radius, int n_halos);

/* ---- rendering ---- */
/* Projects n particles (float32 SoA: positions x,y,z, mass m, density rho,
 * smoothing length h; rho < 0 marks a masked particle) into a HEALPix RING
 * map of 12*nside^2 doubles in flux per steradian (the reference's map after
 * its final division by dOmega).  Inputs and map_out may each be host or
 * device pointers (detected).  accumulate != 0 adds into map_out instead of
 * overwriting it, so chunks of a particle stream can be rendered one call at
 * a time.  1 <= nside <= 8192.  Blocks until map_out is complete when it is a
 * host pointer; otherwise returns with the work queued on the stream. */
dmann_status dmann_render(dmann_ctx *ctx, const float *x, const float *y,
                          const float *z, const float *m, const float *rho,
                          const float *h, int64_t n, int nside, int precision,
                          double *map_out, int accumulate);

/* dmann_render with each particle's velocity dispersion sigmav (code units,
 * the native record's field, src/datatypes.h:46-59), which the somv, somv2
 * and pwave laws need (the plain calls fail with DMANN_ERR_INVALID for those
 * laws); other laws ignore it and accept NULL. */
dmann_status dmann_render_v(dmann_ctx *ctx, const float *x, const float *y,
                            const float *z, const float *m, const float *rho,
                            const float *h, const float *sigmav, int64_t n,
                            int nside, int precision, double *map_out,
                            int accumulate);

/* Streaming form of dmann_render, the shape of MapGenerator::start's loop
 * over DataReader chunks (src/genmap.cpp:67-156): begin zeroes the
 * context's device accumulation planes for one map, every add deposits one
 * chunk of particles into them (inputs host or device), end divides by
 * dOmega into map_out (host or device; accumulate != 0 adds to it).  The
 * FP64 plane carries the sum across chunks, so a streamed map equals a
 * single-call one to the rounding of the FP64 additions.
 *
 * While a map is open (after begin, until end or abort) the context's
 * buffers belong to it: dmann_map_begin, dmann_render(_v),
 * dmann_render_batch and dmann_adjoint on the same context fail with
 * DMANN_ERR_STATE.  dmann_map_abort closes an open map without output (for
 * instance after a failed add); the next begin starts from zero. */
dmann_status dmann_map_begin(dmann_ctx *ctx, int nside, int precision);
dmann_status dmann_map_add(dmann_ctx *ctx, const float *x, const float *y,
                           const float *z, const float *m, const float *rho,
                           const float *h, int64_t n);
dmann_status dmann_map_end(dmann_ctx *ctx, double *map_out, int accumulate);
dmann_status dmann_map_abort(dmann_ctx *ctx);
/* dmann_map_add with the velocity dispersion (as dmann_render_v). */
dmann_status dmann_map_add_v(dmann_ctx *ctx, const float *x, const float *y,
                             const float *z, const float *m, const float *rho,
                             const float *h, const float *sigmav, int64_t n);

/* Renders the same particles for n_obs observers in one call (no reference
 * counterpart: the reference renders one observer per run).  Observer k has
 * the frame rot[9k..9k+8] / opos[3k..3k+2] (as dmann_set_frame) and its own
 * nside[k]; its map goes to maps[k] (12*nside[k]^2 doubles, host or device).
 * The particles are uploaded once; when every map is a device pointer the
 * whole batch is captured into one CUDA graph and launched once, the
 * observers alternating between two workspaces on two streams (the context
 * keeps a second set of per-particle buffers and planes for that).  The context
 * keeps that graph: a later batch with the same inputs, maps, frames, Nside
 * values, units and tuning (and no context buffer reallocated since) launches
 * it again without capturing; one with other frames or maps updates it in
 * place where the graph's shape allows.  Returns when all maps are complete;
 * dmann_get_stats then reports the counters summed over the observers and
 * the graph's device time.  The context's own frame is left unchanged. */
dmann_status dmann_render_batch(dmann_ctx *ctx, const float *x, const float *y,
                                const float *z, const float *m, const float *rho,
                                const float *h, int64_t n, int n_obs,
                                const double *rot, const double *opos,
                                const int *nside, int precision,
                                double *const *maps);

/* ---- differentiation ---- */
/* Adjoint of dmann_render (no reference counterpart), for every flux law:
 * the flux is rho m (m under decay, where dL/drho = 0) over d^2 times the
 * law's factor -- of the velocity dispersion for somv, somv2 and pwave
 * (sigma v is an input, not differentiated: use dmann_adjoint_v), of the
 * particle's position for adiabatic and ann_core_nosom (that factor's own
 * position derivative joins dL/dpos but not dL/dopos; halo-core membership
 * is held fixed).
 * grad_map[p] = dL/dmap[p] for a scalar loss L of the map dmann_render
 * returns for these particles, this nside and the context's frame and units
 * (12*nside^2 doubles, host or device).  Writes dL/d(particle inputs) into
 * grad (6*n doubles, host or device, planes x, y, z, m, rho, h of n each)
 * and dL/d(observer position) into grad_opos (host, 3 doubles).
 *
 * The derivative is that of the map with every particle's disc pixel set
 * and single-pixel decision held fixed (the map is piecewise smooth: it
 * jumps where a pixel centre crosses a disc edge).  Skipped particles (hires
 * mass, rho < 0, invalid geometry) get zero gradient.  The kernel weights are
 * recomputed, not stored: in FP64 with precision DMANN_PLAIN_F64, or with the
 * compensated form's FP32 weights and compensated sums (per-particle
 * epilogue in FP64) with DMANN_COMP_F32.  The observer gradient includes the
 * rotation's dependence on the observer when the frame was set by
 * dmann_set_observer; after dmann_set_frame the rotation is held fixed.
 * Blocks until the gradients are written; dmann_get_stats then reports the
 * adjoint's counters and device time. */
dmann_status dmann_adjoint(dmann_ctx *ctx, const float *x, const float *y,
                           const float *z, const float *m, const float *rho,
                           const float *h, int64_t n, int nside, int precision,
                           const double *grad_map, double *grad,
                           double grad_opos[3]);
/* dmann_adjoint with each particle's velocity dispersion (as dmann_render_v);
 * the somv, somv2 and pwave laws need it, the others accept NULL. */
dmann_status dmann_adjoint_v(dmann_ctx *ctx, const float *x, const float *y,
                             const float *z, const float *m, const float *rho,
                             const float *h, const float *sigmav, int64_t n,
                             int nside, int precision, const double *grad_map,
                             double *grad, double grad_opos[3]);

/* Statistics of the last completed map (synchronises the stream). */
dmann_status dmann_get_stats(const dmann_ctx *ctx, dmann_stats *out);

/* ---- rendering without any allocation ---- */
/* No counterpart in the reference.  For callers that must not allocate GPU
 * memory -- a plug-in inside a host application whose own allocator has
 * reserved the device's memory, or a latency-critical loop where cudaMalloc's
 * implicit synchronisation is not acceptable -- this renders one map with the
 * compensated-FP32 form using only a fixed scratch array compiled into the
 * library (DMANN_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the
 * library until the process exits).  It calls no cudaMalloc, cudaFree or other
 * allocating routine and needs no context.
 *
 * Inputs (float32 SoA, as dmann_render) and map_out (12*nside^2 doubles) must
 * be device pointers; rot / opos / unit_factor / hires_threshold are what
 * dmann_set_frame and dmann_set_units take.  Work is queued on `stream`
 * (a cudaStream_t, NULL = the default stream) of the current device and the
 * call returns without waiting.  The scratch needed is about
 *     8 * 12*nside^2 + 44 * n + 160 * nside + 513 KiB   bytes;
 * a larger problem is rejected with DMANN_ERR_TOO_LARGE (render it in chunks
 * of particles with accumulate = 1).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture.  All calls on a device share the one array: calls that
 * overlap on the GPU (different streams or threads) race and corrupt each
 * other's maps, so serialise them, e.g. on one stream. */
#define DMANN_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
dmann_status dmann_render_noalloc(const float *x, const float *y, const float *z,
                                  const float *m, const float *rho, const float *h,
                                  int64_t n, int nside, const double rot[9],
                                  const double opos[3], double unit_factor,
                                  double hires_threshold, double *map_out,
                                  int accumulate, void *stream);

/* ---- diagnostics ---- */
/* Reduction kinds of dmann_measure_l2_red. */
typedef enum {
    DMANN_PEAK_RED_F32 = 0,   /* red.global.add.f32 */
    DMANN_PEAK_RED_F64 = 1,   /* red.global.add.f64 */
    DMANN_PEAK_COMP_F32 = 2,  /* a two-plane compensated FP32 deposit: returning
                                 FP32 atomic add, exact TwoSum error, FP32 red of
                                 the error */
    DMANN_PEAK_RED_U64 = 3,   /* red.global.add.u64 */
    DMANN_PEAK_RED_F32X2 = 4, /* red.global.add.v2.f32: two consecutive floats per lane */
    DMANN_PEAK_RED_F32X4 = 5  /* red.global.add.v4.f32: four consecutive floats per lane */
} dmann_peak_kind;
/* No reference counterpart.  Measures the rate (operations per second; for
 * the vector kinds, floats added per second) of one kind of global reduction
 * on `device`: a grid of 8 blocks per SM sweeps an array of `bytes` (1 MiB ..
 * 16 GiB; a 400 MB array exceeds the L2) with lanes of a warp on consecutive
 * elements, `reps` times, after one warm-up sweep.  The deposit scatter of the projection is bound by this rate (one
 * reduction per algorithmic deposit). */
dmann_status dmann_measure_l2_red(int device, int kind, int64_t bytes, int reps,
                                  double *ops_per_s);

/* ---- host-only helpers (no context, no GPU) ---- */
/* Parameters::setupParams + setupRotation (src/parameters.cpp:111-152,
 * 183-289): rot = rotmatrix row-major; angles = {otheta, ophi} (may be
 * NULL).  DMANN_ERR_INVALID when opos == cpos. */
dmann_status dmann_observer_rotation(const double opos[3], const double cpos[3],
                                     const double align[3], double rot[9],
                                     double angles[2]);
/* d rot[e] / d opos[k] of dmann_observer_rotation as jac[3*e + k] (e the
 * row-major element of rot), by forward-mode differentiation of the same
 * operations (cpos and align held fixed).  DMANN_ERR_INVALID when
 * opos == cpos. */
dmann_status dmann_observer_rotation_jacobian(const double opos[3],
                                              const double cpos[3],
                                              const double align[3],
                                              double jac[27]);
/* Parameters::setupUnits (src/parameters.cpp:42-82) and the default flux
 * law's unit factor (src/flux/flux_ann_nosom.cpp:13-16).  out = {rho_crit,
 * length_to_cgs, time_to_cgs, density_to_cgs, mass_to_cgs, mass_to_Msun,
 * velocity_to_cgs, annihilation_flux_to_cgs, unit_factor}.  mass_to_Msun
 * = -1 derives the mass unit from rho_crit * L^3, as the reference does. */
dmann_status dmann_code_units(double h100, double Lbox_in_Mpc,
                              double mass_to_Msun, double out[9]);
/* The unit factor of a flux law from the code units of Parameters::setupUnits:
 * the annihilation laws share flux_ann_nosom.cpp:13-16's factor, the decay
 * law has its own (flux_decay.cpp:10-13). */
dmann_status dmann_flux_unit_factor(int flux_model, double h100, double Lbox_in_Mpc,
                                    double mass_to_Msun, double *unit_factor);
/* src/genmap.cpp:52-58: (double)(float)min(masses > 0) * 1.1, the mass at
 * or above which a particle is skipped (FLT_MAX * 1.1 if none positive). */
double dmann_hires_threshold(const double *masses, int n);

#ifdef __cplusplus
}
#endif
#endif /* DMANN_H */
