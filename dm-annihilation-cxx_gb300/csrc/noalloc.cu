// noalloc.cu -- dmann_render_noalloc: the compensated-FP32 render for callers
// that may not allocate device memory.
//
// Every scratch buffer the render needs (ring tables, the key histogram and
// counters, the per-particle prep arrays and disc queue, the FP64
// accumulation plane) is carved out of one fixed array defined below.  The
// array is created when the library is loaded on a GPU and lives until the
// process exits; nothing in this file calls cudaMalloc, cudaFree or any other
// allocating routine.  The kernels are the same ones dmann_render launches.
#include <cmath>
#include <mutex>

#include "../../include/dmann.h"
#include "kernels.cuh"

using namespace dmann;

namespace {

constexpr size_t kScratchBytes = DMANN_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_dev[kMaxDevices];  // device address of g_scratch, per device
int g_num_sms[kMaxDevices];

// Per-ring tables, with the formulas of the context path's host tables.
__global__ void k_ring_tables(int nside, double fact1, double fact2, double *z, double *st,
                              double *th, double *step, float *st32, float *step32) {
    const int n = 4 * nside;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        if (r == 0) {
            z[0] = st[0] = th[0] = step[0] = 0.0;
            st32[0] = step32[0] = 0.0f;
            continue;
        }
        bool have = false;
        double tmp = 0.0, zz;
        int nr;
        if (r < nside) {
            tmp = __dmul_rn((double)((long long)r * r), fact2);
            zz = __dsub_rn(1.0, tmp);
            have = zz > 0.99;
            nr = 4 * r;
        } else if (r <= 3 * nside) {
            zz = __dmul_rn((double)(2 * nside - r), fact1);
            nr = 4 * nside;
        } else {
            const long long ir = 4LL * nside - r;
            tmp = __dmul_rn((double)(ir * ir), fact2);
            zz = __dsub_rn(tmp, 1.0);
            have = zz < -0.99;
            nr = 4 * (int)ir;
        }
        const double s = have ? __dsqrt_rn(__dmul_rn(tmp, __dsub_rn(2.0, tmp)))
                              : __dsqrt_rn(__dmul_rn(__dsub_rn(1.0, zz), __dadd_rn(1.0, zz)));
        z[r] = zz;
        st[r] = s;
        th[r] = have ? atan2(s, zz) : acos(zz);
        step[r] = __ddiv_rn(kTwoPi, (double)nr);
        st32[r] = (float)s;
        step32[r] = (float)step[r];
    }
}

// Byte offsets of the scratch regions for n particles at one Nside.
struct Layout {
    size_t ring, hist, ctr, fsum, acc, theta, phi, ar, flux, cpix, key, queue, total;
};

size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

Layout layout(size_t n, int nside) {
    Layout L;
    const size_t npix = 12 * (size_t)nside * (size_t)nside;
    size_t o = 0;
    L.ring = o;  o = up256(o + (4 * sizeof(double) + 2 * sizeof(float)) * 4 * (size_t)nside);
    L.hist = o;  o = up256(o + sizeof(int) * (size_t)kKeys);
    L.ctr = o;   o = up256(o + sizeof(long long) * C_COUNT);
    L.fsum = o;  o = up256(o + sizeof(double));
    L.acc = o;   o = up256(o + 2 * sizeof(float) * npix);
    L.theta = o; o = up256(o + 8 * n);
    L.phi = o;   o = up256(o + 8 * n);
    L.ar = o;    o = up256(o + 8 * n);
    L.flux = o;  o = up256(o + 8 * n);
    L.cpix = o;  o = up256(o + 4 * n);
    L.key = o;   o = up256(o + 4 * n);
    L.queue = o; o = up256(o + 4 * n);
    L.total = o;
    return L;
}

bool device_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Once per device, with that device current: the device address of the
// scratch array (its host-side name is only a stand-in for it) and the SM
// count.  Called by the first dmann_render_noalloc on each device.
dmann_status setup_device(int dev, void **scratch, int *sms) {
    if (dev < 0 || dev >= kMaxDevices) return DMANN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_dev[dev]) {
        int major = 0, minor = 0, n = 0;
        if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return DMANN_ERR_CUDA;
        }
        if (!(major == 10 && minor == 3)) return DMANN_ERR_NODEVICE;  // built for sm_103a only
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return DMANN_ERR_CUDA;
        }
        g_num_sms[dev] = n;
        g_scratch_dev[dev] = p;
    }
    *scratch = g_scratch_dev[dev];
    *sms = g_num_sms[dev];
    return DMANN_OK;
}

#define NA_CK(call)                              \
    do {                                         \
        if ((call) != cudaSuccess) {             \
            cudaGetLastError();                  \
            return DMANN_ERR_CUDA;               \
        }                                        \
    } while (0)

}  // namespace

extern "C" dmann_status dmann_render_noalloc(const float *x, const float *y, const float *z,
                                             const float *m, const float *rho, const float *h,
                                             int64_t n, int nside, const double rot[9],
                                             const double opos[3], double unit_factor,
                                             double hires_threshold, double *map_out,
                                             int accumulate, void *stream) {
    if (!rot || !opos || !map_out) return DMANN_ERR_INVALID;
    if (n < 0 || n > (int64_t)0x7fffffff || nside < 1 || nside > 8192) return DMANN_ERR_INVALID;
    if (n > 0 && (!x || !y || !z || !m || !rho || !h)) return DMANN_ERR_INVALID;
    if (!(std::isfinite(unit_factor) && unit_factor > 0)) return DMANN_ERR_INVALID;
    for (int i = 0; i < 9; i++)
        if (!std::isfinite(rot[i])) return DMANN_ERR_INVALID;
    const Layout L = layout((size_t)n, nside);
    if (L.total > kScratchBytes) return DMANN_ERR_TOO_LARGE;
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    void *base = nullptr;
    int sms = 0;
    dmann_status st = setup_device(dev, &base, &sms);
    if (st != DMANN_OK) return st;
    // inputs and the map must already be on the GPU: nothing is staged
    const float *in[6] = {x, y, z, m, rho, h};
    if (n > 0)
        for (const float *p : in)
            if (!device_ptr(p)) return DMANN_ERR_INVALID;
    if (!device_ptr(map_out)) return DMANN_ERR_INVALID;

    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *b = (unsigned char *)base;
    const int npix = 12 * nside * nside;
    double *rz = (double *)(b + L.ring), *rst = rz + 4 * nside, *rth = rst + 4 * nside,
           *rstep = rth + 4 * nside;
    float *rst32 = (float *)(rstep + 4 * nside), *rstep32 = rst32 + 4 * nside;

    Hpx g;
    g.nside = nside;
    g.npix = npix;
    g.ncap = 2 * nside * (nside - 1);
    g.nrings = 4 * nside - 1;
    g.fact2 = 4.0 / (double)npix;
    g.fact1 = (double)(nside << 1) * g.fact2;
    g.dOmega = 4 * 3.14159265358979323846 / (double)npix;  // src/datatypes.h:251
    g.theta0 = std::acos(1.0 - g.dOmega / (2.0 * 3.141592));  // src/genmap.cpp:38

    Frame f{};   // every field defined, including those the nosom law never reads
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) f.rot[i][j] = rot[3 * i + j];
        f.opos[i] = opos[i];
    }
    f.unit_factor = unit_factor;
    f.hires_threshold = hires_threshold;
    int e2 = 0;
    std::frexp(unit_factor, &e2);
    f.inv_scale = std::ldexp(1.0, -e2);
    const double scale = std::ldexp(1.0, e2);
    f.flux_model = DMANN_FLUX_ANN_NOSOM;

    Accum acc;
    acc.acc64 = nullptr;
    acc.acc64 = (double *)(b + L.acc);

    // the array keeps the previous call's contents: clear what must start at zero
    NA_CK(cudaMemsetAsync(b + L.hist, 0, sizeof(int) * (size_t)kKeys, s));
    NA_CK(cudaMemsetAsync(b + L.ctr, 0, sizeof(long long) * C_COUNT, s));
    NA_CK(cudaMemsetAsync(b + L.fsum, 0, sizeof(double), s));
    NA_CK(cudaMemsetAsync(b + L.acc, 0, 2 * sizeof(float) * (size_t)npix, s));
    k_ring_tables<<<(4 * nside + 255) / 256, 256, 0, s>>>(nside, g.fact1, g.fact2, rz, rst, rth,
                                                          rstep, rst32, rstep32);
    NA_CK(cudaGetLastError());

    if (n > 0) {
        PrepArgs pa;
        pa.p = {x, y, z, m, rho, h, (int)n};
        pa.f = f;
        pa.g = g;
        pa.out = {(double *)(b + L.theta), (double *)(b + L.phi), (double *)(b + L.ar),
                  (double *)(b + L.flux), (int *)(b + L.cpix), (int *)(b + L.key)};
        pa.hist = (int *)(b + L.hist);
        pa.ctr = (long long *)(b + L.ctr);
        pa.flux_sum = (double *)(b + L.fsum);
        pa.acc = acc;
        pa.precision = DMANN_COMP_F32;
        pa.block_bucket_min = 11;  // discs estimated above 1024 pixels: block per disc
        pa.deposit_singles = 1;
        pa.core_corr = nullptr;
        NA_CK(launch_prep(pa, s));
        NA_CK(launch_scan(pa.hist, pa.ctr, pa.block_bucket_min, s));
        NA_CK(launch_scatter(pa, (int *)(b + L.queue), s));
        DiscArgs da;
        da.g = g;
        da.f = f;
        da.rt = {rz, rst, rth, rstep, rst32, rstep32};
        da.theta = pa.out.theta;
        da.phi = pa.out.phi;
        da.ar = pa.out.ar;
        da.flux = pa.out.flux;
        da.cpix = pa.out.cpix;
        da.queue = (const int *)(b + L.queue);
        da.ctr = pa.ctr;
        da.acc = acc;
        NA_CK(launch_disc_comp(da, sms, 0, 256, s, nullptr));
    }
    NA_CK(launch_finalize(acc, DMANN_COMP_F32, npix, g.dOmega, scale, map_out, accumulate, s));
    return DMANN_OK;
}
