// peaks.cu -- microbenchmarks of the L2 reduction rates that bound the
// deposit scatter of the projection (each algorithmic deposit is one
// reduction into the map).  Measured live by the benchmark so that its
// roofline fraction refers to the GPU it ran on.
//
// Pattern: a persistent grid sweeps an array of `bytes` with lanes of a
// warp on consecutive elements (the layout of the disc kernels' ring runs),
// `reps` times.  Kinds:
//   DMANN_PEAK_RED_F32   red.global.add.f32 (no return value)
//   DMANN_PEAK_RED_F64   red.global.add.f64
//   DMANN_PEAK_RED_U64   red.global.add.u64 (an atomicAdd whose value is unused)
//   DMANN_PEAK_RED_F32X2 red.global.add.v2.f32, DMANN_PEAK_RED_F32X4
//                        red.global.add.v4.f32: a lane adds to two or four
//                        consecutive floats (rates counted in floats)
//   DMANN_PEAK_COMP_F32  a two-plane compensated FP32 deposit (the disc
//                        kernels' earlier form): atom.global.add.f32 that
//                        returns the old value, the exact TwoSum error and a
//                        red.global.add.f32 of the error into a second plane
//                        (two planes of bytes/2 each)
#include <cstdio>

#include "../../include/dmann.h"
#include "kernels.cuh"

namespace dmann {
namespace {

// hi[pix] += v with the rounding error (Knuth's TwoSum on the value the
// atomic returns) added to lo[pix].
__device__ inline void deposit2f(float *hi, float *lo, int pix, float v) {
    const float a = atom_add_f32(hi + pix, v);
    const float s = __fadd_rn(a, v);
    const float bb = __fsub_rn(s, a);
    const float err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    if (err != 0.0f) red_add_f32(lo + pix, err);
}

template <int KIND>
__global__ void __launch_bounds__(256) k_sweep(void *buf, long long n, int reps, float v) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; r++) {
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            if (KIND == DMANN_PEAK_RED_F32) {
                red_add_f32((float *)buf + i, v);
            } else if (KIND == DMANN_PEAK_RED_F64) {
                red_add_f64((double *)buf + i, (double)v);
            } else if (KIND == DMANN_PEAK_RED_F32X2) {
                red_add_v2_f32((float *)buf + 2 * i, v, v);
            } else if (KIND == DMANN_PEAK_RED_F32X4) {
                red_add_v4_f32((float *)buf + 4 * i, v, v, v, v);
            } else if (KIND == DMANN_PEAK_RED_U64) {
                atomicAdd((unsigned long long *)buf + i, (unsigned long long)(v * 1048576.0f));
            } else {
                deposit2f((float *)buf, (float *)buf + n, (int)i, v);
            }
        }
    }
}

}  // namespace
}  // namespace dmann

using namespace dmann;

extern "C" dmann_status dmann_measure_l2_red(int device, int kind, int64_t bytes, int reps,
                                             double *ops_per_s) {
    if (!ops_per_s || reps < 1 || bytes < (1 << 20) || bytes > ((int64_t)1 << 34))
        return DMANN_ERR_INVALID;
    if (kind != DMANN_PEAK_RED_F32 && kind != DMANN_PEAK_RED_F64 && kind != DMANN_PEAK_COMP_F32 &&
        kind != DMANN_PEAK_RED_U64 && kind != DMANN_PEAK_RED_F32X2 && kind != DMANN_PEAK_RED_F32X4)
        return DMANN_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return DMANN_ERR_NODEVICE;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return DMANN_ERR_CUDA;
    void *buf = nullptr;
    if (cudaMalloc(&buf, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        return DMANN_ERR_NOMEM;
    }
    const long long elem = (kind == DMANN_PEAK_RED_F64 || kind == DMANN_PEAK_RED_U64) ? 8 : 4;
    const long long width = kind == DMANN_PEAK_RED_F32X2 ? 2 : kind == DMANN_PEAK_RED_F32X4 ? 4 : 1;
    const long long n = kind == DMANN_PEAK_COMP_F32 ? bytes / (2 * elem) : bytes / (elem * width);
    if (kind == DMANN_PEAK_COMP_F32 && n > 0x7fffffffLL) {
        cudaFree(buf);
        return DMANN_ERR_INVALID;
    }
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    dmann_status st = DMANN_OK;
    const int grid = sms * 8;
    // 1 + 2^-20: the hi plane loses low bits of every addition, so the
    // compensated kind does its error red on every deposit
    const float v = 1.00000095367431640625f;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
        cudaMemsetAsync(buf, 0, (size_t)bytes, s) != cudaSuccess) {
        st = DMANN_ERR_CUDA;
    } else {
        auto launch = [&](int r) {
            if (kind == DMANN_PEAK_RED_F32) k_sweep<DMANN_PEAK_RED_F32><<<grid, 256, 0, s>>>(buf, n, r, v);
            else if (kind == DMANN_PEAK_RED_F64) k_sweep<DMANN_PEAK_RED_F64><<<grid, 256, 0, s>>>(buf, n, r, v);
            else if (kind == DMANN_PEAK_RED_U64) k_sweep<DMANN_PEAK_RED_U64><<<grid, 256, 0, s>>>(buf, n, r, v);
            else if (kind == DMANN_PEAK_RED_F32X2)
                k_sweep<DMANN_PEAK_RED_F32X2><<<grid, 256, 0, s>>>(buf, n, r, v);
            else if (kind == DMANN_PEAK_RED_F32X4)
                k_sweep<DMANN_PEAK_RED_F32X4><<<grid, 256, 0, s>>>(buf, n, r, v);
            else k_sweep<DMANN_PEAK_COMP_F32><<<grid, 256, 0, s>>>(buf, n, r, v);
        };
        launch(1);  // warm-up
        cudaEventRecord(e0, s);
        launch(reps);
        cudaEventRecord(e1, s);
        float ms = 0.0f;
        if (cudaStreamSynchronize(s) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
            !(ms > 0.0f))
            st = DMANN_ERR_CUDA;
        else
            *ops_per_s = (double)n * width * reps / (ms * 1e-3);
    }
    cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(buf);
    return st;
}
