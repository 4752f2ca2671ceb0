// disc_plain.cu -- the plain FP64 form of the disc kernels.
//
// The reference CPU path's arithmetic on the GPU: each disc pixel's centre
// vector as pix2vec computes it (z and sin(theta) of its ring, phi from the
// in-ring index), w = exp(-0.5 (acos(v_pix . v)/ar)^2 / 0.333)
// (src/genmap.cpp:133-145), the FP64 normalisation and w/norm*flux added to
// an FP64 map with FP64 atomics (src/genmap.cpp:148-153).  Compiled with
// -fmad=false so every expression rounds as the CPU path's does; results
// differ from it only by the order of the additions.
#include "plain_form.cuh"

namespace dmann {

namespace {

constexpr int kBT = 256, kRCH = 256;
constexpr int kWPB = 8, kRCHW = 64;

}  // namespace

cudaError_t launch_disc_plain(const DiscArgs &a, int num_sms, int blocks_per_sm, cudaStream_t s,
                              cudaEvent_t mid) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, k_disc_block<PlainForm, kBT, kRCH>, kBT, 0);
    if (e != cudaSuccess) return e;
    int bps = blocks_per_sm > 0 ? min(blocks_per_sm, occ) : occ;
    if (bps < 1) bps = 1;
    k_disc_block<PlainForm, kBT, kRCH><<<num_sms * bps, kBT, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (mid && (e = cudaEventRecord(mid, s)) != cudaSuccess) return e;
    int occw = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occw, k_disc_warp<PlainForm, kWPB, kRCHW>,
                                                      kWPB * 32, 0);
    if (e != cudaSuccess) return e;
    if (occw < 1) occw = 1;
    k_disc_warp<PlainForm, kWPB, kRCHW><<<num_sms * occw, kWPB * 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dmann
