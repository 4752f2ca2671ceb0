// adjoint_common.cuh -- the per-particle epilogue shared by the FP64 adjoint
// (adjoint.cu) and the compensated-FP32 adjoint (disc_comp.cu): given a
// particle's Gb = dL/dF, K T and K V (see adjoint.cu for the formulas), the
// gradient with respect to x, y, z, m, rho, h and its observer terms, for
// every flux law (the law's factor, and its position gradient where it has
// one).
#pragma once
#include "../../include/dmann.h"
#include "kernels.cuh"

namespace dmann {
namespace adj {

constexpr double kInvC2 = 1.0 / 0.333;  // 2 c

struct AdjArgs {
    DiscArgs d;                 // geometry from the prep kernel, queue, counters
    Particles p;                // (p.sigmav: the velocity dispersions of the sigma v laws)
    const double *core_corr;    // ann_core_nosom: each particle's halo-core factor
    const double *core_gln;     //   and d ln(factor) / d pos, [3][n]
    const signed char *cls;     // PClass per particle
    const double *gmap;         // dL/dmap [npix]
    const float *gmap32;        // the same rounded to FP32 (the compensated adjoint)
    double inv_dOmega;
    double *grad;               // [6][n]: x, y, z, m, rho, h
    double *oacc;               // [12]: sum_i dL/du_i (3), dL/dR row-major (9)
};

// u = pos - opos and d exactly as the prep kernel forms them.
__device__ inline double particle_u(const AdjArgs &a, int i, double u[3]) {
    u[0] = (double)a.p.x[i] - a.d.f.opos[0];
    u[1] = (double)a.p.y[i] - a.d.f.opos[1];
    u[2] = (double)a.p.z[i] - a.d.f.opos[2];
    return sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
}

constexpr double kCcgs = 2.99792458e10;   // speed of light, cm/s (src/datatypes.cpp:5-10)

// The flux law's factor s beyond unit_factor rho m / (4 pi d^2) (or m under
// decay) and d ln(s) / d pos (gln; zero unless s depends on the position):
// the sigma v factor of somv, somv2, pwave (src/flux/flux_ann_somv.cpp:16-43,
// flux_ann_somv2.cpp:16-44, flux_ann_pwave.cpp:13-31; sigma v is an input,
// not differentiated), the adiabatic factor squared
// (flux_ann_adiabatic.cpp:17-28, r = |pos - cpos| * 40000) and the halo-core
// factor squared (flux_ann_core_nosom.cpp:14-16; its log-gradient comes from
// the halo-core kernel).
__device__ inline double law_factor(const AdjArgs &a, int i, double gln[3]) {
    gln[0] = gln[1] = gln[2] = 0.0;
    const Frame &f = a.d.f;
    switch (f.flux_model) {
    case DMANN_FLUX_ANN_SOMV: {
        const double v = fmax((double)a.p.sigmav[i] * f.vel_to_cgs / 1.0e5, 1.0);
        return kCcgs / v / 1.0e4;
    }
    case DMANN_FLUX_ANN_SOMV2: {
        const double sv = kCcgs / fmax((double)a.p.sigmav[i] * f.vel_to_cgs / 1.0e5, 5.0);
        return sv * (sv / 1.0e8);
    }
    case DMANN_FLUX_ANN_PWAVE: {
        const double sv = (double)a.p.sigmav[i] * f.vel_to_cgs / kCcgs;
        return sv * sv;
    }
    case DMANN_FLUX_ANN_ADIABATIC: {
        const double dx = (double)a.p.x[i] - f.fcpos[0], dy = (double)a.p.y[i] - f.fcpos[1],
                     dz = (double)a.p.z[i] - f.fcpos[2];
        const double rc = sqrt(dx * dx + dy * dy + dz * dz), r = rc * 40000.0;
        const double t1 = 1 + 0.0355872 * r, t2 = 1 + 0.10888 * pow(r, 0.76);
        const double fac = (14.6534 * pow(t1, 1.76)) / (pow(t2, 3.34211) * pow(r, 0.13));
        if (rc > 0) {
            const double dl =
                1.76 * 0.0355872 / t1 - 3.34211 * 0.10888 * 0.76 * pow(r, -0.24) / t2 - 0.13 / r;
            const double k = 2.0 * dl * 40000.0 / rc;
            gln[0] = k * dx;
            gln[1] = k * dy;
            gln[2] = k * dz;
        }
        return fac * fac;
    }
    case DMANN_FLUX_ANN_CORE_NOSOM: {
        const double c = a.core_corr[i];
        const int n = a.p.n;
#pragma unroll
        for (int k = 0; k < 3; k++) gln[k] = 2.0 * a.core_gln[(size_t)k * n + i];
        return c * c;
    }
    default:
        return 1.0;
    }
}

// Writes particle i's gradient and adds its observer terms to acc.
// Gb = dL/dF; KT = K T and KV = K V (zero for a single-pixel deposit).
__device__ inline void write_grad(const AdjArgs &a, int i, double Gb, double KT,
                                  const double KV[3], bool disc, double acc[12]) {
    double u[3];
    const double d = particle_u(a, i, u);
    const double inv_d = 1.0 / d;
    const double uh[3] = {u[0] * inv_d, u[1] * inv_d, u[2] * inv_d};
    // F = fd rho m s (s the law's factor), or fd m s under the decay law
    // (flux_decay.cpp:9-16, unit_factor then being its own): there dL/drho = 0
    const bool decay = a.d.f.flux_model == DMANN_FLUX_DECAY;
    const double m = (double)a.p.m[i], rho = decay ? 1.0 : (double)a.p.rho[i];
    double gln[3];
    const double fd = a.d.f.unit_factor / (4.0 * kPi * d * d) * law_factor(a, i, gln);  // F / (rho m)
    const double F = fd * rho * m;
    const double w[3] = {-KV[0], -KV[1], KV[2]};                 // D K V
    const double cr = -(2.0 * Gb * F + KT) * inv_d;
    const int n = a.p.n;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const double rw = a.d.f.rot[j][0] * w[0] + a.d.f.rot[j][1] * w[1] + a.d.f.rot[j][2] * w[2];
        const double g = cr * uh[j] + rw * inv_d;
        // the law's own position dependence moves with the particle, not with
        // the observer: it joins dL/dpos but not the observer sums
        a.grad[(size_t)j * n + i] = g + Gb * F * gln[j];
        acc[j] += g;
    }
    a.grad[(size_t)3 * n + i] = Gb * fd * rho;
    a.grad[(size_t)4 * n + i] = decay ? 0.0 : Gb * fd * m;
    a.grad[(size_t)5 * n + i] = disc ? KT / (double)a.p.h[i] : 0.0;
    if (disc) {
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k = 0; k < 3; k++) acc[3 + 3 * j + k] += uh[j] * w[k];
    }
}

// Sum of NV values over a group (one warp, or a block of G threads);
// every thread of the group gets the sums.
template <int G, int NV>
__device__ inline void group_sum(double v[NV], double (*red)[32]) {
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    if (G > 32) {
        const int r = threadIdx.x;
        if ((r & 31) == 0)
#pragma unroll
            for (int k = 0; k < NV; k++) red[k][r >> 5] = v[k];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < G / 32; w++) s += red[k][w];
            v[k] = s;
        }
        __syncthreads();
    }
}

__device__ inline void flush_acc(double *oacc, const double acc[12]) {
#pragma unroll
    for (int k = 0; k < 12; k++)
        if (acc[k] != 0.0) atomicAdd(oacc + k, acc[k]);
}

}  // namespace adj

// disc_comp.cu: the compensated-FP32 adjoint's disc kernels
cudaError_t launch_adjoint_comp_discs(const adj::AdjArgs &a, int num_sms, cudaStream_t s);

}  // namespace dmann
