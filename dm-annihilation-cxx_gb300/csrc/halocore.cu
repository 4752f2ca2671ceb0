// halocore.cu -- the halo-core flux correction of the ann_core_nosom law
// (src/flux/flux_ann_core_nosom.cpp:9-17, src/halocore/halocore.cpp:48-83):
// each particle's flux is multiplied by r^2, where r is the product over all
// halos h of
//     0.55 (d_h / R_h)^-0.9   when 0 < d_h < R_h, else 1,
// d_h the distance from the particle to the halo centre and R_h the halo's
// radius column / (0.73 * 40000) (box units), held in a float.
//
// The reference loops over every halo for every particle (20,048 halos in
// its VL2 table).  Here the halos are bucketed on the host into a uniform
// grid whose cell is at least the largest R_h, so a particle only tests the
// halos of the 27 cells around its own; a particle outside the grid's box
// lies farther than every R_h from every centre.  The distance test runs in
// FP32 with a margin and only candidates take the reference's FP64
// expression, which decides membership and gives the factor; the factors of
// a particle's halos multiply in grid order instead of file order (the
// product differs in the last bits only).  For the adjoint the kernel also
// returns d ln r / d pos = sum over the particle's halos of
// -0.9 (pos - c_h) / d_h^2 (membership held fixed).
#include "kernels.cuh"

namespace dmann {

namespace {

__global__ void __launch_bounds__(256) k_halo_core(HaloGrid g, Particles p, double *corr, double *gln) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float x = p.x[i], y = p.y[i], z = p.z[i];
    double r = 1.0;
    double gx = 0.0, gy = 0.0, gz = 0.0;   // d ln r / d pos: sum of -0.9 (pos - c) / d^2
    const float fx = (x - g.ox) * g.inv_cell, fy = (y - g.oy) * g.inv_cell, fz = (z - g.oz) * g.inv_cell;
    if (fx >= 0.0f && fy >= 0.0f && fz >= 0.0f && fx < (float)g.nx && fy < (float)g.ny && fz < (float)g.nz) {
        const int cx = (int)fx, cy = (int)fy, cz = (int)fz;
        for (int kz = max(cz - 1, 0); kz <= min(cz + 1, g.nz - 1); kz++)
            for (int ky = max(cy - 1, 0); ky <= min(cy + 1, g.ny - 1); ky++) {
                const int row = (kz * g.ny + ky) * g.nx;
                const int c0 = row + max(cx - 1, 0), c1 = row + min(cx + 1, g.nx - 1);
                for (int h = g.cell_start[c0]; h < g.cell_start[c1 + 1]; h++) {
                    // halocore.cpp:70-83: float differences, FP64 distance
                    const float xx = x - g.hx[h], yy = y - g.hy[h], zz = z - g.hz[h];
                    const float rad = g.hr[h];
                    const float s32 = xx * xx + yy * yy + zz * zz;
                    if (s32 > rad * rad * 1.0001f) continue;   // clearly outside
                    const double d = sqrt((double)xx * (double)xx + (double)yy * (double)yy +
                                          (double)zz * (double)zz);
                    if (d < (double)rad && d > 0) {
                        r *= 0.55 * pow(d / (double)rad, -0.9);
                        const double k = -0.9 / (d * d);
                        gx += k * (double)xx;
                        gy += k * (double)yy;
                        gz += k * (double)zz;
                    }
                }
            }
    }
    corr[i] = r;
    if (gln) {
        gln[i] = gx;
        gln[(size_t)p.n + i] = gy;
        gln[2 * (size_t)p.n + i] = gz;
    }
}

}  // namespace

cudaError_t launch_halo_core(const HaloGrid &g, const Particles &p, double *corr, double *grad_ln,
                             cudaStream_t s) {
    if (p.n <= 0) return cudaSuccess;
    k_halo_core<<<(p.n + 255) / 256, 256, 0, s>>>(g, p, corr, grad_ln);
    return cudaGetLastError();
}

}  // namespace dmann
