/*
 * oracle.h -- CPU FP64 oracle for the annihilation sky-map projection.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, the
 * C++ host API, the Python package) links, loads or calls this code.  Only
 * the test suite, the smoke check and the CPU-baseline leg of the benchmark
 * use it, and only as the reference answer / the timed CPU baseline.
 *
 * What it restates (paths relative to the reference project):
 *   - src/genmap.cpp:22-175            MapGenerator::start, the CPU map loop
 *   - src/anglefuncs.cpp:15-52         calc_angles
 *   - src/anglefuncs.cpp:55-71         ang2vec
 *   - src/flux/flux_ann_nosom.cpp:12-23 getflux (the default flux plugin)
 *   - src/parameters.cpp:42-82         Parameters::setupUnits
 *   - src/parameters.cpp:111-152       Parameters::setupParams (observer angles)
 *   - src/parameters.cpp:183-289       Parameters::setupRotation
 *   - src/datatypes.h:248-253          Map::setNside (Npix, dOmega)
 *   - HEALPix C++ 3.00 Healpix_Base RING-scheme ang2pix / pix2vec /
 *     query_disc (non-inclusive) / ring_above / ring2z / get_ring_info_small,
 *     called from src/genmap.cpp:40,106,119,135.  HEALPix is a third-party
 *     library that the reference does not vendor; these functions are
 *     restated from the published scheme (Gorski et al. 2005, ApJ 622:759)
 *     and pinned by identities and a brute-force disc search in the tests.
 *
 * Parity pin: the reference's own genmap.cpp / parameters.cpp /
 * anglefuncs.cpp / datatypes.cpp / flux_ann_nosom.cpp are compiled from the
 * reference sources by oracle/ref_shim (HEALPix and XDR replaced by shims
 * that call the HEALPix functions below) and their maps are committed as
 * golden fixtures under tests/golden/.  The tests check this oracle against
 * those fixtures bit for bit.
 */
#ifndef DMANN_ORACLE_H
#define DMANN_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- HEALPix RING scheme (FP64) ---------------- */
typedef struct {
    int64_t nside, npix, ncap;
    double fact1, fact2;
} orc_hpx;

void    orc_hpx_init(orc_hpx *b, int64_t nside);
int64_t orc_hpx_ang2pix(const orc_hpx *b, double theta, double phi);
void    orc_hpx_pix2vec(const orc_hpx *b, int64_t pix, double v[3]);
void    orc_hpx_pix2ang(const orc_hpx *b, int64_t pix, double *theta, double *phi);
int64_t orc_hpx_ring_above(const orc_hpx *b, double z);
double  orc_hpx_ring2z(const orc_hpx *b, int64_t ring);
void    orc_hpx_ring_info(const orc_hpx *b, int64_t ring, int64_t *startpix,
                          int64_t *ringpix, int *shifted);
/* Non-inclusive query_disc: every pixel whose centre lies within `radius`
 * of (theta, phi).  Writes half-open pixel ranges [lo, hi) in increasing
 * pixel order into ranges[2*k], ranges[2*k+1]; returns the number of ranges
 * (ranges may be NULL to count only; at most 2*4*nside+2 ranges).  The total
 * pixel count is stored into *npix_out when not NULL. */
int64_t orc_hpx_query_disc(const orc_hpx *b, double theta, double phi,
                           double radius, int64_t *ranges, int64_t *npix_out);
/* Same, expanded to the pixel list in increasing order (the vector form the
 * reference calls).  Returns the count; `out` must hold npix entries. */
int64_t orc_hpx_query_disc_list(const orc_hpx *b, double theta, double phi,
                                double radius, int32_t *out);

/* ---------------- Parameters setup (FP64) ---------------- */
typedef struct {
    /* inputs (as read from the info file) */
    double h100, Omega_M, Lbox_in_Mpc, mass_to_Msun, redshift;
    double centerpos[3], obs_pos[3], align_vec[3];
    double particle_masses[10];
    int nside;
    /* derived */
    double rho_crit_in_cgs, length_to_cgs, mass_to_cgs, density_to_cgs,
           time_to_cgs, velocity_to_cgs, annihilation_flux_to_cgs;
    double otheta, ophi;
    double rotmatrix[3][3];
    double unit_factor;       /* flux_ann_nosom.cpp:13-16 */
    double hires_threshold;   /* (double)(float)min(particle_masses>0) * 1.1 */
    int64_t npix;
    double dOmega, theta0;    /* theta0 = acos(1 - dOmega/(2*3.141592)) */
    /* flux law (set before orc_params_setup; 0 = nosom): the reference's
     * link-time getflux plugins in the src/flux directory, see orc_flux */
    int flux_model;
    double decay_unit_factor; /* flux_decay.cpp:10-13 (derived) */
    /* halo table of the ann_core_nosom law (halocore.cpp: x y z radius per
     * line, in file order; not owned) */
    const float *halo_x, *halo_y, *halo_z, *halo_r;
    int n_halos;
    /* 0: the halo-core factor rounds positions and centres to float as
     * halocore.cpp does (the parity path).  1: it takes the unrounded
     * doubles -- the smooth function whose derivative the adjoint returns,
     * for central differences finer than the float rounding. */
    int exact_boost;
} orc_params;

/* Flux laws, in the numbering of the C ABI's dmann_flux. */
enum { ORC_FLUX_NOSOM = 0, ORC_FLUX_SOMV = 1, ORC_FLUX_SOMV2 = 2, ORC_FLUX_PWAVE = 3,
       ORC_FLUX_DECAY = 4, ORC_FLUX_ADIABATIC = 5, ORC_FLUX_CORE_NOSOM = 6 };

/* Fills every derived field from the inputs (setupUnits, setupParams,
 * setupRotation, setNside and the per-map constants of genmap.cpp). */
void orc_params_setup(orc_params *p);

/* ---------------- the map loop ---------------- */
/* Counters filled by orc_render. */
typedef struct {
    int64_t kept, skipped, single_small, single_disc, disc, deposits;
} orc_stats;

/* Restates MapGenerator::start (genmap.cpp:67-156) on SoA float inputs:
 * adds the flux of every kept particle into map[0..npix) (NOT divided by
 * dOmega; call orc_finalize for that).  nthreads <= 1 runs the reference's
 * serial loop; nthreads > 1 shards particles over threads with private maps
 * summed in thread order at the end.  Returns 0 on success. */
int orc_render(const orc_params *p, const float *mass, const float *dens,
               const float *hsmooth, const float *x, const float *y,
               const float *z, int64_t n, double *map, orc_stats *stats,
               int nthreads);

/* orc_render with the particles' velocity dispersion sigmav (float32, code
 * units; needed by the somv, somv2 and pwave laws, may be NULL otherwise). */
int orc_render_v(const orc_params *p, const float *mass, const float *dens,
                 const float *hsmooth, const float *x, const float *y,
                 const float *z, const float *sigmav, int64_t n, double *map,
                 orc_stats *stats, int nthreads);

/* genmap.cpp:161-169: returns totalC = sum(map) and divides map by dOmega. */
double orc_finalize(const orc_params *p, double *map);

/* Per-particle geometry exactly as the loop computes it (for tests):
 * out[0..7] = d, flux, costheta, phi, theta, angular_radius, pix, kept. */
void orc_particle_geom(const orc_params *p, float mass, float dens,
                       float hsmooth, float x, float y, float z, double out[8]);

/* ---------------- the adjoint (FP64 CPU reference) ----------------
 * Loss L = sum_p G[p] map[p], map as orc_finalize leaves it (divided by
 * dOmega).  For one kept particle with u = pos - opos, d = |u|,
 * F = unit_factor rho m / (4 pi d^2), ar = h/d, direction n (ang2vec of the
 * particle's theta, phi: n = D R^T u / d with D = diag(-1, -1, 1), the pi
 * shift of phi) and disc weights w_p = exp(-c alpha_p^2 / ar^2), c = 0.5/0.333,
 * alpha_p = acos(v_p . n), S = sum w_p, the map gets F w_p / S / dOmega.
 * With g = G / dOmega, Gb = sum g_p w_p / S, q_p = (g_p - Gb) w_p,
 * V = sum q_p alpha_p / sin(alpha_p) (v_p - cos(alpha_p) n), T = sum q_p alpha_p^2
 * and K = 2 c F / (S ar^2):
 *   dL/dm = Gb F/m,  dL/drho = Gb F/rho,  dL/dh = K T / h,
 *   dL/dpos = -(2 Gb F + K T)/d u/d + (K/d) R D V,
 *   dL/drot[j][a] = K (D V)_a u_j / d.
 * A single-pixel deposit has Gb = g[cpix] and V = T = 0.  The pixel sets are
 * held fixed. */

/* L_i of one particle from double inputs (no float rounding), and in *sig
 * (may be NULL) a hash of its branch and pixel set: the finite-difference
 * checks use it to confirm the set did not change between the two sides. */
double orc_particle_loss(const orc_params *p, double mass, double dens, double hsmooth,
                         double x, double y, double z, const double *G, uint64_t *sig);

/* orc_particle_loss with a velocity dispersion (the somv, somv2 and pwave
 * laws). */
double orc_particle_loss_v(const orc_params *p, double mass, double dens, double hsmooth,
                           double x, double y, double z, double sigmav, const double *G,
                           uint64_t *sig);

/* orc_particle_loss_v over n particles (sigmav may be NULL). */
void orc_particle_losses_v(const orc_params *p, const double *mass, const double *dens,
                           const double *hsmooth, const double *x, const double *y,
                           const double *z, const double *sigmav, int64_t n, const double *G,
                           double *L, uint64_t *sig);

/* orc_particle_loss over n particles (double SoA inputs). */
void orc_particle_losses(const orc_params *p, const double *mass, const double *dens,
                         const double *hsmooth, const double *x, const double *y,
                         const double *z, int64_t n, const double *G, double *L,
                         uint64_t *sig);

/* grad = [6][n] (x, y, z, m, rho, h); oacc[0..2] = sum_i dL/du_i (u = pos -
 * opos: the geometric terms only), oacc[3..11] = dL/drot (row-major).  Every
 * flux law: the adiabatic and ann_core_nosom factors depend on the particle's
 * position, and d ln(factor) / d pos joins dL/dpos (halo-core membership
 * held fixed).  Returns 0 on success, -2 for an unknown flux law. */
int orc_adjoint(const orc_params *p, const float *mass, const float *dens,
                const float *hsmooth, const float *x, const float *y, const float *z,
                int64_t n, const double *G, double *grad, double oacc[12]);

/* The same with the velocity dispersions of the somv, somv2 and pwave laws
 * (sigmav may be NULL: zero); sigma v is not differentiated. */
int orc_adjoint_v(const orc_params *p, const float *mass, const float *dens,
                  const float *hsmooth, const float *x, const float *y, const float *z,
                  const float *sigmav, int64_t n, const double *G, double *grad,
                  double oacc[12]);

#ifdef __cplusplus
}
#endif
#endif
