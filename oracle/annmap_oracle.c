/*
 * annmap_oracle.c -- FP64 CPU restatement of the reference's CPU map path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): used by the tests as the reference answer,
 * by the smoke check, and as the timed CPU baseline of the benchmark.  The
 * product never links or calls it.
 *
 * Every step below follows the reference line by line, including the
 * float->double promotions and the order of floating-point operations, so
 * that this restatement reproduces the reference's own build bit for bit
 * (checked against golden maps made by oracle/ref_shim).  Two guards differ
 * from the reference only where the reference itself would produce NaN or
 * trap:
 *   - the dot product fed to acos() is clamped to [-1, 1] (genmap.cpp:137
 *     returns NaN when rounding pushes it above 1);
 *   - the progress counter `rec = Np/50` (genmap.cpp:46,71), which divides by
 *     zero for fewer than 50 particles, is not restated (it only prints).
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include "oracle.h"

/* src/datatypes.h:18-26, src/datatypes.cpp:5-10 */
static const double PI = 3.14159265358979323846;
static const double Msun_in_cgs = 1.9889212e+33;
static const double Mpc_in_cgs = 3.08568025e+24;
static const double eV_in_cgs = 1.602e-12;
static const double G_in_cgs = 6.67259e-8;
static const double c_in_cgs = 2.99792458e10;

void orc_params_setup(orc_params *p) {
    /* src/parameters.cpp:42-82 setupUnits (only the fields the map uses) */
    p->rho_crit_in_cgs = 3.0 * pow((100.0 * p->h100 / (Mpc_in_cgs * 1e-5)), 2) /
                         (8 * PI * G_in_cgs);
    p->length_to_cgs = p->Lbox_in_Mpc * Mpc_in_cgs;
    p->time_to_cgs = pow((p->rho_crit_in_cgs * G_in_cgs), (-0.5));
    p->density_to_cgs = p->rho_crit_in_cgs;
    if (p->mass_to_Msun == -1) {
        p->mass_to_cgs = p->density_to_cgs * pow(p->length_to_cgs, 3);
        p->mass_to_Msun = p->mass_to_cgs / Msun_in_cgs;
    } else {
        p->mass_to_cgs = p->mass_to_Msun * Msun_in_cgs;
    }
    p->velocity_to_cgs = p->length_to_cgs / p->time_to_cgs;
    p->annihilation_flux_to_cgs =
        (p->density_to_cgs * p->mass_to_cgs / pow(p->length_to_cgs, 2));

    /* src/flux/flux_ann_nosom.cpp:13-16 */
    p->unit_factor = pow(pow(c_in_cgs, 2) / (eV_in_cgs * 1.0e9), 2) /
                     (Mpc_in_cgs * 1.0e-3) * p->annihilation_flux_to_cgs;

    /* src/flux/flux_decay.cpp:10-13 */
    p->decay_unit_factor = pow(c_in_cgs, 2) / (eV_in_cgs * 1.0e9) / (Mpc_in_cgs * 1.0e-3) *
                           (p->mass_to_cgs / pow(p->length_to_cgs, 2));

    /* src/parameters.cpp:111-152 setupParams: observer angles about the centre */
    const double *opos = p->obs_pos, *cpos = p->centerpos;
    double radius = sqrt(pow(opos[0] - cpos[0], 2.0) + pow(opos[1] - cpos[1], 2.0) +
                         pow(opos[2] - cpos[2], 2.0));
    double otheta = acos((opos[2] - cpos[2]) / radius);
    double ophi = atan2((opos[1] - cpos[1]), (opos[0] - cpos[0]));
    if (ophi < 0.0) ophi += 2.0 * PI;
    p->otheta = otheta;
    p->ophi = ophi;

    /* src/parameters.cpp:183-289 setupRotation */
    double u = 0, v = -cos(otheta), w = sin(otheta) * sin(ophi);
    double rr = sqrt(u * u + v * v + w * w);
    u = u / rr;
    v = v / rr;
    w = w / rr;
    double c = -sin(otheta) * cos(ophi);
    double t = 1.0 - c;
    double s = rr;
    double rotm[3][3];
    if (rr > 0.0) {
        rotm[0][0] = u * u * t + c;
        rotm[0][1] = u * v * t + w * s;
        rotm[0][2] = u * w * t - v * s;
        rotm[1][0] = v * u * t - w * s;
        rotm[1][1] = v * v * t + c;
        rotm[1][2] = v * w * t + u * s;
        rotm[2][0] = w * u * t + v * s;
        rotm[2][1] = w * v * t - u * s;
        rotm[2][2] = w * w * t + c;
    } else {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) rotm[i][j] = (i == j) ? 1.0 : 0.0;
        if (cos(ophi) > 0.0) {
            rotm[0][0] = -1.0;
            rotm[1][1] = -1.0;
        }
    }
    double distance = sqrt(pow(opos[0] - cpos[0], 2.0) + pow(opos[1] - cpos[1], 2.0) +
                           pow(opos[2] - cpos[2], 2.0));
    const double *al = p->align_vec;
    double tv[3] = {cpos[0] + distance * al[0] - opos[0],
                    cpos[1] + distance * al[1] - opos[1],
                    cpos[2] + distance * al[2] - opos[2]};
    double xtmp = tv[0] * rotm[0][0] + tv[1] * rotm[1][0] + tv[2] * rotm[2][0];
    double ytmp = tv[0] * rotm[0][1] + tv[1] * rotm[1][1] + tv[2] * rotm[2][1];
    double ztmp = tv[0] * rotm[0][2] + tv[1] * rotm[1][2] + tv[2] * rotm[2][2];
    (void)xtmp;
    double gamma_t = fabs(atan2(ztmp, ytmp));
    gamma_t *= -1.0;
    double r2[3][3] = {{1.0, 0.0, 0.0},
                       {0.0, cos(gamma_t), sin(gamma_t)},
                       {0.0, -sin(gamma_t), cos(gamma_t)}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double val = 0;
            for (int k = 0; k < 3; k++) val += rotm[i][k] * r2[k][j];
            p->rotmatrix[i][j] = val;
        }

    /* src/datatypes.h:248-253 setNside; src/genmap.cpp:35-38 */
    p->npix = 12 * (int64_t)p->nside * (int64_t)p->nside;
    p->dOmega = 4 * PI / (double)p->npix;
    p->theta0 = acos(1.0 - p->dOmega / (2.0 * 3.141592));

    /* src/genmap.cpp:52-58: hires mass is held in a float */
    float hires = FLT_MAX;
    for (int i = 0; i < 10; i++)
        if (p->particle_masses[i] > 0 && p->particle_masses[i] < hires)
            hires = (float)p->particle_masses[i];
    p->hires_threshold = (double)hires * 1.1;
}

/* src/anglefuncs.cpp:15-52 */
static void calc_angles(double xpos, double ypos, double zpos, double distances,
                        const orc_params *p, double *costheta, double *phi) {
    double vec[3] = {xpos, ypos, zpos};
    double temp[3] = {0, 0, 0};
    for (int i = 0; i < 3; i++) {
        temp[i] = 0;
        for (int j = 0; j < 3; j++) temp[i] += p->rotmatrix[j][i] * vec[j];
    }
    *costheta = temp[2] / distances;
    double ph = atan2(temp[1], temp[0]);
    if (ph < 0) ph += 2.0 * PI;
    ph -= PI;
    if (ph < 0) ph = 2.0 * PI + ph;
    if (ph > 2 * PI) ph = ph - 2.0 * PI;
    *phi = ph;
}

typedef struct {
    double d, flux, costheta, phi, theta, ar;
    int64_t pix;
    int kept;
} geom_t;

/* src/halocore/halocore.cpp:70-83 coreFunc: arguments arrive as floats */
static double core_func(float x, float y, float z, float hxc, float hyc, float hzc,
                        float radius) {
    double xx = (x - hxc);
    double yy = (y - hyc);
    double zz = (z - hzc);
    double r = sqrt(xx * xx + yy * yy + zz * zz);
    double ratio = 1.0;
    if (r < radius) {
        if (r > 0) ratio = 0.55 * pow(r / radius, -0.9);
    }
    return ratio;
}

/* src/halocore/halocore.cpp:52-67 getCorrection, halos in file order */
static double core_correction(const orc_params *p, float x, float y, float z) {
    double xp = x, yp = y, zp = z;
    double r = 1.0;
    for (int i = 0; i < p->n_halos; i++)
        r *= core_func((float)xp, (float)yp, (float)zp, p->halo_x[i], p->halo_y[i], p->halo_z[i],
                       (float)(p->halo_r[i] / (0.73 * 40000.0)));
    return r;
}

/* The same product on unrounded doubles (exact_boost), and its gradient:
 * d ln(prod) / d pos = sum over the halos containing pos of
 * -0.9 (pos - c) / r^2.  Membership is decided as in core_func. */
static double core_correction_exact(const orc_params *p, double x, double y, double z,
                                    double grad_ln[3]) {
    double r = 1.0;
    if (grad_ln) grad_ln[0] = grad_ln[1] = grad_ln[2] = 0.0;
    for (int i = 0; i < p->n_halos; i++) {
        const double dx = x - p->halo_x[i], dy = y - p->halo_y[i], dz = z - p->halo_z[i];
        const double rr = sqrt(dx * dx + dy * dy + dz * dz);
        const double R = (double)(float)(p->halo_r[i] / (0.73 * 40000.0));
        if (rr < R && rr > 0) {
            r *= 0.55 * pow(rr / R, -0.9);
            if (grad_ln) {
                grad_ln[0] += -0.9 * dx / (rr * rr);
                grad_ln[1] += -0.9 * dy / (rr * rr);
                grad_ln[2] += -0.9 * dz / (rr * rr);
            }
        }
    }
    return r;
}

/* src/flux/flux_ann_adiabatic.cpp:17-26: the boost factor f(r) of the
 * adiabatically contracted host, r = |pos - cpos| * 40000 (kpc/h), and
 * d ln f / dr. */
static double adiabatic_factor(double r, double *dlnf_dr) {
    const double a = 1 + 0.0355872 * r, b = 1 + 0.10888 * pow(r, 0.76);
    if (dlnf_dr)
        *dlnf_dr = 1.76 * 0.0355872 / a - 3.34211 * 0.10888 * 0.76 * pow(r, -0.24) / b - 0.13 / r;
    return (14.6534 * pow(a, 1.76)) / (pow(b, 3.34211) * pow(r, 0.13));
}

/* d ln(boost) / d pos of the position-dependent flux laws (the adiabatic
 * factor squared, the halo-core factor squared); zero for the others.  On
 * the parity path the halo-core terms take the float differences of
 * halocore.cpp:70-83 (each term then in double). */
static void boost_grad_ln(const orc_params *p, double x, double y, double z, double g[3]) {
    g[0] = g[1] = g[2] = 0.0;
    if (p->flux_model == ORC_FLUX_ADIABATIC) {
        const double dx = x - p->centerpos[0], dy = y - p->centerpos[1], dz = z - p->centerpos[2];
        const double rc = sqrt(dx * dx + dy * dy + dz * dz);
        if (!(rc > 0)) return;
        double dl;
        adiabatic_factor(rc * 40000.0, &dl);
        const double k = 2.0 * dl * 40000.0 / rc;
        g[0] = k * dx;
        g[1] = k * dy;
        g[2] = k * dz;
    } else if (p->flux_model == ORC_FLUX_CORE_NOSOM) {
        double gl[3] = {0.0, 0.0, 0.0};
        if (p->exact_boost) {
            core_correction_exact(p, x, y, z, gl);
        } else {
            const float xf = (float)x, yf = (float)y, zf = (float)z;
            for (int i = 0; i < p->n_halos; i++) {
                const float xx = xf - p->halo_x[i], yy = yf - p->halo_y[i], zz = zf - p->halo_z[i];
                const double rr = sqrt((double)xx * xx + (double)yy * yy + (double)zz * zz);
                const float R = (float)(p->halo_r[i] / (0.73 * 40000.0));
                if (rr < R && rr > 0) {
                    gl[0] += -0.9 * xx / (rr * rr);
                    gl[1] += -0.9 * yy / (rr * rr);
                    gl[2] += -0.9 * zz / (rr * rr);
                }
            }
        }
        for (int k = 0; k < 3; k++) g[k] = 2.0 * gl[k];
    }
}

/* getflux of the flux law p->flux_model for one particle at distance d, each
 * in the operation order of its plugin (sigmav only read by the laws that
 * use it). */
static double orc_flux(const orc_params *p, double mass, double dens, double sigmav,
                       double px, double py, double pz, double d) {
    const double uf = p->unit_factor;
    switch (p->flux_model) {
    case ORC_FLUX_SOMV: { /* src/flux/flux_ann_somv.cpp:16-43: SAT_V 1 km/s, FACTOR 1e4 */
        double v = sigmav * p->velocity_to_cgs;
        v /= 1.0e5;
        if (v < 1) v = 1;
        double somer_v = c_in_cgs / v / 1.0e4;
        return uf * somer_v * dens * mass / (4.0 * PI * d * d);
    }
    case ORC_FLUX_SOMV2: { /* src/flux/flux_ann_somv2.cpp:16-44: SAT_V 5 km/s, FACTOR 1e8 */
        double v = sigmav * p->velocity_to_cgs;
        v /= 1.0e5;
        if (v < 5) v = 5;
        double somer_v = c_in_cgs / v;
        somer_v *= (somer_v / 1.0e8);
        return uf * somer_v * dens * mass / (4.0 * PI * d * d);
    }
    case ORC_FLUX_PWAVE: { /* src/flux/flux_ann_pwave.cpp:13-31 */
        double somer_v = (sigmav * p->velocity_to_cgs) / c_in_cgs;
        somer_v = somer_v * somer_v;
        return uf * somer_v * dens * mass / (4.0 * PI * d * d);
    }
    case ORC_FLUX_DECAY: /* src/flux/flux_decay.cpp:9-16 */
        return p->decay_unit_factor * mass / (4.0 * PI * d * d);
    case ORC_FLUX_ADIABATIC: { /* src/flux/flux_ann_adiabatic.cpp:10-33 */
        double dx = px - p->centerpos[0];
        double dy = py - p->centerpos[1];
        double dz = pz - p->centerpos[2];
        double r = sqrt(dx * dx + dy * dy + dz * dz) * 40000.0;
        double factor = (14.6534 * pow(1 + 0.0355872 * r, 1.76)) /
                        (pow(1 + 0.10888 * pow(r, 0.76), 3.34211) * pow(r, 0.13));
        double fluxes = uf * dens * mass / (4.0 * PI * d * d);
        fluxes *= (factor * factor);
        return fluxes;
    }
    case ORC_FLUX_CORE_NOSOM: { /* src/flux/flux_ann_core_nosom.cpp:9-17 */
        double r = p->exact_boost ? core_correction_exact(p, px, py, pz, NULL)
                                  : core_correction(p, (float)px, (float)py, (float)pz);
        return r * r * uf * dens * mass / (4.0 * PI * d * d);
    }
    default: /* src/flux/flux_ann_nosom.cpp:12-23 */
        return uf * dens * mass / (4.0 * PI * d * d);
    }
}

/* genmap.cpp:82-106 for one particle.  The inputs are the float values
 * promoted to double (the finite-difference checks pass unrounded doubles). */
static void particle_geom_dv(const orc_params *p, const orc_hpx *hb, double mass,
                             double dens, double hsmooth, double px, double py,
                             double pz, double sigmav, geom_t *g) {
    g->kept = 0;
    if (mass >= p->hires_threshold || dens < 0) return;
    g->kept = 1;
    double ox = p->obs_pos[0], oy = p->obs_pos[1], oz = p->obs_pos[2];
    double dx = px - ox, dy = py - oy, dz = pz - oz;
    g->d = sqrt(dx * dx + dy * dy + dz * dz);
    g->flux = orc_flux(p, mass, dens, sigmav, px, py, pz, g->d);
    calc_angles(dx, dy, dz, g->d, p, &g->costheta, &g->phi);
    double ct = g->costheta;
    if (ct > 1.0) ct = 1.0; /* acos argument guard */
    if (ct < -1.0) ct = -1.0;
    g->theta = acos(ct);
    g->ar = hsmooth / g->d;
    g->pix = orc_hpx_ang2pix(hb, g->theta, g->phi);
}

static void particle_geom_d(const orc_params *p, const orc_hpx *hb, double mass,
                            double dens, double hsmooth, double px, double py,
                            double pz, geom_t *g) {
    particle_geom_dv(p, hb, mass, dens, hsmooth, px, py, pz, 0.0, g);
}

static void particle_geom(const orc_params *p, const orc_hpx *hb, float mass,
                          float dens, float hsmooth, float px, float py,
                          float pz, geom_t *g) {
    particle_geom_d(p, hb, (double)mass, (double)dens, (double)hsmooth,
                    (double)px, (double)py, (double)pz, g);
}

void orc_particle_geom(const orc_params *p, float mass, float dens,
                       float hsmooth, float x, float y, float z, double out[8]) {
    orc_hpx hb;
    orc_hpx_init(&hb, p->nside);
    geom_t g;
    memset(&g, 0, sizeof g);
    particle_geom(p, &hb, mass, dens, hsmooth, x, y, z, &g);
    out[0] = g.d;
    out[1] = g.flux;
    out[2] = g.costheta;
    out[3] = g.phi;
    out[4] = g.theta;
    out[5] = g.ar;
    out[6] = (double)g.pix;
    out[7] = (double)g.kept;
}

typedef struct {
    const orc_params *p;
    const float *m, *rho, *h, *x, *y, *z, *sv;
    int64_t i0, i1;
    double *map;
    orc_stats st;
    int rc;
} job_t;

static void *render_range(void *arg) {
    job_t *J = (job_t *)arg;
    const orc_params *p = J->p;
    orc_hpx hb;
    orc_hpx_init(&hb, p->nside);
    int32_t *list = (int32_t *)malloc(sizeof(int32_t) * (size_t)p->npix);
    double *weight = (double *)malloc(sizeof(double) * (size_t)p->npix);
    if (!list || !weight) {
        free(list);
        free(weight);
        J->rc = -1;
        return NULL;
    }
    double *map = J->map;
    memset(&J->st, 0, sizeof J->st);
    for (int64_t i = J->i0; i < J->i1; i++) {
        geom_t g;
        particle_geom_dv(p, &hb, (double)J->m[i], (double)J->rho[i], (double)J->h[i],
                         (double)J->x[i], (double)J->y[i], (double)J->z[i],
                         J->sv ? (double)J->sv[i] : 0.0, &g);
        if (!g.kept) {
            J->st.skipped++;
            continue;
        }
        J->st.kept++;
        /* anglefuncs.cpp:55-71 ang2vec */
        double sz = sin(g.theta);
        double vx = sz * cos(g.phi), vy = sz * sin(g.phi), vz = cos(g.theta);
        /* genmap.cpp:107-110 */
        if (2.0 * g.ar < p->theta0) {
            map[g.pix] += g.flux;
            J->st.single_small++;
            J->st.deposits++;
            continue;
        }
        /* genmap.cpp:119-128 */
        int64_t npd = orc_hpx_query_disc_list(&hb, g.theta, g.phi, 2.0 * g.ar, list);
        if (npd < 2) {
            map[g.pix] += g.flux;
            J->st.single_disc++;
            J->st.deposits++;
            continue;
        }
        J->st.disc++;
        J->st.deposits += npd;
        /* genmap.cpp:132-145 */
        double weight_norm = 0.0;
        for (int64_t j = 0; j < npd; j++) {
            double pv[3];
            orc_hpx_pix2vec(&hb, list[j], pv);
            double dot = pv[0] * vx + pv[1] * vy + pv[2] * vz;
            if (dot > 1.0) dot = 1.0; /* acos argument guard */
            if (dot < -1.0) dot = -1.0;
            double d2 = acos(dot) / g.ar;
            d2 = d2 * d2;
            weight[j] = exp(-0.5 * d2 / 0.333);
            weight_norm += weight[j];
        }
        /* genmap.cpp:148-153 */
        for (int64_t j = 0; j < npd; j++) {
            weight[j] = weight[j] / weight_norm;
            map[list[j]] += weight[j] * g.flux;
        }
    }
    free(list);
    free(weight);
    J->rc = 0;
    return NULL;
}

int orc_render(const orc_params *p, const float *mass, const float *dens,
               const float *hsmooth, const float *x, const float *y,
               const float *z, int64_t n, double *map, orc_stats *stats,
               int nthreads) {
    return orc_render_v(p, mass, dens, hsmooth, x, y, z, NULL, n, map, stats, nthreads);
}

int orc_render_v(const orc_params *p, const float *mass, const float *dens,
                 const float *hsmooth, const float *x, const float *y,
                 const float *z, const float *sigmav, int64_t n, double *map,
                 orc_stats *stats, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (n < (int64_t)nthreads * 4) nthreads = 1;
    job_t *jobs = (job_t *)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) {
        free(jobs);
        free(th);
        return -1;
    }
    int rc = 0;
    for (int t = 0; t < nthreads; t++) {
        job_t *J = &jobs[t];
        J->p = p;
        J->m = mass; J->rho = dens; J->h = hsmooth;
        J->x = x; J->y = y; J->z = z; J->sv = sigmav;
        J->i0 = n * t / nthreads;
        J->i1 = n * (t + 1) / nthreads;
        if (nthreads == 1) {
            J->map = map;
        } else {
            J->map = (double *)calloc((size_t)p->npix, sizeof(double));
            if (!J->map) rc = -1;
        }
    }
    if (rc == 0) {
        if (nthreads == 1) {
            render_range(&jobs[0]);
        } else {
            for (int t = 0; t < nthreads; t++)
                pthread_create(&th[t], NULL, render_range, &jobs[t]);
            for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
            for (int t = 0; t < nthreads; t++) {
                const double *pm = jobs[t].map;
                for (int64_t k = 0; k < p->npix; k++) map[k] += pm[k];
            }
        }
    }
    orc_stats tot;
    memset(&tot, 0, sizeof tot);
    for (int t = 0; t < nthreads; t++) {
        if (jobs[t].rc != 0) rc = -1;
        tot.kept += jobs[t].st.kept;
        tot.skipped += jobs[t].st.skipped;
        tot.single_small += jobs[t].st.single_small;
        tot.single_disc += jobs[t].st.single_disc;
        tot.disc += jobs[t].st.disc;
        tot.deposits += jobs[t].st.deposits;
        if (nthreads > 1) free(jobs[t].map);
    }
    if (stats) *stats = tot;
    free(jobs);
    free(th);
    return rc;
}

double orc_finalize(const orc_params *p, double *map) {
    double totalC = 0;
    for (int64_t i = 0; i < p->npix; i++) {
        totalC += map[i];
        map[i] /= p->dOmega;
    }
    return totalC;
}

/* ------------------------------------------------------------------ adjoint
 * The derivative of L = sum_p G[p] map[p] (map after the dOmega division)
 * with the disc pixel sets held fixed; see oracle.h for the formulas. */

/* Disc pixels and weights of one kept particle; returns the pixel count, or
 * -1 for a single-pixel deposit (genmap.cpp:107-128). */
static int64_t disc_pixels(const orc_params *p, const orc_hpx *hb, const geom_t *g,
                           int32_t *list) {
    if (2.0 * g->ar < p->theta0) return -1;
    int64_t npd = orc_hpx_query_disc_list(hb, g->theta, g->phi, 2.0 * g->ar, list);
    return npd < 2 ? -1 : npd;
}

static void ang2vec(const geom_t *g, double v[3]) {
    double sz = sin(g->theta);
    v[0] = sz * cos(g->phi);
    v[1] = sz * sin(g->phi);
    v[2] = cos(g->theta);
}

/* w of one disc pixel exactly as genmap.cpp:133-143 computes it; also
 * returns the pixel vector and the angle. */
static double pixel_weight(const orc_hpx *hb, int32_t pix, const double v[3], double ar,
                           double pv[3], double *alpha, double *dotc) {
    orc_hpx_pix2vec(hb, pix, pv);
    double dot = pv[0] * v[0] + pv[1] * v[1] + pv[2] * v[2];
    if (dot > 1.0) dot = 1.0;
    if (dot < -1.0) dot = -1.0;
    double a = acos(dot);
    double d2 = a / ar;
    d2 = d2 * d2;
    *alpha = a;
    *dotc = dot;
    return exp(-0.5 * d2 / 0.333);
}

double orc_particle_loss(const orc_params *p, double mass, double dens, double hsmooth,
                         double x, double y, double z, const double *G, uint64_t *sig) {
    return orc_particle_loss_v(p, mass, dens, hsmooth, x, y, z, 0.0, G, sig);
}

double orc_particle_loss_v(const orc_params *p, double mass, double dens, double hsmooth,
                           double x, double y, double z, double sigmav, const double *G,
                           uint64_t *sig) {
    orc_hpx hb;
    orc_hpx_init(&hb, p->nside);
    geom_t g;
    memset(&g, 0, sizeof g);
    particle_geom_dv(p, &hb, mass, dens, hsmooth, x, y, z, sigmav, &g);
    uint64_t hsig = 1469598103934665603ull; /* FNV-1a over the branch and pixels */
#define SIG(v) do { hsig ^= (uint64_t)(v); hsig *= 1099511628211ull; } while (0)
    double L = 0.0;
    if (!g.kept || !(g.d > 0.0)) {
        SIG(0);
    } else {
        int32_t *list = (int32_t *)malloc(sizeof(int32_t) * (size_t)p->npix);
        int64_t npd = list ? disc_pixels(p, &hb, &g, list) : -1;
        if (npd < 0) {
            SIG(1);
            SIG(g.pix);
            L = G[g.pix] * g.flux / p->dOmega;
        } else {
            double v[3];
            ang2vec(&g, v);
            SIG(2);
            double S = 0.0;
            for (int64_t j = 0; j < npd; j++) {
                double pv[3], a, dc;
                S += pixel_weight(&hb, list[j], v, g.ar, pv, &a, &dc);
                SIG(list[j]);
            }
            for (int64_t j = 0; j < npd; j++) {
                double pv[3], a, dc;
                double w = pixel_weight(&hb, list[j], v, g.ar, pv, &a, &dc);
                L += G[list[j]] * ((w / S) * g.flux) / p->dOmega;
            }
        }
        free(list);
    }
#undef SIG
    if (sig) *sig = hsig;
    return L;
}

void orc_particle_losses(const orc_params *p, const double *mass, const double *dens,
                         const double *hsmooth, const double *x, const double *y,
                         const double *z, int64_t n, const double *G, double *L,
                         uint64_t *sig) {
    for (int64_t i = 0; i < n; i++)
        L[i] = orc_particle_loss(p, mass[i], dens[i], hsmooth[i], x[i], y[i], z[i], G,
                                 sig ? sig + i : NULL);
}

void orc_particle_losses_v(const orc_params *p, const double *mass, const double *dens,
                           const double *hsmooth, const double *x, const double *y,
                           const double *z, const double *sigmav, int64_t n, const double *G,
                           double *L, uint64_t *sig) {
    for (int64_t i = 0; i < n; i++)
        L[i] = orc_particle_loss_v(p, mass[i], dens[i], hsmooth[i], x[i], y[i], z[i],
                                   sigmav ? sigmav[i] : 0.0, G, sig ? sig + i : NULL);
}

int orc_adjoint(const orc_params *p, const float *mass, const float *dens,
                const float *hsmooth, const float *x, const float *y, const float *z,
                int64_t n, const double *G, double *grad, double oacc[12]) {
    return orc_adjoint_v(p, mass, dens, hsmooth, x, y, z, NULL, n, G, grad, oacc);
}

int orc_adjoint_v(const orc_params *p, const float *mass, const float *dens,
                  const float *hsmooth, const float *x, const float *y, const float *z,
                  const float *sigmav, int64_t n, const double *G, double *grad,
                  double oacc[12]) {
    /* every law: the flux is rho m (or m under decay) over d^2 times a
       factor of sigma v (somv, somv2, pwave) or of the position (adiabatic,
       ann_core_nosom), whose log-gradient joins the position gradient */
    if (p->flux_model < 0 || p->flux_model > 6) return -2;
    orc_hpx hb;
    orc_hpx_init(&hb, p->nside);
    int32_t *list = (int32_t *)malloc(sizeof(int32_t) * (size_t)p->npix);
    if (!list) return -1;
    const double inv_dO = 1.0 / p->dOmega;
    for (int k = 0; k < 12; k++) oacc[k] = 0.0;
    for (int64_t i = 0; i < n; i++) {
        for (int k = 0; k < 6; k++) grad[k * n + i] = 0.0;
        geom_t g;
        const double sv = sigmav ? (double)sigmav[i] : 0.0;
        particle_geom_dv(p, &hb, (double)mass[i], (double)dens[i], (double)hsmooth[i],
                         (double)x[i], (double)y[i], (double)z[i], sv, &g);
        if (!g.kept || !(g.d > 0.0) || !isfinite(g.flux) || !isfinite(g.ar)) continue;
        double Gb, KT = 0.0, KV[3] = {0.0, 0.0, 0.0};
        int64_t npd = disc_pixels(p, &hb, &g, list);
        if (npd < 0) {
            Gb = G[g.pix] * inv_dO;
        } else {
            double v[3];
            ang2vec(&g, v);
            double S = 0.0, A = 0.0;
            for (int64_t j = 0; j < npd; j++) {
                double pv[3], a, dc;
                double w = pixel_weight(&hb, list[j], v, g.ar, pv, &a, &dc);
                S += w;
                A += G[list[j]] * w;
            }
            double Gm = A / S;
            double V[3] = {0.0, 0.0, 0.0}, T = 0.0;
            for (int64_t j = 0; j < npd; j++) {
                double pv[3], a, dc;
                double w = pixel_weight(&hb, list[j], v, g.ar, pv, &a, &dc);
                double q = (G[list[j]] - Gm) * w;
                double e[3] = {pv[0] - dc * v[0], pv[1] - dc * v[1], pv[2] - dc * v[2]};
                double sa = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                double f = sa > 0.0 ? q * a / sa : 0.0;
                for (int k = 0; k < 3; k++) V[k] += f * e[k];
                T += q * a * a;
            }
            double K = (1.0 / 0.333) * g.flux / (S * g.ar * g.ar) * inv_dO;
            Gb = Gm * inv_dO;
            KT = K * T;
            for (int k = 0; k < 3; k++) KV[k] = K * V[k];
        }
        double u[3] = {(double)x[i] - p->obs_pos[0], (double)y[i] - p->obs_pos[1],
                       (double)z[i] - p->obs_pos[2]};
        double d = g.d;
        double uh[3] = {u[0] / d, u[1] / d, u[2] / d};
        /* F = fd rho m with fd the law's flux per unit rho m (its sigma v
           factor included), or fd m under the decay law
           (src/flux/flux_decay.cpp:9-16): then dL/drho = 0 */
        int decay = p->flux_model == 4;
        double fd = orc_flux(p, 1.0, 1.0, sv, (double)x[i], (double)y[i], (double)z[i], d);
        double rho_f = decay ? 1.0 : (double)dens[i];
        double F = fd * rho_f * (double)mass[i];
        double w[3] = {-KV[0], -KV[1], KV[2]}; /* D K V, D = diag(-1,-1,1) */
        double cr = -(2.0 * Gb * F + KT) / d;
        double gb[3];   /* the boost's own position dependence (not the observer's) */
        boost_grad_ln(p, (double)x[i], (double)y[i], (double)z[i], gb);
        for (int j = 0; j < 3; j++) {
            double rw = p->rotmatrix[j][0] * w[0] + p->rotmatrix[j][1] * w[1] +
                        p->rotmatrix[j][2] * w[2];
            double gj = cr * uh[j] + rw / d;
            grad[j * n + i] = gj + Gb * F * gb[j];
            oacc[j] += gj;
        }
        grad[3 * n + i] = Gb * fd * rho_f;
        grad[4 * n + i] = decay ? 0.0 : Gb * fd * (double)mass[i];
        if (npd >= 0) {
            grad[5 * n + i] = KT / (double)hsmooth[i];
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++) oacc[3 + 3 * j + k] += uh[j] * w[k];
        }
    }
    free(list);
    return 0;
}
