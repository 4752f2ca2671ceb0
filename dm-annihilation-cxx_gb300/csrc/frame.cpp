// frame.cpp -- observer rotation, code units and the hires-mass threshold.
// Built with -ffp-contract=off so the FP64 results are those of the
// reference's own build on any host (x86 or Arm).
#include "frame.h"

#include <cfloat>
#include <cmath>

namespace dmann {

namespace {
constexpr double PI = 3.14159265358979323846;       // src/datatypes.h:18-26
constexpr double Msun_in_cgs = 1.9889212e+33;       // src/datatypes.cpp:5-10
constexpr double Mpc_in_cgs = 3.08568025e+24;
constexpr double eV_in_cgs = 1.602e-12;
constexpr double G_in_cgs = 6.67259e-8;
constexpr double c_in_cgs = 2.99792458e10;
}  // namespace

bool observer_rotation(const double opos[3], const double cpos[3], const double align[3],
                       double rot[9], double *otheta_out, double *ophi_out) {
    // setupParams (parameters.cpp:137-150)
    const double radius = std::sqrt(std::pow(opos[0] - cpos[0], 2.0) + std::pow(opos[1] - cpos[1], 2.0) +
                                    std::pow(opos[2] - cpos[2], 2.0));
    if (!(radius > 0.0)) return false;
    const double otheta = std::acos((opos[2] - cpos[2]) / radius);
    double ophi = std::atan2((opos[1] - cpos[1]), (opos[0] - cpos[0]));
    if (ophi < 0.0) ophi += 2.0 * PI;
    if (otheta_out) *otheta_out = otheta;
    if (ophi_out) *ophi_out = ophi;

    // setupRotation (parameters.cpp:188-237): rotate the centre direction
    // r = -(sin t cos p, sin t sin p, cos t) onto e1 about r x e1.
    double u = 0, v = -std::cos(otheta), w = std::sin(otheta) * std::sin(ophi);
    const double rr = std::sqrt(u * u + v * v + w * w);
    u = u / rr;
    v = v / rr;
    w = w / rr;
    const double c = -std::sin(otheta) * std::cos(ophi);
    const double t = 1.0 - c;
    const double s = rr;
    double m[3][3];
    if (rr > 0.0) {
        m[0][0] = u * u * t + c;
        m[0][1] = u * v * t + w * s;
        m[0][2] = u * w * t - v * s;
        m[1][0] = v * u * t - w * s;
        m[1][1] = v * v * t + c;
        m[1][2] = v * w * t + u * s;
        m[2][0] = w * u * t + v * s;
        m[2][1] = w * v * t - u * s;
        m[2][2] = w * w * t + c;
    } else {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) m[i][j] = (i == j) ? 1.0 : 0.0;
        if (std::cos(ophi) > 0.0) {
            m[0][0] = -1.0;
            m[1][1] = -1.0;
        }
    }
    // parameters.cpp:240-287: roll about x so the alignment vector, seen
    // from the observer, lies in the horizontal plane.
    const double distance = radius;
    const double tv[3] = {cpos[0] + distance * align[0] - opos[0],
                          cpos[1] + distance * align[1] - opos[1],
                          cpos[2] + distance * align[2] - opos[2]};
    const double ytmp = tv[0] * m[0][1] + tv[1] * m[1][1] + tv[2] * m[2][1];
    const double ztmp = tv[0] * m[0][2] + tv[1] * m[1][2] + tv[2] * m[2][2];
    const double gamma = -std::fabs(std::atan2(ztmp, ytmp));
    const double r2[3][3] = {{1.0, 0.0, 0.0},
                             {0.0, std::cos(gamma), std::sin(gamma)},
                             {0.0, -std::sin(gamma), std::cos(gamma)}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double val = 0;
            for (int k = 0; k < 3; k++) val += m[i][k] * r2[k][j];
            rot[3 * i + j] = val;
        }
    return true;
}

void setup_units(double h100, double Lbox_in_Mpc, double mass_to_Msun, CodeUnits *u) {
    u->rho_crit_in_cgs = 3.0 * std::pow((100.0 * h100 / (Mpc_in_cgs * 1e-5)), 2) / (8 * PI * G_in_cgs);
    u->length_to_cgs = Lbox_in_Mpc * Mpc_in_cgs;
    u->time_to_cgs = std::pow((u->rho_crit_in_cgs * G_in_cgs), (-0.5));
    u->density_to_cgs = u->rho_crit_in_cgs;
    if (mass_to_Msun == -1) {
        u->mass_to_cgs = u->density_to_cgs * std::pow(u->length_to_cgs, 3);
        u->mass_to_Msun = u->mass_to_cgs / Msun_in_cgs;
    } else {
        u->mass_to_Msun = mass_to_Msun;
        u->mass_to_cgs = u->mass_to_Msun * Msun_in_cgs;
    }
    u->velocity_to_cgs = u->length_to_cgs / u->time_to_cgs;
    u->annihilation_flux_to_cgs = (u->density_to_cgs * u->mass_to_cgs / std::pow(u->length_to_cgs, 2));
}

double nosom_unit_factor(const CodeUnits &u) {
    return std::pow(std::pow(c_in_cgs, 2) / (eV_in_cgs * 1.0e9), 2) / (Mpc_in_cgs * 1.0e-3) *
           u.annihilation_flux_to_cgs;
}

double hires_threshold(const double *masses, int n) {
    float hires = FLT_MAX;
    for (int i = 0; i < n; i++)
        if (masses[i] > 0 && masses[i] < hires) hires = (float)masses[i];
    return (double)hires * 1.1;
}

}  // namespace dmann
