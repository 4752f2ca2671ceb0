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

namespace {

// Forward-mode dual number with three tangents (derivatives with respect to
// the observer's x, y, z).  Only the operations the rotation set-up uses.
struct Dual3 {
    double v, d[3];
    Dual3(double x = 0.0) : v(x), d{0.0, 0.0, 0.0} {}
};
inline Dual3 mk(double v, double d0, double d1, double d2) {
    Dual3 r(v);
    r.d[0] = d0;
    r.d[1] = d1;
    r.d[2] = d2;
    return r;
}
inline Dual3 chain(const Dual3 &a, double v, double dv) {
    return mk(v, dv * a.d[0], dv * a.d[1], dv * a.d[2]);
}
inline Dual3 operator+(const Dual3 &a, const Dual3 &b) {
    return mk(a.v + b.v, a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]);
}
inline Dual3 operator-(const Dual3 &a, const Dual3 &b) {
    return mk(a.v - b.v, a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]);
}
inline Dual3 operator-(const Dual3 &a) { return mk(-a.v, -a.d[0], -a.d[1], -a.d[2]); }
inline Dual3 operator*(const Dual3 &a, const Dual3 &b) {
    return mk(a.v * b.v, a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1],
              a.d[2] * b.v + a.v * b.d[2]);
}
inline Dual3 operator/(const Dual3 &a, const Dual3 &b) {
    const double q = a.v / b.v;
    return mk(q, (a.d[0] - q * b.d[0]) / b.v, (a.d[1] - q * b.d[1]) / b.v,
              (a.d[2] - q * b.d[2]) / b.v);
}
inline bool operator<(const Dual3 &a, double b) { return a.v < b; }
inline bool operator>(const Dual3 &a, double b) { return a.v > b; }
inline Dual3 &operator+=(Dual3 &a, const Dual3 &b) { return a = a + b; }
inline Dual3 sqrt(const Dual3 &a) {
    const double r = std::sqrt(a.v);
    return chain(a, r, 0.5 / r);
}
inline Dual3 pow(const Dual3 &a, double e) {  // only e = 2 occurs
    return chain(a, std::pow(a.v, e), e * std::pow(a.v, e - 1.0));
}
inline Dual3 sin(const Dual3 &a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
inline Dual3 cos(const Dual3 &a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
inline Dual3 acos(const Dual3 &a) {
    return chain(a, std::acos(a.v), -1.0 / std::sqrt((1.0 - a.v) * (1.0 + a.v)));
}
inline Dual3 atan2(const Dual3 &y, const Dual3 &x) {
    const double r2 = x.v * x.v + y.v * y.v;
    return mk(std::atan2(y.v, x.v), (x.v * y.d[0] - y.v * x.d[0]) / r2,
              (x.v * y.d[1] - y.v * x.d[1]) / r2, (x.v * y.d[2] - y.v * x.d[2]) / r2);
}
inline Dual3 fabs(const Dual3 &a) { return a.v < 0.0 ? -a : a; }
inline double value(const Dual3 &a) { return a.v; }
inline double value(double a) { return a; }

// setupParams + setupRotation for a scalar type T (double, or Dual3 for the
// derivatives).  With T = double the operations and their order are those
// of the reference (src/parameters.cpp:137-150, 188-287).
template <class T>
bool rotation_t(const T opos[3], const double cpos[3], const double align[3], T rot[9],
                double *otheta_out, double *ophi_out) {
    using std::acos;
    using std::atan2;
    using std::cos;
    using std::fabs;
    using std::pow;
    using std::sin;
    using std::sqrt;
    // setupParams (parameters.cpp:137-150)
    const T radius = sqrt(pow(opos[0] - cpos[0], 2.0) + pow(opos[1] - cpos[1], 2.0) +
                          pow(opos[2] - cpos[2], 2.0));
    if (!(value(radius) > 0.0)) return false;
    const T otheta = acos((opos[2] - cpos[2]) / radius);
    T ophi = atan2((opos[1] - cpos[1]), (opos[0] - cpos[0]));
    if (ophi < 0.0) ophi += T(2.0 * PI);
    if (otheta_out) *otheta_out = value(otheta);
    if (ophi_out) *ophi_out = value(ophi);

    // setupRotation (parameters.cpp:188-237): rotate the centre direction
    // r = -(sin t cos p, sin t sin p, cos t) onto e1 about r x e1.
    T u = T(0.0), v = -cos(otheta), w = sin(otheta) * sin(ophi);
    const T rr = sqrt(u * u + v * v + w * w);
    u = u / rr;
    v = v / rr;
    w = w / rr;
    const T c = -sin(otheta) * cos(ophi);
    const T t = T(1.0) - c;
    const T s = rr;
    T m[3][3];
    if (value(rr) > 0.0) {
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
            for (int j = 0; j < 3; j++) m[i][j] = T((i == j) ? 1.0 : 0.0);
        if (std::cos(value(ophi)) > 0.0) {
            m[0][0] = T(-1.0);
            m[1][1] = T(-1.0);
        }
    }
    // parameters.cpp:240-287: roll about x so the alignment vector, seen
    // from the observer, lies in the horizontal plane.
    const T distance = radius;
    const T tv[3] = {T(cpos[0]) + distance * T(align[0]) - opos[0],
                     T(cpos[1]) + distance * T(align[1]) - opos[1],
                     T(cpos[2]) + distance * T(align[2]) - opos[2]};
    const T ytmp = tv[0] * m[0][1] + tv[1] * m[1][1] + tv[2] * m[2][1];
    const T ztmp = tv[0] * m[0][2] + tv[1] * m[1][2] + tv[2] * m[2][2];
    const T gamma = -fabs(atan2(ztmp, ytmp));
    const T r2[3][3] = {{T(1.0), T(0.0), T(0.0)},
                        {T(0.0), cos(gamma), sin(gamma)},
                        {T(0.0), -sin(gamma), cos(gamma)}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            T val = T(0.0);
            for (int k = 0; k < 3; k++) val += m[i][k] * r2[k][j];
            rot[3 * i + j] = val;
        }
    return true;
}

}  // namespace

bool observer_rotation(const double opos[3], const double cpos[3], const double align[3],
                       double rot[9], double *otheta_out, double *ophi_out) {
    return rotation_t<double>(opos, cpos, align, rot, otheta_out, ophi_out);
}

bool observer_rotation_jacobian(const double opos[3], const double cpos[3], const double align[3],
                                double jac[27]) {
    Dual3 o[3] = {mk(opos[0], 1, 0, 0), mk(opos[1], 0, 1, 0), mk(opos[2], 0, 0, 1)};
    Dual3 r[9];
    if (!rotation_t<Dual3>(o, cpos, align, r, nullptr, nullptr)) return false;
    for (int e = 0; e < 9; e++)
        for (int k = 0; k < 3; k++) jac[3 * e + k] = r[e].d[k];
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

double decay_unit_factor(const CodeUnits &u) {
    const double decay_flux_to_cgs = (u.mass_to_cgs / std::pow(u.length_to_cgs, 2));
    return std::pow(c_in_cgs, 2) / (eV_in_cgs * 1.0e9) / (Mpc_in_cgs * 1.0e-3) * decay_flux_to_cgs;
}

double hires_threshold(const double *masses, int n) {
    float hires = FLT_MAX;
    for (int i = 0; i < n; i++)
        if (masses[i] > 0 && masses[i] < hires) hires = (float)masses[i];
    return (double)hires * 1.1;
}

}  // namespace dmann
