// frame.h -- host-side observer frame and unit set-up shared by the C ABI
// (dmann_set_observer) and the C++ Parameters class.
#pragma once

namespace dmann {

// Parameters::setupParams + setupRotation (src/parameters.cpp:111-152,
// 183-289): the observer's angles about the halo centre, the axis-angle
// rotation taking the centre direction to -x, then the roll about x that
// makes the alignment vector horizontal.  rot is rotmatrix[3][3] row-major.
// Returns false when opos == cpos (the reference's angles are NaN there).
bool observer_rotation(const double opos[3], const double cpos[3], const double align[3],
                       double rot[9], double *otheta, double *ophi);

// d rot[e] / d opos[k] of observer_rotation, jac[3 e + k] (e the row-major
// element index), by forward-mode differentiation of the same operations.
// The roll angle's |.| and the degenerate-axis branch are differentiated
// piecewise.  Returns false when opos == cpos.
bool observer_rotation_jacobian(const double opos[3], const double cpos[3], const double align[3],
                                double jac[27]);

// Unit factor of the default flux law (src/flux/flux_ann_nosom.cpp:13-16)
// from the code units of Parameters::setupUnits (src/parameters.cpp:42-82).
struct CodeUnits {
    double rho_crit_in_cgs, length_to_cgs, time_to_cgs, density_to_cgs, mass_to_cgs,
        mass_to_Msun, velocity_to_cgs, annihilation_flux_to_cgs;
};
void setup_units(double h100, double Lbox_in_Mpc, double mass_to_Msun, CodeUnits *u);
double nosom_unit_factor(const CodeUnits &u);
// The decay law's unit factor (src/flux/flux_decay.cpp:10-13).
double decay_unit_factor(const CodeUnits &u);

// genmap.cpp:52-58,82: the hires mass is held in a float; particles with
// mass >= hires * 1.1 are skipped.  masses[0..n) are the particle_masses.
double hires_threshold(const double *masses, int n);

}  // namespace dmann
