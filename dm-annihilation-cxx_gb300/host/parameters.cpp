// parameters.cpp -- Parameters: the reference's info-file configuration
// (src/parameters.cpp:291-483 for the keys and tokenisation, :42-289 for the
// derived fields, whose unit and rotation set-up is the library's own
// restatement in frame.cpp, reached through the C ABI).
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "annmap.hpp"

namespace annmap {

void Map::setNside(int nside) {
    Nside = nside;
    Npix = 12LL * nside * nside;
    dOmega = 4 * 3.14159265358979323846 / (double)Npix;   // datatypes.h:251
    theta0 = 0;
}

namespace {

// Tokens of one line split on spaces (strtok(" ") semantics: runs of spaces
// separate, empty tokens do not exist).
std::vector<std::string> tokens(const std::string &line) {
    std::vector<std::string> t;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && line[i] == ' ') i++;
        size_t j = i;
        while (j < line.size() && line[j] != ' ') j++;
        if (j > i) t.push_back(line.substr(i, j - i));
        i = j;
    }
    return t;
}

}  // namespace

Parameters::Parameters(const std::string &info_file) {
    std::ifstream f(info_file);
    if (!f.is_open()) throw std::runtime_error("Info file incorrect: " + info_file);
    std::stringstream ss;
    ss << f.rdbuf();
    map.setNside(512);
    parse(ss.str());
    setup();
}

Parameters Parameters::fromText(const std::string &text) {
    Parameters p;
    p.map.setNside(512);
    p.parse(text);
    p.setup();
    return p;
}

void Parameters::parse(const std::string &text) {
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        const std::vector<std::string> t = tokens(line);
        if (t.empty() || t[0][0] == '#') continue;
        const std::string &key = t[0];
        // values start at the third token (the second is "=")
        auto val = [&](size_t k) -> const char * {
            if (t.size() < 3 + k) throw std::runtime_error("info file: key '" + key + "' lacks a value");
            return t[2 + k].c_str();
        };
        auto vec3 = [&](double *d) {
            for (int k = 0; k < 3; k++) d[k] = std::atof(val(k));
        };
        if (key == "Omega_M") info.Omega_M = std::atof(val(0));
        else if (key == "h100") info.h100 = std::atof(val(0));
        else if (key == "n_s") info.n_s = std::atof(val(0));
        else if (key == "sigma_8") info.sigma_8 = std::atof(val(0));
        else if (key == "Lbox_in_Mpc") info.Lbox_in_Mpc = std::atof(val(0));
        else if (key == "mass_to_Msun") info.mass_to_Msun = std::atof(val(0));
        else if (key == "particle_masses") {
            for (size_t k = 0; k + 2 < t.size() && k < (size_t)MAX_NUM_MASS_RES; k++)
                info.particle_masses[k] = std::atof(val(k));
            (void)val(0);
        } else if (key == "particle_numbers") {
            for (size_t k = 0; k + 2 < t.size() && k < (size_t)MAX_NUM_MASS_RES; k++)
                info.particle_numbers[k] = std::atol(val(k));
            (void)val(0);
        } else if (key == "centerpos") vec3(info.centerpos);
        else if (key == "centervel") vec3(info.centervel);
        else if (key == "align_vec") {
            vec3(align_vector_);
            have_align_ = true;
        } else if (key == "obs_pos") {
            vec3(obs_pos_);
            have_obs_ = true;
        } else if (key == "nside") map.setNside(std::atoi(val(0)));
        else if (key == "test") testNum = std::atoi(val(0));
        else if (key == "datafile") nativeDatafile = val(0);
        else if (key == "partfile") { partFile = val(0); isNative = false; }
        else if (key == "densfile") { densFile = val(0); isNative = false; }
        else if (key == "hsmfile") { hsmFile = val(0); isNative = false; }
        else if (key == "vdspfile") { dspFile = val(0); isNative = false; }
        else if (key == "outputmap") outputFileName = val(0);
        else if (key == "mem_buffer") memParts = std::atoi(val(0));
        else if (key == "mask") { maskFileName = val(0); isMask = true; }
        // the halo keys (Mvir_in_Msun, params_NFW, ...) are read by the
        // reference but not used by the map path
    }
}

void Parameters::setup() {
    if (!have_obs_ || !have_align_) throw std::runtime_error("info file lacks obs_pos / align_vec");
    double u[9];
    dmann_code_units(info.h100, info.Lbox_in_Mpc, info.mass_to_Msun, u);
    rho_crit_in_cgs = u[0];
    codeunits.length_to_cgs = u[1];
    codeunits.time_to_cgs = u[2];
    codeunits.density_to_cgs = u[3];
    codeunits.mass_to_cgs = u[4];
    codeunits.mass_to_Msun = u[5];
    codeunits.velocity_to_cgs = u[6];
    codeunits.annihilation_flux_to_cgs = u[7];
    codeunits.length_to_Mpc = info.Lbox_in_Mpc;
    unit_factor = u[8];
    // setupParams (parameters.cpp:111-152)
    params.z = redshift_;
    for (int k = 0; k < 3; k++) {
        params.cpos[k] = info.centerpos[k];
        params.cvel[k] = info.centervel[k];
        params.opos[k] = obs_pos_[k];
    }
    params.Lbox_in_Mpc = info.Lbox_in_Mpc;
    int j = 0;
    for (int i = 0; i < MAX_NUM_MASS_RES; i++) {
        params.particle_masses[i] = 0;
        params.particle_numbers[i] = 0;
        params.particle_masses_in_Msun[i] = 0;
    }
    for (int i = 0; i < MAX_NUM_MASS_RES; i++) {
        if (info.particle_masses[i] > 0) {
            params.particle_numbers[j] = info.particle_numbers[i];
            params.particle_masses[j] = info.particle_masses[i];
            params.particle_masses_in_Msun[j] = info.particle_masses[i] * codeunits.mass_to_cgs / 1.9889212e+33;
            j++;
        }
    }
    setObserver(obs_pos_, align_vector_);
}

void Parameters::setObserver(const double opos[3], const double *align) {
    double o[3] = {opos[0], opos[1], opos[2]};
    for (int k = 0; k < 3; k++) {
        obs_pos_[k] = o[k];
        params.opos[k] = o[k];
        if (align) align_vector_[k] = align[k];
    }
    double rot[9], ang[2];
    if (dmann_observer_rotation(params.opos, params.cpos, align_vector_, rot, ang) != DMANN_OK)
        throw std::runtime_error("observer position equals the halo centre");
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) rotmatrix[i][k] = rot[3 * i + k];
    params.otheta = ang[0];
    params.ophi = ang[1];
}

double Parameters::fluxUnitFactor(int flux_model) const {
    if (flux_model == DMANN_FLUX_ANN_NOSOM) return unit_factor;
    double u = 0;
    if (dmann_flux_unit_factor(flux_model, info.h100, info.Lbox_in_Mpc, info.mass_to_Msun, &u) != DMANN_OK)
        throw std::runtime_error("unknown flux law");
    return u;
}

double Parameters::hiresThreshold() const {
    return dmann_hires_threshold(params.particle_masses, MAX_NUM_MASS_RES);
}

void Parameters::printParameters() const {
    std::printf("Nside %d, Npix %lld, dOmega %g\n", map.Nside, (long long)map.Npix, map.dOmega);
    std::printf("observer (%g %g %g), centre (%g %g %g), otheta %g ophi %g\n", params.opos[0],
                params.opos[1], params.opos[2], params.cpos[0], params.cpos[1], params.cpos[2],
                params.otheta, params.ophi);
    std::printf("unit factor %.17g, hires threshold %.9g, buffer %d, test %d\n", unit_factor,
                hiresThreshold(), memParts, testNum);
}

}  // namespace annmap
