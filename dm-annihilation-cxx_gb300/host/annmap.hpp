// annmap.hpp -- the C++ host API of the GB300 sky-map projection: the
// reference's Parameters / DataReader / MapGenerator classes
// (src/parameters.h:4-57, src/datareader.h:14-119, src/mapgenerator.h:8-26),
// re-implemented on top of the C ABI of include/dmann.h (libdmann.so).
//
// The classes keep the reference's names, member names, call order and
// semantics (info-file keys and tokenisation, the native particle file with
// its byte mask, chunked reading through a memory buffer, the FP64 RING map in
// flux per steradian after the dOmega division, saveToFits).  Differences:
//   - failures throw std::runtime_error instead of printf + exit(1);
//   - MapGenerator::start() streams chunks to the GPU through two pinned
//     host buffers and two device buffers, so reading and converting the next
//     chunk overlaps the upload and rendering of the current one;
//   - MapGenerator takes the precision form (DMANN_COMP_F32 default) and the
//     CUDA device; totalFlux() returns the reference's "Total Conts";
//   - the XDR / tipsy input path of DataReader is not provided.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "dmann.h"

namespace annmap {

typedef double MAPTYPE;                      // src/datatypes.h:29
constexpr int MAX_NUM_MASS_RES = 10;         // src/datatypes.h:31

// One native-file record (src/datatypes.h:46-59): twelve float32 fields.
struct DMParticle {
    float mass, dens, hsmooth;
    float posx, posy, posz;
    float velx, vely, velz;
    float sigmav, eps, phi;
};
static_assert(sizeof(DMParticle) == 48, "native record is 48 bytes");

struct Info {                                // src/datatypes.h:171-186 (the fields used)
    double Omega_M = 0, h100 = 0, n_s = 0, sigma_8 = 0, Lbox_in_Mpc = 0, mass_to_Msun = -1.0;
    double particle_masses[MAX_NUM_MASS_RES] = {0};
    long particle_numbers[MAX_NUM_MASS_RES] = {0};
    double centerpos[3] = {0, 0, 0}, centervel[3] = {0, 0, 0};
};

struct Codeunits {                           // src/datatypes.h:203-213
    double mass_to_cgs = 0, mass_to_Msun = 0, length_to_Mpc = 0, length_to_cgs = 0,
           time_to_cgs = 0, velocity_to_cgs = 0, density_to_cgs = 0,
           annihilation_flux_to_cgs = 0;
};

struct Params {                              // src/datatypes.h:220-232
    double z = 0;
    double cpos[3] = {0, 0, 0}, cvel[3] = {0, 0, 0}, opos[3] = {0, 0, 0};
    double otheta = 0, ophi = 0, Lbox_in_Mpc = 0;
    long particle_numbers[MAX_NUM_MASS_RES] = {0};
    double particle_masses[MAX_NUM_MASS_RES] = {0};
    double particle_masses_in_Msun[MAX_NUM_MASS_RES] = {0};
};

struct Map {                                 // src/datatypes.h:236-254
    int Nside = 512;
    int64_t Npix = 12LL * 512 * 512;
    double dOmega = 0, theta0 = 0;
    void setNside(int nside);
};

class Parameters {
public:
    explicit Parameters(const std::string &info_file);
    // The same, from the text of an info file.
    static Parameters fromText(const std::string &text);

    Info info;
    Codeunits codeunits;
    Params params;
    Map map;
    double rotmatrix[3][3];
    double rho_crit_in_cgs = 0;
    double unit_factor = 1.0;   // the default flux law's factor (flux_ann_nosom.cpp:13-16)

    int memParts = 10000000;    // particles per buffered chunk ("mem_buffer")
    int testNum = -1;           // "test": render only the first testNum particles

    std::string partFile, densFile, hsmFile, dspFile;
    std::string nativeDatafile;
    std::string maskFileName;
    std::string outputFileName;
    bool isNative = true;
    bool isMask = false;

    // Mass at or above which a particle is skipped (genmap.cpp:52-58).
    double hiresThreshold() const;
    // The unit factor of a flux law (dmann_flux_unit_factor).
    double fluxUnitFactor(int flux_model) const;
    // Moves the observer (and optionally the alignment vector) and redoes the
    // rotation; the reference keeps these private.
    void setObserver(const double opos[3], const double *align = nullptr);
    void printParameters() const;

private:
    Parameters() = default;
    void parse(const std::string &text);
    void setup();
    double align_vector_[3] = {0, 0, 1};
    double obs_pos_[3] = {0, 0, 0};
    bool have_align_ = false, have_obs_ = false;
    double redshift_ = 0;
};

class DataReader {
public:
    // Native file (int32 count, then 48-byte records); optional byte mask
    // file (int32 count, one byte per particle; 0 masks: dens = -1).
    DataReader(const std::string &path, bool isMask = false, const std::string &maskfile = "");
    // Tipsy XDR particle file (big-endian: header time, nbodies, ndim, nsph,
    // ndark, nstar, pad; then gas, dark and star records -- only the dark
    // ones are read, src/datareader.cpp:120-190) with the density, smoothing
    // length and velocity dispersion side files of "smooth" (native int32
    // count of all bodies, then one float per body, gas first).  With
    // isSingleFile the side files are not read and those fields are 0.
    DataReader(const std::string &partfile, const std::string &densfile,
               const std::string &hsmoothfile, const std::string &sigmafile, bool isMask = false,
               const std::string &maskfile = "", bool isSingleFile = false);
    ~DataReader();
    DataReader(const DataReader &) = delete;
    DataReader &operator=(const DataReader &) = delete;

    int getPartNum() const { return testnum_ != -1 ? testnum_ : (int)partNumbers_; }
    void setTest(int tn);
    void setBuf(unsigned int mem);
    unsigned int getBufSize() const { return memParts_; }        // particles in the buffer
    unsigned int getBufCapacity() const { return memBuffer_; }   // the chunk size
    bool open();
    bool isOpen() const { return open_; }
    bool hasNext() const;
    void loadBuffer();                       // reads the next chunk into the buffer
    DMParticle *getBuf() { return buffer_.data(); }
    int getMemparts() const { return (int)memParts_; }
    bool readParticle(DMParticle *part);     // one particle at a time
    void close();

private:
    std::string path_, maskPath_;
    std::string densPath_, hsmPath_, sigmaPath_;
    bool isMask_;
    bool isNative_ = true, isSingleFile_ = false;
    void *dfp_ = nullptr, *hfp_ = nullptr, *sfp_ = nullptr;   // FILE * of the side files
    std::vector<unsigned char> raw_;
    bool open_ = false;
    void *fp_ = nullptr, *mfp_ = nullptr;    // FILE *
    unsigned int partNumbers_ = 0;
    unsigned int readCursor_ = 0;            // particles consumed from the file
    unsigned int memBuffer_ = 10000000;
    unsigned int memParts_ = 0;              // particles in the buffer
    unsigned int memCursor_ = 0;
    int testnum_ = -1;
    std::vector<DMParticle> buffer_;
    std::vector<unsigned char> mask_;
};

class MapGenerator {
public:
    // flux_model: a dmann_flux law (the reference links one getflux plugin
    // per build; here it is chosen per generator).
    MapGenerator(Parameters *par, DataReader *reader, int precision = DMANN_COMP_F32,
                 int device = 0, int flux_model = DMANN_FLUX_ANN_NOSOM);
    ~MapGenerator();
    MapGenerator(const MapGenerator &) = delete;
    MapGenerator &operator=(const MapGenerator &) = delete;

    void start();
    void saveToFits(const std::string &fits_file, bool isVerbose = false);
    // The halo table the ann_core_nosom law reads (default as the reference:
    // ./halocore/VL2_Halos.data, relative to the working directory).
    void setHaloFile(const std::string &path) { halo_file_ = path; }
    bool isFinished() const { return isFinished_; }
    MAPTYPE *getMap() { return map_; }
    int getNside() const { return par_->map.Nside; }
    double totalFlux() const { return total_flux_; }   // "Total Conts" (genmap.cpp:161-172)
    const dmann_stats &stats() const { return stats_; }

private:
    Parameters *par_;
    DataReader *reader_;
    int precision_, device_, flux_model_;
    bool isFinished_ = false;
    MAPTYPE *map_ = nullptr;
    double total_flux_ = 0;
    dmann_stats stats_{};
    std::string halo_file_ = "./halocore/VL2_Halos.data";
};

// The ann_core_nosom law's halo table (src/halocore/halocore.cpp:16-45): one
// halo per line, x y z radius.  Throws on an empty or short file.
struct HaloTable {
    std::vector<float> x, y, z, radius;
};
HaloTable readHaloTable(const std::string &path);

// HEALPix FITS map (the layout of write_Healpix_map_to_fits with FP64 data:
// empty primary HDU, one BINTABLE with column "signal").
void writeHealpixFits(const std::string &path, const double *map, int64_t npix,
                      const char *ordering = "RING");

}  // namespace annmap
