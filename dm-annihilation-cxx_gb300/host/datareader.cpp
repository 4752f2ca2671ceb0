// datareader.cpp -- DataReader over the reference's particle files
// (src/datareader.cpp:100-350): the native file (an int32 particle count,
// then 48-byte records, src/datatypes.h:46-59) or a Tipsy XDR file of dark
// particles with the density / hsmooth / sigmav side files of "smooth"
// (src/tipsy_io.c:159-192 for the XDR records, decoded here from big-endian
// bytes).  An optional mask file holds an int32 count and one byte per
// particle, a zero byte sets dens = -1 (datareader.cpp:263-271).  setTest
// caps the particle count, setBuf sets the chunk size, open() loads the
// first chunk, loadBuffer() the next one.
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "annmap.hpp"

namespace annmap {

DataReader::DataReader(const std::string &path, bool isMask, const std::string &maskfile)
    : path_(path), maskPath_(maskfile), isMask_(isMask) {}

DataReader::DataReader(const std::string &partfile, const std::string &densfile,
                       const std::string &hsmoothfile, const std::string &sigmafile, bool isMask,
                       const std::string &maskfile, bool isSingleFile)
    : path_(partfile), maskPath_(maskfile), densPath_(densfile), hsmPath_(hsmoothfile),
      sigmaPath_(sigmafile), isMask_(isMask), isNative_(false), isSingleFile_(isSingleFile) {}

DataReader::~DataReader() { close(); }

void DataReader::setTest(int tn) { testnum_ = tn; }

void DataReader::setBuf(unsigned int mem) {
    memBuffer_ = mem > 0 ? mem : 1;
    buffer_.clear();
    memParts_ = 0;
    memCursor_ = 0;
}

namespace {

uint32_t be32(const unsigned char *b) {
    return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}
float be_float(const unsigned char *b) {
    const uint32_t u = be32(b);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// A side file of "smooth": int32 count of all bodies, then one float each;
// positioned after the gas bodies.
FILE *open_side(const std::string &path, int32_t nbodies, int32_t nsph, const char *what) {
    FILE *f = std::fopen(path.c_str(), "rb");
    int32_t np = -1;
    if (!f || std::fread(&np, sizeof np, 1, f) != 1 || np != nbodies) {
        if (f) std::fclose(f);
        throw std::runtime_error(std::string("Particle numbers in ") + what + " not match: " + path);
    }
    if (nsph > 0 && std::fseek(f, (long)nsph * 4, SEEK_CUR) != 0) {
        std::fclose(f);
        throw std::runtime_error(std::string("cannot skip the gas entries of ") + path);
    }
    return f;
}

}  // namespace

bool DataReader::open() {
    close();
    FILE *f = std::fopen(path_.c_str(), "rb");
    if (!f) throw std::runtime_error("Datafile error: " + path_);
    int32_t n = 0;
    if (isNative_) {
        if (std::fread(&n, sizeof n, 1, f) != 1 || n < 0) {
            std::fclose(f);
            throw std::runtime_error("Datafile error (no particle count): " + path_);
        }
    } else {
        // XDR header: double time, int nbodies, ndim, nsph, ndark, nstar, pad
        unsigned char h[32];
        if (std::fread(h, 1, 32, f) != 32) {
            std::fclose(f);
            throw std::runtime_error("Problem reading tipsy header: " + path_);
        }
        const int32_t nbodies = (int32_t)be32(h + 8), nsph = (int32_t)be32(h + 16),
                      ndark = (int32_t)be32(h + 20);
        if (nbodies < 0 || nsph < 0 || ndark < 0) {
            std::fclose(f);
            throw std::runtime_error("Problem reading tipsy header: " + path_);
        }
        n = ndark;
        // the gas records (12 floats each) precede the dark ones
        if (std::fseek(f, 32 + (long)nsph * 48, SEEK_SET) != 0) {
            std::fclose(f);
            throw std::runtime_error("cannot skip the gas particles of " + path_);
        }
        if (!isSingleFile_) {
            try {
                dfp_ = open_side(densPath_, nbodies, nsph, "density");
                hfp_ = open_side(hsmPath_, nbodies, nsph, "hsmooth");
                sfp_ = open_side(sigmaPath_, nbodies, nsph, "sigmav");
            } catch (...) {
                std::fclose(f);
                close();
                throw;
            }
        }
    }
    fp_ = f;
    partNumbers_ = (unsigned int)n;
    if (isMask_) {
        FILE *m = std::fopen(maskPath_.c_str(), "rb");
        int32_t nm = -1;
        if (!m || std::fread(&nm, sizeof nm, 1, m) != 1 || nm != n) {
            if (m) std::fclose(m);
            close();
            throw std::runtime_error("Particle numbers in mask file not match: " + maskPath_);
        }
        mfp_ = m;
    }
    if (testnum_ != -1 && (int)partNumbers_ > testnum_) partNumbers_ = (unsigned int)testnum_;
    buffer_.resize(memBuffer_);
    readCursor_ = 0;
    memParts_ = 0;
    memCursor_ = 0;
    open_ = true;
    loadBuffer();
    return true;
}

bool DataReader::hasNext() const { return open_ && readCursor_ < partNumbers_; }

// The buffer holds particles [readCursor_, readCursor_ + memParts_); the
// next chunk starts where it ends.
void DataReader::loadBuffer() {
    if (!open_) throw std::runtime_error("DataReader not open");
    readCursor_ += memParts_;
    memCursor_ = 0;
    const unsigned int rest = partNumbers_ - readCursor_;
    memParts_ = rest > memBuffer_ ? memBuffer_ : rest;
    if (memParts_ == 0) return;
    if (isNative_) {
        if (std::fread(buffer_.data(), sizeof(DMParticle), memParts_, (FILE *)fp_) != memParts_)
            throw std::runtime_error("Datafile error (short read): " + path_);
    } else {
        // dark records: mass, pos[3], vel[3], eps, phi as big-endian floats
        raw_.resize((size_t)memParts_ * 36);
        if (std::fread(raw_.data(), 36, memParts_, (FILE *)fp_) != memParts_)
            throw std::runtime_error("Error reading dark particle from input file: " + path_);
        std::vector<float> side(isSingleFile_ ? 0 : 3 * (size_t)memParts_);
        if (!isSingleFile_) {
            FILE *sf[3] = {(FILE *)dfp_, (FILE *)hfp_, (FILE *)sfp_};
            for (int k = 0; k < 3; k++)
                if (std::fread(side.data() + (size_t)k * memParts_, 4, memParts_, sf[k]) != memParts_)
                    throw std::runtime_error("short read in a density / hsmooth / sigmav file");
        }
        for (unsigned int i = 0; i < memParts_; i++) {
            const unsigned char *b = raw_.data() + (size_t)i * 36;
            DMParticle &p = buffer_[i];
            p.mass = be_float(b);
            p.posx = be_float(b + 4);
            p.posy = be_float(b + 8);
            p.posz = be_float(b + 12);
            p.velx = be_float(b + 16);
            p.vely = be_float(b + 20);
            p.velz = be_float(b + 24);
            p.eps = be_float(b + 28);
            p.phi = be_float(b + 32);
            p.dens = isSingleFile_ ? 0.0f : side[i];
            p.hsmooth = isSingleFile_ ? 0.0f : side[memParts_ + i];
            p.sigmav = isSingleFile_ ? 0.0f : side[2 * (size_t)memParts_ + i];
        }
    }
    if (isMask_) {
        mask_.resize(memParts_);
        if (std::fread(mask_.data(), 1, memParts_, (FILE *)mfp_) != memParts_)
            throw std::runtime_error("Mask file error (short read): " + maskPath_);
        for (unsigned int i = 0; i < memParts_; i++)
            if (mask_[i] == 0) buffer_[i].dens = -1.0f;
    }
}

bool DataReader::readParticle(DMParticle *part) {
    if (!hasNext()) return false;
    if (memCursor_ == memParts_) {
        loadBuffer();
        if (memParts_ == 0) return false;
    }
    std::memcpy(part, &buffer_[memCursor_], sizeof(DMParticle));
    memCursor_++;
    if (memCursor_ == memParts_ && readCursor_ + memParts_ >= partNumbers_) {
        readCursor_ += memParts_;   // the stream is exhausted
        memParts_ = 0;
        memCursor_ = 0;
    }
    return true;
}

void DataReader::close() {
    for (void **f : {&fp_, &mfp_, &dfp_, &hfp_, &sfp_}) {
        if (*f) std::fclose((FILE *)*f);
        *f = nullptr;
    }
    open_ = false;
}

}  // namespace annmap
