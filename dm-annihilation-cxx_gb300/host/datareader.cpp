// datareader.cpp -- DataReader over the reference's native particle file
// (src/datareader.cpp:100-350): an int32 particle count, then 48-byte
// records (src/datatypes.h:46-59); an optional mask file holds an int32
// count and one byte per particle, a zero byte sets dens = -1
// (datareader.cpp:263-271).  setTest caps the particle count, setBuf sets
// the chunk size, open() loads the first chunk, loadBuffer() the next one.
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "annmap.hpp"

namespace annmap {

DataReader::DataReader(const std::string &path, bool isMask, const std::string &maskfile)
    : path_(path), maskPath_(maskfile), isMask_(isMask) {}

DataReader::~DataReader() { close(); }

void DataReader::setTest(int tn) { testnum_ = tn; }

void DataReader::setBuf(unsigned int mem) {
    memBuffer_ = mem > 0 ? mem : 1;
    buffer_.clear();
    memParts_ = 0;
    memCursor_ = 0;
}

bool DataReader::open() {
    close();
    FILE *f = std::fopen(path_.c_str(), "rb");
    if (!f) throw std::runtime_error("Datafile error: " + path_);
    int32_t n = 0;
    if (std::fread(&n, sizeof n, 1, f) != 1 || n < 0) {
        std::fclose(f);
        throw std::runtime_error("Datafile error (no particle count): " + path_);
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
    if (std::fread(buffer_.data(), sizeof(DMParticle), memParts_, (FILE *)fp_) != memParts_)
        throw std::runtime_error("Datafile error (short read): " + path_);
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
    if (fp_) std::fclose((FILE *)fp_);
    if (mfp_) std::fclose((FILE *)mfp_);
    fp_ = mfp_ = nullptr;
    open_ = false;
}

}  // namespace annmap
