// mapgenerator.cpp -- MapGenerator::start() on the GPU (the loop of
// src/genmap.cpp:22-175 with the CPU path's semantics): the observer frame
// and units from Parameters, then every DataReader chunk converted from the
// 48-byte records to float32 SoA and deposited into the context's map, then
// the dOmega division into an FP64 host map.
//
// Chunk pipeline: two pinned host SoA buffers and two device SoA buffers
// alternate.  For chunk k the host waits until slot k%2 is free (the render
// of chunk k-2 has finished), converts the records into its pinned buffer,
// queues the host-to-device copies and the deposit kernels on the context's
// stream and at once reads chunk k+1 from the file while the GPU works.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <sys/stat.h>

#include "annmap.hpp"

namespace annmap {

namespace {

struct Ctx {
    dmann_ctx *c = nullptr;
    explicit Ctx(int device) {
        dmann_status st = dmann_create(&c, device);
        if (st != DMANN_OK)
            throw std::runtime_error("dmann_create failed (status " + std::to_string(st) +
                                     "): a GB300 (sm_103) device is required");
    }
    ~Ctx() { dmann_destroy(c); }
    void check(dmann_status st) const {
        if (st != DMANN_OK) throw std::runtime_error(std::string("dmann: ") + dmann_last_error(c));
    }
};

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// The pinned and device buffers of the two pipeline slots.
struct Slots {
    size_t cap = 0;
    float *host[2] = {nullptr, nullptr};   // 7 * cap floats each (pinned): x y z m rho h sigmav
    float *dev[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    explicit Slots(size_t capacity) : cap(capacity) {
        for (int k = 0; k < 2; k++) {
            cuda_check(cudaHostAlloc((void **)&host[k], 7 * cap * sizeof(float), cudaHostAllocDefault),
                       "pinned chunk buffer");
            cuda_check(cudaMalloc((void **)&dev[k], 7 * cap * sizeof(float)), "device chunk buffer");
            cuda_check(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming), "event");
        }
    }
    ~Slots() {
        for (int k = 0; k < 2; k++) {
            if (done[k]) cudaEventSynchronize(done[k]), cudaEventDestroy(done[k]);
            if (dev[k]) cudaFree(dev[k]);
            if (host[k]) cudaFreeHost(host[k]);
        }
    }
};

}  // namespace

MapGenerator::MapGenerator(Parameters *par, DataReader *reader, int precision, int device,
                           int flux_model)
    : par_(par), reader_(reader), precision_(precision), device_(device), flux_model_(flux_model) {}

MapGenerator::~MapGenerator() { std::free(map_); }

void MapGenerator::start() {
    Ctx ctx(device_);
    ctx.check(dmann_set_frame(ctx.c, &par_->rotmatrix[0][0], par_->params.opos));
    ctx.check(dmann_set_units(ctx.c, par_->fluxUnitFactor(flux_model_), par_->hiresThreshold(),
                              flux_model_));
    ctx.check(dmann_set_flux_params(ctx.c, par_->codeunits.velocity_to_cgs, par_->params.cpos));
    if (flux_model_ == DMANN_FLUX_ANN_CORE_NOSOM) {
        const HaloTable t = readHaloTable(halo_file_);
        ctx.check(dmann_set_halo_cores(ctx.c, t.x.data(), t.y.data(), t.z.data(), t.radius.data(),
                                       (int)t.x.size()));
    }
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    cudaStream_t s = nullptr;
    cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    struct StreamGuard {   // the context goes back to its own stream before s is destroyed
        dmann_ctx *c;
        cudaStream_t s;
        ~StreamGuard() {
            cudaStreamSynchronize(s);
            dmann_set_stream(c, nullptr);
            cudaStreamDestroy(s);
        }
    } sg{ctx.c, s};
    ctx.check(dmann_set_stream(ctx.c, s));
    if (!reader_->isOpen()) reader_->open();
    const int nside = par_->map.Nside;
    ctx.check(dmann_map_begin(ctx.c, nside, precision_));
    {
        Slots slots(reader_->getBufCapacity() > 0 ? reader_->getBufCapacity() : 1);
        int k = 0;
        while (reader_->hasNext()) {   // genmap.cpp:67
            const DMParticle *p = reader_->getBuf();
            const size_t n = (size_t)reader_->getMemparts();
            const int slot = k & 1;
            cuda_check(cudaEventSynchronize(slots.done[slot]), "chunk slot");
            float *h = slots.host[slot], *d = slots.dev[slot];
            const size_t cap = slots.cap;
            float *hx = h, *hy = h + cap, *hz = h + 2 * cap, *hm = h + 3 * cap, *hr = h + 4 * cap,
                  *hh = h + 5 * cap, *hv = h + 6 * cap;
            for (size_t i = 0; i < n; i++) {   // records -> SoA
                hx[i] = p[i].posx;
                hy[i] = p[i].posy;
                hz[i] = p[i].posz;
                hm[i] = p[i].mass;
                hr[i] = p[i].dens;
                hh[i] = p[i].hsmooth;
                hv[i] = p[i].sigmav;
            }
            for (int f = 0; f < 7; f++)
                cuda_check(cudaMemcpyAsync(d + f * cap, h + f * cap, n * sizeof(float),
                                           cudaMemcpyHostToDevice, s),
                           "chunk upload");
            ctx.check(dmann_map_add_v(ctx.c, d, d + cap, d + 2 * cap, d + 3 * cap, d + 4 * cap,
                                      d + 5 * cap, d + 6 * cap, (int64_t)n));
            cuda_check(cudaEventRecord(slots.done[slot], s), "chunk event");
            reader_->loadBuffer();   // genmap.cpp:155, overlapping the GPU work
            k++;
        }
        std::free(map_);
        map_ = (MAPTYPE *)std::calloc((size_t)par_->map.Npix, sizeof(MAPTYPE));
        if (!map_) throw std::runtime_error("map allocation failed");
        ctx.check(dmann_map_end(ctx.c, map_, 0));   // divides by dOmega (genmap.cpp:168)
    }
    ctx.check(dmann_get_stats(ctx.c, &stats_));
    total_flux_ = stats_.total_flux;
    isFinished_ = true;
}

HaloTable readHaloTable(const std::string &path) {
    std::ifstream f(path);
    if (!f.is_open()) throw std::runtime_error("cannot open halo file " + path);
    HaloTable t;
    std::string line;
    size_t lines = 0;
    std::string all;
    while (std::getline(f, line)) {
        lines++;
        all += line;
        all += ' ';
    }
    if (lines == 0) throw std::runtime_error("empty halo file " + path);
    std::istringstream in(all);
    for (size_t i = 0; i < lines; i++) {
        float v[4];
        for (int k = 0; k < 4; k++)
            if (!(in >> v[k])) throw std::runtime_error("halo file " + path + ": short record");
        t.x.push_back(v[0]);
        t.y.push_back(v[1]);
        t.z.push_back(v[2]);
        t.radius.push_back(v[3]);
    }
    return t;
}

void MapGenerator::saveToFits(const std::string &fits_file, bool isVerbose) {
    if (!isFinished()) {
        std::printf("Map not generated yet");
        return;
    }
    const std::string path = fits_file.empty() ? par_->outputFileName : fits_file;
    struct stat sb;
    if (stat(path.c_str(), &sb) == 0) {
        // mapgenerator.cpp:44-55: an existing file is replaced (after a
        // prompt in verbose mode)
        std::printf("File exists! Owerite...\n");
        if (isVerbose) {
            char t = 0;
            if (std::scanf(" %c", &t) != 1 || t != 'y') return;
        }
        std::remove(path.c_str());
    }
    writeHealpixFits(path, map_, par_->map.Npix, "RING");
}

}  // namespace annmap
