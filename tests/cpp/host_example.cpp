// Uses the C++ host API the way the reference's main.cpp uses its classes
// (src/main.cpp:35-66): Parameters from an info file, a DataReader with the
// info file's test limit and buffer, and -- when a GPU is present and the
// second argument is "render" -- MapGenerator::start and saveToFits.
// Prints what it read as one JSON line.
#include <cstdio>
#include <cstring>
#include <exception>

#include "annmap.hpp"

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    try {
        annmap::Parameters par(argv[1]);
        annmap::DataReader reader(par.nativeDatafile, par.isMask, par.maskFileName);
        reader.setTest(par.testNum);
        reader.setBuf((unsigned)par.memParts);
        reader.open();
        long long n = 0, masked = 0, chunks = 0;
        double msum = 0;
        while (reader.hasNext()) {
            const annmap::DMParticle *p = reader.getBuf();
            for (int i = 0; i < reader.getMemparts(); i++, n++) {
                msum += p[i].mass;
                masked += p[i].dens < 0;
            }
            chunks++;
            reader.loadBuffer();
        }
        reader.close();
        double total = -1;
        if (argc > 2 && std::strcmp(argv[2], "render") == 0) {
            reader.open();
            annmap::MapGenerator gen(&par, &reader);
            gen.start();
            reader.close();
            gen.saveToFits(par.outputFileName, false);
            total = gen.totalFlux();
        }
        std::printf("{\"nside\": %d, \"particles\": %lld, \"masked\": %lld, \"chunks\": %lld, "
                    "\"mass_sum\": %.17g, \"rot00\": %.17g, \"unit_factor\": %.17g, "
                    "\"total_flux\": %.17g}\n",
                    par.map.Nside, n, masked, chunks, msum, par.rotmatrix[0][0], par.unit_factor, total);
        return 0;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
