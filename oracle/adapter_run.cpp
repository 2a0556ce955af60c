// Runs a scene file through the reference simulator with the GPU drop-in
// solvers selected (src/Simulation.cpp compiled with -include
// sph_gpu_select.h; built by `make adapter`): Simulation::importScene, then
// Simulation::step n times with frame output on (SceneLoader::writeFluid
// writes the frames next to the scene file, as the reference's own run
// does), then the final positions and velocities from the solver's device
// context, as records {char name[48]; char type; uint64 count; payload}.
//
// It needs the reference's sources (to build) and a GPU (to run) on the same
// machine.
#include "Simulation.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../sph_gb300/adapter/sph_gpu_solvers.h"

static void put(FILE* f, const std::string& name, const std::vector<double>& v)
{
    char buf[48];
    std::memset(buf, 0, sizeof buf);
    std::strncpy(buf, name.c_str(), sizeof buf - 1);
    const char t = 'd';
    const uint64_t n = v.size();
    std::fwrite(buf, 1, sizeof buf, f);
    std::fwrite(&t, 1, 1, f);
    std::fwrite(&n, sizeof n, 1, f);
    if (n) std::fwrite(v.data(), 8, n, f);
}

static sph_ctx* context_of(SPHSolver* s)
{
    if (auto* d = dynamic_cast<GpuDFSPHSolver*>(s)) return d->context();
    if (auto* p = dynamic_cast<GpuPCISPHSolver*>(s)) return p->context();
    if (auto* w = dynamic_cast<GpuWCSPHSolver*>(s)) return w->context();
    return nullptr;
}

int main(int argc, char** argv)
{
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s scene.json steps out.bin\n", argv[0]);
        return 2;
    }
    Simulation* sim = Simulation::getCurrent();
    sim->activateSave(true);
    if (!sim->importScene(argv[1])) {
        std::fprintf(stderr, "importScene failed\n");
        return 3;
    }
    sph_ctx* ctx = context_of(sim->getSolver());
    if (!ctx) {
        std::fprintf(stderr, "the GPU solvers are not selected in this build\n");
        return 4;
    }
    const int steps = std::atoi(argv[2]);
    for (int k = 0; k < steps; ++k) sim->step();
    unsigned nf = 0, nb = 0;
    sph_ctx_num_particles(ctx, &nf, &nb);
    std::vector<double> x(3 * (size_t)nf), v(3 * (size_t)nf);
    if (nf && (sph_ctx_download(ctx, SPH_FIELD_POSITION, x.data()) || sph_ctx_download(ctx, SPH_FIELD_VELOCITY, v.data()))) {
        std::fprintf(stderr, "download: %s\n", sph_ctx_last_error(ctx));
        return 5;
    }
    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 6;
    put(f, "x", x);
    put(f, "v", v);
    put(f, "time", {sim->getTime()});
    std::fclose(f);
    return 0;
}
