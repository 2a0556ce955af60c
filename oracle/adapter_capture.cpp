// Test driver for the GPU drop-in solvers' scene capture (CPU only; built
// with the reference's own sources and its CPU solvers by `make adapter`).
//
// Imports a scene file through the reference's Simulation::importScene
// (src/Simulation.cpp:331-494), then reads the imported scene the way the GPU
// solvers' init() does (sph_gpu::capture_scene) and writes what it read --
// the scene descriptor, fluid, boundary points and normals, emitters -- as
// records {char name[48]; char type; uint64 count; payload} (oracle
// read_dump's format).  The Python side compares them with the library's own
// reading of the same file and with the reference's state.
//
// Run with stdin from /dev/null (printInfo waits on getchar) and stdout
// redirected (the reference logs every step).
#include "Simulation.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../sph_gb300/adapter/sph_gpu_solvers.h"

static FILE* g_out = nullptr;

static void put(const std::string& name, const std::vector<double>& v)
{
    char buf[48];
    std::memset(buf, 0, sizeof buf);
    std::strncpy(buf, name.c_str(), sizeof buf - 1);
    const char t = 'd';
    const uint64_t n = v.size();
    std::fwrite(buf, 1, sizeof buf, g_out);
    std::fwrite(&t, 1, 1, g_out);
    std::fwrite(&n, sizeof n, 1, g_out);
    if (n) std::fwrite(v.data(), 8, n, g_out);
}
static void put1(const std::string& name, double x) { put(name, std::vector<double>{x}); }

int main(int argc, char** argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s scene.json out.bin\n", argv[0]);
        return 2;
    }
    Simulation* sim = Simulation::getCurrent();
    if (!sim->importScene(argv[1])) {
        std::fprintf(stderr, "importScene failed\n");
        return 3;
    }
    sph_gpu::CapturedScene s;
    std::string err;
    if (!sph_gpu::capture_scene(sim, sim->getSolver(), &s, &err)) {
        std::fprintf(stderr, "capture_scene: %s\n", err.c_str());
        return 4;
    }
    g_out = std::fopen(argv[2], "wb");
    if (!g_out) return 5;
    const sph_scene_desc& d = s.desc;
    put1("desc.simulation_method", d.simulation_method);
    put1("desc.boundary_method", d.boundary_method);
    put1("desc.precision", d.precision);
    put1("desc.particle_radius", d.particle_radius);
    put("desc.gravity", std::vector<double>(d.gravity, d.gravity + 3));
    put1("desc.time_step", d.time_step);
    put1("desc.min_time_step", d.min_time_step);
    put1("desc.max_time_step", d.max_time_step);
    put1("desc.fps", d.fps);
    put1("desc.density0", d.density0);
    put1("desc.stiffness", d.stiffness);
    put1("desc.gamma", d.gamma);
    put1("desc.max_error", d.max_error);
    put1("desc.max_error_v", d.max_error_v);
    put1("desc.cfl_factor", d.cfl_factor);
    put1("desc.min_iterations", d.min_iterations);
    put1("desc.max_iterations", d.max_iterations);
    put1("desc.min_iterations_v", d.min_iterations_v);
    put1("desc.max_iterations_v", d.max_iterations_v);
    put1("desc.viscosity_method", d.viscosity_method);
    put1("desc.viscosity", d.viscosity);
    put1("desc.boundary_viscosity", d.boundary_viscosity);
    put1("desc.surface_tension_method", d.surface_tension_method);
    put1("desc.surface_tension", d.surface_tension);
    put1("desc.adhesion_method", d.adhesion_method);
    put1("desc.adhesion", d.adhesion);
    put1("desc.has_cube", d.has_cube);
    put("desc.cube", {d.cube_min[0], d.cube_min[1], d.cube_min[2], d.cube_max[0], d.cube_max[1], d.cube_max[2]});
    put1("desc.bh_normal_fct", d.bh_normal_fct);
    put1("desc.bh_tangential_fct", d.bh_tangential_fct);
    put("x", s.x);
    put("v", s.v);
    put("boundary", s.boundary);
    put("bh_points", s.bh_points);
    put("bh_normals", s.bh_normals);
    std::vector<double> em;
    for (const sph_gpu::CapturedEmitter& e : s.emitters) {
        const double row[] = {(double)e.type, (double)e.num, e.r[0], e.r[1], e.r[2], e.v, e.q[0], e.q[1], e.q[2], e.q[3],
                              e.start, e.width, e.height, e.spacing, e.paused ? 1.0 : 0.0};
        em.insert(em.end(), row, row + 15);
    }
    put("emitters", em);
    put1("num_fluid_total", s.num_fluid_total);
    put1("time", s.time);
    std::fclose(g_out);
    return 0;
}
