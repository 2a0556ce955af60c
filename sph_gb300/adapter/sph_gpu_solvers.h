// GPU drop-in solvers for the reference simulator (josemanuel28v/SPH).
//
// GpuWCSPHSolver, GpuPCISPHSolver and GpuDFSPHSolver derive from the
// reference's own solver classes (src/WCSPHSolver.h, src/PCISPHSolver.h,
// src/DFSPHSolver.h), so Simulation::importScene's setters
// (src/Simulation.cpp:354-378, static_cast to the CPU solver type) and every
// getter keep working, and override the plugin interface of SPHSolver
// (src/SPHSolver.h:37-39):
//
//   init()        reads the scene the Simulation singleton holds -- time
//                 settings, fluid model 0 (active particles, rest density,
//                 non-pressure forces, emitters), the boundary models (Akinci
//                 points, cube bounds, PCISPH points with normals) -- and the
//                 solver's own parameters, and creates one device context
//                 (include/sph_gb300.h) that owns the scene from then on;
//   step()        one sph_ctx_step on the GPU, then the Simulation's time,
//                 time step and the fluid model's active count follow the
//                 device; when SceneLoader::writeFluid is about to write a
//                 frame (src/Simulation.cpp:172-181, the predicate of
//                 TimeManager::hasToSave, src/TimeManager.h:101-110) the
//                 positions and velocities are downloaded into the fluid
//                 model first;
//   resizeData()  the base class's (FluidModel::addEmitter calls it before
//                 init, src/FluidModel.cpp:136).
//
// The reference's non-pressure-force objects stay owned by the fluid model
// (src/FluidModel.cpp:24-25); their coefficients are passed to the device,
// which computes them.  The reference compiles with these solvers selected by
// building src/Simulation.cpp with `-include sph_gpu_select.h` (the factory,
// src/Simulation.cpp:207-231, then creates them for the same method ids);
// oracle/Makefile's `adapter` target does exactly that.
//
// Library-only settings (arithmetic form, pair-list width, lanes per
// particle) come from sph_gpu_set_defaults; the default is the FP32
// production form with 64-slot pair lists.
#pragma once

#include <string>
#include <vector>

#include "DFSPHSolver.h"
#include "PCISPHSolver.h"
#include "SPHSolver.h"
#include "Simulation.h"
#include "WCSPHSolver.h"

#include "../../include/sph_gb300.h"

namespace sph_gpu {

// An emitter as FluidModel::addEmitter received it (src/Emitter.cpp:10-29).
struct CapturedEmitter {
    int type = 0;
    unsigned num = 0;
    double r[3] = {0, 0, 0};
    double v = 0;
    double q[4] = {1, 0, 0, 0};  // w, x, y, z
    double start = 0, width = 0, height = 0, spacing = 0;
    bool paused = false;
};

// The scene of the Simulation singleton, as the GPU context takes it.
struct CapturedScene {
    sph_scene_desc desc{};
    std::vector<double> x, v;                     // fluid model 0's active particles (xyz)
    std::vector<double> boundary;                 // Akinci boundary points (xyz)
    std::vector<double> bh_points, bh_normals;    // PCISPH boundary model points and normals
    std::vector<CapturedEmitter> emitters;
    unsigned num_fluid_total = 0;                 // FluidModel::getNumParticles (active + emitter slots)
    double time = 0;
};

// Library-only settings for solvers initialised afterwards (precision,
// neighbor_list_max, threads_per_particle, domain box); NULL restores the
// defaults.
void sph_gpu_set_defaults(const sph_scene_desc* base);

// Reads the scene that `sim` holds and `solver`'s parameters.  Returns false
// with *err set for what the device path does not take: more than one fluid
// model, boundary models of mixed kinds.
bool capture_scene(Simulation* sim, SPHSolver* solver, CapturedScene* out, std::string* err);

// The device context of one scene, shared by the three solvers.
class GpuSceneLink {
public:
    ~GpuSceneLink();
    // sph_ctx_create + the scene + sph_ctx_init; false with *err on failure.
    bool create(const CapturedScene& s, std::string* err);
    // One step; the Simulation's time and time step follow the device.
    bool step(Simulation* sim, FluidModel* fm, unsigned* steps, unsigned* iterations, unsigned* sum_iterations,
              std::string* err);
    sph_ctx* ctx() const { return ctx_; }

private:
    bool download_fluid(FluidModel* fm, std::string* err);
    sph_ctx* ctx_ = nullptr;
    std::vector<double> buf_x_, buf_v_;
};

}  // namespace sph_gpu

class GpuWCSPHSolver : public WCSPHSolver {
public:
    void init() override;
    void step() override;
    void resizeData() override { WCSPHSolver::resizeData(); }
    sph_ctx* context() const { return link_.ctx(); }

private:
    sph_gpu::GpuSceneLink link_;
};

class GpuPCISPHSolver : public PCISPHSolver {
public:
    void init() override;
    void step() override;
    void resizeData() override { PCISPHSolver::resizeData(); }
    sph_ctx* context() const { return link_.ctx(); }

private:
    sph_gpu::GpuSceneLink link_;
};

class GpuDFSPHSolver : public DFSPHSolver {
public:
    void init() override;
    void step() override;
    void resizeData() override { DFSPHSolver::resizeData(); }
    sph_ctx* context() const { return link_.ctx(); }

private:
    sph_gpu::GpuSceneLink link_;
};
