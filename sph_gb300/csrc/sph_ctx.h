// The C ABI's context (sph_api.cu, sph_scene_io.cpp): a scene plus the
// host-side bookkeeping of Simulation::step (Simulation.cpp:148-182) and
// TimeManager (TimeManager.h:20-110): the simulated-time window in which
// steps run and the frame counter of the frame export.
#pragma once

#include <limits>
#include <string>

#include "sph_scene_base.h"

namespace sph {
class FrameWriter;  // sph_scene_io.cpp: frame files written by a host thread
}

struct sph_ctx {
    sph::SceneBase* scene = nullptr;
    std::string err;
    // While `track` is set every step reads the simulated time on the host:
    // steps outside [t_start, t_end] are skipped and TimeManager::hasToSave
    // is evaluated after each step (Simulation.cpp:152,171-178).
    bool track = false;
    double t_start = -std::numeric_limits<double>::infinity();
    double t_end = std::numeric_limits<double>::infinity();
    bool save = false;        // Simulation::activateSave: write a frame file when hasToSave fires
    std::string name;         // scene path; frame files are named after it (SceneLoader.cpp:202-212)
    unsigned frame = 1;       // TimeManager::frame, first frame 1 (TimeManager.h:45)
    double last_save = 0.0;   // TimeManager::lastTimeSave
    sph::FrameWriter* writer = nullptr;  // created with the first frame
};

namespace sph {
// Simulation::step for a tracked context (sph_scene_io.cpp).
int tracked_step(sph_ctx* ctx);
// Wait until every queued frame file is written; the first write error, if
// any, is returned (and stored in ctx->err).
int frames_flush(sph_ctx* ctx);
// frames_flush, then stop the writer thread (before the scene is freed).
int frames_close(sph_ctx* ctx);
}  // namespace sph
