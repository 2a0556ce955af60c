// Type-erased scene interface shared by the C ABI (sph_api.cu) and the two
// numeric forms of the scene (sph_scene_f32.cu, sph_scene_f64.cu).
#pragma once

#include <string>
#include <vector>

#include "../../include/sph_gb300.h"

namespace sph {

#define SPH_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            fail(std::string(#call) + ": " + cudaGetErrorString(e_));                   \
            return SPH_ERR_CUDA;                                                        \
        }                                                                               \
    } while (0)

// Host restatements of the scene-construction helpers (sph_api.cu).
long long sample_box(double support_radius, const double mn[3], const double mx[3], double* out);
long long sample_sphere(double particle_radius, const double c[3], double radius, double* out);
long long fluid_block(double r, const double mn[3], const double mx[3], double* out);

struct SceneBase {
    sph_scene_desc d{};
    std::string err;
    std::vector<double> hx, hv, hb;   // staged points before init
    bool inited = false;
    virtual ~SceneBase() {}
    void fail(const std::string& m) { err = m; }
    virtual int init() = 0;
    virtual int step(int n) = 0;
    virtual int step_timed(int n, float* ms) = 0;
    virtual int sync() = 0;
    virtual int set_graph(int on) = 0;
    virtual int download(int field, double* out) = 0;
    virtual int stats(sph_stats* s) = 0;
    virtual int neighbors(int* cells, int* rank, int* off, int* nbr, int* boff, int* bnbr, long long* totals) = 0;
    virtual int launch_count(unsigned long long* out) = 0;
    virtual int set_profiling(int on) = 0;
    virtual int profile(char* buf, size_t len) = 0;
    virtual unsigned nfluid() const = 0;
    virtual unsigned nboundary() const = 0;
};

SceneBase* make_scene_f32(const sph_scene_desc& d);
SceneBase* make_scene_f64(const sph_scene_desc& d);

}  // namespace sph
