// Type-erased scene interface shared by the C ABI (sph_api.cu) and the two
// numeric forms of the scene (sph_scene_f32.cu, sph_scene_f64.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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
long long sample_pcisph_box(double support_radius, const double mn[3], const double mx[3], int inverted, double* out,
                            double* normals);
long long fluid_block(double r, const double mn[3], const double mx[3], double* out);
long long emitter_group(int type, double particle_radius, double width, double height, double* out);
// sph_mesh.cpp: AkinciBoundaryModel::addGeometry's surface samples of an OBJ
// file (xyz per point); -1 and *err on failure.
long long sample_mesh(const char* path, double max_distance, std::vector<double>* out, std::string* err);

// An emitter as FluidModel::addEmitter receives it (FluidModel.cpp:124),
// with its group (Emitter::buildSquareGroup / buildCircleGroup) sampled.
struct EmitterSpec {
    int type = 0;
    unsigned num = 0;
    double r[3] = {0, 0, 0};
    double v = 0;
    double q[4] = {1, 0, 0, 0};   // w, x, y, z
    double start = 0, width = 0, height = 0, spacing = 0;
    std::vector<double> group;    // xyz per point, emitter frame
};

// Where a downloadable field lives on the device (sorted order), for
// conversion kernels outside the scene's own translation unit.
struct FieldView {
    const void* v4 = nullptr;     // P4<R> array, or nullptr for scalar fields
    const void* s = nullptr;      // R array for scalar fields
    const uint32_t* id = nullptr;
    const uint32_t* cell = nullptr;
    int nx = 0, ny = 0, nz = 0, ox = 0, oy = 0, oz = 0;
    double h = 0.0;
    int kind = 0;                 // 0 vector, 1 position, 2 scalar
    unsigned n = 0;               // points
    size_t count = 0;             // doubles written
    bool fp64 = false;
    int device = 0;
    cudaStream_t stream = nullptr;
};

struct SceneBase {
    sph_scene_desc d{};
    std::string err;
    std::vector<double> hx, hv, hb;   // staged points before init
    std::vector<double> hbn;          // PCISPH boundary model: a normal per boundary point
    std::vector<EmitterSpec> hem;     // emitters, in the order they were added
    bool inited = false;
    virtual ~SceneBase() {}
    void fail(const std::string& m) { err = m; }
    virtual int init() = 0;
    virtual int step(int n) = 0;
    virtual int step_timed(int n, float* ms) = 0;
    virtual int sync() = 0;
    virtual int set_graph(int on) = 0;
    virtual int set_grid_growth(int on) = 0;
    virtual int pause_emitters(int pause) = 0;
    virtual int download(int field, double* out) = 0;
    // Positions (absolute, FP64) and velocities of the active particles in
    // original order into host memory x, v (pinned, 3 * active values each),
    // queued on the scene's stream; `done` is recorded after the copies.
    // *count_out receives the count copied.  Returns without waiting.
    virtual int capture_async(double* x, double* v, cudaEvent_t done, unsigned* count_out) = 0;
    virtual int stats(sph_stats* s) = 0;
    virtual int neighbors(int* cells, int* rank, int* off, int* nbr, int* boff, int* bnbr, long long* totals) = 0;
    virtual int pair_lists(int* count, int* off, int* nbr, long long* total) = 0;
    virtual int field_view(int field, FieldView* v) = 0;
    virtual int launch_count(unsigned long long* out) = 0;
    virtual int set_profiling(int on) = 0;
    virtual int profile(char* buf, size_t len) = 0;
    virtual int phase_profile(char* buf, size_t len) = 0;
    virtual unsigned nfluid() const = 0;
    virtual unsigned nboundary() const = 0;
};

SceneBase* make_scene_f32(const sph_scene_desc& d);
// sph_noalloc.cu
int download_noalloc(SceneBase* scene, int field, double* out, std::string* err);
SceneBase* make_scene_f64(const sph_scene_desc& d);

}  // namespace sph
