// FP32 production form of the scene (cell-relative positions, FP64
// reductions); compiled separately so the two forms build in parallel.
#include "sph_scene.cuh"

namespace sph {
SceneBase* make_scene_f32(const sph_scene_desc& d) { return new Scene<float>(d); }
}  // namespace sph
