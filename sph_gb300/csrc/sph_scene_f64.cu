// FP64 parity form of the scene (absolute positions, the reference's
// expression order); compiled separately so the two forms build in parallel.
#include "sph_scene.cuh"

namespace sph {
SceneBase* make_scene_f64(const sph_scene_desc& d) { return new Scene<double>(d); }
}  // namespace sph
