// Matrix-transform subset of the GLM API, written for this project (see
// ../glm.hpp).  rotate(m, angle, axis) returns m * R where R is the rotation
// by `angle` radians about the normalised `axis` (Rodrigues' formula).
#ifndef SPH_ORACLE_GLM_SHIM_MATRIX_TRANSFORM_HPP
#define SPH_ORACLE_GLM_SHIM_MATRIX_TRANSFORM_HPP

#include "../glm.hpp"

namespace glm {

template <typename T>
tmat4<T> rotate(const tmat4<T>& m, T angle, const tvec3<T>& axis_in)
{
    const T c = std::cos(angle), s = std::sin(angle);
    const tvec3<T> a = normalize(axis_in);
    const tvec3<T> t = a * (T(1) - c);
    tmat4<T> r(T(1));
    r[0][0] = c + t.x * a.x;       r[0][1] = t.x * a.y + s * a.z; r[0][2] = t.x * a.z - s * a.y;
    r[1][0] = t.y * a.x - s * a.z; r[1][1] = c + t.y * a.y;       r[1][2] = t.y * a.z + s * a.x;
    r[2][0] = t.z * a.x + s * a.y; r[2][1] = t.z * a.y - s * a.x; r[2][2] = c + t.z * a.z;
    return m * r;
}

}  // namespace glm

#endif
