// Matrix-transform subset of the GLM API, written for this project (see
// ../glm.hpp).  rotate(m, angle, axis): R, the rotation by `angle` radians
// about the normalised `axis` (Rodrigues' formula, t = (1 - cos) axis), and
// columns 0-2 of the result as m[0] R[c][0] + m[1] R[c][1] + m[2] R[c][2]
// (left to right), column 3 copied from m, as GLM documents and computes it.
#ifndef SPH_ORACLE_GLM_SHIM_MATRIX_TRANSFORM_HPP
#define SPH_ORACLE_GLM_SHIM_MATRIX_TRANSFORM_HPP

#include "../glm.hpp"

namespace glm {

template <typename T>
tmat4<T> rotate(const tmat4<T>& m, T angle, const tvec3<T>& axis_in)
{
    const T c = std::cos(angle), s = std::sin(angle);
    const tvec3<T> a = normalize(axis_in);
    const tvec3<T> t = (T(1) - c) * a;
    T r[3][3];
    r[0][0] = c + t.x * a.x;       r[0][1] = t.x * a.y + s * a.z; r[0][2] = t.x * a.z - s * a.y;
    r[1][0] = t.y * a.x - s * a.z; r[1][1] = c + t.y * a.y;       r[1][2] = t.y * a.z + s * a.x;
    r[2][0] = t.z * a.x + s * a.y; r[2][1] = t.z * a.y - s * a.x; r[2][2] = c + t.z * a.z;
    tmat4<T> out;
    for (int col = 0; col < 3; ++col)
        out[col] = m[0] * r[col][0] + m[1] * r[col][1] + m[2] * r[col][2];
    out[3] = m[3];
    return out;
}

}  // namespace glm

#endif
