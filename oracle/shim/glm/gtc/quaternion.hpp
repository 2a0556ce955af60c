// Quaternion subset of the GLM API, written for this project (see ../glm.hpp).
// Component order of the 4-scalar constructor is (w, x, y, z), as in GLM's
// default configuration; rotation of a vector v by unit quaternion q is
// q * v * conj(q).  The Euler-angle constructor takes (pitch, yaw, roll) in
// radians about x, y, z as GLM documents.
#ifndef SPH_ORACLE_GLM_SHIM_QUATERNION_HPP
#define SPH_ORACLE_GLM_SHIM_QUATERNION_HPP

#include "../glm.hpp"

namespace glm {

template <typename T>
struct tquat {
    T x, y, z, w;
    tquat() : x(0), y(0), z(0), w(1) {}
    template <typename A, typename B, typename C, typename D>
    tquat(A w_, B x_, C y_, D z_)
        : x(static_cast<T>(x_)), y(static_cast<T>(y_)), z(static_cast<T>(z_)), w(static_cast<T>(w_)) {}
    // Euler angles (radians) about x, y, z.
    tquat(const tvec3<T>& euler)
    {
        T cx = std::cos(euler.x * T(0.5)), sx = std::sin(euler.x * T(0.5));
        T cy = std::cos(euler.y * T(0.5)), sy = std::sin(euler.y * T(0.5));
        T cz = std::cos(euler.z * T(0.5)), sz = std::sin(euler.z * T(0.5));
        w = cx * cy * cz + sx * sy * sz;
        x = sx * cy * cz - cx * sy * sz;
        y = cx * sy * cz + sx * cy * sz;
        z = cx * cy * sz - sx * sy * cz;
    }
};

template <typename T>
tvec3<T> operator*(const tquat<T>& q, const tvec3<T>& v)
{
    // v' = v + 2 w (u x v) + 2 u x (u x v), u = (x, y, z)
    tvec3<T> u(q.x, q.y, q.z);
    tvec3<T> uv = cross(u, v);
    tvec3<T> uuv = cross(u, uv);
    return v + ((uv * q.w) + uuv) * T(2);
}

template <typename T>
tvec4<T> operator*(const tquat<T>& q, const tvec4<T>& v)
{
    tvec3<T> r = q * tvec3<T>(v.x, v.y, v.z);
    return tvec4<T>(r.x, r.y, r.z, v.w);
}

typedef tquat<double> dquat;
typedef tquat<float> quat;

}  // namespace glm

#endif
