// Minimal GLM-API-compatible header written for this project.
//
// It exists only so that the reference simulator's own C++ sources can be
// compiled headless as a test oracle (the real GLM library is not installed
// here).  It covers exactly the subset those sources use: 3/4-component
// vectors of double/float/int, a 4x4 matrix, a quaternion, and the free
// functions length, dot, normalize, floor, ceil, abs, min, max, pow, clamp,
// cross, rotate.
//
// Semantics follow GLM's documented definitions:
//   length(v)    = sqrt(dot(v, v))
//   dot(a, b)    = (a.x*b.x + a.y*b.y) + a.z*b.z      (left to right)
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
//   conversions between vector types are implicit and component-wise
//   (static_cast), as in GLM without GLM_FORCE_EXPLICIT_CTOR.
#ifndef SPH_ORACLE_GLM_SHIM_HPP
#define SPH_ORACLE_GLM_SHIM_HPP

#include <cmath>
#include <cstddef>
#include <algorithm>

namespace glm {

template <typename T> struct tvec4;

template <typename T>
struct tvec3 {
    T x, y, z;
    tvec3() : x(0), y(0), z(0) {}
    template <typename S>
    explicit tvec3(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)) {}
    template <typename A, typename B, typename C>
    tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U>
    tvec3(const tvec3<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    template <typename U>
    tvec3(const tvec4<U>& o);

    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }

    tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    tvec3& operator*=(const tvec3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    tvec3& operator/=(const tvec3& o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
    tvec3& operator+=(T s) { x += s; y += s; z += s; return *this; }
    tvec3& operator-=(T s) { x -= s; y -= s; z -= s; return *this; }
    tvec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    tvec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
};

template <typename T>
struct tvec4 {
    T x, y, z, w;
    tvec4() : x(0), y(0), z(0), w(0) {}
    template <typename S>
    explicit tvec4(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)), w(static_cast<T>(s)) {}
    template <typename A, typename B, typename C, typename D>
    tvec4(A a, B b, C c, D d)
        : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
    template <typename U, typename D>
    tvec4(const tvec3<U>& v, D d)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(d)) {}
    template <typename U>
    tvec4(const tvec4<U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)), w(static_cast<T>(o.w)) {}

    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }

    tvec4& operator+=(const tvec4& o) { x += o.x; y += o.y; z += o.z; w += o.w; return *this; }
    tvec4& operator-=(const tvec4& o) { x -= o.x; y -= o.y; z -= o.z; w -= o.w; return *this; }
    tvec4& operator*=(T s) { x *= s; y *= s; z *= s; w *= s; return *this; }
};

template <typename T>
template <typename U>
tvec3<T>::tvec3(const tvec4<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}

// ---- vec3 arithmetic --------------------------------------------------------
template <typename T> tvec3<T> operator-(const tvec3<T>& a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <typename T> tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> tvec3<T> operator-(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> tvec3<T> operator*(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> tvec3<T> operator/(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <typename T> tvec3<T> operator+(const tvec3<T>& a, T s) { return tvec3<T>(a.x + s, a.y + s, a.z + s); }
template <typename T> tvec3<T> operator-(const tvec3<T>& a, T s) { return tvec3<T>(a.x - s, a.y - s, a.z - s); }
template <typename T> tvec3<T> operator*(const tvec3<T>& a, T s) { return tvec3<T>(a.x * s, a.y * s, a.z * s); }
template <typename T> tvec3<T> operator/(const tvec3<T>& a, T s) { return tvec3<T>(a.x / s, a.y / s, a.z / s); }
template <typename T> tvec3<T> operator+(T s, const tvec3<T>& a) { return tvec3<T>(s + a.x, s + a.y, s + a.z); }
template <typename T> tvec3<T> operator-(T s, const tvec3<T>& a) { return tvec3<T>(s - a.x, s - a.y, s - a.z); }
template <typename T> tvec3<T> operator*(T s, const tvec3<T>& a) { return tvec3<T>(s * a.x, s * a.y, s * a.z); }
template <typename T> tvec3<T> operator/(T s, const tvec3<T>& a) { return tvec3<T>(s / a.x, s / a.y, s / a.z); }
template <typename T> bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <typename T> bool operator!=(const tvec3<T>& a, const tvec3<T>& b) { return !(a == b); }

// ---- vec4 arithmetic --------------------------------------------------------
template <typename T> tvec4<T> operator+(const tvec4<T>& a, const tvec4<T>& b) { return tvec4<T>(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
template <typename T> tvec4<T> operator-(const tvec4<T>& a, const tvec4<T>& b) { return tvec4<T>(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <typename T> tvec4<T> operator*(const tvec4<T>& a, T s) { return tvec4<T>(a.x * s, a.y * s, a.z * s, a.w * s); }
template <typename T> tvec4<T> operator*(T s, const tvec4<T>& a) { return tvec4<T>(s * a.x, s * a.y, s * a.z, s * a.w); }

typedef tvec3<double> dvec3;
typedef tvec4<double> dvec4;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;
typedef tvec3<int> ivec3;
typedef tvec4<int> ivec4;

// ---- scalar functions (GLM exposes these for scalars too) -------------------
template <typename T> T abs(T a) { return a < T(0) ? -a : a; }
template <typename T> T min(T a, T b) { return b < a ? b : a; }
template <typename T> T max(T a, T b) { return a < b ? b : a; }
template <typename T> T clamp(T a, T lo, T hi) { return min(max(a, lo), hi); }
inline double ceil(double a) { return std::ceil(a); }
inline float ceil(float a) { return std::ceil(a); }
inline double floor(double a) { return std::floor(a); }
inline float floor(float a) { return std::floor(a); }
inline double pow(double a, double b) { return std::pow(a, b); }
inline float pow(float a, float b) { return std::pow(a, b); }
inline double sqrt(double a) { return std::sqrt(a); }

// ---- geometric functions ---------------------------------------------------
template <typename T> T dot(const tvec3<T>& a, const tvec3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> T dot(const tvec4<T>& a, const tvec4<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <typename T> T length(const tvec3<T>& a) { return std::sqrt(dot(a, a)); }
template <typename T> T length(const tvec4<T>& a) { return std::sqrt(dot(a, a)); }
template <typename T> tvec3<T> normalize(const tvec3<T>& a) { return a * (T(1) / std::sqrt(dot(a, a))); }
template <typename T> tvec3<T> cross(const tvec3<T>& a, const tvec3<T>& b)
{
    return tvec3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename T> tvec3<T> floor(const tvec3<T>& a) { return tvec3<T>(std::floor(a.x), std::floor(a.y), std::floor(a.z)); }
template <typename T> tvec3<T> ceil(const tvec3<T>& a) { return tvec3<T>(std::ceil(a.x), std::ceil(a.y), std::ceil(a.z)); }
template <typename T> tvec3<T> abs(const tvec3<T>& a) { return tvec3<T>(abs(a.x), abs(a.y), abs(a.z)); }
template <typename T> tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <typename T> tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

// ---- 4x4 matrix (column-major, m[c] is column c) ----------------------------
template <typename T>
struct tmat4 {
    tvec4<T> m[4];
    tmat4() : tmat4(T(1)) {}
    explicit tmat4(T d)
    {
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r) m[c][r] = (c == r) ? d : T(0);
    }
    tvec4<T>& operator[](int c) { return m[c]; }
    const tvec4<T>& operator[](int c) const { return m[c]; }
};

// m * v as GLM evaluates it: (m[0] v.x + m[1] v.y) + (m[2] v.z + m[3] v.w)
template <typename T>
tvec4<T> operator*(const tmat4<T>& a, const tvec4<T>& v)
{
    tvec4<T> r;
    for (int row = 0; row < 4; ++row)
        r[row] = (a[0][row] * v.x + a[1][row] * v.y) + (a[2][row] * v.z + a[3][row] * v.w);
    return r;
}

template <typename T>
tmat4<T> operator*(const tmat4<T>& a, const tmat4<T>& b)
{
    tmat4<T> r(T(0));
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            T s = 0;
            for (int k = 0; k < 4; ++k) s += a[k][row] * b[c][k];
            r[c][row] = s;
        }
    return r;
}

typedef tmat4<double> dmat4;
typedef tmat4<float> mat4;

}  // namespace glm

#endif
