// Mesh boundaries, host side: AkinciBoundaryModel::addGeometry /
// sampleGeometry (AkinciBoundayModel.cpp:78-98,166-221), which read a
// triangulated OBJ file (the reference's vendored extern/OBJLoader.h),
// sample its surface with the regular per-triangle sampling of its vendored
// extern/RegularTriangleSampling.cpp (vertices, then the unique edges, then
// lines parallel to each face's longest edge, every sample at most
// maxDistance from the next), and place the samples with a fixed rotation of
// pi/2 about x.  Restated here in this project's own code, with the
// reference's arithmetic: the reader and the sampler work in FP32 (the
// vendored code's Real is float), sums over a vector's three components
// group as a0 + (a1 + a2) (Eigen's unrolled reduction), and the placement is
// FP64 with GLM's rotate and matrix-vector product.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "sph_scene_base.h"

namespace sph {
namespace {

struct V3f {
    float x, y, z;
};
V3f operator+(V3f a, V3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3f operator-(V3f a, V3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3f operator*(float s, V3f a) { return {s * a.x, s * a.y, s * a.z}; }
V3f operator/(V3f a, float s) { return {a.x / s, a.y / s, a.z / s}; }
float dot(V3f a, V3f b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
float norm(V3f a) { return std::sqrt(dot(a, a)); }

// Splits on the delimiter characters, dropping empty tokens (StringTools::tokenize).
std::vector<std::string> tokens(const std::string& s, char delim)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && s[i] == delim) ++i;
        if (i >= s.size()) break;
        size_t j = i;
        while (j < s.size() && s[j] != delim) ++j;
        out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

bool to_float(const std::string& t, float* v)
{
    char* end = nullptr;
    *v = std::strtof(t.c_str(), &end);  // a leading number, as std::stof reads it
    return end != t.c_str();
}

bool to_int(const std::string& t, int* v)
{
    char* end = nullptr;
    const long x = std::strtol(t.c_str(), &end, 10);
    *v = (int)x;
    return end != t.c_str();
}

// OBJLoader::loadObj with unit scale: "v" positions and the position
// indices of "f" triangles; the face syntax (v, v/vt, v//vn, v/vt/vn) is
// decided by whether "vt" / "vn" lines were seen before the face.
bool read_obj(const std::string& path, std::vector<V3f>* x, std::vector<unsigned>* faces, std::string* err)
{
    std::ifstream f(path);
    if (!f) { *err = "cannot read " + path; return false; }
    std::string line;
    bool vt = false, vn = false;
    unsigned lineno = 0;
    while (std::getline(f, line)) {
        ++lineno;
        const std::vector<std::string> head = tokens(line, ' ');
        if (head.empty()) continue;
        const std::string& type = head[0];
        auto bad = [&](const char* what) {
            *err = path + ":" + std::to_string(lineno) + ": " + what;
            return false;
        };
        if (type == "v") {
            const std::vector<std::string> t = tokens(line.substr(line.find('v') + 1), ' ');
            V3f p;
            if (t.size() < 3 || !to_float(t[0], &p.x) || !to_float(t[1], &p.y) || !to_float(t[2], &p.z))
                return bad("a vertex needs three numbers");
            p.x = p.x * 1.0f; p.y = p.y * 1.0f; p.z = p.z * 1.0f;
            x->push_back(p);
        } else if (type == "vt") {
            vt = true;
        } else if (type == "vn") {
            vn = true;
        } else if (type == "f") {
            const std::vector<std::string> t = tokens(line.substr(line.find('f') + 1), ' ');
            if (t.size() < 3) return bad("a face needs three vertices");
            for (int i = 0; i < 3; ++i) {
                int idx;
                const std::string first = (vn || vt) ? (tokens(t[i], '/').empty() ? std::string() : tokens(t[i], '/')[0]) : t[i];
                if (!to_int(first, &idx)) return bad("bad face index");
                if (idx < 1) return bad("face indices must be positive (relative indices are not supported)");
                faces->push_back((unsigned)(idx - 1));
            }
        }
    }
    for (unsigned v : *faces)
        if (v >= x->size()) { *err = path + ": a face refers to a vertex that does not exist"; return false; }
    return true;
}

// Samples an edge or a line of this length gets (ceil(l / d) + 1, ends
// included), or 0 when that count is beyond what one boundary can hold.
constexpr float kMaxSamples = 268435456.0f;  // 2^28
unsigned samples_along(float l, float d)
{
    const float n = std::ceil(l / d) + 1.0f;
    return n < kMaxSamples ? (unsigned)n : 0u;
}

// RegularTriangleSampling::sampleMesh in FP32.  False when the mesh would
// need more than 2^28 samples (an edge, a line or the whole surface).
bool sample_surface(const std::vector<V3f>& vx, const std::vector<unsigned>& faces, float d, std::vector<V3f>* out)
{
    // vertices
    out->insert(out->end(), vx.begin(), vx.end());
    // unique edges, smaller index first, sorted
    std::vector<std::pair<unsigned, unsigned>> edges;
    const size_t nf = faces.size() / 3;
    edges.reserve(3 * nf);
    for (size_t i = 0; i < nf; ++i)
        for (int c = 0; c < 3; ++c) {
            unsigned a = faces[3 * i + c], b = faces[3 * i + (c + 1) % 3];
            if (a > b) std::swap(a, b);
            edges.emplace_back(a, b);
        }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    // edge interiors: ceil(l / d) + 1 points end to end, ends skipped
    for (const auto& e : edges) {
        const V3f v0 = vx[e.first];
        const V3f dir = vx[e.second] - v0;
        const float l = norm(dir);
        const unsigned numSamples = samples_along(l, d);
        if (numSamples == 0 || out->size() + numSamples > (size_t)kMaxSamples) return false;
        if (numSamples == 1) { out->push_back(v0); continue; }
        for (unsigned i = 1; i < numSamples - 1; i++) out->push_back(v0 + ((float)i / (float)(numSamples - 1)) * dir);
    }
    // face interiors: lines parallel to the longest edge, ends skipped
    for (size_t f = 0; f < nf; ++f) {
        const unsigned* fc = &faces[3 * f];
        V3f v0{0, 0, 0}, base{0, 0, 0}, toTop{0, 0, 0};
        float l2 = 0;
        for (unsigned c = 0; c < 3; c++) {
            const V3f v = vx[fc[(c + 1) % 3]] - vx[fc[c]];
            const float le2 = dot(v, v);
            if (le2 > l2) {
                l2 = le2;
                v0 = vx[fc[c]];
                base = v;
                toTop = vx[fc[(c + 2) % 3]] - vx[fc[c]];
            }
        }
        if (!(l2 > 0.0f)) continue;  // all three corners coincide: nothing to sample inside
        const float l = std::sqrt(l2);
        const V3f bn = base / l;
        const float h = norm(toTop - dot(bn, toTop) * bn);
        const unsigned numLines = samples_along(h, d);
        if (numLines == 0) return false;
        for (unsigned line = 1; line < numLines - 1; line++) {
            V3f lineStart = v0;
            const float alpha = (float)line / (float)(numLines - 1);
            lineStart = lineStart + alpha * toTop;
            const float lineLength = (1.0f - alpha) * l;
            const unsigned numSamples = samples_along(lineLength, d);
            if (numSamples == 0 || out->size() + numSamples > (size_t)kMaxSamples) return false;
            for (unsigned i = 1; i < numSamples - 1; i++)
                out->push_back(lineStart + (((float)i * lineLength) / (float)(numSamples - 1)) * bn);
        }
    }
    return true;
}

// GLM's rotate(m, angle, axis) and m * v on column-major 4x4 FP64 matrices.
struct M4 {
    double c[4][4];  // c[col][row]
};
M4 rotate(const M4& m, double angle, const double axis_in[3])
{
    const double cs = std::cos(angle), sn = std::sin(angle);
    const double inv = 1.0 / std::sqrt(axis_in[0] * axis_in[0] + axis_in[1] * axis_in[1] + axis_in[2] * axis_in[2]);
    const double a[3] = {axis_in[0] * inv, axis_in[1] * inv, axis_in[2] * inv};
    const double t[3] = {(1.0 - cs) * a[0], (1.0 - cs) * a[1], (1.0 - cs) * a[2]};
    double r[3][3];
    r[0][0] = cs + t[0] * a[0]; r[0][1] = t[0] * a[1] + sn * a[2]; r[0][2] = t[0] * a[2] - sn * a[1];
    r[1][0] = t[1] * a[0] - sn * a[2]; r[1][1] = cs + t[1] * a[1]; r[1][2] = t[1] * a[2] + sn * a[0];
    r[2][0] = t[2] * a[0] + sn * a[1]; r[2][1] = t[2] * a[1] - sn * a[0]; r[2][2] = cs + t[2] * a[2];
    M4 out;
    for (int col = 0; col < 3; ++col)
        for (int row = 0; row < 4; ++row)
            out.c[col][row] = m.c[0][row] * r[col][0] + m.c[1][row] * r[col][1] + m.c[2][row] * r[col][2];
    for (int row = 0; row < 4; ++row) out.c[3][row] = m.c[3][row];
    return out;
}

}  // namespace

// AkinciBoundaryModel::addGeometry: samples at most max_distance apart,
// rotated by (pi/2, 0, 0) about x, y, z, unit scale, no translation.
long long sample_mesh(const char* path, double max_distance, std::vector<double>* out, std::string* err)
{
    std::vector<V3f> vx;
    std::vector<unsigned> faces;
    if (!read_obj(path, &vx, &faces, err)) return -1;
    const float d = (float)max_distance;
    if (!(d > 0.0f) || !std::isfinite(d)) { *err = "the maximum sample distance must be positive"; return -1; }
    std::vector<V3f> s;
    if (!sample_surface(vx, faces, d, &s)) {
        *err = "the mesh needs more than 2^28 samples at this distance";
        return -1;
    }
    M4 id;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) id.c[i][j] = i == j ? 1.0 : 0.0;
    const double ax[3] = {1.0, 0.0, 0.0}, ay[3] = {0.0, 1.0, 0.0}, az[3] = {0.0, 0.0, 1.0};
    M4 rot = rotate(id, M_PI * 0.5, ax);
    rot = rotate(rot, 0.0, ay);
    rot = rotate(rot, 0.0, az);
    out->resize(3 * s.size());
    for (size_t i = 0; i < s.size(); ++i) {
        const double v[4] = {(double)s[i].x, (double)s[i].y, (double)s[i].z, 1.0};
        for (int row = 0; row < 3; ++row) {
            const double p = (rot.c[0][row] * v[0] + rot.c[1][row] * v[1]) + (rot.c[2][row] * v[2] + rot.c[3][row] * v[3]);
            (*out)[3 * i + row] = p + 0.0;  // += translate (0, 0, 0)
        }
    }
    return (long long)s.size();
}

}  // namespace sph
