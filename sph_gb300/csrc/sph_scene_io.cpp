// Scene files and frame export, host side of the C ABI:
//   * SceneLoader::readConfiguration (SceneLoader.cpp:9-198) and
//     Simulation::importScene (Simulation.cpp:331-494): a JSON scene file
//     into a context, through the same public entry points a C caller uses;
//   * SceneLoader::writeFluid (SceneLoader.cpp:200-264): the fluid state as
//     a JSON frame file;
//   * Simulation::step / run (Simulation.cpp:148-190) with TimeManager's
//     frame clock (TimeManager.h:101-110): the time window and frame output.
// The JSON reader is this project's own (a small recursive-descent parser
// over the JSON grammar, numbers through strtod).
#include <algorithm>
#include <charconv>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <system_error>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sph_gb300.h"
#include "sph_ctx.h"

namespace sph {
namespace {

// ---------------------------------------------------------------------------
// JSON values and reader
// ---------------------------------------------------------------------------
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } k = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    // the last occurrence wins for a repeated key, as an object assignment would
    const JVal* at(const char* key) const
    {
        if (k != Obj) return nullptr;
        for (size_t i = obj.size(); i-- > 0;)
            if (obj[i].first == key) return &obj[i].second;
        return nullptr;
    }
    size_t size() const { return k == Arr ? arr.size() : k == Obj ? obj.size() : 0; }
};

class JsonReader {
public:
    JsonReader(const char* b, const char* e) : p_(b), e_(e) {}
    bool parse(JVal* out, std::string* err)
    {
        ws();
        if (!value(out, 0)) { *err = msg_; return false; }
        ws();
        if (p_ != e_) { fail("trailing characters after the document"); *err = msg_; return false; }
        return true;
    }

private:
    const char* p_;
    const char* e_;
    std::string msg_;

    bool fail(const char* m)
    {
        if (msg_.empty()) msg_ = std::string("JSON: ") + m;
        return false;
    }
    void ws()
    {
        while (p_ < e_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char* s)
    {
        const size_t n = std::strlen(s);
        if ((size_t)(e_ - p_) < n || std::strncmp(p_, s, n) != 0) return fail("invalid literal");
        p_ += n;
        return true;
    }
    static void utf8(std::string& o, unsigned cp)
    {
        if (cp < 0x80) o += (char)cp;
        else if (cp < 0x800) { o += (char)(0xC0 | (cp >> 6)); o += (char)(0x80 | (cp & 0x3F)); }
        else if (cp < 0x10000) {
            o += (char)(0xE0 | (cp >> 12)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F));
        } else {
            o += (char)(0xF0 | (cp >> 18)); o += (char)(0x80 | ((cp >> 12) & 0x3F));
            o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F));
        }
    }
    bool hex4(unsigned* v)
    {
        if (e_ - p_ < 4) return fail("short \\u escape");
        unsigned r = 0;
        for (int i = 0; i < 4; ++i) {
            const char c = *p_++;
            r <<= 4;
            if (c >= '0' && c <= '9') r |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') r |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') r |= (unsigned)(c - 'A' + 10);
            else return fail("bad \\u escape");
        }
        *v = r;
        return true;
    }
    bool string(std::string* o)
    {
        ++p_;  // opening quote
        while (p_ < e_) {
            const char c = *p_++;
            if (c == '"') return true;
            if ((unsigned char)c < 0x20) return fail("control character in string");
            if (c != '\\') { *o += c; continue; }
            if (p_ >= e_) break;
            const char x = *p_++;
            switch (x) {
                case '"': *o += '"'; break;
                case '\\': *o += '\\'; break;
                case '/': *o += '/'; break;
                case 'b': *o += '\b'; break;
                case 'f': *o += '\f'; break;
                case 'n': *o += '\n'; break;
                case 'r': *o += '\r'; break;
                case 't': *o += '\t'; break;
                case 'u': {
                    unsigned cp;
                    if (!hex4(&cp)) return false;
                    if (cp >= 0xD800 && cp < 0xDC00 && e_ - p_ >= 6 && p_[0] == '\\' && p_[1] == 'u') {
                        p_ += 2;
                        unsigned lo;
                        if (!hex4(&lo)) return false;
                        if (lo < 0xDC00 || lo >= 0xE000) return fail("bad surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(*o, cp);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        return fail("unterminated string");
    }
    bool number(JVal* v)
    {
        const char* s = p_;
        if (p_ < e_ && *p_ == '-') ++p_;
        if (p_ >= e_ || !(*p_ >= '0' && *p_ <= '9')) return fail("bad number");
        if (*p_ == '0') ++p_;
        else while (p_ < e_ && *p_ >= '0' && *p_ <= '9') ++p_;
        if (p_ < e_ && *p_ == '.') {
            ++p_;
            if (p_ >= e_ || !(*p_ >= '0' && *p_ <= '9')) return fail("bad number");
            while (p_ < e_ && *p_ >= '0' && *p_ <= '9') ++p_;
        }
        if (p_ < e_ && (*p_ == 'e' || *p_ == 'E')) {
            ++p_;
            if (p_ < e_ && (*p_ == '+' || *p_ == '-')) ++p_;
            if (p_ >= e_ || !(*p_ >= '0' && *p_ <= '9')) return fail("bad number");
            while (p_ < e_ && *p_ >= '0' && *p_ <= '9') ++p_;
        }
        const std::string text(s, p_);
        v->k = JVal::Num;
        v->num = std::strtod(text.c_str(), nullptr);  // correctly rounded
        return true;
    }
    bool value(JVal* v, int depth)
    {
        if (depth > 200) return fail("nesting too deep");
        if (p_ >= e_) return fail("unexpected end of document");
        const char c = *p_;
        if (c == '{') {
            ++p_;
            v->k = JVal::Obj;
            ws();
            if (p_ < e_ && *p_ == '}') { ++p_; return true; }
            for (;;) {
                ws();
                if (p_ >= e_ || *p_ != '"') return fail("expected a key");
                std::string key;
                if (!string(&key)) return false;
                ws();
                if (p_ >= e_ || *p_ != ':') return fail("expected ':'");
                ++p_;
                ws();
                v->obj.emplace_back(std::move(key), JVal());
                if (!value(&v->obj.back().second, depth + 1)) return false;
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == '}') { ++p_; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p_;
            v->k = JVal::Arr;
            ws();
            if (p_ < e_ && *p_ == ']') { ++p_; return true; }
            for (;;) {
                ws();
                v->arr.emplace_back();
                if (!value(&v->arr.back(), depth + 1)) return false;
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == ']') { ++p_; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') { v->k = JVal::Str; return string(&v->str); }
        if (c == 't') { v->k = JVal::Bool; v->b = true; return lit("true"); }
        if (c == 'f') { v->k = JVal::Bool; v->b = false; return lit("false"); }
        if (c == 'n') { v->k = JVal::Null; return lit("null"); }
        return number(v);
    }
};

// Typed access with the key path in error messages.  A missing or mistyped
// required key is an error, as the reference's reads of it would throw; a
// missing list counts as empty (a null value has size 0).
struct Access {
    std::string err;
    bool ok() const { return err.empty(); }
    const JVal* need(const JVal* o, const char* key, const std::string& where)
    {
        const JVal* v = o ? o->at(key) : nullptr;
        if (!v && ok()) err = "scene file: missing " + where + key;
        return v;
    }
    double num(const JVal* o, const char* key, const std::string& where)
    {
        const JVal* v = need(o, key, where);
        if (!v) return 0.0;
        if (v->k == JVal::Num) return v->num;
        if (v->k == JVal::Bool) return v->b ? 1.0 : 0.0;
        if (ok()) err = "scene file: " + where + key + " is not a number";
        return 0.0;
    }
    int integer(const JVal* o, const char* key, const std::string& where)
    {
        const double x = num(o, key, where);
        if (ok() && (x != std::floor(x) || std::fabs(x) > 2147483647.0)) err = "scene file: " + where + key + " is not an integer";
        return (int)x;
    }
    bool boolean(const JVal* o, const char* key, const std::string& where) { return num(o, key, where) != 0.0; }
    void vec(const JVal* o, const char* key, const std::string& where, double* out, int n)
    {
        const JVal* v = need(o, key, where);
        if (!v) return;
        if (v->k != JVal::Arr || (int)v->arr.size() < n) {
            if (ok()) err = "scene file: " + where + key + " needs " + std::to_string(n) + " numbers";
            return;
        }
        for (int i = 0; i < n; ++i) {
            if (v->arr[i].k != JVal::Num) {
                if (ok()) err = "scene file: " + where + key + " needs numbers";
                return;
            }
            out[i] = v->arr[i].num;
        }
    }
    const JVal* list(const JVal* o, const char* key)
    {
        const JVal* v = o ? o->at(key) : nullptr;
        return (v && v->k == JVal::Arr) ? v : nullptr;
    }
};

int check(sph_ctx* ctx, int rc, const char* what, std::string* err)
{
    if (rc != SPH_OK && err->empty()) {
        const char* m = ctx ? sph_ctx_last_error(ctx) : "";
        *err = std::string(what) + ": " + (m && *m ? m : "failed");
    }
    return rc;
}

thread_local std::string g_load_error;

// readConfiguration + importScene up to (not including) init().
int load_scene(const char* path, const sph_scene_desc* base, sph_ctx** out, std::string* err)
{
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) { *err = std::string("cannot read ") + path; return SPH_ERR_INVALID; }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    JVal root;
    JsonReader rd(text.data(), text.data() + text.size());
    if (!rd.parse(&root, err)) return SPH_ERR_INVALID;
    Access A;

    // SceneLoader::readSceneInfo SceneLoader.cpp:38-77
    sph_scene_desc d;
    if (base) d = *base;
    else sph_scene_desc_init(&d);
    const JVal* cfg = A.need(&root, "Configuration", "");
    const std::string C = "Configuration.";
    const double startTime = A.num(cfg, "startTime", C), endTime = A.num(cfg, "endTime", C);
    d.time_step = A.num(cfg, "timeStep", C);
    d.fps = A.num(cfg, "fps", C);
    d.min_time_step = A.num(cfg, "minTimeStep", C);
    d.max_time_step = A.num(cfg, "maxTimeStep", C);
    const double cfl = A.num(cfg, "cflFactor", C);
    d.particle_radius = A.num(cfg, "particleRadius", C);
    d.boundary_method = A.integer(cfg, "boundaryMethod", C);
    d.simulation_method = A.integer(cfg, "simulationMethod", C);
    A.vec(cfg, "gravity", C, d.gravity, 3);
    if (!A.ok()) { *err = A.err; return SPH_ERR_INVALID; }
    // importScene Simulation.cpp:346-382: the solver takes its own settings
    if (d.simulation_method == SPH_WCSPH) {
        d.stiffness = A.num(cfg, "stiffness", C);
        d.gamma = A.num(cfg, "gamma", C);
    } else if (d.simulation_method == SPH_PCISPH) {
        d.max_error = A.num(cfg, "eta", C);
        d.min_iterations = A.integer(cfg, "minIterations", C);
        d.max_iterations = A.integer(cfg, "maxIterations", C);
    } else if (d.simulation_method == SPH_DFSPH) {
        d.max_error = A.num(cfg, "eta", C);
        d.max_error_v = A.num(cfg, "etaV", C);
        d.cfl_factor = cfl;
        d.min_iterations = A.integer(cfg, "minIterations", C);
        d.max_iterations = A.integer(cfg, "maxIterations", C);
        d.min_iterations_v = A.integer(cfg, "minIterationsV", C);
        d.max_iterations_v = A.integer(cfg, "maxIterationsV", C);
    } else {
        *err = "scene file: Configuration.simulationMethod must be 0 (WCSPH), 1 (PCISPH) or 2 (DFSPH)";
        return SPH_ERR_INVALID;
    }
    if (d.boundary_method < 0 || d.boundary_method > 2) {
        *err = "scene file: Configuration.boundaryMethod must be 0, 1 or 2";
        return SPH_ERR_INVALID;
    }

    // SceneLoader::readFluidInfo SceneLoader.cpp:79-141
    const JVal* fl = A.need(&root, "Fluid", "");
    const std::string F = "Fluid.";
    d.viscosity_method = A.integer(fl, "viscosityMethod", F);
    d.surface_tension_method = A.integer(fl, "surfaceTensionMethod", F);
    d.adhesion_method = A.integer(fl, "adhesionMethod", F);
    const JVal* models = A.list(fl, "FluidModel");
    if (A.ok() && (!models || models->size() != 1)) {
        *err = "scene file: Fluid.FluidModel must hold exactly one fluid model (one fluid phase per scene)";
        return SPH_ERR_UNSUPPORTED;
    }
    if (!A.ok()) { *err = A.err; return SPH_ERR_INVALID; }
    const JVal* fm = &models->arr[0];
    const std::string M = "Fluid.FluidModel[0].";
    d.density0 = A.num(fm, "density0", M);
    d.viscosity = 0.0; d.boundary_viscosity = 0.0; d.surface_tension = 0.0; d.adhesion = 0.0;
    if (d.viscosity_method > -1) {
        d.viscosity = A.num(fm, "viscosity", M);
        d.boundary_viscosity = A.num(fm, "boundaryViscosity", M);
    }
    if (d.surface_tension_method > -1) d.surface_tension = A.num(fm, "surfaceTension", M);
    if (d.adhesion_method > -1) d.adhesion = A.num(fm, "adhesion", M);
    struct Block { double mn[3], mx[3]; };
    std::vector<Block> blocks;
    if (const JVal* bl = A.list(fm, "fluidBlocks"))
        for (size_t j = 0; j < bl->arr.size(); ++j) {
            Block b{};
            const std::string W = M + "fluidBlocks[" + std::to_string(j) + "].";
            A.vec(&bl->arr[j], "min", W, b.mn, 3);
            A.vec(&bl->arr[j], "max", W, b.mx, 3);
            blocks.push_back(b);
        }
    struct Emit { int type; unsigned num; double r[3], v, q[4], start, w, h, spacing; };
    std::vector<Emit> emits;
    if (const JVal* el = A.list(fm, "emitters"))
        for (size_t j = 0; j < el->arr.size(); ++j) {
            Emit e{};
            const JVal* o = &el->arr[j];
            const std::string W = M + "emitters[" + std::to_string(j) + "].";
            A.vec(o, "position", W, e.r, 3);
            A.vec(o, "rotation", W, e.q, 4);
            e.v = A.num(o, "velocity", W);
            const double num = A.num(o, "numParticles", W);
            if (A.ok() && !(num >= 0.0 && num <= 4294967295.0 && num == std::floor(num)))
                A.err = "scene file: " + W + "numParticles must be a non-negative integer";
            e.num = (unsigned)num;
            e.start = A.num(o, "startTime", W);
            e.type = A.integer(o, "type", W);
            e.w = A.num(o, "width", W);
            e.h = A.num(o, "height", W);
            e.spacing = A.num(o, "spacing", W);
            emits.push_back(e);
        }

    // SceneLoader::readBoundaryInfo SceneLoader.cpp:143-198
    struct Shape { double a[3], b[3]; double radius; int inverted; };
    std::vector<Shape> boxes, spheres;
    std::vector<std::pair<std::string, double>> meshes;  // OBJ path, spacing in particle diameters
    const JVal* bnd = A.list(&root, "Boundary");
    if (bnd && bnd->arr.size() > 1) {
        // the reference builds one model per entry, and AkinciBoundaryModel::
        // computeVolume then indexes its own points with every model's
        // neighbour ids (AkinciBoundayModel.cpp:32-36, Simulation.h:39-44)
        *err = "scene file: more than one Boundary entry; put every shape in one entry";
        return SPH_ERR_UNSUPPORTED;
    }
    if (bnd && bnd->arr.size() == 1) {
        const JVal* b = &bnd->arr[0];
        const std::string B = "Boundary[0].";
        const bool bh = d.boundary_method == SPH_BOUNDARY_PCISPH;
        if (bh) {
            d.bh_normal_fct = A.num(b, "normalFct", B);
            d.bh_tangential_fct = A.num(b, "tangFct", B);
        }
        if (const JVal* bl = A.list(b, "box"))
            for (size_t j = 0; j < bl->arr.size(); ++j) {
                Shape s{};
                const std::string W = B + "box[" + std::to_string(j) + "].";
                if (bh) s.inverted = A.boolean(&bl->arr[j], "inverted", W) ? 1 : 0;
                A.vec(&bl->arr[j], "min", W, s.a, 3);
                A.vec(&bl->arr[j], "max", W, s.b, 3);
                boxes.push_back(s);
            }
        if (const JVal* sl = A.list(b, "sphere"))
            for (size_t j = 0; j < sl->arr.size(); ++j) {
                Shape s{};
                const std::string W = B + "sphere[" + std::to_string(j) + "].";
                if (bh) s.inverted = A.boolean(&sl->arr[j], "inverted", W) ? 1 : 0;
                A.vec(&sl->arr[j], "pos", W, s.a, 3);
                s.radius = A.num(&sl->arr[j], "radius", W);
                spheres.push_back(s);
            }
        if (const JVal* gl = A.list(b, "geometry"))
            for (size_t j = 0; j < gl->arr.size(); ++j) {
                const std::string W = B + "geometry[" + std::to_string(j) + "].";
                const JVal* pth = A.need(&gl->arr[j], "path", W);
                if (pth && pth->k != JVal::Str && A.ok()) A.err = "scene file: " + W + "path is not a string";
                const double spacing = A.num(&gl->arr[j], "spacing", W);
                if (A.ok()) meshes.emplace_back(pth->str, spacing);
            }
    }
    if (!A.ok()) { *err = A.err; return SPH_ERR_INVALID; }
    // importScene never creates a cube boundary model (Simulation.cpp:419-490)
    d.has_cube = 0;

    // importScene Simulation.cpp:346-490, through the public entry points
    sph_ctx* ctx = nullptr;
    int rc = sph_ctx_create(&d, &ctx);
    if (rc != SPH_OK) { *err = "scene file: the configuration was rejected (sph_ctx_create)"; return rc; }
    auto bail = [&](int code) { sph_ctx_destroy(ctx); return code; };
    for (const Block& b : blocks)  // Simulation::buildFluidBlock Simulation.cpp:512-539
        if (check(ctx, sph_ctx_add_fluid_block(ctx, b.mn, b.mx), "fluid block", err)) return bail(SPH_ERR_INVALID);
    for (const Emit& e : emits)  // FluidModel::addEmitter Simulation.cpp:407-418
        if (check(ctx, sph_ctx_add_emitter(ctx, e.type, e.num, e.r, e.v, e.q, e.start, e.w, e.h, e.spacing), "emitter", err))
            return bail(SPH_ERR_INVALID);
    if (d.boundary_method == SPH_BOUNDARY_AKINCI) {  // Simulation.cpp:427-446
        for (const Shape& s : boxes)
            if (check(ctx, sph_ctx_add_boundary_box(ctx, s.a, s.b), "boundary box", err)) return bail(SPH_ERR_INVALID);
        for (const Shape& s : spheres)
            if (check(ctx, sph_ctx_add_boundary_sphere(ctx, s.a, s.radius), "boundary sphere", err)) return bail(SPH_ERR_INVALID);
        for (const auto& m : meshes)  // addGeometry(path, spacing * particleRadius * 2.0)
            if (check(ctx, sph_ctx_add_boundary_mesh(ctx, m.first.c_str(), m.second * d.particle_radius * 2.0), "boundary mesh", err))
                return bail(SPH_ERR_INVALID);
    } else if (d.boundary_method == SPH_BOUNDARY_PCISPH) {  // Simulation.cpp:447-487
        for (const Shape& s : boxes)
            if (check(ctx, sph_ctx_add_pcisph_box(ctx, s.a, s.b, s.inverted), "boundary box", err)) return bail(SPH_ERR_INVALID);
        for (const Shape& s : spheres)
            if (check(ctx, sph_ctx_add_pcisph_sphere(ctx, s.a, s.radius, s.inverted), "boundary sphere", err))
                return bail(SPH_ERR_INVALID);
    }
    // Simulation::step runs while startTime <= time <= endTime; frames are
    // named after the scene path (Simulation.cpp:334)
    ctx->track = true;
    ctx->t_start = startTime;
    ctx->t_end = endTime;
    ctx->name = path;
    *out = ctx;
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// Frame export
// ---------------------------------------------------------------------------

// A finite double as the shortest decimal string that reads back to the
// same value, laid out as nlohmann::json writes numbers: with decimal point
// position n (value = 0.d1..dk x 10^n), "ddd00.0" for k <= n <= 15, "dd.dd"
// for 0 < n <= 15, "0.00dd" for -4 < n <= 0, otherwise "d.ddde+XX" (two
// exponent digits at least); non-finite values are written as null.
void put_double(std::string& o, double v)
{
    if (!std::isfinite(v)) { o += "null"; return; }
    if (std::signbit(v)) { o += '-'; v = -v; }
    if (v == 0.0) { o += "0.0"; return; }
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::scientific);
    // "d[.ddd]e[+-]XX"
    std::string digits;
    const char* q = buf;
    for (; q < r.ptr && *q != 'e'; ++q)
        if (*q != '.') digits += *q;
    const int e10 = std::atoi(std::string(q + 1, static_cast<const char*>(r.ptr)).c_str());
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    const int k = (int)digits.size();
    const int n = e10 + 1;
    if (k <= n && n <= 15) {
        o += digits;
        o.append((size_t)(n - k), '0');
        o += ".0";
    } else if (0 < n && n <= 15) {
        o.append(digits, 0, (size_t)n);
        o += '.';
        o.append(digits, (size_t)n, std::string::npos);
    } else if (-4 < n && n <= 0) {
        o += "0.";
        o.append((size_t)(-n), '0');
        o += digits;
    } else {
        o += digits[0];
        if (k > 1) { o += '.'; o.append(digits, 1, std::string::npos); }
        const int x = n - 1;
        o += 'e';
        o += x < 0 ? '-' : '+';
        const int ax = x < 0 ? -x : x;
        if (ax < 10) o += '0';
        o += std::to_string(ax);
    }
}

// The frame file's text: keys in sorted order, no whitespace; every slot of
// the fluid model (slots emitters have not filled yet hold zeros),
// "positions" and "velocities" absent when there are none
// (SceneLoader.cpp:214-257).
void frame_text(std::string& o, unsigned na, unsigned total, const double* x, const double* v, double time, double dt)
{
    o.clear();
    o.reserve(64 + (size_t)total * 120);
    o += "{\"numActiveParticles\":" + std::to_string(na) + ",\"numParticles\":" + std::to_string(total);
    auto triples = [&](const char* key, const double* a) {
        o += ",\"";
        o += key;
        o += "\":[";
        for (unsigned i = 0; i < total; ++i) {
            if (i) o += ',';
            o += '[';
            for (int c = 0; c < 3; ++c) {
                if (c) o += ',';
                put_double(o, i < na ? a[3 * (size_t)i + c] : 0.0);
            }
            o += ']';
        }
        o += ']';
    };
    if (total) triples("positions", x);
    o += ",\"time\":";
    put_double(o, time);
    o += ",\"timeStep\":";
    put_double(o, dt);
    if (total) triples("velocities", v);
    o += '}';
}

int write_text(const std::string& path, const std::string& o, std::string* err)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { *err = "cannot write " + path; return SPH_ERR_INVALID; }
    const size_t w = std::fwrite(o.data(), 1, o.size(), f);
    const int cl = std::fclose(f);
    if (w != o.size() || cl != 0) { *err = "cannot write " + path; return SPH_ERR_INVALID; }
    return SPH_OK;
}

int write_frame(sph_ctx* ctx, const std::string& path, std::string* err)
{
    sph_stats st;
    int rc = sph_ctx_get_stats(ctx, &st);
    if (rc != SPH_OK) { *err = sph_ctx_last_error(ctx); return rc; }
    const unsigned na = st.num_fluid, total = st.num_fluid_total;
    std::vector<double> x(3 * (size_t)na), v(3 * (size_t)na);
    if (na) {
        if ((rc = sph_ctx_download(ctx, SPH_FIELD_POSITION, x.data())) != SPH_OK ||
            (rc = sph_ctx_download(ctx, SPH_FIELD_VELOCITY, v.data())) != SPH_OK) {
            *err = sph_ctx_last_error(ctx);
            return rc;
        }
    }
    std::string o;
    frame_text(o, na, total, x.data(), v.data(), st.time, st.dt);
    return write_text(path, o, err);
}

// SceneLoader::writeFluid's file name: the frame number zero-padded to four
// digits, "_" + it inserted before the scene path's last five characters
// (".json").  Numbers of five digits and more are written unpadded.
std::string frame_name(const std::string& scene, unsigned frame)
{
    std::string num = std::to_string(frame);
    while (num.size() < 4) num = "0" + num;
    return scene.substr(0, scene.size() - 5) + "_" + num + scene.substr(scene.size() - 5);
}

double sim_time(sph_ctx* ctx, int* rc)
{
    sph_stats st;
    *rc = sph_ctx_get_stats(ctx, &st);
    return st.time;
}

}  // namespace

// Frame files written off the step loop: a frame is captured into pinned
// host memory on the scene's stream (positions and velocities in original
// order), and a host thread waits for the copy, formats the text and writes
// the file while the next steps run.  Two capture buffers: a third frame
// waits for the oldest file to be written.
class FrameWriter {
public:
    explicit FrameWriter(int device) : device_(device) { th_ = std::thread([this] { loop(); }); }
    ~FrameWriter()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
        for (Slot& s : slots_) {
            if (s.x) cudaFreeHost(s.x);
            if (s.v) cudaFreeHost(s.v);
            if (s.ev) cudaEventDestroy(s.ev);
        }
    }

    // Capture the current state and queue its file.
    int submit(SceneBase* scene, const std::string& path, unsigned total, double time, double dt, std::string* err)
    {
        int k = -1;
        {
            std::unique_lock<std::mutex> lk(m_);
            done_cv_.wait(lk, [&] { return !slots_[0].busy || !slots_[1].busy; });
            if (!err_.empty()) { *err = err_; return SPH_ERR_INVALID; }
            k = slots_[0].busy ? 1 : 0;
            slots_[k].busy = true;
        }
        Slot& s = slots_[k];
        const size_t need = 3 * (size_t)std::max(total, 1u);
        if (s.cap < need) {
            if (s.x) cudaFreeHost(s.x);
            if (s.v) cudaFreeHost(s.v);
            s.x = s.v = nullptr;
            s.cap = 0;
            if (cudaMallocHost((void**)&s.x, need * sizeof(double)) != cudaSuccess ||
                cudaMallocHost((void**)&s.v, need * sizeof(double)) != cudaSuccess) {
                release(k);
                *err = "cannot allocate pinned memory for frame capture";
                return SPH_ERR_CUDA;
            }
            s.cap = need;
        }
        if (!s.ev && cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess) {
            release(k);
            *err = "cannot create an event for frame capture";
            return SPH_ERR_CUDA;
        }
        unsigned na = 0;
        const int rc = scene->capture_async(s.x, s.v, s.ev, &na);
        if (rc != SPH_OK) {
            release(k);
            *err = scene->err;
            return rc;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            q_.push_back(Job{path, k, na, total, time, dt});
        }
        cv_.notify_all();
        return SPH_OK;
    }

    // Wait for every queued file; the first error since the last flush.
    int flush(std::string* err)
    {
        std::unique_lock<std::mutex> lk(m_);
        done_cv_.wait(lk, [&] { return q_.empty() && !slots_[0].busy && !slots_[1].busy; });
        if (!err_.empty()) {
            *err = err_;
            err_.clear();
            return SPH_ERR_INVALID;
        }
        return SPH_OK;
    }

private:
    struct Slot {
        double* x = nullptr;
        double* v = nullptr;
        size_t cap = 0;
        cudaEvent_t ev = nullptr;
        bool busy = false;
    };
    struct Job {
        std::string path;
        int slot;
        unsigned na, total;
        double time, dt;
    };

    void release(int k)
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            slots_[k].busy = false;
        }
        done_cv_.notify_all();
    }

    void loop()
    {
        cudaSetDevice(device_);
        std::string text;
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_ || !q_.empty(); });
                if (q_.empty()) return;  // stop requested and nothing left
                j = q_.front();
                q_.pop_front();
            }
            Slot& s = slots_[j.slot];
            std::string e;
            if (cudaEventSynchronize(s.ev) != cudaSuccess) e = "frame capture failed on the device";
            if (e.empty()) {
                frame_text(text, j.na, j.total, s.x, s.v, j.time, j.dt);
                write_text(j.path, text, &e);
            }
            {
                std::lock_guard<std::mutex> lk(m_);
                if (!e.empty() && err_.empty()) err_ = e;
                slots_[j.slot].busy = false;
            }
            done_cv_.notify_all();
        }
    }

    int device_;
    std::thread th_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    std::deque<Job> q_;
    Slot slots_[2];
    std::string err_;
    bool stop_ = false;
};

// Simulation::step Simulation.cpp:148-182: one solver step if the time is
// inside [startTime, endTime], then TimeManager::hasToSave (frame clock) and,
// with saving on, SceneLoader::writeFluid.
int tracked_step(sph_ctx* ctx)
{
    int rc;
    const double t = sim_time(ctx, &rc);
    if (rc != SPH_OK) return rc;
    if (!(t >= ctx->t_start && t <= ctx->t_end)) return SPH_OK;
    rc = ctx->scene->step(1);
    if (rc != SPH_OK) { ctx->err = ctx->scene->err; return rc; }
    sph_stats st;
    rc = sph_ctx_get_stats(ctx, &st);
    if (rc != SPH_OK) return rc;
    const double fps = ctx->scene->d.fps;
    if (st.time - ctx->last_save >= 1.0 / fps) {
        ctx->last_save = (double)ctx->frame / fps;
        if (ctx->save) {
            std::string err;
            if (!ctx->writer) {
                int dev = 0;
                cudaGetDevice(&dev);
                ctx->writer = new FrameWriter(dev);
            }
            rc = ctx->writer->submit(ctx->scene, frame_name(ctx->name, ctx->frame), st.num_fluid_total, st.time, st.dt,
                                     &err);
            if (rc != SPH_OK) { ctx->err = err; return rc; }
        }
        ctx->frame += 1;
    }
    return SPH_OK;
}

int frames_flush(sph_ctx* ctx)
{
    if (!ctx->writer) return SPH_OK;
    std::string err;
    const int rc = ctx->writer->flush(&err);
    if (rc != SPH_OK) ctx->err = err;
    return rc;
}

int frames_close(sph_ctx* ctx)
{
    const int rc = frames_flush(ctx);
    delete ctx->writer;
    ctx->writer = nullptr;
    return rc;
}

}  // namespace sph

extern "C" {

const char* sph_scene_load_error(void) { return sph::g_load_error.c_str(); }

int sph_ctx_load_scene(const char* json_path, const sph_scene_desc* base, sph_ctx** out)
{
    sph::g_load_error.clear();
    if (!json_path || !out) { sph::g_load_error = "invalid argument"; return SPH_ERR_INVALID; }
    const int rc = sph::load_scene(json_path, base, out, &sph::g_load_error);
    return rc;
}

int sph_ctx_import_scene(const char* json_path, const sph_scene_desc* base, sph_ctx** out)
{
    int rc = sph_ctx_load_scene(json_path, base, out);
    if (rc != SPH_OK) return rc;
    rc = sph_ctx_init(*out);
    if (rc != SPH_OK) {
        sph::g_load_error = std::string("sph_ctx_init: ") + sph_ctx_last_error(*out);
        sph_ctx_destroy(*out);
        *out = nullptr;
    }
    return rc;
}

int sph_ctx_set_time_window(sph_ctx* ctx, double start_time, double end_time)
{
    if (!ctx || std::isnan(start_time) || std::isnan(end_time)) return SPH_ERR_INVALID;
    ctx->track = true;
    ctx->t_start = start_time;
    ctx->t_end = end_time;
    return SPH_OK;
}

int sph_ctx_set_frame_output(sph_ctx* ctx, const char* scene_path, int active)
{
    if (!ctx) return SPH_ERR_INVALID;
    if (scene_path) {
        if (std::strlen(scene_path) < 5) {
            ctx->err = "the frame output path must end in .json";
            return SPH_ERR_INVALID;
        }
        ctx->name = scene_path;
    }
    if (active && ctx->name.size() < 5) {
        ctx->err = "no scene path for the frame files";
        return SPH_ERR_INVALID;
    }
    if (!active && sph::frames_flush(ctx) != SPH_OK) return SPH_ERR_INVALID;
    ctx->save = active != 0;
    ctx->track = true;
    return SPH_OK;
}

int sph_ctx_get_frame(const sph_ctx* ctx, unsigned* frame)
{
    if (!ctx || !frame) return SPH_ERR_INVALID;
    *frame = ctx->frame;
    return SPH_OK;
}

int sph_ctx_write_frame(sph_ctx* ctx, const char* path)
{
    if (!ctx || !path) return SPH_ERR_INVALID;
    if (sph::frames_flush(ctx) != SPH_OK) return SPH_ERR_INVALID;
    std::string err;
    const int rc = sph::write_frame(ctx, path, &err);
    if (rc != SPH_OK) ctx->err = err;
    return rc;
}

int sph_ctx_run(sph_ctx* ctx, unsigned long long max_steps, unsigned long long* steps_done)
{
    if (!ctx) return SPH_ERR_INVALID;
    unsigned long long done = 0;
    int rc = SPH_OK;
    const sph_scene_desc& d = ctx->scene->d;
    // no time step exceeds max(max dt, initial dt) (the DFSPH CFL step is
    // clamped to the max, the other solvers keep the initial step)
    const double dmax = std::max(d.max_time_step, d.time_step);
    while (done < max_steps) {
        const double t = sph::sim_time(ctx, &rc);
        if (rc != SPH_OK) break;
        if (!(t >= ctx->t_start && t <= ctx->t_end)) break;
        unsigned long long chunk = 1;
        if (!ctx->track) chunk = max_steps - done;
        else if (!ctx->save && std::isfinite(ctx->t_end)) {
            // steps that provably start inside the window run untracked;
            // the frame clock is not advanced for them
            const double k = std::floor((ctx->t_end - t) / dmax) - 1.0;
            if (k > 1.0) chunk = (unsigned long long)std::min(k, 4096.0);
            chunk = std::min(chunk, max_steps - done);
        }
        if (chunk > 1 || !ctx->track) {
            const unsigned long long c = std::min<unsigned long long>(chunk, 1u << 30);
            rc = ctx->scene->step((int)c);
            if (rc != SPH_OK) { ctx->err = ctx->scene->err; break; }
            done += c;
        } else {
            rc = sph::tracked_step(ctx);
            if (rc != SPH_OK) break;
            done += 1;
        }
    }
    if (steps_done) *steps_done = done;
    const int fr = sph::frames_flush(ctx);
    return rc != SPH_OK ? rc : fr;
}

}  // extern "C"
