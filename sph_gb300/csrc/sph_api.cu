// C ABI of sph_gb300 (include/sph_gb300.h).  No C++ exception crosses this
// boundary; every entry point returns an SPH_* status.
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "../../include/sph_gb300.h"
#include "sph_ctx.h"
#include "sph_scene_base.h"

#include <cuda_runtime.h>

namespace sph {

// AkinciBoundaryModel::sampleCube AkinciBoundayModel.cpp:100-134: the
// surface nodes of an (nx+1) x (ny+1) x (nz+1) lattice, spacing ~h/2.
long long sample_box(double supportRadius, const double mn[3], const double mx[3], double* out)
{
    const double lx = std::fabs(mn[0] - mx[0]), ly = std::fabs(mn[1] - mx[1]), lz = std::fabs(mn[2] - mx[2]);
    const unsigned nx = (unsigned)std::ceil(lx / (0.5 * supportRadius));
    const unsigned ny = (unsigned)std::ceil(ly / (0.5 * supportRadius));
    const unsigned nz = (unsigned)std::ceil(lz / (0.5 * supportRadius));
    const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
    long long count = 0;
    for (unsigned i = 0; i <= nx; i++)
        for (unsigned j = 0; j <= ny; j++)
            for (unsigned k = 0; k <= nz; k++) {
                const bool surface = (i == 0 || i == nx) || (j == 0 || j == ny) || (k == 0 || k == nz);
                if (!surface) continue;
                if (out) {
                    out[3 * count] = i * dx + mn[0];
                    out[3 * count + 1] = j * dy + mn[1];
                    out[3 * count + 2] = k * dz + mn[2];
                }
                ++count;
            }
    return count;
}

// AkinciBoundaryModel::sampleSphere AkinciBoundayModel.cpp:136-164:
// equal-area latitude rings, 1.5x the surface / particle-disc count.
// PCISPHBoundaryModel::sampleCube PCISPHBoundaryModel.cpp:56-184: the box's
// surface at a spacing of at most 0.45 h per axis; each point carries the
// normal of its face, or the normalised mean of its two (edge) or three
// (corner) faces' normals, pointing into the box, negated unless `inverted`
// (addCube :7-30).
long long sample_pcisph_box(double supportRadius, const double mn[3], const double mx[3], int inverted, double* out,
                            double* normals)
{
    double len[3], step[3];
    unsigned cnt[3];
    for (int a = 0; a < 3; ++a) {
        len[a] = std::fabs(mn[a] - mx[a]);
        cnt[a] = (unsigned)std::ceil(len[a] / (0.45 * supportRadius));
        step[a] = len[a] / cnt[a];
    }
    // into-the-box normal of the low / high face of each axis
    const double lo[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, hi[3][3] = {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
    const double sign = inverted ? 1.0 : -1;
    long long count = 0;
    for (unsigned i = 0; i <= cnt[0]; i++)
        for (unsigned j = 0; j <= cnt[1]; j++)
            for (unsigned k = 0; k <= cnt[2]; k++) {
                const unsigned idx[3] = {i, j, k};
                int faces = 0;
                const double* f[3];
                // faces in the order x, z, y: the order the reference adds them in
                const int order[3] = {0, 2, 1};
                for (int q = 0; q < 3; ++q) {
                    const int a = order[q];
                    if (idx[a] == 0) f[faces++] = lo[a];
                    else if (idx[a] == cnt[a]) f[faces++] = hi[a];
                }
                if (!faces) continue;
                double n[3] = {f[0][0], f[0][1], f[0][2]};
                if (faces > 1) {
                    for (int q = 1; q < faces; ++q)
                        for (int a = 0; a < 3; ++a) n[a] = n[a] + f[q][a];
                    for (int a = 0; a < 3; ++a) n[a] = faces == 2 ? n[a] * 0.5 : n[a] / 3.0;
                    const double inv = 1.0 / std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                    for (int a = 0; a < 3; ++a) n[a] = n[a] * inv;
                }
                if (out) {
                    for (int a = 0; a < 3; ++a) out[3 * count + a] = idx[a] * step[a] + mn[a];
                    for (int a = 0; a < 3; ++a) normals[3 * count + a] = sign * n[a];
                }
                count++;
            }
    return count;
}

long long sample_sphere(double particleRadius, const double c[3], double radius, double* out)
{
    const double separation = 1.5;
    const unsigned num = (unsigned)std::floor(4.0 * M_PI * radius * radius / (M_PI * particleRadius * particleRadius) * separation);
    const double a = 4.0 * M_PI / num;
    const double dd = std::sqrt(a);
    const int m_theta = (int)std::round(M_PI / dd);
    const double d_theta = M_PI / m_theta;
    const double d_phi = a / d_theta;
    long long count = 0;
    for (int m = 0; m < m_theta; ++m) {
        const double theta = M_PI * (m + 0.5) / m_theta;
        const int m_phi = (int)std::round(2.0 * M_PI * std::sin(theta) / d_phi);
        for (int n = 0; n < m_phi; ++n) {
            const double phi = 2.0 * M_PI * n / m_phi;
            const double x = std::sin(theta) * std::cos(phi);
            const double y = std::sin(theta) * std::sin(phi);
            const double z = std::cos(theta);
            if (out) {
                out[3 * count] = radius * x + c[0];
                out[3 * count + 1] = radius * y + c[1];
                out[3 * count + 2] = radius * z + c[2];
            }
            ++count;
        }
    }
    return count;
}

// Simulation::buildFluidBlock Simulation.cpp:512-539: lattice at spacing 2r
// starting at min + r.
long long fluid_block(double r, const double mn[3], const double mx[3], double* out)
{
    const double dist = 2.0 * r;
    const int px = (int)std::floor((mx[0] - mn[0]) / dist + 1e-5);
    const int py = (int)std::floor((mx[1] - mn[1]) / dist + 1e-5);
    const int pz = (int)std::floor((mx[2] - mn[2]) / dist + 1e-5);
    long long count = 0;
    for (int i = 0; i < px; ++i)
        for (int j = 0; j < py; ++j)
            for (int k = 0; k < pz; ++k) {
                if (out) {
                    out[3 * count] = i * dist + (mn[0] + r);
                    out[3 * count + 1] = j * dist + (mn[1] + r);
                    out[3 * count + 2] = k * dist + (mn[2] + r);
                }
                ++count;
            }
    return count;
}

// Emitter::buildCircleGroup / buildSquareGroup Emitter.cpp:31-79: the
// group of points emitted each time, in the emitter's frame (z = 0).
// Circle: the centre and rings of radius (i + 1) 2r, i < floor((width - r) /
// 2r), each with floor(2 pi radius / 2r) points at equal angles from the +y
// axis (x = R sin a, y = R cos a).  Square: a floor(width / 2r) x
// floor(height / 2r) lattice at spacing 2r centred on the origin, x outer.
// (A negative level count, which the reference converts to unsigned
// unchecked, is taken as zero.)
long long emitter_group(int type, double particleRadius, double width, double height, double* out)
{
    long long count = 0;
    auto put = [&](double x, double y) {
        if (out) {
            out[3 * count] = x;
            out[3 * count + 1] = y;
            out[3 * count + 2] = 0.0;
        }
        ++count;
    };
    if (type == SPH_EMITTER_CIRCLE) {
        const double dist = 2.0 * particleRadius;
        const double lv = std::floor((width - 0.5 * dist) / dist);
        const unsigned numLevels = lv > 0.0 ? (unsigned)lv : 0u;
        put(0.0, 0.0);
        for (unsigned i = 0; i < numLevels; ++i) {
            const double radius = (i + 1) * dist;
            const double l = 2.0 * M_PI * radius;
            const unsigned nParts = (unsigned)std::floor(l / dist);
            const double inc = 2 * M_PI / nParts;
            for (unsigned k = 0; k < nParts; ++k) {
                const double angle = k * inc;
                put(radius * std::sin(angle), radius * std::cos(angle));
            }
        }
    } else {
        const double dist = particleRadius * 2.0;
        const double fx = std::floor(width / dist), fy = std::floor(height / dist);
        const unsigned numX = fx > 0.0 ? (unsigned)fx : 0u, numY = fy > 0.0 ? (unsigned)fy : 0u;
        const double realWidth = (numX - 1) * dist;
        const double realHeight = (numY - 1) * dist;
        for (unsigned i = 0; i < numX; ++i)
            for (unsigned j = 0; j < numY; ++j) put(realWidth * 0.5 - i * dist, realHeight * 0.5 - j * dist);
    }
    return count;
}

}  // namespace sph

static int bad(sph_ctx* ctx, const char* m)
{
    if (ctx) ctx->err = m;
    return SPH_ERR_INVALID;
}

static int relay(sph_ctx* ctx, int rc)
{
    if (rc != SPH_OK && ctx && ctx->scene) ctx->err = ctx->scene->err;
    return rc;
}

extern "C" {

int sph_scene_desc_init(sph_scene_desc* d)
{
    if (!d) return SPH_ERR_INVALID;
    std::memset(d, 0, sizeof *d);
    d->simulation_method = SPH_DFSPH;
    d->boundary_method = SPH_BOUNDARY_AKINCI;
    d->precision = SPH_PRECISION_F32;
    d->particle_radius = 0.025;
    d->gravity[1] = -9.81;
    d->time_step = 0.0001;       // TimeManager.h:44
    d->min_time_step = 0.00001;
    d->max_time_step = 0.005;
    d->fps = 60.0;
    d->density0 = 1000.0;        // FluidModel.cpp:98
    d->stiffness = 1000.0;
    d->gamma = 7.0;
    d->max_error = 0.01;         // SPHSolver.cpp:18
    d->max_error_v = 0.001;
    d->cfl_factor = 1.0;         // DFSPHSolver.cpp:21
    d->min_iterations = -1;
    d->max_iterations = -1;
    d->min_iterations_v = -1;
    d->max_iterations_v = -1;
    d->viscosity_method = -1;
    d->surface_tension_method = -1;
    d->adhesion_method = -1;
    d->cube_max[0] = d->cube_max[1] = d->cube_max[2] = 1.0;
    d->threads_per_particle = 0;
    d->neighbor_list_max = 64;
    d->bh_normal_fct = 0.0;
    d->bh_tangential_fct = 1.0;
    return SPH_OK;
}

int sph_ctx_create(const sph_scene_desc* desc, sph_ctx** out)
{
    if (!desc || !out) return SPH_ERR_INVALID;
    *out = nullptr;
    if (desc->simulation_method < 0 || desc->simulation_method > 2) return SPH_ERR_INVALID;
    if (desc->boundary_method < 0 || desc->boundary_method > 2) return SPH_ERR_INVALID;
    if (!(desc->particle_radius > 0.0) || !(desc->density0 > 0.0) || !(desc->time_step > 0.0) || !(desc->fps > 0.0))
        return SPH_ERR_INVALID;
    sph_ctx* c = new (std::nothrow) sph_ctx();
    if (!c) return SPH_ERR_INVALID;
    try {
        c->scene = desc->precision == SPH_PRECISION_F64 ? sph::make_scene_f64(*desc) : sph::make_scene_f32(*desc);
    } catch (...) {
        delete c;
        return SPH_ERR_INVALID;
    }
    *out = c;
    return SPH_OK;
}

int sph_ctx_destroy(sph_ctx* ctx)
{
    if (!ctx) return SPH_ERR_INVALID;
    sph::frames_close(ctx);  // queued frame files are written first
    delete ctx->scene;
    delete ctx;
    return SPH_OK;
}

int sph_ctx_set_fluid(sph_ctx* ctx, const double* x, const double* v, unsigned n)
{
    if (!ctx || (!x && n)) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "fluid must be set before sph_ctx_init");
    try {
        ctx->scene->hx.assign(x, x + 3 * (size_t)n);
        if (v) ctx->scene->hv.assign(v, v + 3 * (size_t)n);
        else ctx->scene->hv.assign(3 * (size_t)n, 0.0);
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    return SPH_OK;
}

int sph_ctx_add_fluid_block(sph_ctx* ctx, const double mn[3], const double mx[3])
{
    if (!ctx || !mn || !mx) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "fluid must be added before sph_ctx_init");
    const double r = ctx->scene->d.particle_radius;
    const long long m = sph::fluid_block(r, mn, mx, nullptr);
    try {
        auto& hx = ctx->scene->hx;
        auto& hv = ctx->scene->hv;
        if (hv.size() != hx.size()) hv.assign(hx.size(), 0.0);
        const size_t at = hx.size();
        hx.resize(at + 3 * (size_t)m);
        hv.resize(at + 3 * (size_t)m, 0.0);
        sph::fluid_block(r, mn, mx, hx.data() + at);
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    return SPH_OK;
}

static int add_boundary(sph_ctx* ctx, const double* pts, long long m, const double* normals = nullptr)
{
    const bool pcisph = ctx->scene->d.boundary_method == SPH_BOUNDARY_PCISPH;
    if (pcisph && !normals)
        return bad(ctx, "the PCISPH boundary model needs normals: use sph_ctx_add_pcisph_box / _sphere");
    try {
        auto& hb = ctx->scene->hb;
        hb.insert(hb.end(), pts, pts + 3 * m);
        if (pcisph) ctx->scene->hbn.insert(ctx->scene->hbn.end(), normals, normals + 3 * m);
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    return SPH_OK;
}

int sph_ctx_add_pcisph_box(sph_ctx* ctx, const double mn[3], const double mx[3], int inverted)
{
    if (!ctx || !mn || !mx) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    if (ctx->scene->d.boundary_method != SPH_BOUNDARY_PCISPH) return bad(ctx, "boundary_method is not SPH_BOUNDARY_PCISPH");
    const double h = 4.0 * ctx->scene->d.particle_radius;
    const long long m = sph::sample_pcisph_box(h, mn, mx, inverted, nullptr, nullptr);
    std::vector<double> pts, nrm;
    try {
        pts.resize(3 * m + 1);
        nrm.resize(3 * m + 1);
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    sph::sample_pcisph_box(h, mn, mx, inverted, pts.data(), nrm.data());
    return add_boundary(ctx, pts.data(), m, nrm.data());
}

int sph_ctx_add_pcisph_sphere(sph_ctx* ctx, const double c[3], double radius, int inverted)
{
    if (!ctx || !c || !(radius > 0.0)) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    if (ctx->scene->d.boundary_method != SPH_BOUNDARY_PCISPH) return bad(ctx, "boundary_method is not SPH_BOUNDARY_PCISPH");
    const double r = ctx->scene->d.particle_radius;
    const long long m = sph::sample_sphere(r, c, radius, nullptr);
    std::vector<double> pts, nrm;
    try {
        pts.resize(3 * m + 1);
        nrm.resize(3 * m + 1);
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    sph::sample_sphere(r, c, radius, pts.data());
    // PCISPHBoundaryModel::addSphere :32-54: inv * (centre - point), not normalised
    const double sign = inverted ? 1.0 : -1;
    for (long long q = 0; q < m; ++q)
        for (int a = 0; a < 3; ++a) nrm[3 * q + a] = sign * (c[a] - pts[3 * q + a]);
    return add_boundary(ctx, pts.data(), m, nrm.data());
}

int sph_ctx_add_boundary_box(sph_ctx* ctx, const double mn[3], const double mx[3])
{
    if (!ctx || !mn || !mx) return bad(ctx, "invalid argument");
    if (ctx->scene->d.boundary_method == SPH_BOUNDARY_PCISPH) return sph_ctx_add_pcisph_box(ctx, mn, mx, 1);
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    const double h = 4.0 * ctx->scene->d.particle_radius;
    const long long m = sph::sample_box(h, mn, mx, nullptr);
    std::string tmp;
    double* buf = new (std::nothrow) double[3 * m + 1];
    if (!buf) return bad(ctx, "out of host memory");
    sph::sample_box(h, mn, mx, buf);
    const int rc = add_boundary(ctx, buf, m);
    delete[] buf;
    return rc;
}

int sph_ctx_add_boundary_sphere(sph_ctx* ctx, const double c[3], double radius)
{
    if (!ctx || !c || !(radius > 0.0)) return bad(ctx, "invalid argument");
    if (ctx->scene->d.boundary_method == SPH_BOUNDARY_PCISPH) return sph_ctx_add_pcisph_sphere(ctx, c, radius, 0);
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    const double r = ctx->scene->d.particle_radius;
    const long long m = sph::sample_sphere(r, c, radius, nullptr);
    double* buf = new (std::nothrow) double[3 * m + 1];
    if (!buf) return bad(ctx, "out of host memory");
    sph::sample_sphere(r, c, radius, buf);
    const int rc = add_boundary(ctx, buf, m);
    delete[] buf;
    return rc;
}

int sph_ctx_add_boundary_mesh(sph_ctx* ctx, const char* obj_path, double max_distance)
{
    if (!ctx || !obj_path) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    if (ctx->scene->d.boundary_method != SPH_BOUNDARY_AKINCI)
        return bad(ctx, "mesh boundaries belong to the Akinci boundary model (AkinciBoundaryModel::addGeometry)");
    std::vector<double> pts;
    std::string err;
    long long m;
    try {
        m = sph::sample_mesh(obj_path, max_distance, &pts, &err);
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    if (m < 0) {
        ctx->err = err;
        return SPH_ERR_INVALID;
    }
    if (m > 0xffffffffll) return bad(ctx, "too many mesh samples");
    return add_boundary(ctx, pts.data(), (unsigned)m);
}

int sph_ctx_add_pcisph_points(sph_ctx* ctx, const double* x, const double* normals, unsigned n)
{
    if (!ctx || (n && (!x || !normals))) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    if (ctx->scene->d.boundary_method != SPH_BOUNDARY_PCISPH) return bad(ctx, "boundary_method is not SPH_BOUNDARY_PCISPH");
    return add_boundary(ctx, x, n, normals);
}

int sph_ctx_add_boundary_points(sph_ctx* ctx, const double* x, unsigned n)
{
    if (!ctx || (!x && n)) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "boundary must be added before sph_ctx_init");
    return add_boundary(ctx, x, n);
}

int sph_ctx_add_emitter(sph_ctx* ctx, int type, unsigned num_particles, const double position[3], double velocity,
                        const double rotation[4], double start_time, double width, double height, double spacing)
{
    if (!ctx || !position || !rotation) return bad(ctx, "invalid argument");
    if (ctx->scene->inited) return bad(ctx, "emitters must be added before sph_ctx_init");
    if (type != SPH_EMITTER_SQUARE && type != SPH_EMITTER_CIRCLE)
        return bad(ctx, "emitter type must be SPH_EMITTER_SQUARE (0) or SPH_EMITTER_CIRCLE (1)");
    if (ctx->scene->hem.size() >= 64) return bad(ctx, "at most 64 emitters per scene");
    const double vals[] = {position[0], position[1], position[2], velocity, rotation[0], rotation[1], rotation[2],
                           rotation[3], start_time, width, height, spacing};
    for (double x : vals)
        if (!std::isfinite(x)) return bad(ctx, "emitter parameters must be finite");
    try {
        sph::EmitterSpec e;
        e.type = type;
        e.num = num_particles;
        for (int k = 0; k < 3; ++k) e.r[k] = position[k];
        for (int k = 0; k < 4; ++k) e.q[k] = rotation[k];
        e.v = velocity;
        e.start = start_time;
        e.width = width;
        e.height = height;
        e.spacing = spacing;
        const double r = ctx->scene->d.particle_radius;
        const long long m = sph::emitter_group(type, r, width, height, nullptr);
        if (m > (1ll << 24)) return bad(ctx, "emitter group larger than 2^24 particles");
        e.group.resize(3 * (size_t)m);
        sph::emitter_group(type, r, width, height, e.group.data());
        ctx->scene->hem.push_back(std::move(e));
    } catch (...) {
        return bad(ctx, "out of host memory");
    }
    return SPH_OK;
}

int sph_ctx_pause_emitters(sph_ctx* ctx, int pause)
{
    if (!ctx) return SPH_ERR_INVALID;
    return relay(ctx, ctx->scene->pause_emitters(pause));
}

int sph_ctx_init(sph_ctx* ctx)
{
    if (!ctx) return SPH_ERR_INVALID;
    return relay(ctx, ctx->scene->init());
}

int sph_ctx_step(sph_ctx* ctx, int nsteps)
{
    if (!ctx || nsteps < 0) return bad(ctx, "invalid argument");
    if (!ctx->track) return relay(ctx, ctx->scene->step(nsteps));
    for (int k = 0; k < nsteps; ++k) {
        const int rc = sph::tracked_step(ctx);
        if (rc != SPH_OK) return rc;
    }
    return SPH_OK;
}

int sph_ctx_step_timed(sph_ctx* ctx, int nsteps, float* elapsed_ms)
{
    if (!ctx || nsteps < 0 || !elapsed_ms) return bad(ctx, "invalid argument");
    return relay(ctx, ctx->scene->step_timed(nsteps, elapsed_ms));
}

int sph_ctx_synchronize(sph_ctx* ctx)
{
    if (!ctx) return SPH_ERR_INVALID;
    if (!ctx->scene->inited) return SPH_OK;
    const int rc = relay(ctx, ctx->scene->sync());
    if (rc != SPH_OK) return rc;
    return sph::frames_flush(ctx);  // and every queued frame file is on disk
}

int sph_ctx_set_graph(sph_ctx* ctx, int enable)
{
    if (!ctx) return SPH_ERR_INVALID;
    return relay(ctx, ctx->scene->set_graph(enable));
}

int sph_ctx_set_grid_growth(sph_ctx* ctx, int enable)
{
    if (!ctx) return SPH_ERR_INVALID;
    return relay(ctx, ctx->scene->set_grid_growth(enable));
}

int sph_ctx_get_desc(const sph_ctx* ctx, sph_scene_desc* out)
{
    if (!ctx || !out) return SPH_ERR_INVALID;
    *out = ctx->scene->d;
    return SPH_OK;
}

int sph_ctx_num_particles(const sph_ctx* ctx, unsigned* nf, unsigned* nb)
{
    if (!ctx) return SPH_ERR_INVALID;
    if (nf) *nf = ctx->scene->nfluid();
    if (nb) *nb = ctx->scene->nboundary();
    return SPH_OK;
}

int sph_ctx_download(sph_ctx* ctx, int field, double* out)
{
    if (!ctx || !out) return bad(ctx, "invalid argument");
    return relay(ctx, ctx->scene->download(field, out));
}

int sph_ctx_download_noalloc(sph_ctx* ctx, int field, double* out)
{
    if (!ctx || !out) return bad(ctx, "invalid argument");
    std::string err;
    const int rc = sph::download_noalloc(ctx->scene, field, out, &err);
    if (rc != SPH_OK) ctx->err = err;
    return rc;
}

int sph_ctx_get_stats(sph_ctx* ctx, sph_stats* out)
{
    if (!ctx || !out) return bad(ctx, "invalid argument");
    return relay(ctx, ctx->scene->stats(out));
}

const char* sph_ctx_last_error(const sph_ctx* ctx)
{
    if (!ctx) return "null context";
    return ctx->err.c_str();
}

int sph_ctx_neighbors(sph_ctx* ctx, int* cells, int* cell_rank, int* nbr_off, int* nbr, int* bnbr_off, int* bnbr,
                      long long* totals)
{
    if (!ctx) return SPH_ERR_INVALID;
    return relay(ctx, ctx->scene->neighbors(cells, cell_rank, nbr_off, nbr, bnbr_off, bnbr, totals));
}

int sph_ctx_pair_lists(sph_ctx* ctx, int* count, int* off, int* nbr, long long* total)
{
    if (!ctx) return SPH_ERR_INVALID;
    if (nbr && !off) return bad(ctx, "nbr needs off");
    return relay(ctx, ctx->scene->pair_lists(count, off, nbr, total));
}

long long sph_sample_box(double support_radius, const double mn[3], const double mx[3], double* out)
{
    if (!mn || !mx || !(support_radius > 0.0)) return -1;
    return sph::sample_box(support_radius, mn, mx, out);
}

long long sph_sample_pcisph_box(double support_radius, const double mn[3], const double mx[3], int inverted,
                                double* out, double* normals)
{
    if (!mn || !mx || !(support_radius > 0.0) || (out && !normals)) return -1;
    return sph::sample_pcisph_box(support_radius, mn, mx, inverted, out, normals);
}

long long sph_sample_sphere(double particle_radius, const double c[3], double radius, double* out)
{
    if (!c || !(particle_radius > 0.0) || !(radius > 0.0)) return -1;
    return sph::sample_sphere(particle_radius, c, radius, out);
}

long long sph_sample_mesh(const char* obj_path, double max_distance, double* out)
{
    if (!obj_path) return -1;
    std::vector<double> pts;
    std::string err;
    long long m;
    try {
        m = sph::sample_mesh(obj_path, max_distance, &pts, &err);
    } catch (...) {
        return -1;
    }
    if (m > 0 && out) std::memcpy(out, pts.data(), pts.size() * sizeof(double));
    return m;
}

long long sph_emitter_group(int type, double particle_radius, double width, double height, double* out)
{
    if ((type != SPH_EMITTER_SQUARE && type != SPH_EMITTER_CIRCLE) || !(particle_radius > 0.0) || !std::isfinite(width) ||
        !std::isfinite(height))
        return -1;
    return sph::emitter_group(type, particle_radius, width, height, out);
}

long long sph_fluid_block(double particle_radius, const double mn[3], const double mx[3], double* out)
{
    if (!mn || !mx || !(particle_radius > 0.0)) return -1;
    return sph::fluid_block(particle_radius, mn, mx, out);
}

int sph_ctx_get_launch_count(sph_ctx* ctx, unsigned long long* out)
{
    if (!ctx || !out) return bad(ctx, "invalid argument");
    return relay(ctx, ctx->scene->launch_count(out));
}

int sph_ctx_set_profiling(sph_ctx* ctx, int enable)
{
    if (!ctx) return SPH_ERR_INVALID;
    return relay(ctx, ctx->scene->set_profiling(enable));
}

int sph_ctx_get_profile(sph_ctx* ctx, char* buf, unsigned long long len)
{
    if (!ctx) return SPH_ERR_INVALID;
    if (!ctx->scene->inited) return bad(ctx, "not initialised");
    const int n = ctx->scene->profile(buf, (size_t)len);
    if (n < 0) return relay(ctx, n);
    return n;
}

int sph_ctx_get_phase_profile(sph_ctx* ctx, char* buf, unsigned long long len)
{
    if (!ctx) return SPH_ERR_INVALID;
    if (!ctx->scene->inited) return bad(ctx, "not initialised");
    const int n = ctx->scene->phase_profile(buf, (size_t)len);
    if (n < 0) return relay(ctx, n);
    return n;
}

int sph_select_device(int device)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return SPH_ERR_INVALID;
    return cudaSetDevice(device) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

const char* sph_version(void) { return "sph_gb300 0.1 (sm_103a)"; }

}  // extern "C"
