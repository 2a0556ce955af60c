// Host side of one scene: device buffers, the grid build, and the per-step
// orchestration of WCSPHSolver::step (WCSPHSolver.cpp:14-78),
// PCISPHSolver::step (PCISPHSolver.cpp:21-81) and DFSPHSolver::step
// (DFSPHSolver.cpp:38-112) as sequences of kernels on one CUDA stream.
//
// Solver loops whose trip count depends on a convergence test run either
// host-driven (kernels of finished loops exit at once; the host reads the
// loop flag every few iterations) or, in graph mode, as CUDA-graph
// conditional WHILE nodes whose condition the reduction kernels set on the
// device, so a whole step is one graph launch with no host round trip.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "sph_scene_base.h"
#include "sph_kernels.cuh"
#include "sph_lists.cuh"
#include "sph_phase.cuh"

namespace sph {

// Kernel coefficients, evaluated in double as each reference kernel's
// setSupportRadius does (CubicSpline.h:18-26, Poly6.h:19-28, Spiky.h:18-27,
// ViscoK.h:18-26, Cohesion.h:20-27), the particle mass of
// Simulation::initMasses (Simulation.cpp:134-146), the plugin selection of
// FluidModel::set*Force (FluidModel.cpp:73-122) and the solver limits
// (defaults SPHSolver.cpp:12-19, DFSPHSolver.cpp:10-22).
template <typename R>
void scene_constants(const sph_scene_desc& d, Consts<R>* out_c, LoopLimits* out_l, double* out_h, double* out_mass)
{
    const double r = d.particle_radius;
    const double sr = 4.0 * r;
    const double pi = M_PI;
    const double h3 = sr * sr * sr;
    const double h6 = sr * sr * sr * sr * sr * sr;
    const double h9 = sr * sr * sr * sr * sr * sr * sr * sr * sr;
    const double diameter = 2.0 * r;
    const double mass = d.density0 * std::pow(diameter, 3.0);
    Consts<R> c{};
    c.h = (R)sr;
    c.inv_h = (R)(1.0 / sr);
    c.h2 = (R)(sr * sr);
    c.cull2 = (R)(sr * sr * (sizeof(R) == 8 ? (1.0 + 1e-12) : (1.0 + 1e-6)));
    c.inv_density0 = 1.0 / (double)(R)d.density0;
    c.cs_k = (R)(8.0 / (pi * h3));
    c.cs_l = (R)(48.0 / (pi * h3));
    c.p6_h2 = (R)(sr * sr);
    c.p6_value = (R)(315.0 / (64.0 * M_PI * h9));
    c.p6_grad = (R)(945.0 / (32.0 * M_PI * h9));
    c.sp_value = (R)(15.0 / (M_PI * h6));
    c.sp_grad = (R)(45.0 / (M_PI * h6));
    c.vk_lapl = (R)(45 / (M_PI * h6));
    c.co_c1 = (R)(32.0 / (M_PI * h9));
    c.co_c2 = (R)(h6 / 64.0);
    c.mass = (R)mass;
    c.density0 = (R)d.density0;
    c.eps = (R)1e-5;
    c.gx = (R)d.gravity[0]; c.gy = (R)d.gravity[1]; c.gz = (R)d.gravity[2];
    c.stiffness = (R)d.stiffness;
    c.gamma = (R)d.gamma;
    c.k_eos = (R)(d.stiffness * d.density0 / d.gamma);
    c.visc = (R)d.viscosity;
    c.bvisc = (R)d.boundary_viscosity;
    c.st = (R)d.surface_tension;
    c.adh = (R)d.adhesion;
    for (int k = 0; k < 3; ++k) { c.cube_min[k] = (R)d.cube_min[k]; c.cube_max[k] = (R)d.cube_max[k]; }
    c.has_cube = (d.boundary_method == SPH_BOUNDARY_CUBE && d.has_cube) ? 1 : 0;
    // warm start: Akinci boundaries take 2 k_i, the PCISPH model k_i (DFSPHSolver.cpp:646-672)
    c.bwarm = (R)(d.boundary_method == SPH_BOUNDARY_PCISPH ? 1.0 : 2.0);
    c.bh_nf = (R)d.bh_normal_fct;
    c.bh_tf = (R)d.bh_tangential_fct;
    int fl = 0;
    if (d.viscosity_method > -1 && d.viscosity != 0.0) {
        if (d.viscosity_method == SPH_VISCOSITY_STANDARD) fl |= F_STD_VISC;
        else if (d.viscosity_method == SPH_VISCOSITY_ARTIFICIAL) fl |= F_ART_VISC;
        else if (d.viscosity_method == SPH_VISCOSITY_XSPH) fl |= F_XSPH;
        if (d.boundary_viscosity != 0.0) fl |= F_BVISC;
    }
    if (d.surface_tension_method == SPH_SURFACE_TENSION_AKINCI && d.surface_tension != 0.0) fl |= F_SURFACE_TENSION;
    if (d.adhesion_method == SPH_ADHESION_AKINCI && d.adhesion != 0.0) fl |= F_ADHESION;
    c.force_flags = fl;
    LoopLimits l{};
    l.maxError = 0.01; l.minIt = 3; l.maxIt = 100; l.maxErrorV = 0.001; l.minItV = 1; l.maxItV = 100;
    l.cflFactor = 1.0;
    if (d.simulation_method == SPH_DFSPH) { l.minIt = 2; l.maxIt = 100; }
    if (d.simulation_method != SPH_WCSPH) l.maxError = d.max_error;
    if (d.simulation_method == SPH_DFSPH) { l.maxErrorV = d.max_error_v; l.cflFactor = d.cfl_factor; }
    if (d.min_iterations >= 0) l.minIt = (unsigned)d.min_iterations;
    if (d.max_iterations >= 0) l.maxIt = (unsigned)d.max_iterations;
    if (d.min_iterations_v >= 0) l.minItV = (unsigned)d.min_iterations_v;
    if (d.max_iterations_v >= 0) l.maxItV = (unsigned)d.max_iterations_v;
    l.particleRadius = d.particle_radius;
    // TimeManager::setMinTimeStep keeps min(minTs, 1/fps) (TimeManager.h:55)
    const double minFPSTimeStep = 1.0 / d.fps;
    l.minTs = minFPSTimeStep < d.min_time_step ? minFPSTimeStep : d.min_time_step;
    l.maxTs = d.max_time_step;
    *out_c = c;
    *out_l = l;
    *out_h = sr;
    *out_mass = mass;
}

// Dense cell box over the domain (given, or the points' bounds widened by
// rel_margin of their extent) with a two-cell margin, and the column-Morton
// tables of its key space.
struct GridPlan {
    int o[3] = {0, 0, 0}, nn[3] = {0, 0, 0};
    std::vector<uint32_t> mx, my;
    uint64_t nkeys = 0;
};

// cover_points: a given domain is widened to hold every point too.
// The dense cell box with origin cell o and nn cells per axis: its column
// Morton tables and key count (the part of a plan that follows from the box).
inline int grid_plan_box(const int o[3], const int nn[3], GridPlan* out, std::string* err)
{
    GridPlan p;
    for (int k = 0; k < 3; ++k) { p.o[k] = o[k]; p.nn[k] = nn[k]; }
    if (p.nn[0] > 2048 || p.nn[1] > 2048 || p.nn[2] > 1024 || p.nn[0] < 1 || p.nn[1] < 1 || p.nn[2] < 1) {
        *err = "grid box too large for the cell packing (max 2048 x 2048 x 1024 cells)";
        return SPH_ERR_CAPACITY;
    }
    int bx = 0, by = 0;
    while ((1 << bx) < p.nn[0]) ++bx;
    while ((1 << by) < p.nn[1]) ++by;
    p.mx.assign(p.nn[0], 0u);
    p.my.assign(p.nn[1], 0u);
    // interleave bit k of x and y (x first) while both have bits left
    int pos = 0;
    std::vector<int> px(bx), py(by);
    for (int k = 0; k < std::max(bx, by); ++k) {
        if (k < bx) px[k] = pos++;
        if (k < by) py[k] = pos++;
    }
    for (int v = 0; v < p.nn[0]; ++v) {
        uint32_t m = 0;
        for (int k = 0; k < bx; ++k) if (v >> k & 1) m |= 1u << px[k];
        p.mx[v] = m;
    }
    for (int v = 0; v < p.nn[1]; ++v) {
        uint32_t m = 0;
        for (int k = 0; k < by; ++k) if (v >> k & 1) m |= 1u << py[k];
        p.my[v] = m;
    }
    p.nkeys = (1ull << (bx + by)) * (uint64_t)p.nn[2];
    if (p.nkeys > (1ull << 30)) { *err = "grid key space too large"; return SPH_ERR_CAPACITY; }
    *out = std::move(p);
    return SPH_OK;
}

// A set of points, xyz per point (n doubles).
struct PointSpan {
    const double* p;
    size_t n;
    PointSpan(const double* ptr, size_t count) : p(ptr), n(count) {}
    PointSpan(const std::vector<double>& v) : p(v.data()), n(v.size()) {}
    size_t size() const { return n; }
    double operator[](size_t i) const { return p[i]; }
};

// known_box (lo xyz, hi xyz): the points' bounding box, already formed (by
// the same rule: points with a non-finite coordinate left out); the point
// spans are then not read.
inline int grid_plan(const sph_scene_desc& d, PointSpan hx, PointSpan hb, bool akinci, PointSpan he, double h,
                     GridPlan* out, std::string* err, double rel_margin = 0.05, bool cover_points = false,
                     const double* known_box = nullptr)
{
    double lo[3], hi[3];
    bool given = false;
    for (int k = 0; k < 3; ++k) given |= d.domain_max[k] > d.domain_min[k];
    // non-finite points (a corrupted input) do not shape the box: the upload
    // keeps them in a border cell and the solver's reductions flag them
    auto acc = [&](const PointSpan& v) {
        for (size_t i = 0; i + 2 < v.size(); i += 3) {
            if (!std::isfinite(v[i]) || !std::isfinite(v[i + 1]) || !std::isfinite(v[i + 2])) continue;
            for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], v[i + k]); hi[k] = std::max(hi[k], v[i + k]); }
        }
    };
    if (given) {
        for (int k = 0; k < 3; ++k) { lo[k] = d.domain_min[k]; hi[k] = d.domain_max[k]; }
        if (cover_points) {
            acc(hx);
            acc(he);
            if (akinci) acc(hb);
        }
    } else {
        for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
        if (known_box) {
            for (int k = 0; k < 3; ++k) { lo[k] = known_box[k]; hi[k] = known_box[3 + k]; }
        } else {
            acc(hx);
            acc(he);
            if (akinci) acc(hb);
        }
        if (d.boundary_method == SPH_BOUNDARY_CUBE && d.has_cube)
            for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], d.cube_min[k]); hi[k] = std::max(hi[k], d.cube_max[k]); }
        for (int k = 0; k < 3; ++k) {
            const double ext = hi[k] - lo[k];
            lo[k] -= rel_margin * ext;
            hi[k] += rel_margin * ext;
        }
    }
    if (!(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2])) {
        *err = "no point with finite coordinates to place the grid box";
        return SPH_ERR_INVALID;
    }
    int o[3], nn[3];
    for (int k = 0; k < 3; ++k) {
        o[k] = (int)std::floor(lo[k] / h) - 2;
        nn[k] = (int)std::floor(hi[k] / h) + 3 - o[k];
    }
    return grid_plan_box(o, nn, out, err);
}

template <typename T> struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t count)
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = count;
        return cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T));
    }
};

template <typename R> class Scene : public SceneBase {
public:
    explicit Scene(const sph_scene_desc& desc) { d = desc; }
    ~Scene() override
    {
        for (int k = 0; k < 2; ++k)
            if (gexec_[k]) cudaGraphExecDestroy(gexec_[k]);
        if (st_) cudaStreamDestroy(st_);
        if (st2_) cudaStreamDestroy(st2_);
        if (h_sc_) cudaFreeHost(h_sc_);
        if (h_esc_) cudaFreeHost(h_esc_);
        if (esc_ev_) cudaEventDestroy(esc_ev_);
        for (auto& p : pending_) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
        for (auto e : events_) cudaEventDestroy(e);
        for (auto e : tev_) if (e) cudaEventDestroy(e);
    }

    unsigned nfluid() const override { return inited ? active() : (unsigned)(hx.size() / 3); }
    unsigned nboundary() const override { return inited ? nb_ : (unsigned)(hb.size() / 3); }

    // ------------------------------------------------------------------
    int init() override
    {
        if (inited) { fail("scene already initialised"); return SPH_ERR_INVALID; }
        int G = d.threads_per_particle;
        if (G == 0) {
            // by default enough lanes for ~160k walking threads: a small
            // scene's walks run out of warps to hide their load latency with
            // one lane per particle (8,000 WCSPH particles: 2.4x faster at 8)
            const unsigned long long n = std::max<unsigned long long>(hx.size() / 3, 1ull);
            const unsigned long long want = (160000ull + n - 1) / n;
            G = want >= 8 ? 8 : want >= 4 ? 4 : want >= 2 ? 2 : 1;
            // PCISPH / WCSPH from 40k particles: one lane over candidate lists
            // beats lanes splitting the cell walks (81k PCISPH drop: 0.45 vs
            // 0.64 ms/step)
            if ((d.simulation_method == SPH_PCISPH || d.simulation_method == SPH_WCSPH) && d.neighbor_list_max > 0 &&
                d.boundary_method != SPH_BOUNDARY_PCISPH && n >= 40000ull)
                G = 1;
        }
        G_ = (G == 2 || G == 4 || G == 8) ? G : 1;
        SPH_CUDA(cudaGetDevice(&device_));
        SPH_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        SPH_CUDA(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
        ls_ = st_;
        SPH_CUDA(cudaMallocHost((void**)&h_sc_, sizeof(DevScalars)));
        SPH_CUDA(cudaMallocHost((void**)&h_esc_, sizeof(unsigned)));
        *h_esc_ = 0u;
        SPH_CUDA(cudaEventCreateWithFlags(&esc_ev_, cudaEventDisableTiming));
        n0_ = (unsigned)(hx.size() / 3);
        akinci_ = d.boundary_method == SPH_BOUNDARY_AKINCI ? 1 : 0;
        bh_ = d.boundary_method == SPH_BOUNDARY_PCISPH ? 1 : 0;
        hasb_ = akinci_ || bh_;
        if (bh_) grow_ = false;  // cell lifetimes are tied to the key space
        nb_ = hasb_ ? (unsigned)(hb.size() / 3) : 0u;
        // FluidModel::addEmitter FluidModel.cpp:124-143: every emitter's
        // particles get slots up front; emission only activates them
        nem_ = (int)hem.size();
        {
            unsigned long long cap = n0_;
            for (const EmitterSpec& e : hem) cap += e.num;
            if (cap > (1ull << 31)) { fail("fluid plus emitter particles exceed 2^31"); return SPH_ERR_CAPACITY; }
            n_ = (unsigned)cap;
        }
        if (n_ == 0) { fail("no fluid particles"); return SPH_ERR_INVALID; }
        if (bh_ && hbn.size() != hb.size()) {
            fail("the PCISPH boundary model needs a normal per boundary point (sph_ctx_add_pcisph_box / _sphere)");
            return SPH_ERR_INVALID;
        }
        setup_constants();
        int rc = setup_grid();
        if (rc) return rc;
        rc = allocate();
        if (rc) return rc;
        // scalars
        DevScalars s{};
        s.dt = d.time_step;
        s.scaling = pcisph_scaling();
        s.n_active = n0_;
        SPH_CUDA(cudaMemcpyAsync(sc_.p, &s, sizeof s, cudaMemcpyHostToDevice, st_));
        // fluid upload
        {
            DevBuf<double> tx, tv;
            SPH_CUDA(tx.alloc(hx.size()));
            SPH_CUDA(tv.alloc(hx.size()));
            if (hv.size() != hx.size()) hv.assign(hx.size(), 0.0);
            if (n0_) {
                SPH_CUDA(cudaMemcpyAsync(tx.p, hx.data(), hx.size() * 8, cudaMemcpyHostToDevice, st_));
                SPH_CUDA(cudaMemcpyAsync(tv.p, hv.data(), hv.size() * 8, cudaMemcpyHostToDevice, st_));
                k_upload_fluid<R><<<blocks(n0_, 256), 256, 0, st_>>>(tx.p, tv.p, n0_, 0, F(), gv_, hd_, sc_.p);
                SPH_CUDA(cudaGetLastError());
            }
            rc = upload_emitters();
            if (rc) return rc;
            SPH_CUDA(cudaStreamSynchronize(st_));
        }
        // boundary upload, sort, volumes (SPHSolver::init SPHSolver.cpp:22-39)
        if (nb_) {
            DevBuf<double> tb;
            SPH_CUDA(tb.alloc(hb.size()));
            SPH_CUDA(cudaMemcpyAsync(tb.p, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st_));
            k_upload_boundary<R><<<blocks(nb_, 256), 256, 0, st_>>>(tb.p, nb_, B(0), gv_, hd_, sc_.p);
            SPH_CUDA(cudaGetLastError());
            DevBuf<double> tn;
            if (bh_) {
                // PCISPH boundary model: normals, and the model's mass (the fluid's,
                // Simulation.cpp:464-468) as the walks' boundary weight
                SPH_CUDA(tn.alloc(hbn.size()));
                SPH_CUDA(cudaMemcpyAsync(tn.p, hbn.data(), hbn.size() * 8, cudaMemcpyHostToDevice, st_));
                k_bh_upload<R><<<blocks(nb_, 256), 256, 0, st_>>>(tn.p, nb_, B(0), c_.mass);
                SPH_CUDA(cudaGetLastError());
            }
            k_cell_count<<<blocks(nb_, 256), 256, 0, st_>>>(nb_, B(0).cell, key_.p, slot_.p, count_.p, gv_);
            if (bh_) k_bh_mark_cells<<<blocks(nb_, 256), 256, 0, st_>>>(nb_, key_.p, cell_epoch_.p);
            rc = scan(bstarts_.p);
            if (rc) return rc;
            k_scatter<<<blocks(nb_, 256), 256, 0, st_>>>(nb_, key_.p, slot_.p, bstarts_.p, tmp_.p);
            k_gather_boundary<R><<<blocks(nb_, 256), 256, 0, st_>>>(nb_, tmp_.p, key_.p, bstarts_.p, B(0), B(1));
            SPH_CUDA(cudaGetLastError());
            if (akinci_) k_boundary_psi<R><<<blocks(nb_, 128), 128, 0, st_>>>(B(1), gv_, bstarts_.p, c_);
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaStreamSynchronize(st_));
        } else {
            SPH_CUDA(cudaMemsetAsync(bstarts_.p, 0, (nkeys_ + 1) * sizeof(uint32_t), st_));
        }
        rc = build_grid(false);
        if (rc) return rc;
        if (d.simulation_method == SPH_DFSPH) {
            // DFSPHSolver::init DFSPHSolver.cpp:24-36
            rc = lists_ ? launch_build_lists() : launch_density(true, false);
            if (rc) return rc;
            launch_bh_boundary(0);
        }
        SPH_CUDA(cudaStreamSynchronize(st_));
        inited = true;
        return SPH_OK;
    }

    int step(int nsteps) override
    {
        if (!inited) { fail("sph_ctx_init has not been called"); return SPH_ERR_INVALID; }
        for (int s = 0; s < nsteps; ++s) {
            int rc;
            if (grow_ && esc_pending_ && cudaEventQuery(esc_ev_) == cudaSuccess) {
                esc_pending_ = false;
                if (*h_esc_) {
                    rc = grow_grid();
                    if (rc) return rc;
                }
            }
            {
                Phase ph(phases_, "Step computation", ls_, false, prof_);
                rc = graph_ ? graph_step() : one_step();
            }
            if (rc) return rc;
            // every kGrowthCheck steps, read the escape flag without waiting
            if (grow_ && !esc_pending_ && ++since_check_ >= kGrowthCheck) {
                since_check_ = 0;
                SPH_CUDA(cudaMemcpyAsync(h_esc_, &sc_.p->escaped, sizeof(unsigned), cudaMemcpyDeviceToHost, st_));
                SPH_CUDA(cudaEventRecord(esc_ev_, st_));
                esc_pending_ = true;
            }
        }
        return SPH_OK;
    }

    int set_grid_growth(int on) override
    {
        grow_ = on != 0 && !bh_;
        if (on && bh_) { fail("the grid box of the PCISPH boundary model does not grow"); return SPH_ERR_UNSUPPORTED; }
        return SPH_OK;
    }

    // The reference hashes cells without bounds (HashTable.h:79-102); the
    // dense box here grows instead.  Between steps: the box is re-planned
    // around every point (fluid where it is now, boundary, emitters) with a
    // 25 % margin on the same cell lattice, cells are shifted into it (a
    // particle kept in a border cell is re-binned from its true offset), the
    // static boundary is re-sorted and its volumes recomputed, the fluid is
    // re-sorted and the DFSPH densities, alpha factors and lists rebuilt at
    // the same positions (same values: sums run in the geometric walk order,
    // which the box does not change), and the step graphs are re-captured.
    // A box beyond the cell packing's limits stays as it is, and growth stops.
    int grow_grid()
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        const unsigned na = active();
        std::vector<double> xs(3 * (size_t)na);
        int rc = download(SPH_FIELD_POSITION, xs.data());
        if (rc) return rc;
        // a particle with non-finite coordinates (a scene that blew up) has no
        // place in any box: plan around the finite ones
        size_t keep = 0;
        for (size_t k = 0; k + 2 < xs.size(); k += 3)
            if (std::isfinite(xs[k]) && std::isfinite(xs[k + 1]) && std::isfinite(xs[k + 2])) {
                xs[keep] = xs[k]; xs[keep + 1] = xs[k + 1]; xs[keep + 2] = xs[k + 2];
                keep += 3;
            }
        xs.resize(keep);
        if (keep == 0) { grow_ = false; return SPH_OK; }
        sph_scene_desc dd = d;
        for (int k = 0; k < 3; ++k) dd.domain_min[k] = dd.domain_max[k] = 0.0;
        GridPlan p;
        std::string perr;
        if (grid_plan(dd, xs, hb, hasb_ != 0, emitter_points(), hd_, &p, &perr, 0.25) != SPH_OK) {
            grow_ = false;
            return SPH_OK;
        }
        const int sx = gv_.ox - p.o[0], sy = gv_.oy - p.o[1], sz = gv_.oz - p.o[2];
        // graph-run kernels so far, before the graphs go
        SPH_CUDA(cudaMemcpy(h_sc_, sc_.p, sizeof(DevScalars), cudaMemcpyDeviceToHost));
        if (graph_) graph_launches_ += graph_kernels();
        snap_it_ = h_sc_->sumIterations;
        snap_itv_ = h_sc_->sumIterationsV;
        for (int k = 0; k < 2; ++k) {
            if (gexec_[k]) cudaGraphExecDestroy(gexec_[k]);
            gexec_[k] = nullptr;
            gsteps_[k] = 0;
            for (int q = 0; q < 3; ++q) gshape_[k][q] = 0;
        }
        rc = use_grid(p);
        if (rc) return rc;
        SPH_CUDA(count_.alloc(nkeys_)); SPH_CUDA(starts_.alloc(nkeys_ + 1)); SPH_CUDA(bstarts_.alloc(nkeys_ + 1));
        SPH_CUDA(tile_sums_.alloc(blocks(nkeys_, kScanTile)));
        SPH_CUDA(cudaMemsetAsync(count_.p, 0, nkeys_ * sizeof(uint32_t), st_));
        Fluid<R> f = F();
        k_shift_cells<<<blocks(n_, 256), 256, 0, st_>>>(n_, f.na, f.cell, sx, sy, sz);
        k_cell_update<R, false, false><<<blocks(n_, 256), 256, 0, st_>>>(n_, f.pos, f.vel, f.cell, key_.p, slot_.p, count_.p,
                                                                         gv_, c_.h, hd_, sc_.p, nullptr, nullptr, f.na);
        SPH_CUDA(cudaGetLastError());
        if (nb_) {
            // boundary points kept in border cells (outside a given domain)
            // are re-binned too; the weights in w are rewritten with psi below
            k_shift_cells<<<blocks(nb_, 256), 256, 0, st_>>>(nb_, nullptr, B(1).cell, sx, sy, sz);
            k_cell_update<R, false, false><<<blocks(nb_, 256), 256, 0, st_>>>(nb_, B(1).pos, B(1).pos, B(1).cell, key_.p,
                                                                              slot_.p, count_.p, gv_, c_.h, hd_, sc_.p);
            k_cell_count<<<blocks(nb_, 256), 256, 0, st_>>>(nb_, B(1).cell, key_.p, slot_.p, count_.p, gv_);
            SPH_CUDA(cudaGetLastError());
            rc = scan(bstarts_.p);
            if (rc) return rc;
            k_scatter<<<blocks(nb_, 256), 256, 0, st_>>>(nb_, key_.p, slot_.p, bstarts_.p, tmp_.p);
            k_gather_boundary<R><<<blocks(nb_, 256), 256, 0, st_>>>(nb_, tmp_.p, key_.p, bstarts_.p, B(1), B(0));
            std::swap(bd_[0], bd_[1]);
            if (akinci_) k_boundary_psi<R><<<blocks(nb_, 128), 128, 0, st_>>>(B(1), gv_, bstarts_.p, c_);
            SPH_CUDA(cudaGetLastError());
        } else {
            SPH_CUDA(cudaMemsetAsync(bstarts_.p, 0, (nkeys_ + 1) * sizeof(uint32_t), st_));
        }
        SPH_CUDA(cudaMemsetAsync(&sc_.p->escaped, 0, sizeof(unsigned), st_));
        rc = build_grid(false);
        if (rc) return rc;
        if (d.simulation_method == SPH_DFSPH) {
            rc = lists_ ? launch_build_lists() : launch_density(true, false);
            if (rc) return rc;
        }
        SPH_CUDA(cudaStreamSynchronize(st_));
        ++growths_;
        return SPH_OK;
    }

    // nsteps steps bracketed by CUDA events on the scene's stream; waits and
    // returns the elapsed device time.
    int step_timed(int nsteps, float* ms) override
    {
        if (!inited) { fail("sph_ctx_init has not been called"); return SPH_ERR_INVALID; }
        if (!tev_[0]) {
            SPH_CUDA(cudaEventCreate(&tev_[0]));
            SPH_CUDA(cudaEventCreate(&tev_[1]));
        }
        SPH_CUDA(cudaEventRecord(tev_[0], st_));
        const int rc = step(nsteps);
        if (rc) return rc;
        SPH_CUDA(cudaEventRecord(tev_[1], st_));
        SPH_CUDA(cudaEventSynchronize(tev_[1]));
        SPH_CUDA(cudaEventElapsedTime(ms, tev_[0], tev_[1]));
        return SPH_OK;
    }

    int sync() override
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    int set_graph(int on) override
    {
        const bool want = on != 0;
        if (want == graph_) return SPH_OK;
        if (inited) {
            SPH_CUDA(cudaMemcpyAsync(h_sc_, sc_.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, st_));
            SPH_CUDA(cudaStreamSynchronize(st_));
            if (want) {
                snap_it_ = h_sc_->sumIterations;
                snap_itv_ = h_sc_->sumIterationsV;
                gsteps_[0] = gsteps_[1] = 0;
            } else {
                graph_launches_ += graph_kernels();
            }
        }
        graph_ = want;
        return SPH_OK;
    }

    // Kernels run by graph steps since the last snapshot: per step the fixed
    // part of the captured graph, plus each loop body times the iterations it
    // ran (h_sc_ must be current).
    unsigned long long graph_kernels() const
    {
        unsigned long long k = 0;
        for (int q = 0; q < 2; ++q) k += gsteps_[q] * (unsigned long long)gshape_[q][0];
        const unsigned long long b1 = std::max(gshape_[0][1], gshape_[1][1]);
        const unsigned long long b2 = std::max(gshape_[0][2], gshape_[1][2]);
        k += b1 * (h_sc_->sumIterations - snap_it_) + b2 * (h_sc_->sumIterationsV - snap_itv_);
        return k;
    }

    int pause_emitters(int pause) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        if (!nem_) return SPH_OK;
        k_emit_pause<<<1, kMaxEmitters, 0, st_>>>(em_.p, nem_, pause ? 1u : 0u, sc_.p);
        SPH_CUDA(cudaGetLastError());
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    int launch_count(unsigned long long* out) override
    {
        if (!inited) { *out = 0; return SPH_OK; }
        SPH_CUDA(cudaMemcpyAsync(h_sc_, sc_.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        *out = launches_ + graph_launches_ + (graph_ ? graph_kernels() : 0ull);
        return SPH_OK;
    }

    int set_profiling(int on) override
    {
        prof_ = on != 0;
        return SPH_OK;
    }

    // Phase times (CUDA events, profiling on) since the last call.
    int phase_profile(char* buf, size_t len) override
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        const int n = phases_.report(buf, len);
        if (n < 0) { fail(cudaGetErrorString((cudaError_t)-n)); return SPH_ERR_CUDA; }
        return n;
    }
    // a named phase of the host-driven step (nothing while capturing)
    Phase phase(const char* name) { return Phase(phases_, name, ls_, capturing_, prof_); }

    // "name count total_ms" per kernel name, for the launches timed since the
    // last call (host-driven steps with profiling on).
    int profile(char* buf, size_t len) override
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        std::vector<std::string> names;
        std::vector<double> ms;
        std::vector<unsigned long long> cnt;
        for (auto& p : pending_) {
            float t = 0.f;
            SPH_CUDA(cudaEventElapsedTime(&t, p.a, p.b));
            size_t q = 0;
            while (q < names.size() && names[q] != p.name) ++q;
            if (q == names.size()) { names.push_back(p.name); ms.push_back(0.0); cnt.push_back(0); }
            ms[q] += t;
            cnt[q] += 1;
            events_.push_back(p.a);
            events_.push_back(p.b);
        }
        pending_.clear();
        std::string outs;
        char line[256];
        for (size_t q = 0; q < names.size(); ++q) {
            std::snprintf(line, sizeof line, "%s %llu %.6f\n", names[q].c_str(), cnt[q], ms[q]);
            outs += line;
        }
        if (buf && len) {
            std::strncpy(buf, outs.c_str(), len - 1);
            buf[len - 1] = 0;
        }
        return (int)outs.size();
    }

    int download(int field, double* out) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        const bool bnd = field == SPH_FIELD_BOUNDARY_POSITION || field == SPH_FIELD_BOUNDARY_VOLUME ||
                         field == SPH_FIELD_BOUNDARY_DENSITY || field == SPH_FIELD_BOUNDARY_PRESSURE;
        if ((field == SPH_FIELD_BOUNDARY_DENSITY || field == SPH_FIELD_BOUNDARY_PRESSURE) && !bh_) {
            fail("boundary densities and pressures exist for the PCISPH boundary model only");
            return SPH_ERR_INVALID;
        }
        if ((field == SPH_FIELD_PRESSURE_ACC && pacc_.n < n_) || (field == SPH_FIELD_NORMAL && normal_.n < n_)) {
            fail("this solver configuration keeps no such field");
            return SPH_ERR_INVALID;
        }
        const unsigned n = bnd ? nb_ : active();
        const bool vec = field == SPH_FIELD_POSITION || field == SPH_FIELD_VELOCITY || field == SPH_FIELD_ACCELERATION ||
                         field == SPH_FIELD_PRESSURE_ACC || field == SPH_FIELD_NORMAL ||
                         field == SPH_FIELD_BOUNDARY_POSITION;
        const size_t count = (size_t)n * (vec ? 3 : 1);
        if (count == 0) return SPH_OK;
        DevBuf<double> o;
        SPH_CUDA(o.alloc(count));
        Fluid<R> f = F();
        Boundary<R> b = B(1);
        const P4<R>* v4 = nullptr;
        const R* s = nullptr;
        int kind = 0;
        switch (field) {
            case SPH_FIELD_POSITION: v4 = f.pos; kind = 1; break;
            case SPH_FIELD_VELOCITY: v4 = f.vel; break;
            case SPH_FIELD_ACCELERATION: v4 = f.acc; break;
            case SPH_FIELD_PRESSURE_ACC: v4 = f.pacc; break;
            case SPH_FIELD_NORMAL: v4 = f.normal; break;
            case SPH_FIELD_DENSITY: s = f.rho; kind = 2; break;
            case SPH_FIELD_PRESSURE: s = f.press; kind = 2; break;
            case SPH_FIELD_ALPHA: s = f.alpha; kind = 2; break;
            case SPH_FIELD_PRED_DENSITY: s = f.pred; kind = 2; break;
            case SPH_FIELD_DIV_ERROR: s = f.div; kind = 2; break;
            case SPH_FIELD_KAPPA: s = f.kappa; kind = 2; break;
            case SPH_FIELD_KAPPA_V: s = f.kappav; kind = 2; break;
            case SPH_FIELD_BOUNDARY_POSITION: v4 = b.pos; kind = 1; break;
            case SPH_FIELD_BOUNDARY_VOLUME: s = b.psi; kind = 2; break;
            case SPH_FIELD_BOUNDARY_DENSITY: s = b.dens; kind = 2; break;
            case SPH_FIELD_BOUNDARY_PRESSURE: s = b.press; kind = 2; break;
            default: fail("unknown field"); return SPH_ERR_INVALID;
        }
        k_download<R><<<blocks(n, 256), 256, 0, st_>>>(n, v4, s, bnd ? b.id : f.id, bnd ? b.cell : f.cell, gv_, hd_, kind,
                                                      o.p);
        SPH_CUDA(cudaGetLastError());
        SPH_CUDA(cudaMemcpyAsync(out, o.p, count * 8, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    int capture_async(double* hx, double* hv, cudaEvent_t done, unsigned* count_out) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        const unsigned n = active();
        *count_out = n;
        if (cap_x_.n < 3 * (size_t)n_) {
            SPH_CUDA(cap_x_.alloc(3 * (size_t)n_));
            SPH_CUDA(cap_v_.alloc(3 * (size_t)n_));
        }
        if (n) {
            Fluid<R> f = F();
            k_download<R><<<blocks(n, 256), 256, 0, st_>>>(n, f.pos, nullptr, f.id, f.cell, gv_, hd_, 1, cap_x_.p);
            k_download<R><<<blocks(n, 256), 256, 0, st_>>>(n, f.vel, nullptr, f.id, f.cell, gv_, hd_, 0, cap_v_.p);
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaMemcpyAsync(hx, cap_x_.p, 3 * (size_t)n * 8, cudaMemcpyDeviceToHost, st_));
            SPH_CUDA(cudaMemcpyAsync(hv, cap_v_.p, 3 * (size_t)n * 8, cudaMemcpyDeviceToHost, st_));
        }
        SPH_CUDA(cudaEventRecord(done, st_));
        return SPH_OK;
    }

    int field_view(int field, FieldView* v) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        const bool bnd = field == SPH_FIELD_BOUNDARY_POSITION || field == SPH_FIELD_BOUNDARY_VOLUME ||
                         field == SPH_FIELD_BOUNDARY_DENSITY || field == SPH_FIELD_BOUNDARY_PRESSURE;
        if ((field == SPH_FIELD_BOUNDARY_DENSITY || field == SPH_FIELD_BOUNDARY_PRESSURE) && !bh_) {
            fail("boundary densities and pressures exist for the PCISPH boundary model only");
            return SPH_ERR_INVALID;
        }
        if ((field == SPH_FIELD_PRESSURE_ACC && pacc_.n < n_) || (field == SPH_FIELD_NORMAL && normal_.n < n_)) {
            fail("this solver configuration keeps no such field");
            return SPH_ERR_INVALID;
        }
        Fluid<R> f = F();
        Boundary<R> b = B(1);
        FieldView o;
        o.n = bnd ? nb_ : active();
        o.id = bnd ? b.id : f.id;
        o.cell = bnd ? b.cell : f.cell;
        switch (field) {
            case SPH_FIELD_POSITION: o.v4 = f.pos; o.kind = 1; break;
            case SPH_FIELD_VELOCITY: o.v4 = f.vel; break;
            case SPH_FIELD_ACCELERATION: o.v4 = f.acc; break;
            case SPH_FIELD_PRESSURE_ACC: o.v4 = f.pacc; break;
            case SPH_FIELD_NORMAL: o.v4 = f.normal; break;
            case SPH_FIELD_DENSITY: o.s = f.rho; o.kind = 2; break;
            case SPH_FIELD_PRESSURE: o.s = f.press; o.kind = 2; break;
            case SPH_FIELD_ALPHA: o.s = f.alpha; o.kind = 2; break;
            case SPH_FIELD_PRED_DENSITY: o.s = f.pred; o.kind = 2; break;
            case SPH_FIELD_DIV_ERROR: o.s = f.div; o.kind = 2; break;
            case SPH_FIELD_KAPPA: o.s = f.kappa; o.kind = 2; break;
            case SPH_FIELD_KAPPA_V: o.s = f.kappav; o.kind = 2; break;
            case SPH_FIELD_BOUNDARY_POSITION: o.v4 = b.pos; o.kind = 1; break;
            case SPH_FIELD_BOUNDARY_VOLUME: o.s = b.psi; o.kind = 2; break;
            case SPH_FIELD_BOUNDARY_DENSITY: o.s = b.dens; o.kind = 2; break;
            case SPH_FIELD_BOUNDARY_PRESSURE: o.s = b.press; o.kind = 2; break;
            default: fail("unknown field"); return SPH_ERR_INVALID;
        }
        o.count = (size_t)o.n * (o.kind == 2 ? 1 : 3);
        o.nx = gv_.nx; o.ny = gv_.ny; o.nz = gv_.nz; o.ox = gv_.ox; o.oy = gv_.oy; o.oz = gv_.oz;
        o.h = hd_;
        o.fp64 = sizeof(R) == 8;
        o.device = device_;
        o.stream = st_;
        *v = o;
        return SPH_OK;
    }

    int stats(sph_stats* out) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        unsigned long long ls[2] = {0, 0};
        if (lists_) {
            SPH_CUDA(cudaMemsetAsync(lstat_.p, 0, 2 * sizeof(unsigned long long), st_));
            const unsigned na = active();
            k_list_stats<<<blocks(na, 256), 256, 0, st_>>>(na, lcount_.p, kmax_, lstat_.p);
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaMemcpyAsync(ls, lstat_.p, sizeof ls, cudaMemcpyDeviceToHost, st_));
        }
        SPH_CUDA(cudaMemcpyAsync(h_sc_, sc_.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        const DevScalars& s = *h_sc_;
        std::memset(out, 0, sizeof *out);
        out->list_pairs = ls[0];
        out->list_overflow = (unsigned)ls[1];
        out->time = s.time;
        out->dt = s.dt;
        out->avg_density_error = s.avgDensError;
        out->avg_divergence_error = s.avgDivError;
        out->max_density_error = s.maxDensityError;
        out->max_velocity = s.maxVel;
        out->iterations = s.iterations;
        out->iterations_v = s.iterationsV;
        out->steps = s.steps;
        out->status = s.status;
        out->sum_iterations = s.sumIterations;
        out->sum_iterations_v = s.sumIterationsV;
        out->num_fluid = nem_ ? s.n_active : n_;
        out->num_fluid_total = n_;
        out->num_boundary = nb_;
        out->grid_growths = growths_;
        return SPH_OK;
    }

    int neighbors(int* cells, int* rank, int* off, int* nbr, int* boff, int* bnbr, long long* totals) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        const unsigned na = active();
        DevBuf<int> cnt, bcnt, dcells, drank;
        SPH_CUDA(cnt.alloc(na));
        SPH_CUDA(bcnt.alloc(na));
        SPH_CUDA(dcells.alloc(3 * (size_t)na));
        SPH_CUDA(drank.alloc(na));
        Fluid<R> f = F();
        Boundary<R> b = B(1);
        k_neighbors<R><<<blocks(n_, 128), 128, 0, st_>>>(f, b.pos, b.id, b.cell, gv_, starts_.p, bstarts_.p, c_, hd_, nullptr,
                                                         nullptr, cnt.p, bcnt.p, nullptr, nullptr, dcells.p, drank.p);
        SPH_CUDA(cudaGetLastError());
        std::vector<int> hc(na), hbc(na);
        SPH_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, na * 4, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaMemcpyAsync(hbc.data(), bcnt.p, na * 4, cudaMemcpyDeviceToHost, st_));
        if (cells) SPH_CUDA(cudaMemcpyAsync(cells, dcells.p, 3 * (size_t)na * 4, cudaMemcpyDeviceToHost, st_));
        if (rank) SPH_CUDA(cudaMemcpyAsync(rank, drank.p, (size_t)na * 4, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        std::vector<int> ho(na + 1), hbo(na + 1);
        long long a = 0, bt = 0;
        for (unsigned i = 0; i < na; ++i) {
            ho[i] = (int)a; hbo[i] = (int)bt;
            a += hc[i]; bt += hbc[i];
        }
        ho[na] = (int)a; hbo[na] = (int)bt;
        if (totals) { totals[0] = a; totals[1] = bt; }
        if (off) std::memcpy(off, ho.data(), (na + 1) * 4);
        if (boff) std::memcpy(boff, hbo.data(), (na + 1) * 4);
        if (nbr || bnbr) {
            DevBuf<int> doff, dboff, dn, dbn;
            SPH_CUDA(doff.alloc(na + 1));
            SPH_CUDA(dboff.alloc(na + 1));
            SPH_CUDA(dn.alloc((size_t)std::max<long long>(a, 1)));
            SPH_CUDA(dbn.alloc((size_t)std::max<long long>(bt, 1)));
            SPH_CUDA(cudaMemcpyAsync(doff.p, ho.data(), (na + 1) * 4, cudaMemcpyHostToDevice, st_));
            SPH_CUDA(cudaMemcpyAsync(dboff.p, hbo.data(), (na + 1) * 4, cudaMemcpyHostToDevice, st_));
            k_neighbors<R><<<blocks(n_, 128), 128, 0, st_>>>(f, b.pos, b.id, b.cell, gv_, starts_.p, bstarts_.p, c_, hd_,
                                                             doff.p, dboff.p, nullptr, nullptr, dn.p, dbn.p, nullptr,
                                                             nullptr);
            SPH_CUDA(cudaGetLastError());
            if (nbr && a) SPH_CUDA(cudaMemcpyAsync(nbr, dn.p, a * 4, cudaMemcpyDeviceToHost, st_));
            if (bnbr && bt) SPH_CUDA(cudaMemcpyAsync(bnbr, dbn.p, bt * 4, cudaMemcpyDeviceToHost, st_));
            SPH_CUDA(cudaStreamSynchronize(st_));
        }
        return SPH_OK;
    }

    // The DFSPH pair lists as the last grid build stored them (original
    // order; see sph_ctx_pair_lists).
    int pair_lists(int* count, int* off, int* nbr, long long* total) override
    {
        if (!inited) { fail("not initialised"); return SPH_ERR_INVALID; }
        if (!lists_) { fail("the scene keeps no pair lists (DFSPH with neighbor_list_max > 0 only)"); return SPH_ERR_UNSUPPORTED; }
        const unsigned na = active();
        const Fluid<R> f = F();
        const Lists<R> L = LS();
        const uint32_t stride = n_;
        const cudaError_t e = dump_pair_lists(
            na, kmax_, st_,
            [&](const int* doff, int* dcnt, int* dn) {
                k_pair_lists<R><<<blocks(na, 256), 256, 0, st_>>>(na, 0u, stride, f.id, L, doff, dcnt, dn);
            },
            count, off, nbr, total);
        SPH_CUDA(e);
        return SPH_OK;
    }

private:
    // ------------------------------------------------------------------
    static unsigned blocks(size_t n, unsigned b) { return (unsigned)std::max<size_t>(1, (n + b - 1) / b); }

    Fluid<R> F() const { return fl_[cur_]; }
    Lists<R> LS() const
    {
        return Lists<R>{pairs_.p, lcount_.p, bgrad_.p, kbuf_.p, kmax_, posh_.p, &sc_.p->status, nullptr, nullptr};
    }
    Boundary<R> B(int k) const { return bd_[k]; }

    // Kernel coefficients, evaluated in double as each reference kernel's
    // setSupportRadius does (CubicSpline.h:18-26, Poly6.h:19-28,
    // Spiky.h:18-27, ViscoK.h:18-26, Cohesion.h:20-27), and the particle
    // mass of Simulation::initMasses (Simulation.cpp:134-146).
    void setup_constants()
    {
        scene_constants<R>(d, &c_, &lim_, &hd_, &mass_);
    }

    // PCISPHSolver::computeScalingFactor PCISPHSolver.cpp:389-421 (Poly6
    // gradient on a 3x3x3 lattice prototype at spacing 2r, init-time dt).
    double pcisph_scaling() const
    {
        const double sr = hd_;
        const double h9 = sr * sr * sr * sr * sr * sr * sr * sr * sr;
        const double gradCoef = 945.0 / (32.0 * M_PI * h9);
        const double h2 = sr * sr;
        const double dist = 2.0 * d.particle_radius;
        double sg[3] = {0, 0, 0}, sumSqGrad = 0;
        for (int i = -1; i <= 1; i++)
            for (int j = -1; j <= 1; j++)
                for (int k = -1; k <= 1; k++) {
                    double r[3] = {(double)-i * dist, (double)-j * dist, (double)-k * dist};
                    const double mod_r = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                    const double mod_r2 = mod_r * mod_r;
                    double gr[3] = {0, 0, 0};
                    if (mod_r2 <= h2) {
                        const double diff = h2 - mod_r2;
                        const double s = -diff * diff * gradCoef;
                        gr[0] = s * r[0]; gr[1] = s * r[1]; gr[2] = s * r[2];
                    }
                    sg[0] += gr[0]; sg[1] += gr[1]; sg[2] += gr[2];
                    sumSqGrad += gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2];
                }
        const double beta = 2 * std::pow(mass_ * d.time_step / d.density0, 2);
        const double dotSumGrad = sg[0] * sg[0] + sg[1] * sg[1] + sg[2] * sg[2];
        return -1.0 / (beta * (-dotSumGrad - sumSqGrad));
    }

    // Dense cell box over the domain with a margin; column-Morton key space.
    // The emitters' groups where they are placed (rotated, translated).
    std::vector<double> emitter_points() const
    {
        std::vector<double> he;
        for (const EmitterSpec& e : hem)
            for (size_t k = 0; k + 2 < e.group.size(); k += 3) {
                const double v[3] = {e.group[k], e.group[k + 1], e.group[k + 2]};
                const double* q = e.q;
                const double uv[3] = {q[2] * v[2] - v[1] * q[3], q[3] * v[0] - v[2] * q[1], q[1] * v[1] - v[0] * q[2]};
                const double uuv[3] = {q[2] * uv[2] - uv[1] * q[3], q[3] * uv[0] - uv[2] * q[1], q[1] * uv[1] - uv[0] * q[2]};
                for (int c = 0; c < 3; ++c) he.push_back(v[c] + (uv[c] * q[0] + uuv[c]) * 2.0 + e.r[c]);
            }
        return he;
    }

    int setup_grid()
    {
        GridPlan p;
        // a box that grows starts around every point (a given domain widened)
        const int rc = grid_plan(d, hx, hb, hasb_ != 0, emitter_points(), hd_, &p, &err, 0.05, grow_);
        if (rc) return rc;
        return use_grid(p);
    }

    // Installs a planned box: key count, Morton tables, the grid view.
    int use_grid(const GridPlan& p)
    {
        nkeys_ = (uint32_t)p.nkeys;
        SPH_CUDA(mortx_.alloc(p.nn[0]));
        SPH_CUDA(morty_.alloc(p.nn[1]));
        SPH_CUDA(cudaMemcpy(mortx_.p, p.mx.data(), p.nn[0] * 4, cudaMemcpyHostToDevice));
        SPH_CUDA(cudaMemcpy(morty_.p, p.my.data(), p.nn[1] * 4, cudaMemcpyHostToDevice));
        gv_.nx = p.nn[0]; gv_.ny = p.nn[1]; gv_.nz = p.nn[2];
        gv_.ox = p.o[0]; gv_.oy = p.o[1]; gv_.oz = p.o[2];
        gv_.mortx = mortx_.p;
        gv_.morty = morty_.p;
        return SPH_OK;
    }

    int allocate()
    {
        const size_t n = n_, nb = std::max(nb_, 1u);
        for (int k = 0; k < 2; ++k) {
            SPH_CUDA(pos_[k].alloc(n)); SPH_CUDA(vel_[k].alloc(n)); SPH_CUDA(kappa_[k].alloc(n));
            SPH_CUDA(kappav_[k].alloc(n)); SPH_CUDA(cell_[k].alloc(n)); SPH_CUDA(id_[k].alloc(n));
            SPH_CUDA(pred_[k].alloc(n));
            SPH_CUDA(cudaMemsetAsync(pred_[k].p, 0, n * sizeof(R), st_));
            SPH_CUDA(bpos_[k].alloc(nb)); SPH_CUDA(bcell_[k].alloc(nb)); SPH_CUDA(bid_[k].alloc(nb));
        }
        SPH_CUDA(bpsi_.alloc(nb));
        SPH_CUDA(acc_.alloc(n)); SPH_CUDA(xk_.alloc(n)); SPH_CUDA(rho_.alloc(n)); SPH_CUDA(alpha_.alloc(n));
        SPH_CUDA(div_.alloc(n)); SPH_CUDA(press_.alloc(n));
        const bool pci = d.simulation_method == SPH_PCISPH;
        const bool st = (c_.force_flags & F_SURFACE_TENSION) != 0;
        SPH_CUDA(predR_.alloc(pci ? n : 1)); SPH_CUDA(predV_.alloc(pci ? n : 1)); SPH_CUDA(pacc_.alloc(pci ? n : 1));
        const bool bh = d.boundary_method == SPH_BOUNDARY_PCISPH;
        SPH_CUDA(normal_.alloc(st || bh ? n : 1));
        SPH_CUDA(normal2_.alloc(bh ? n : 1));
        for (int k = 0; k < 2; ++k) SPH_CUDA(bnrm_[k].alloc(bh ? nb : 1));
        SPH_CUDA(bdens_.alloc(bh ? nb : 1)); SPH_CUDA(bpress_.alloc(bh ? nb : 1)); SPH_CUDA(bdp_.alloc(bh ? nb : 1));
        SPH_CUDA(cell_epoch_.alloc(bh ? nkeys_ : 1));
        SPH_CUDA(cudaMemsetAsync(cell_epoch_.p, 0xFF, cell_epoch_.n * sizeof(uint32_t), st_));  // no cell exists yet
        if (bh) {
            SPH_CUDA(cudaMemsetAsync(bdens_.p, 0, nb * sizeof(R), st_));
            SPH_CUDA(cudaMemsetAsync(bpress_.p, 0, nb * sizeof(R), st_));
            SPH_CUDA(cudaMemsetAsync(bdp_.p, 0, nb * sizeof(R), st_));
        }
        lists_ = d.simulation_method == SPH_DFSPH && d.neighbor_list_max > 0;
        kmax_ = lists_ ? (uint32_t)d.neighbor_list_max : 0u;
        // PCISPH / WCSPH candidate lists: one lane per particle, Akinci or no
        // boundary (the PCISPH boundary model moves predicted positions after
        // the prediction), indices below 2^27
        cands_ = (d.simulation_method == SPH_PCISPH || d.simulation_method == SPH_WCSPH) && d.neighbor_list_max > 0 &&
                 G_ == 1 && !bh_ && n < (size_t)kCandIdxMask;
        if (cands_) {
            ckmax_ = (uint32_t)d.neighbor_list_max;
            SPH_CUDA(cand_.alloc((size_t)ckmax_ * n));
            SPH_CUDA(candn_.alloc(n));
            SPH_CUDA(cudaMemsetAsync(candn_.p, 0, n * sizeof(uint32_t), st_));
        }
        SPH_CUDA(pairs_.alloc(lists_ ? (size_t)kmax_ * n : 1));
        SPH_CUDA(lcount_.alloc(lists_ ? n : 1));
        SPH_CUDA(bgrad_.alloc(lists_ ? n : 1));
        SPH_CUDA(kbuf_.alloc(n));
        // FP32 pair lists: half-precision positions for the build's cull
        // (particle pairs, the last one whole); written by every gather
        if (lists_ && sizeof(R) == 4) {
            SPH_CUDA(posh_.alloc(n / 2 + 2));  // a spare word past the last pair for the cull
            SPH_CUDA(cudaMemsetAsync(posh_.p, 0, (n / 2 + 2) * sizeof(uint4), st_));
        }
        SPH_CUDA(cudaMemsetAsync(lcount_.p, 0, lcount_.n * sizeof(uint32_t), st_));
        SPH_CUDA(cudaMemsetAsync(kbuf_.p, 0, n * sizeof(R), st_));
        SPH_CUDA(lstat_.alloc(2));
        const size_t nmax = std::max(n, nb);
        SPH_CUDA(key_.alloc(nmax)); SPH_CUDA(slot_.alloc(nmax)); SPH_CUDA(tmp_.alloc(nmax));
        SPH_CUDA(count_.alloc(nkeys_)); SPH_CUDA(starts_.alloc(nkeys_ + 1)); SPH_CUDA(bstarts_.alloc(nkeys_ + 1));
        SPH_CUDA(tile_sums_.alloc(blocks(nkeys_, kScanTile)));
        SPH_CUDA(cudaMemsetAsync(count_.p, 0, nkeys_ * sizeof(uint32_t), st_));
        SPH_CUDA(partials_.alloc(blocks(n * 8, kBlock) + blocks(n, 256) + 64));
        SPH_CUDA(sc_.alloc(1));
        SPH_CUDA(cudaMemsetAsync(sc_.p, 0, sizeof(DevScalars), st_));
        SPH_CUDA(cudaMemsetAsync(normal_.p, 0, normal_.n * sizeof(P4<R>), st_));
        SPH_CUDA(cudaMemsetAsync(normal2_.p, 0, normal2_.n * sizeof(P4<R>), st_));
        SPH_CUDA(cudaMemsetAsync(pacc_.p, 0, pacc_.n * sizeof(P4<R>), st_));
        SPH_CUDA(cudaMemsetAsync(alpha_.p, 0, n * sizeof(R), st_));
        SPH_CUDA(cudaMemsetAsync(div_.p, 0, n * sizeof(R), st_));
        SPH_CUDA(cudaMemsetAsync(rho_.p, 0, n * sizeof(R), st_));
        for (int k = 0; k < 2; ++k) {
            Fluid<R>& f = fl_[k];
            f.pos = pos_[k].p; f.vel = vel_[k].p; f.kappa = kappa_[k].p; f.kappav = kappav_[k].p;
            f.cell = cell_[k].p; f.id = id_[k].p; f.pred = pred_[k].p;
            f.acc = acc_.p; f.xk = xk_.p; f.predR = predR_.p; f.predV = predV_.p; f.pacc = pacc_.p;
            f.normal = (bh && k == 1) ? normal2_.p : normal_.p;
            f.rho = rho_.p; f.alpha = alpha_.p; f.div = div_.p; f.press = press_.p;
            f.n = (uint32_t)n_;
            f.na = nem_ ? &sc_.p->n_active : nullptr;
            Boundary<R>& b = bd_[k];
            b.pos = bpos_[k].p; b.cell = bcell_[k].p; b.id = bid_[k].p; b.psi = bpsi_.p; b.n = nb_;
            b.nrm = bh ? bnrm_[k].p : nullptr;
            b.dens = bh ? bdens_.p : nullptr;
            b.press = bh ? bpress_.p : nullptr;
            b.dp = bh ? bdp_.p : nullptr;
        }
        cur_ = 0;
        return SPH_OK;
    }

    // Exclusive scan of count_ into out (nkeys + 1 entries); zeroes count_.
    int scan(uint32_t* out)
    {
        const unsigned nt = blocks(nkeys_, kScanTile);
        run("k_scan_tiles", [&] { k_scan_tiles<<<nt, kScanThreads, 0, ls_>>>(nkeys_, count_.p, out, tile_sums_.p); });
        run("k_scan_tile_sums", [&] { k_scan_tile_sums<<<1, 1024, 0, ls_>>>(nt, tile_sums_.p, out, nkeys_); });
        run("k_scan_add", [&] { k_scan_add<<<nt, kScanThreads, 0, ls_>>>(nkeys_, tile_sums_.p, out); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // SPHSolver::insertFluidParticles + neighborhoodSearch
    // (SPHSolver.cpp:172-221): recompute cells (after the position update
    // when MOVE), counting sort by cell key, in-cell order by id.
    int build_grid(bool move)
    {
        Fluid<R> a = F();
        uint32_t* ce = bh_ ? cell_epoch_.p : nullptr;
        if (bh_) run("k_bh_epoch", [&] { k_bh_epoch<<<1, 1, 0, ls_>>>(sc_.p); });
        if (move)
            run("k_cell_update", [&] { k_cell_update<R, true><<<blocks(n_, 256), 256, 0, ls_>>>(n_, a.pos, a.vel, a.cell, key_.p, slot_.p, count_.p, gv_,
                                                                     c_.h, hd_, sc_.p, ce, nullptr, a.na); });
        else
            run("k_cell_update", [&] { k_cell_update<R, false><<<blocks(n_, 256), 256, 0, ls_>>>(n_, a.pos, a.vel, a.cell, key_.p, slot_.p, count_.p,
                                                                      gv_, c_.h, hd_, sc_.p, ce, nullptr, a.na); });
        SPH_CUDA(cudaGetLastError());
        int rc = scan(starts_.p);
        if (rc) return rc;
        run("k_scatter", [&] { k_scatter<<<blocks(n_, 256), 256, 0, ls_>>>(n_, key_.p, slot_.p, starts_.p, tmp_.p, a.na); });
        run("k_gather_fluid", [&] { k_gather_fluid<R><<<blocks(n_, 256), 256, 0, ls_>>>(n_, tmp_.p, key_.p, starts_.p, fl_[cur_], fl_[1 - cur_],
                                                                                  posh_.p); });
        SPH_CUDA(cudaGetLastError());
        cur_ = 1 - cur_;
        return SPH_OK;
    }

    template <typename Fn> void withG(Fn&& fn)
    {
        switch (G_) {
            case 2: fn(std::integral_constant<int, 2>{}); break;
            case 4: fn(std::integral_constant<int, 4>{}); break;
            case 8: fn(std::integral_constant<int, 8>{}); break;
            default: fn(std::integral_constant<int, 1>{}); break;
        }
    }
    unsigned wblocks() const { return blocks((size_t)n_ * G_, kBlock); }

    int launch_density(bool alpha, bool eos)
    {
        Fluid<R> f = F();
        const P4<R>* bp = bd_[1].pos;
        withG([&](auto gt) {
            constexpr int G = decltype(gt)::value;
            if (alpha)
                run("k_density", [&] { k_density<R, G, true, false><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_); });
            else if (eos)
                run("k_density", [&] { k_density<R, G, false, true><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_); });
            else
                run("k_density", [&] { k_density<R, G, false, false><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_); });
        });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // Densities (EOS: and WCSPH pressures) with the step's candidate lists.
    template <bool EOS> int launch_density_cand()
    {
        Fluid<R> f = F();
        const R reach = c_.h + cand_margin();
        run("k_density_cand", [&] { k_density_cand<R, EOS><<<blocks(n_, kBlock), kBlock, 0, ls_>>>(
            f, bd_[1].pos, gv_, starts_.p, bstarts_.p, c_, akinci_, reach * reach, cand_.p, candn_.p, ckmax_); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // Densities, alpha and the DFSPH pair lists after a grid build.
    int launch_build_lists()
    {
        Fluid<R> f = F();
        const P4<R>* bp = bd_[1].pos;
        Lists<R> L = LS();
        run("k_build_lists", [&] { k_build_lists<R><<<blocks(n_, kBlock), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, L); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // ---- PCISPH boundary model passes (no-ops for other boundary models) ----
    // Boundary densities (MODE 0), + WCSPH pressures (1), or the PCISPH
    // predicted densities and pressure update inside the loop (2).
    void launch_bh_boundary(int mode)
    {
        if (!bh_ || !nb_) return;
        Fluid<R> f = F();
        Boundary<R> b = B(1);
        const unsigned nbk = blocks(nb_, 128);
        if (mode == 0) run("k_bh_boundary", [&] { k_bh_boundary<R, 0><<<nbk, 128, 0, ls_>>>(b, f, gv_, starts_.p, bstarts_.p, c_, sc_.p); });
        else if (mode == 1) run("k_bh_boundary", [&] { k_bh_boundary<R, 1><<<nbk, 128, 0, ls_>>>(b, f, gv_, starts_.p, bstarts_.p, c_, sc_.p); });
        else run("k_bh_boundary", [&] { k_bh_boundary<R, 2><<<nbk, 128, 0, ls_>>>(b, f, gv_, starts_.p, bstarts_.p, c_, sc_.p); });
    }
    // Positions and cells after the integration (and MOVE: after the DFSPH
    // position update), then PCISPHBoundaryModel::correctPositions (MODE 0 /
    // 1) and, when VEL, ::correctVelocities (PRED for PCISPH).
    template <bool MOVE, int MODE, bool VEL, bool PRED> void launch_bh_after_move()
    {
        Fluid<R> f = F();
        // PCISPH: the predicted positions move into the new cell frames too
        P4<R>* carry = MODE == 1 ? f.predR : nullptr;
        run("k_cell_update", [&] { k_cell_update<R, MOVE, false><<<blocks(n_, 256), 256, 0, ls_>>>(n_, f.pos, f.vel, f.cell, key_.p, slot_.p,
                                                                                             count_.p, gv_, c_.h, hd_, sc_.p, nullptr,
                                                                                             carry, f.na); });
        run("k_bh_collide", [&] { k_bh_collide<R, MODE><<<blocks(n_, 128), 128, 0, ls_>>>(f, B(1), gv_, bstarts_.p, c_, sc_.p,
                                                                                          cell_epoch_.p); });
        if (VEL) run("k_bh_correct_velocities", [&] { k_bh_correct_velocities<R, PRED><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_); });
    }
    // DFSPHSolver::step :51-57: correctVelocities after predictVelocities.
    void launch_bh_velocities()
    {
        if (bh_) run("k_bh_correct_velocities", [&] { k_bh_correct_velocities<R, false><<<blocks(n_, 256), 256, 0, ls_>>>(F(), c_); });
    }
    // updatePositions, then (PCISPH boundary model) correctPositions
    // DFSPHSolver.cpp:65-75, then the grid build.
    int dfsph_move_and_build()
    {
        if (!bh_ && !nem_) {
            auto ph = phase("Fill grid");  // with the position update fused in
            return build_grid(true);
        }
        if (bh_) {
            auto ph = phase("Boundary handling");
            launch_bh_after_move<true, 0, false, false>();
        } else {
            Fluid<R> f = F();
            run("k_cell_update", [&] { k_cell_update<R, true, false><<<blocks(n_, 256), 256, 0, ls_>>>(n_, f.pos, f.vel, f.cell, key_.p, slot_.p,
                                                                                              count_.p, gv_, c_.h, hd_, sc_.p, nullptr,
                                                                                              nullptr, f.na); });
        }
        launch_emit();  // Simulation::emitParticles DFSPHSolver.cpp:77, before the grid fill
        auto ph = phase("Fill grid");
        return build_grid(false);
    }

    // Simulation::emitParticles (Simulation.cpp:325-329) at the current time.
    void launch_emit()
    {
        if (!nem_) return;
        const unsigned flags = (d.simulation_method == SPH_PCISPH ? EMIT_PCISPH : 0u) | (normal_.n >= n_ ? EMIT_NORMALS : 0u);
        Fluid<R> f = F();
        run("k_emit", [&] { k_emit<R><<<1, 256, 0, ls_>>>(f, em_.p, nem_, egroup_.p, gv_, hd_, d.gravity[0], d.gravity[1],
                                                          d.gravity[2], sc_.p, &sc_.p->n_active, flags); });
    }

    // Emitter state and the group table on the device.
    int upload_emitters()
    {
        if (!nem_) return SPH_OK;
        if (nem_ > kMaxEmitters) { fail("at most 64 emitters per scene"); return SPH_ERR_INVALID; }
        std::vector<EmitterDev> he(nem_);
        std::vector<double> tab;
        for (int e = 0; e < nem_; ++e) {
            const EmitterSpec& s = hem[e];
            EmitterDev& o = he[e];
            for (int k = 0; k < 3; ++k) o.r[k] = s.r[k];
            for (int k = 0; k < 4; ++k) o.q[k] = s.q[k];
            o.v = s.v;
            o.next = s.start;
            // Emitter::emitSquare / emitCircle Emitter.cpp:127,159
            const double dist = 2.0 * d.particle_radius;
            o.period = s.spacing * 1.105 * dist / s.v;
            o.remaining = s.num;
            o.first = (uint32_t)(tab.size() / 3);
            o.count = (uint32_t)(s.group.size() / 3);
            o.pause = 0;
            tab.insert(tab.end(), s.group.begin(), s.group.end());
        }
        SPH_CUDA(em_.alloc(nem_));
        SPH_CUDA(egroup_.alloc(tab.size()));
        SPH_CUDA(cudaMemcpyAsync(em_.p, he.data(), nem_ * sizeof(EmitterDev), cudaMemcpyHostToDevice, st_));
        if (!tab.empty()) SPH_CUDA(cudaMemcpyAsync(egroup_.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));  // the host tables are freed on return
        return SPH_OK;
    }

    // getNumActiveParticles: the device count for scenes with emitters.
    unsigned active() const
    {
        if (!inited) return n0_;
        if (!nem_) return n_;
        unsigned v = 0;
        if (cudaStreamSynchronize(st_) != cudaSuccess) return 0;
        if (cudaMemcpy(&v, &sc_.p->n_active, sizeof v, cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
        return v;
    }
    const R* bdp() const { return bh_ ? bdp_.p : nullptr; }

    // DFSPHSolver::step DFSPHSolver.cpp:38-112 over the pair lists.
    int dfsph_step_lists()
    {
        int rc = SPH_OK;
        if (c_.force_flags) {
            auto ph = phase("npForces");
            rc = launch_npforces();
        }
        if (rc) return rc;
        const unsigned nb = blocks(n_, kBlock);
        {
            Fluid<R> f = F();
            const P4<R>* bp = bd_[1].pos;
            Lists<R> L = LS();
            run("k_dfsph_cfl", [&] { k_dfsph_cfl<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_, sc_.p, lim_, partials_.p); });
            run("k_dfsph_predict_v_warm", [&] { k_dfsph_predict_v_warm_list<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_, sc_.p, L.kbuf); });
            launch_bh_velocities();
            auto ph = phase("Density solver");
            run("k_dfsph_correct_list", [&] { k_dfsph_correct_list<R, 0><<<nb, kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, L); });
            SPH_CUDA(cudaGetLastError());
            // correctDensityError DFSPHSolver.cpp:311-406
            rc = solve_loop(1,
                [&](cudaGraphConditionalHandle h) {
                    run("k_dfsph_predict_density_list", [&] { k_dfsph_predict_density_list<R, true><<<nb, kBlock, 0, ls_>>>(
                        f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h, L); });
                },
                [&](cudaGraphConditionalHandle h) {
                    run("k_dfsph_correct_list", [&] { k_dfsph_correct_list<R, 1><<<nb, kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, L); });
                    run("k_dfsph_predict_density_list", [&] { k_dfsph_predict_density_list<R, false><<<nb, kBlock, 0, ls_>>>(
                        f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h, L); });
                },
                lim_.minIt, lim_.maxIt);
            if (rc) return rc;
        }
        rc = dfsph_move_and_build();  // updatePositions + fill grid + neighbour search
        if (rc) return rc;
        {
            auto ph = phase("Neigh search+Densities+Alpha factor");
            rc = launch_build_lists();  // computeDensities + computeAlpha + pair lists
            if (rc) return rc;
            launch_bh_boundary(0);
        }
        {
            Fluid<R> f = F();
            const P4<R>* bp = bd_[1].pos;
            Lists<R> L = LS();
            // correctDivergenceError DFSPHSolver.cpp:494-590
            auto ph = phase("Divergence solver");
            rc = solve_loop(2,
                [&](cudaGraphConditionalHandle h) {
                    run("k_dfsph_divergence_list", [&] { k_dfsph_divergence_list<R, true><<<nb, kBlock, 0, ls_>>>(
                        f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h, L); });
                },
                [&](cudaGraphConditionalHandle h) {
                    run("k_dfsph_correct_list", [&] { k_dfsph_correct_list<R, 2><<<nb, kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, L); });
                    run("k_dfsph_divergence_list", [&] { k_dfsph_divergence_list<R, false><<<nb, kBlock, 0, ls_>>>(
                        f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h, L); });
                },
                lim_.minItV, lim_.maxIt);
            if (rc) return rc;
        }
        if (c_.has_cube) {
            Fluid<R> f = F();
            auto ph = phase("Boundary handling");
            run("k_dfsph_cube", [&] { k_dfsph_cube<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, gv_, hd_, c_); });
        }
        run("k_finish_step", [&] { k_finish_step<<<1, 1, 0, ls_>>>(sc_.p); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // Simulation::computeNonPressureForces (Simulation.cpp:313-323)
    int launch_npforces()
    {
        if (!c_.force_flags) return SPH_OK;
        Fluid<R> f = F();
        const P4<R>* bp = bd_[1].pos;
        withG([&](auto gt) {
            constexpr int G = decltype(gt)::value;
            const CandLists L = CL();
            if (c_.force_flags & F_SURFACE_TENSION)
                run("k_st_normals", [&] { k_st_normals<R, G><<<wblocks(), kBlock, 0, ls_>>>(f, gv_, starts_.p, c_, L); });
            run("k_npforce", [&] { k_npforce<R, G><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, akinci_, sc_.p, L); });
        });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // A solver loop: init(h) launches the kernel that sets the first loop
    // test, body(h) one iteration whose last kernel sets the next.  Host mode
    // reads the flag back every few iterations (finished-loop kernels exit at
    // once); capture mode makes it a conditional WHILE node.
    template <typename Init, typename Body> int solve_loop(int loop_id, Init&& init, Body&& body, unsigned minIt, unsigned maxIt)
    {
        if (capturing_) {
            cudaStreamCaptureStatus cs;
            cudaGraph_t g;
            const cudaGraphNode_t* deps = nullptr;
            size_t ndeps = 0;
            SPH_CUDA(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &g, nullptr, nullptr, nullptr));
            cudaGraphConditionalHandle h;
            SPH_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
            init(h);
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &g, &deps, nullptr, &ndeps));
            cudaGraphNodeParams p{};
            p.type = cudaGraphNodeTypeConditional;
            p.conditional.handle = h;
            p.conditional.type = cudaGraphCondTypeWhile;
            p.conditional.size = 1;
            cudaGraphNode_t node;
            SPH_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
            cudaGraph_t bodyg = p.conditional.phGraph_out[0];
            SPH_CUDA(cudaStreamUpdateCaptureDependencies(st_, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            SPH_CUDA(cudaStreamBeginCaptureToGraph(st2_, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
            ls_ = st2_;
            loop_ctx_ = loop_id;
            body(h);
            loop_ctx_ = 0;
            ls_ = st_;
            cudaGraph_t out;
            SPH_CUDA(cudaStreamEndCapture(st2_, &out));
            return SPH_OK;
        }
        init((cudaGraphConditionalHandle)0);
        SPH_CUDA(cudaGetLastError());
        unsigned launched = 0;
        const unsigned first = std::min(std::max(minIt, 1u) + 1u, maxIt);
        while (launched < maxIt) {
            unsigned batch = launched == 0 ? first : 2u;
            batch = std::min(batch, maxIt - launched);
            for (unsigned b = 0; b < batch; ++b) body((cudaGraphConditionalHandle)0);
            SPH_CUDA(cudaGetLastError());
            launched += batch;
            SPH_CUDA(cudaMemcpyAsync(&h_sc_->active, &sc_.p->active, sizeof(unsigned), cudaMemcpyDeviceToHost, st_));
            SPH_CUDA(cudaStreamSynchronize(st_));
            if (!h_sc_->active) break;
        }
        return SPH_OK;
    }

    // Every launch of the step path goes through run(): it counts launches
    // (host mode), records how many kernels a captured step holds per loop
    // body (graph mode), and brackets the launch with CUDA events when
    // profiling is on.
    template <typename Fn> void run(const char* name, Fn&& fn)
    {
        if (capturing_) { ++cap_count_[loop_ctx_]; fn(); return; }
        ++launches_;
        if (!prof_) { fn(); return; }
        cudaEvent_t a = take_event(), b = take_event();
        cudaEventRecord(a, ls_);
        fn();
        cudaEventRecord(b, ls_);
        pending_.push_back({name, a, b});
    }
    cudaEvent_t take_event()
    {
        if (!events_.empty()) { cudaEvent_t e = events_.back(); events_.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }

    // DFSPHSolver::step DFSPHSolver.cpp:38-112
    int dfsph_step()
    {
        int rc = SPH_OK;
        if (c_.force_flags) {
            auto ph = phase("npForces");
            rc = launch_npforces();
        }
        if (rc) return rc;
        {
            Fluid<R> f = F();
            run("k_dfsph_cfl", [&] { k_dfsph_cfl<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_, sc_.p, lim_, partials_.p); });
            run("k_dfsph_predict_v_warm", [&] { k_dfsph_predict_v_warm<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_, sc_.p); });
            SPH_CUDA(cudaGetLastError());
            launch_bh_velocities();
            const P4<R>* bp = bd_[1].pos;
            auto ph = phase("Density solver");
            withG([&](auto gt) {
                constexpr int G = decltype(gt)::value;
                run("k_dfsph_correct", [&] { k_dfsph_correct<R, G, 0><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p); });
            });
            SPH_CUDA(cudaGetLastError());
            // correctDensityError DFSPHSolver.cpp:311-406
            rc = solve_loop(1, 
                [&](cudaGraphConditionalHandle h) {
                    withG([&](auto gt) {
                        constexpr int G = decltype(gt)::value;
                        run("k_dfsph_predict_density", [&] { k_dfsph_predict_density<R, G, true><<<wblocks(), kBlock, 0, ls_>>>(
                            f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h); });
                    });
                },
                [&](cudaGraphConditionalHandle h) {
                    withG([&](auto gt) {
                        constexpr int G = decltype(gt)::value;
                        run("k_dfsph_correct", [&] { k_dfsph_correct<R, G, 1><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_,
                                                                                 sc_.p); });
                        run("k_dfsph_predict_density", [&] { k_dfsph_predict_density<R, G, false><<<wblocks(), kBlock, 0, ls_>>>(
                            f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h); });
                    });
                },
                lim_.minIt, lim_.maxIt);
            if (rc) return rc;
        }
        rc = dfsph_move_and_build();  // updatePositions + fill grid + neighbour search
        if (rc) return rc;
        {
            auto ph = phase("Densities+Alpha factor");
            rc = launch_density(true, false);  // computeDensities + computeAlpha
            if (rc) return rc;
            launch_bh_boundary(0);
        }
        {
            Fluid<R> f = F();
            const P4<R>* bp = bd_[1].pos;
            // correctDivergenceError DFSPHSolver.cpp:494-590
            auto ph = phase("Divergence solver");
            rc = solve_loop(2, 
                [&](cudaGraphConditionalHandle h) {
                    withG([&](auto gt) {
                        constexpr int G = decltype(gt)::value;
                        run("k_dfsph_divergence", [&] { k_dfsph_divergence<R, G, true><<<wblocks(), kBlock, 0, ls_>>>(
                            f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h); });
                    });
                },
                [&](cudaGraphConditionalHandle h) {
                    withG([&](auto gt) {
                        constexpr int G = decltype(gt)::value;
                        run("k_dfsph_correct", [&] { k_dfsph_correct<R, G, 2><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_,
                                                                                 sc_.p); });
                        run("k_dfsph_divergence", [&] { k_dfsph_divergence<R, G, false><<<wblocks(), kBlock, 0, ls_>>>(
                            f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, sc_.p, lim_, partials_.p, h); });
                    });
                },
                lim_.minItV, lim_.maxIt);
            if (rc) return rc;
        }
        if (c_.has_cube) {
            Fluid<R> f = F();
            auto ph = phase("Boundary handling");
            run("k_dfsph_cube", [&] { k_dfsph_cube<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, gv_, hd_, c_); });
        }
        run("k_finish_step", [&] { k_finish_step<<<1, 1, 0, ls_>>>(sc_.p); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // WCSPHSolver::step WCSPHSolver.cpp:14-78
    int wcsph_step()
    {
        int rc;
        {
            auto ph = phase("Fill grid");
            rc = build_grid(false);
        }
        if (rc) return rc;
        {
            auto ph = phase("Densities+Pressures");  // the equation of state is fused into the density pass
            rc = cands_ ? launch_density_cand<true>() : launch_density(false, true);
            if (rc) return rc;
            launch_bh_boundary(1);
        }
        Fluid<R> f = F();
        const P4<R>* bp = bd_[1].pos;
        const R* dp = bdp();
        {
            auto ph = phase("Pressure force");
            withG([&](auto gt) {
                constexpr int G = decltype(gt)::value;
                run("k_wcsph_pressure_force", [&] { k_wcsph_pressure_force<R, G><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_, dp, CL()); });
            });
            SPH_CUDA(cudaGetLastError());
        }
        {
            auto ph = phase("NPForces");
            rc = launch_npforces();
        }
        if (rc) return rc;
        {
            auto ph = phase("Integratio");
            run("k_integrate", [&] { k_integrate<R, false><<<blocks(n_, 256), 256, 0, ls_>>>(f, gv_, hd_, c_, sc_.p); });
        }
        if (bh_) {
            auto ph = phase("Boundary Handling");
            launch_bh_after_move<false, 0, true, false>();  // WCSPHSolver.cpp:62-72
        }
        launch_emit();  // WCSPHSolver.cpp:75
        run("k_finish_step", [&] { k_finish_step<<<1, 1, 0, ls_>>>(sc_.p); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // PCISPHSolver::step PCISPHSolver.cpp:21-81
    int pcisph_step()
    {
        int rc;
        {
            auto ph = phase("Fill grid");
            rc = build_grid(false);
        }
        if (rc) return rc;
        {
            auto ph = phase("Densities");
            if (cands_) {
                rc = launch_density_cand<false>();   // densities and the step's candidate lists
                if (rc) return rc;
            } else {
                rc = launch_density(false, false);
                if (rc) return rc;
            }
            launch_bh_boundary(0);
        }
        {
            auto ph = phase("npForces");
            rc = launch_npforces();
        }
        if (rc) return rc;
        Fluid<R> f = F();
        const P4<R>* bp = bd_[1].pos;
        const R* dp = bdp();
        {
            auto ph = phase("Pressure solver");
            run("k_pcisph_init", [&] { k_pcisph_init<R><<<blocks(n_, 256), 256, 0, ls_>>>(f); });
            if (bh_ && nb_) run("k_bh_zero_pressure", [&] { k_bh_zero_pressure<R><<<blocks(nb_, 256), 256, 0, ls_>>>(B(1)); });
            rc = solve_loop(1,
                [&](cudaGraphConditionalHandle h) { run("k_pcisph_loop_begin", [&] { k_pcisph_loop_begin<<<1, 1, 0, ls_>>>(sc_.p, lim_, h); }); },
                [&](cudaGraphConditionalHandle h) {
                    if (cands_)
                    run("k_pcisph_predict", [&] { k_pcisph_predict<R, true><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_, sc_.p); });
                else
                    run("k_pcisph_predict", [&] { k_pcisph_predict<R><<<blocks(n_, 256), 256, 0, ls_>>>(f, c_, sc_.p); });
                    if (bh_)  // correctPredPositions PCISPHSolver.cpp:367-377
                        run("k_bh_collide", [&] { k_bh_collide<R, 2><<<blocks(n_, 128), 128, 0, ls_>>>(f, B(1), gv_, bstarts_.p, c_, sc_.p,
                                                                                                  cell_epoch_.p); });
                    withG([&](auto gt) {
                        constexpr int G = decltype(gt)::value;
                        const CandLists L = CL();
                        const float margin = (float)cand_margin();
                        run("k_pcisph_density_pressure", [&] { k_pcisph_density_pressure<R, G><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_,
                                                                                       hasb_, sc_.p, lim_, partials_.p, L, margin); });
                        launch_bh_boundary(2);
                        run("k_pcisph_pressure_acc", [&] { k_pcisph_pressure_acc<R, G><<<wblocks(), kBlock, 0, ls_>>>(f, bp, gv_, starts_.p, bstarts_.p, c_, hasb_,
                                                                                   sc_.p, dp, L); });
                    });
                    run("k_pcisph_loop_next", [&] { k_pcisph_loop_next<<<1, 1, 0, ls_>>>(sc_.p, lim_, h); });
                },
                lim_.minIt, lim_.maxIt);
        }
        if (rc) return rc;
        {
            auto ph = phase("Integration");
            run("k_integrate", [&] { k_integrate<R, true><<<blocks(n_, 256), 256, 0, ls_>>>(f, gv_, hd_, c_, sc_.p); });
        }
        if (bh_) {
            auto ph = phase("Boundary handling");
            launch_bh_after_move<false, 1, true, true>();  // PCISPHSolver.cpp:65-75
        }
        launch_emit();  // PCISPHSolver.cpp:78
        run("k_finish_step", [&] { k_finish_step<<<1, 1, 0, ls_>>>(sc_.p); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    int one_step()
    {
        switch (d.simulation_method) {
            case SPH_WCSPH: return wcsph_step();
            case SPH_PCISPH: return pcisph_step();
            default: return lists_ ? dfsph_step_lists() : dfsph_step();
        }
    }

    // One graph per buffer parity (each step swaps the sorted buffers once).
    int graph_step()
    {
        const int k = cur_;
        if (!gexec_[k]) {
            cudaGraph_t g;
            SPH_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
            capturing_ = true;
            cap_count_[0] = cap_count_[1] = cap_count_[2] = 0;
            const int rc = one_step();
            capturing_ = false;
            for (int q = 0; q < 3; ++q) gshape_[k][q] = cap_count_[q];
            cudaError_t e = cudaStreamEndCapture(st_, &g);
            if (rc) { if (e == cudaSuccess) cudaGraphDestroy(g); cur_ = k; return rc; }
            SPH_CUDA(e);
            SPH_CUDA(cudaGraphInstantiate(&gexec_[k], g, 0));
            cudaGraphDestroy(g);
            cur_ = k;  // capture recorded the swap; the launch performs it
        }
        SPH_CUDA(cudaGraphLaunch(gexec_[k], st_));
        ++gsteps_[k];
        cur_ = 1 - k;
        return SPH_OK;
    }

    // ------------------------------------------------------------------
    cudaStream_t st_ = nullptr, st2_ = nullptr, ls_ = nullptr;
    DevScalars* h_sc_ = nullptr;
    Consts<R> c_{};
    LoopLimits lim_{};
    GridView gv_{};
    double hd_ = 0, mass_ = 0;
    unsigned n_ = 0, nb_ = 0;   // fluid slots (initial fluid + emitter reservations), boundary points
    unsigned n0_ = 0;           // fluid particles at init
    int nem_ = 0;               // emitters
    DevBuf<EmitterDev> em_;
    DevBuf<double> egroup_;
    DevBuf<double> cap_x_, cap_v_;  // staging of asynchronous frame captures
    DevBuf<uint4> posh_;            // FP32 pair lists: half-precision positions (build cull, particle pairs)
    int akinci_ = 0;   // Akinci boundary model: boundary terms in the forces too
    int bh_ = 0;       // PCISPH boundary model
    int hasb_ = 0;     // boundary particles take part in the solver sums
    int device_ = 0;
    int G_ = 1;
    uint32_t nkeys_ = 0;
    int cur_ = 0;
    bool graph_ = false, capturing_ = false;
    cudaGraphExec_t gexec_[2] = {nullptr, nullptr};
    int loop_ctx_ = 0;
    unsigned cap_count_[3] = {0, 0, 0};
    static constexpr unsigned kGrowthCheck = 16;
    bool grow_ = true, esc_pending_ = false;
    unsigned since_check_ = 0, growths_ = 0;
    unsigned* h_esc_ = nullptr;
    cudaEvent_t esc_ev_ = nullptr;
    unsigned gshape_[2][3] = {{0, 0, 0}, {0, 0, 0}};
    unsigned long long gsteps_[2] = {0, 0};
    unsigned long long launches_ = 0, graph_launches_ = 0, snap_it_ = 0, snap_itv_ = 0;
    bool prof_ = false;
    PhaseLog phases_;
    cudaEvent_t tev_[2] = {nullptr, nullptr};
    struct Timed { const char* name; cudaEvent_t a, b; };
    std::vector<Timed> pending_;
    std::vector<cudaEvent_t> events_;
    Fluid<R> fl_[2]{};
    Boundary<R> bd_[2]{};
    DevBuf<P4<R>> pos_[2], vel_[2], bpos_[2];
    DevBuf<R> kappa_[2], kappav_[2], pred_[2];
    DevBuf<uint32_t> cell_[2], id_[2], bcell_[2], bid_[2];
    DevBuf<P4<R>> acc_, xk_, predR_, predV_, pacc_, normal_, normal2_;
    DevBuf<R> rho_, alpha_, div_, press_, bpsi_;
    DevBuf<P4<R>> bnrm_[2];
    DevBuf<R> bdens_, bpress_, bdp_;
    DevBuf<uint32_t> cell_epoch_;  // PCISPH boundary model: first grid build at which each cell exists
    DevBuf<uint32_t> mortx_, morty_, key_, slot_, tmp_, count_, starts_, bstarts_, tile_sums_;
    DevBuf<double> partials_;
    DevBuf<P4<R>> pairs_, bgrad_;
    DevBuf<uint32_t> lcount_;
    DevBuf<R> kbuf_;
    DevBuf<unsigned long long> lstat_;
    bool lists_ = false;
    uint32_t kmax_ = 0;
    bool cands_ = false;            // PCISPH candidate lists (CandLists)
    uint32_t ckmax_ = 0;
    DevBuf<uint32_t> cand_, candn_;
    CandLists CL() const
    {
        return cands_ ? CandLists{cand_.p, candn_.p, ckmax_, &sc_.p->status} : CandLists{nullptr, nullptr, 0u, nullptr};
    }
    // the lists' reach beyond h: predicted displacements up to half of it keep them exact
    R cand_margin() const { return (R)0.1 * c_.h; }
    DevBuf<DevScalars> sc_;
};

}  // namespace sph
