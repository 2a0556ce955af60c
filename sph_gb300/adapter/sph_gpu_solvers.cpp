// GPU drop-in solvers for the reference simulator: see sph_gpu_solvers.h.
//
// The scene is read from the reference's live objects.  Fields the reference
// keeps protected without a getter (a cube model's bounds, a PCISPH model's
// normals, a fluid model's emitters and their settings, the DFSPH CFL
// factor, Simulation::activeSave) are read through member pointers formed in
// a derived class's scope, which C++ allows for protected members; no
// reference source is changed.
#include "sph_gpu_solvers.h"

#include <cmath>
#include <cstdio>
#include <mutex>
#include <stdexcept>

#include "AdhesionForce.h"
#include "AkinciBoundaryModel.h"
#include "ArtificialViscosity.h"
#include "CubeBoundaryModel.h"
#include "Emitter.h"
#include "FluidModel.h"
#include "PCISPHBoundaryModel.h"
#include "StandardViscosityForce.h"
#include "SurfaceTensionAkinci.h"
#include "XSPHViscosity.h"

namespace sph_gpu {
namespace {

// Member pointers to protected state (formed in derived scopes).
struct FluidModelAccess : FluidModel {
    static std::vector<Emitter> FluidModel::*emitters_ptr() { return &FluidModelAccess::emitters; }
};
struct EmitterAccess : Emitter {
    static unsigned int Emitter::*type_ptr() { return &EmitterAccess::type; }
    static unsigned int Emitter::*num_ptr() { return &EmitterAccess::numParticles; }
    static Vector3r Emitter::*r_ptr() { return &EmitterAccess::r; }
    static Real Emitter::*v_ptr() { return &EmitterAccess::v; }
    static Quat4r Emitter::*rot_ptr() { return &EmitterAccess::rot; }
    static Real Emitter::*start_ptr() { return &EmitterAccess::startTime; }
    static Real Emitter::*width_ptr() { return &EmitterAccess::width; }
    static Real Emitter::*height_ptr() { return &EmitterAccess::height; }
    static Real Emitter::*spacing_ptr() { return &EmitterAccess::spacing; }
    static bool Emitter::*pause_ptr() { return &EmitterAccess::pause; }
};
struct CubeAccess : CubeBoundaryModel {
    static Vector3r* CubeBoundaryModel::*min_ptr() { return &CubeAccess::min; }
    static Vector3r* CubeBoundaryModel::*max_ptr() { return &CubeAccess::max; }
};
struct PCISPHModelAccess : PCISPHBoundaryModel {
    static std::vector<Vector3r> PCISPHBoundaryModel::*normals_ptr() { return &PCISPHModelAccess::n; }
};
struct DFSPHAccess : DFSPHSolver {
    static Real DFSPHSolver::*cfl_ptr() { return &DFSPHAccess::cflFactor; }
};
struct SimulationAccess : Simulation {
    static bool Simulation::*active_save_ptr() { return &SimulationAccess::activeSave; }
};

std::mutex g_mutex;
sph_scene_desc g_base;
bool g_base_set = false;

sph_scene_desc defaults()
{
    sph_scene_desc d;
    sph_scene_desc_init(&d);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_base_set) {
        d.precision = g_base.precision;
        d.threads_per_particle = g_base.threads_per_particle;
        d.neighbor_list_max = g_base.neighbor_list_max;
        for (int k = 0; k < 3; ++k) { d.domain_min[k] = g_base.domain_min[k]; d.domain_max[k] = g_base.domain_max[k]; }
    }
    return d;
}

void put3(std::vector<double>* out, const Vector3r& p)
{
    out->push_back(p.x);
    out->push_back(p.y);
    out->push_back(p.z);
}

}  // namespace

void sph_gpu_set_defaults(const sph_scene_desc* base)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    g_base_set = base != nullptr;
    if (base) g_base = *base;
}

bool capture_scene(Simulation* sim, SPHSolver* solver, CapturedScene* out, std::string* err)
{
    CapturedScene s;
    sph_scene_desc& d = s.desc;
    d = defaults();
    // settings importScene gives the Simulation (Simulation.cpp:346-355)
    d.simulation_method = sim->getSimulationMethod();
    d.boundary_method = sim->getBoundaryHandlingMethod();
    d.particle_radius = sim->getParticleRadius();
    const Vector3r g = sim->getGravity();
    d.gravity[0] = g.x; d.gravity[1] = g.y; d.gravity[2] = g.z;
    d.time_step = sim->getTimeStep();
    d.fps = sim->getFPS();
    d.min_time_step = sim->getMinTimeStep();  // already min(minTimeStep, 1/fps) (TimeManager.h:55)
    d.max_time_step = sim->getMaxTimeStep();
    s.time = sim->getTime();
    // the solver's own parameters (Simulation.cpp:357-378)
    if (auto* w = dynamic_cast<WCSPHSolver*>(solver)) {
        d.stiffness = w->getStiffness();
        d.gamma = w->getGamma();
    } else if (auto* p = dynamic_cast<PCISPHSolver*>(solver)) {
        d.max_error = p->getMaxError();
        d.min_iterations = (int)p->getMinIterations();
        d.max_iterations = (int)p->getMaxIterations();
    } else if (auto* f = dynamic_cast<DFSPHSolver*>(solver)) {
        d.max_error = f->getMaxError();
        d.max_error_v = f->getMaxErrorV();
        d.cfl_factor = f->*DFSPHAccess::cfl_ptr();
        d.min_iterations = (int)f->getMinIterations();
        d.max_iterations = (int)f->getMaxIterations();
        d.min_iterations_v = (int)f->getMinIterationsV();
        d.max_iterations_v = (int)f->getMaxIterationsV();
    } else {
        *err = "unknown solver type";
        return false;
    }
    // fluid model 0: the device path holds one fluid phase per scene
    if (sim->numberFluidModels() != 1) {
        *err = "the GPU solvers take exactly one fluid model";
        return false;
    }
    FluidModel* fm = sim->getFluidModel(0);
    d.density0 = fm->getRefDensity();
    const unsigned na = fm->getNumActiveParticles();
    s.num_fluid_total = fm->getNumParticles();
    s.x.reserve(3 * (size_t)na);
    s.v.reserve(3 * (size_t)na);
    for (unsigned i = 0; i < na; ++i) {
        put3(&s.x, fm->getPosition(i));
        put3(&s.v, fm->getVelocity(i));
    }
    // non-pressure forces: the methods the Simulation selected and each force
    // object's coefficients (FluidModel.cpp:73-122; no object, no force)
    d.viscosity_method = sim->getViscosityMethod();
    d.surface_tension_method = sim->getSurfaceTensionMethod();
    d.adhesion_method = sim->getAdhesionMethod();
    d.viscosity = d.boundary_viscosity = d.surface_tension = d.adhesion = 0.0;
    for (unsigned k = 0; k < fm->numberNonPressureForces(); ++k) {
        NonPressureForce* npf = fm->getNonPressureForce(k);
        if (auto* x = dynamic_cast<XSPHViscosity*>(npf)) {
            d.viscosity = x->getViscosity();
            d.boundary_viscosity = x->getBoundaryViscosity();
        } else if (auto* sv = dynamic_cast<StandardViscosityForce*>(npf)) {
            d.viscosity = sv->getViscosity();
            d.boundary_viscosity = sv->getBoundaryViscosity();
        } else if (auto* av = dynamic_cast<ArtificialViscosity*>(npf)) {
            d.viscosity = av->getViscosity();
            d.boundary_viscosity = av->getBoundaryViscosity();
        } else if (auto* st = dynamic_cast<SurfaceTensionAkinci*>(npf)) {
            d.surface_tension = st->getSurfaceTension();
        } else if (auto* ad = dynamic_cast<AdhesionForce*>(npf)) {
            d.adhesion = ad->getAdhesion();
        }
    }
    // emitters (FluidModel::addEmitter, FluidModel.cpp:124-143)
    for (const Emitter& e : fm->*FluidModelAccess::emitters_ptr()) {
        CapturedEmitter c;
        c.type = (int)(e.*EmitterAccess::type_ptr());
        c.num = e.*EmitterAccess::num_ptr();
        const Vector3r& r = e.*EmitterAccess::r_ptr();
        c.r[0] = r.x; c.r[1] = r.y; c.r[2] = r.z;
        c.v = e.*EmitterAccess::v_ptr();
        const Quat4r& q = e.*EmitterAccess::rot_ptr();
        c.q[0] = q.w; c.q[1] = q.x; c.q[2] = q.y; c.q[3] = q.z;
        c.start = e.*EmitterAccess::start_ptr();
        c.width = e.*EmitterAccess::width_ptr();
        c.height = e.*EmitterAccess::height_ptr();
        c.spacing = e.*EmitterAccess::spacing_ptr();
        c.paused = e.*EmitterAccess::pause_ptr();
        s.emitters.push_back(c);
    }
    // boundary models of the Simulation's boundary method (the solvers read
    // only those, e.g. SPHSolver.cpp:60-90)
    d.has_cube = 0;
    bool bh_factors = false;
    for (unsigned b = 0; b < sim->numberBoundaryModels(); ++b) {
        BoundaryModel* bm = sim->getBoundaryModel(b);
        if (d.boundary_method == SPH_BOUNDARY_AKINCI) {
            if (auto* ak = dynamic_cast<AkinciBoundaryModel*>(bm))
                for (const Vector3r& p : ak->getPosition()) put3(&s.boundary, p);
        } else if (d.boundary_method == SPH_BOUNDARY_CUBE) {
            if (auto* cb = dynamic_cast<CubeBoundaryModel*>(bm)) {
                if (d.has_cube) {
                    *err = "the GPU solvers take one cube boundary model";
                    return false;
                }
                const Vector3r* mn = cb->*CubeAccess::min_ptr();
                const Vector3r* mx = cb->*CubeAccess::max_ptr();
                d.has_cube = 1;
                d.cube_min[0] = mn->x; d.cube_min[1] = mn->y; d.cube_min[2] = mn->z;
                d.cube_max[0] = mx->x; d.cube_max[1] = mx->y; d.cube_max[2] = mx->z;
            }
        } else if (auto* ph = dynamic_cast<PCISPHBoundaryModel*>(bm)) {
            if (bh_factors && (ph->getNormalFct() != d.bh_normal_fct || ph->getTangentialFct() != d.bh_tangential_fct)) {
                *err = "the GPU solvers take PCISPH boundary models with one pair of collision factors";
                return false;
            }
            bh_factors = true;
            d.bh_normal_fct = ph->getNormalFct();
            d.bh_tangential_fct = ph->getTangentialFct();
            const std::vector<Vector3r>& nrm = ph->*PCISPHModelAccess::normals_ptr();
            for (unsigned i = 0; i < ph->getNumParticles(); ++i) {
                put3(&s.bh_points, ph->getPosition(i));
                put3(&s.bh_normals, nrm[i]);
            }
        }
    }
    *out = std::move(s);
    return true;
}

GpuSceneLink::~GpuSceneLink()
{
    if (ctx_) sph_ctx_destroy(ctx_);
}

bool GpuSceneLink::create(const CapturedScene& s, std::string* err)
{
    auto fail = [&](const char* what) {
        *err = std::string(what) + ": " + (ctx_ ? sph_ctx_last_error(ctx_) : "invalid scene settings");
        if (ctx_) sph_ctx_destroy(ctx_);
        ctx_ = nullptr;
        return false;
    };
    if (s.time != 0.0) {
        *err = "the device context starts at time 0; initialise the solver before stepping";
        return false;
    }
    if (ctx_) sph_ctx_destroy(ctx_);
    ctx_ = nullptr;
    // the cube's bounds are part of the descriptor, so they are set before
    // the context exists
    if (sph_ctx_create(&s.desc, &ctx_) != SPH_OK) return fail("sph_ctx_create");
    const unsigned n = (unsigned)(s.x.size() / 3);
    if (sph_ctx_set_fluid(ctx_, s.x.data(), s.v.data(), n) != SPH_OK) return fail("sph_ctx_set_fluid");
    for (const CapturedEmitter& e : s.emitters)
        if (sph_ctx_add_emitter(ctx_, e.type, e.num, e.r, e.v, e.q, e.start, e.width, e.height, e.spacing) != SPH_OK)
            return fail("sph_ctx_add_emitter");
    if (!s.boundary.empty() &&
        sph_ctx_add_boundary_points(ctx_, s.boundary.data(), (unsigned)(s.boundary.size() / 3)) != SPH_OK)
        return fail("sph_ctx_add_boundary_points");
    if (!s.bh_points.empty() &&
        sph_ctx_add_pcisph_points(ctx_, s.bh_points.data(), s.bh_normals.data(), (unsigned)(s.bh_points.size() / 3)) !=
            SPH_OK)
        return fail("sph_ctx_add_pcisph_points");
    if (sph_ctx_set_graph(ctx_, 1) != SPH_OK) return fail("sph_ctx_set_graph");
    if (sph_ctx_init(ctx_) != SPH_OK) return fail("sph_ctx_init");
    bool paused = !s.emitters.empty();
    for (const CapturedEmitter& e : s.emitters) paused = paused && e.paused;
    if (paused && sph_ctx_pause_emitters(ctx_, 1) != SPH_OK) return fail("sph_ctx_pause_emitters");
    return true;
}

bool GpuSceneLink::download_fluid(FluidModel* fm, std::string* err)
{
    unsigned nf = 0, nb = 0;
    if (sph_ctx_num_particles(ctx_, &nf, &nb) != SPH_OK) { *err = sph_ctx_last_error(ctx_); return false; }
    buf_x_.resize(3 * (size_t)nf);
    buf_v_.resize(3 * (size_t)nf);
    if (nf && (sph_ctx_download(ctx_, SPH_FIELD_POSITION, buf_x_.data()) != SPH_OK ||
               sph_ctx_download(ctx_, SPH_FIELD_VELOCITY, buf_v_.data()) != SPH_OK)) {
        *err = sph_ctx_last_error(ctx_);
        return false;
    }
    for (unsigned i = 0; i < nf && i < fm->getNumParticles(); ++i) {
        fm->setPosition(i, Vector3r(buf_x_[3 * i], buf_x_[3 * i + 1], buf_x_[3 * i + 2]));
        fm->setVelocity(i, Vector3r(buf_v_[3 * i], buf_v_[3 * i + 1], buf_v_[3 * i + 2]));
    }
    return true;
}

bool GpuSceneLink::step(Simulation* sim, FluidModel* fm, unsigned* steps, unsigned* iterations,
                        unsigned* sum_iterations, std::string* err)
{
    if (!ctx_) { *err = "not initialised"; return false; }
    sph_stats st;
    if (sph_ctx_step(ctx_, 1) != SPH_OK || sph_ctx_get_stats(ctx_, &st) != SPH_OK) {
        *err = sph_ctx_last_error(ctx_);
        return false;
    }
    // what the reference's solvers leave behind each step
    // (DFSPHSolver.cpp:111,867, WCSPHSolver.cpp:77,225, PCISPHSolver.cpp:80)
    sim->setTimeStep(st.dt);
    sim->setTime(st.time);
    fm->setNumActiveParticles(st.num_fluid);
    *steps = st.steps;
    *iterations = st.iterations;
    *sum_iterations = (unsigned)st.sum_iterations;
    // Simulation::step writes a frame right after this returns when
    // TimeManager::hasToSave holds (Simulation.cpp:172-181): its test, whose
    // last save time is (frame - 1) / fps, without its side effect
    const Real fps = sim->getFPS();
    const bool due = sim->getTime() - (Real)(sim->getFrame() - 1) / fps >= 1.0 / fps;
    if (due && sim->*SimulationAccess::active_save_ptr()) return download_fluid(fm, err);
    return true;
}

}  // namespace sph_gpu

namespace {

void raise(const char* where, const std::string& err)
{
    std::fprintf(stderr, "%s: %s\n", where, err.c_str());
    throw std::runtime_error(std::string(where) + ": " + err);
}

template <typename S> void init_link(S* solver, sph_gpu::GpuSceneLink* link, const char* where)
{
    sph_gpu::CapturedScene scene;
    std::string err;
    Simulation* sim = Simulation::getCurrent();
    if (!sph_gpu::capture_scene(sim, solver, &scene, &err) || !link->create(scene, &err)) raise(where, err);
}

}  // namespace

void GpuWCSPHSolver::init()
{
    init_link(this, &link_, "GpuWCSPHSolver::init");
}

void GpuWCSPHSolver::step()
{
    std::string err;
    Simulation* sim = Simulation::getCurrent();
    if (!link_.step(sim, sim->getFluidModel(0), &steps, &iterations, &sumIterations, &err))
        raise("GpuWCSPHSolver::step", err);
}

void GpuPCISPHSolver::init()
{
    init_link(this, &link_, "GpuPCISPHSolver::init");
}

void GpuPCISPHSolver::step()
{
    std::string err;
    Simulation* sim = Simulation::getCurrent();
    if (!link_.step(sim, sim->getFluidModel(0), &steps, &iterations, &sumIterations, &err))
        raise("GpuPCISPHSolver::step", err);
}

void GpuDFSPHSolver::init()
{
    init_link(this, &link_, "GpuDFSPHSolver::init");
}

void GpuDFSPHSolver::step()
{
    std::string err;
    Simulation* sim = Simulation::getCurrent();
    if (!link_.step(sim, sim->getFluidModel(0), &steps, &iterations, &sumIterations, &err))
        raise("GpuDFSPHSolver::step", err);
}
