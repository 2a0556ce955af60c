// Headless driver for the reference simulator (josemanuel28v/SPH), used only
// as a test oracle.  It replaces the reference's GLUT front end
// (src/main.cpp:21-52, src/OGL.cpp:465-484): it builds a scene through the
// reference's own public C++ API, the same calls Simulation::importScene makes
// (src/Simulation.cpp:331-494), runs Simulation::step() a fixed number of
// times (never Simulation::run(), which does not terminate,
// src/Simulation.cpp:184-190) and writes the solver state to a binary file.
//
// Scene input: a text file of "key values..." lines (written by
// oracle/refscene.py); fluid particles come from a binary file so that every
// implementation starts from the same bits.
//
// Output: a sequence of records  {char name[48]; char type; uint64 count;
// payload}  with type 'd' (double), 'i' (int32) or 'u' (uint32).
//
// The reference's per-step LOG output goes to stdout; run with stdout
// redirected.  printInfo() waits on getchar() (src/Simulation.cpp:619): run
// with stdin from /dev/null.
#include "Simulation.h"
#include "FluidModel.h"
#include "SPHSolver.h"
#include "DFSPHSolver.h"
#include "PCISPHSolver.h"
#include "WCSPHSolver.h"
#include "AkinciBoundaryModel.h"
#include "CubeBoundaryModel.h"
#include "PCISPHBoundaryModel.h"
#include "CubicSpline.h"
#include "HashTable.h"

#include <omp.h>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>


// Read access to protected solver state through member pointers (legal C++:
// a member pointer formed in a derived class's scope applies to the base).
struct DFSPHAccess : DFSPHSolver {
    static std::vector<std::vector<Real>> DFSPHSolver::*kvPtr() { return &DFSPHAccess::kv; }
    static unsigned int DFSPHSolver::*itVPtr() { return &DFSPHAccess::iterationsV; }
    static Real DFSPHSolver::*avgDensPtr() { return &DFSPHAccess::avgDensError; }
    static Real DFSPHSolver::*avgDivPtr() { return &DFSPHAccess::avgDivError; }
};
struct SolverAccess : SPHSolver {
    static unsigned int SPHSolver::*itPtr() { return &SolverAccess::iterations; }
    static unsigned int SPHSolver::*sumItPtr() { return &SolverAccess::sumIterations; }
};
struct PCISPHAccess : PCISPHSolver {
    static Real PCISPHSolver::*maxErrPtr() { return &PCISPHAccess::maxDensityError; }
    static std::vector<Real> PCISPHSolver::*scalingPtr() { return &PCISPHAccess::scalingFactor; }
};

static FILE* g_out = nullptr;

static void put(const std::string& name, char type, const void* data, uint64_t count, size_t esize)
{
    char buf[48];
    std::memset(buf, 0, sizeof buf);
    std::strncpy(buf, name.c_str(), sizeof buf - 1);
    std::fwrite(buf, 1, sizeof buf, g_out);
    std::fwrite(&type, 1, 1, g_out);
    std::fwrite(&count, sizeof count, 1, g_out);
    if (count) std::fwrite(data, esize, count, g_out);
}
static void putd(const std::string& n, const std::vector<double>& v) { put(n, 'd', v.data(), v.size(), 8); }
static void puti(const std::string& n, const std::vector<int32_t>& v) { put(n, 'i', v.data(), v.size(), 4); }
static void putscalar(const std::string& n, double x) { put(n, 'd', &x, 1, 8); }

static std::vector<double> flat(const std::vector<Vector3r>& v, size_t n)
{
    std::vector<double> o(3 * n);
    for (size_t i = 0; i < n; ++i) { o[3 * i] = v[i].x; o[3 * i + 1] = v[i].y; o[3 * i + 2] = v[i].z; }
    return o;
}

struct Spec {
    int method = 2, boundary = 2;
    double radius = 0.025, g[3] = {0, -9.81, 0};
    double dt = 1e-4, min_dt = 1e-5, max_dt = 5e-3, fps = 60;
    double density0 = 1000, stiffness = 1000, gamma = 7;
    double eta = 0.001, eta_v = 0.001, cfl = 1.0;
    int min_it = -1, max_it = -1, min_it_v = -1, max_it_v = -1;
    int visc_method = -1, st_method = -1, adh_method = -1;
    double visc = 0, bvisc = 0, st = 0, adh = 0;
    bool has_cube = false;
    double cube[6] = {0, 0, 0, 1, 1, 1};
    std::vector<std::vector<double>> boxes, spheres;
    std::vector<std::vector<double>> bh_boxes, bh_spheres;  // + inverted flag
    std::vector<std::pair<std::string, double>> geometries;  // OBJ path, spacing (in 2r)
    // type num rx ry rz v qw qx qy qz start width height spacing
    std::vector<std::vector<double>> emitters;
    double bh_normal_fct = 0, bh_tang_fct = 1;
    std::string fluid, out;
    std::string json;         // a scene file: Simulation::importScene builds everything
    int save = 0;             // Simulation::activateSave (frames next to the scene file)
    int steps = 1;
    int dump_neighbors = 0;   // 1: neighbour sets after init and after step 1
    int dump_every = 1;       // dump full state every k steps (0: only the last)
};

static Spec read_spec(const char* path)
{
    Spec s;
    std::ifstream f(path);
    if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string k;
        if (!(is >> k) || k[0] == '#') continue;
        if (k == "method") is >> s.method;
        else if (k == "boundary") is >> s.boundary;
        else if (k == "radius") is >> s.radius;
        else if (k == "gravity") is >> s.g[0] >> s.g[1] >> s.g[2];
        else if (k == "dt") is >> s.dt;
        else if (k == "min_dt") is >> s.min_dt;
        else if (k == "max_dt") is >> s.max_dt;
        else if (k == "fps") is >> s.fps;
        else if (k == "density0") is >> s.density0;
        else if (k == "stiffness") is >> s.stiffness;
        else if (k == "gamma") is >> s.gamma;
        else if (k == "eta") is >> s.eta;
        else if (k == "eta_v") is >> s.eta_v;
        else if (k == "cfl") is >> s.cfl;
        else if (k == "min_it") is >> s.min_it;
        else if (k == "max_it") is >> s.max_it;
        else if (k == "min_it_v") is >> s.min_it_v;
        else if (k == "max_it_v") is >> s.max_it_v;
        else if (k == "visc_method") is >> s.visc_method;
        else if (k == "visc") is >> s.visc;
        else if (k == "bvisc") is >> s.bvisc;
        else if (k == "st_method") is >> s.st_method;
        else if (k == "st") is >> s.st;
        else if (k == "adh_method") is >> s.adh_method;
        else if (k == "adh") is >> s.adh;
        else if (k == "cube") { s.has_cube = true; for (double& c : s.cube) is >> c; }
        else if (k == "box") { std::vector<double> b(6); for (double& c : b) is >> c; s.boxes.push_back(b); }
        else if (k == "sphere") { std::vector<double> b(4); for (double& c : b) is >> c; s.spheres.push_back(b); }
        else if (k == "bh_box") { std::vector<double> b(7); for (double& c : b) is >> c; s.bh_boxes.push_back(b); }
        else if (k == "bh_sphere") { std::vector<double> b(5); for (double& c : b) is >> c; s.bh_spheres.push_back(b); }
        else if (k == "geometry") { std::string p; double sp; is >> p >> sp; s.geometries.emplace_back(p, sp); }
        else if (k == "emitter") { std::vector<double> b(14); for (double& c : b) is >> c; s.emitters.push_back(b); }
        else if (k == "bh_normal_fct") is >> s.bh_normal_fct;
        else if (k == "bh_tang_fct") is >> s.bh_tang_fct;
        else if (k == "fluid") is >> s.fluid;
        else if (k == "json") is >> s.json;
        else if (k == "save") is >> s.save;
        else if (k == "out") is >> s.out;
        else if (k == "steps") is >> s.steps;
        else if (k == "dump_neighbors") is >> s.dump_neighbors;
        else if (k == "dump_every") is >> s.dump_every;
        else { std::fprintf(stderr, "unknown key %s\n", k.c_str()); std::exit(2); }
    }
    return s;
}

// Neighbour sets as the reference's walks see them: the candidates of the
// particle's cell (src/Simulation.h:24-29) that lie within the cubic
// spline's support, using the same predicate as CubicSpline::W
// (q = length(ri - rj) / h, q <= 1; src/CubicSpline.h:28-33).
static void dump_neighbors(const std::string& tag, Simulation* sim)
{
    HashTable* grid = sim->getGrid();
    FluidModel* fm = sim->getFluidModel(0);
    const unsigned n = fm->getNumActiveParticles();
    const double h = sim->getSupportRadius();
    std::vector<int32_t> cells(3 * n), rank(n), offs(n + 1), nbr, cand(n), boffs(n + 1), bnbr;
    offs[0] = 0; boffs[0] = 0;
    for (unsigned i = 0; i < n; ++i) {
        Vector3r& ri = fm->getPosition(i);
        Vector3i cellId = floor(ri / h);
        cells[3 * i] = cellId.x; cells[3 * i + 1] = cellId.y; cells[3 * i + 2] = cellId.z;
        auto it = grid->table.find(cellId);
        int r = -1;
        if (it != grid->table.end()) {
            const auto& pts = it->second.points;
            for (size_t q = 0; q < pts.size(); ++q) if (pts[q].id == i) { r = (int)q; break; }
            cand[i] = (int)it->second.neighbors.size();
            for (auto& pi : it->second.neighbors) {
                Vector3r& rj = fm->getPosition(pi.id);
                const double q = length(ri - rj) / h;
                if (q <= 1.0) nbr.push_back((int32_t)pi.id);
            }
            for (auto& pi : it->second.boundary_neighbors) {
                Vector3r& rb = sim->getBoundaryModel(pi.pointSetId)->getPosition(pi.id);
                const double q = length(ri - rb) / h;
                if (q <= 1.0) bnbr.push_back((int32_t)pi.id);
            }
        }
        rank[i] = r;
        offs[i + 1] = (int32_t)nbr.size();
        boffs[i + 1] = (int32_t)bnbr.size();
    }
    puti(tag + ".cell", cells);
    puti(tag + ".cell_rank", rank);
    puti(tag + ".cand", cand);
    puti(tag + ".nbr_off", offs);
    puti(tag + ".nbr", nbr);
    puti(tag + ".bnbr_off", boffs);
    puti(tag + ".bnbr", bnbr);
}

static void dump_state(const std::string& tag, Simulation* sim, const Spec& s)
{
    FluidModel* fm = sim->getFluidModel(0);
    const unsigned n = fm->getNumActiveParticles();
    std::vector<Vector3r> x(n), v(n), a(n);
    std::vector<double> rho(n), p(n);
    for (unsigned i = 0; i < n; ++i) {
        x[i] = fm->getPosition(i); v[i] = fm->getVelocity(i); a[i] = fm->getAcceleration(i);
        rho[i] = fm->getDensity(i); p[i] = fm->getPressure(i);
    }
    putd(tag + ".x", flat(x, n));
    putd(tag + ".v", flat(v, n));
    putd(tag + ".a", flat(a, n));
    putd(tag + ".rho", rho);
    putd(tag + ".p", p);
    putscalar(tag + ".time", sim->getTime());
    putscalar(tag + ".dt", sim->getTimeStep());
    SPHSolver* solver = sim->getSolver();
    putscalar(tag + ".iterations", (double)(solver->*SolverAccess::itPtr()));
    if (s.method == Simulation::DFSPH_METHOD) {
        DFSPHSolver* d = static_cast<DFSPHSolver*>(solver);
        std::vector<double> alpha(n), div(n), pred(n), k(n), kv(n);
        for (unsigned i = 0; i < n; ++i) {
            alpha[i] = d->getAlpha(0, i); div[i] = d->getDivError(0, i);
            pred[i] = d->getPredDensity(0, i); k[i] = d->getDivergenceError(0)[i];
            kv[i] = (d->*DFSPHAccess::kvPtr())[0][i];
        }
        putd(tag + ".alpha", alpha); putd(tag + ".div", div); putd(tag + ".pred", pred);
        putd(tag + ".k", k); putd(tag + ".kv", kv);
        putscalar(tag + ".iterationsV", (double)(d->*DFSPHAccess::itVPtr()));
        putscalar(tag + ".avgDensError", d->*DFSPHAccess::avgDensPtr());
        putscalar(tag + ".avgDivError", d->*DFSPHAccess::avgDivPtr());
    }
    if (s.boundary == Simulation::PCISPH_BOUNDARY_METHOD && sim->numberBoundaryModels() > 0) {
        PCISPHBoundaryModel* bm = static_cast<PCISPHBoundaryModel*>(sim->getBoundaryModel(0));
        std::vector<double> bd(bm->size()), bp(bm->size());
        for (unsigned i = 0; i < bm->size(); ++i) { bd[i] = bm->getDensity(i); bp[i] = bm->getPressure(i); }
        std::vector<Vector3r> nrm(n);
        for (unsigned i = 0; i < n; ++i) nrm[i] = fm->getNormal(i);
        putd(tag + ".bdens", bd);
        putd(tag + ".bpress", bp);
        putd(tag + ".normal", flat(nrm, n));
    }
    if (s.method == Simulation::PCISPH_METHOD) {
        PCISPHSolver* pc = static_cast<PCISPHSolver*>(solver);
        std::vector<double> pacc(3 * n);
        for (unsigned i = 0; i < n; ++i) {
            Vector3r q = pc->getPressureAcc(0, i);
            pacc[3 * i] = q.x; pacc[3 * i + 1] = q.y; pacc[3 * i + 2] = q.z;
        }
        putd(tag + ".pacc", pacc);
        putscalar(tag + ".maxDensityError", pc->*PCISPHAccess::maxErrPtr());
        putscalar(tag + ".scaling", (pc->*PCISPHAccess::scalingPtr())[0]);
    }
}

int main(int argc, char** argv)
{
    if (argc < 2) { std::fprintf(stderr, "usage: ref_driver scene.txt\n"); return 2; }
    Spec s = read_spec(argv[1]);

    g_out = std::fopen(s.out.c_str(), "wb");
    if (!g_out) { std::fprintf(stderr, "cannot open %s\n", s.out.c_str()); return 2; }

    Simulation* sim = Simulation::getCurrent();
    FluidModel* fm = nullptr;
    if (!s.json.empty()) {
        // the reference's own scene-file path (SceneLoader::readConfiguration
        // + Simulation::importScene, which ends with init())
        if (!sim->importScene(s.json)) { std::fprintf(stderr, "importScene failed\n"); return 3; }
        s.method = sim->getSimulationMethod();
        s.boundary = sim->getBoundaryHandlingMethod();
        sim->activateSave(s.save != 0);
        fm = sim->getFluidModel(0);
    } else {
        std::vector<Vector3r> pos, vel;
        {
            FILE* f = std::fopen(s.fluid.c_str(), "rb");
            if (!f) { std::fprintf(stderr, "cannot open %s\n", s.fluid.c_str()); return 2; }
            uint64_t n = 0;
            if (std::fread(&n, 8, 1, f) != 1) return 2;
            std::vector<double> buf(6 * n);
            if (std::fread(buf.data(), 8, 6 * n, f) != 6 * n) return 2;
            std::fclose(f);
            pos.resize(n); vel.resize(n);
            for (uint64_t i = 0; i < n; ++i) {
                pos[i] = Vector3r(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]);
                vel[i] = Vector3r(buf[3 * n + 3 * i], buf[3 * n + 3 * i + 1], buf[3 * n + 3 * i + 2]);
            }
        }
        // Same sequence of calls as Simulation::importScene (src/Simulation.cpp:346-487).
        sim->setTimeStep(s.dt);
        sim->setFPS(s.fps);
        sim->setMinTimeStep(s.min_dt);
        sim->setMaxTimeStep(s.max_dt);
        sim->setStartTime(0.0);
        sim->setEndTime(1e30);
        sim->setSimulationMethod(s.method);
        sim->setBoundaryMethod(s.boundary);
        sim->setGravity(Vector3r(s.g[0], s.g[1], s.g[2]));
        sim->setParticleRadius(s.radius);
        SPHSolver* solver = sim->getSolver();
        if (s.method == Simulation::WCSPH_METHOD) {
            WCSPHSolver* w = static_cast<WCSPHSolver*>(solver);
            w->setStiffness(s.stiffness);
            w->setGamma(s.gamma);
        } else if (s.method == Simulation::PCISPH_METHOD) {
            solver->setMaxError(s.eta);
            if (s.min_it >= 0) solver->setMinIterations(s.min_it);
            if (s.max_it >= 0) solver->setMaxIterations(s.max_it);
        } else {
            DFSPHSolver* d = static_cast<DFSPHSolver*>(solver);
            d->setMaxError(s.eta);
            d->setMaxErrorV(s.eta_v);
            d->setCFLFactor(s.cfl);
            if (s.min_it >= 0) d->setMinIterations(s.min_it);
            if (s.max_it >= 0) d->setMaxIterations(s.max_it);
            if (s.min_it_v >= 0) d->setMinIterationsV(s.min_it_v);
            if (s.max_it_v >= 0) d->setMaxIterationsV(s.max_it_v);
        }
        sim->setViscosityMethod(s.visc_method);
        sim->setSurfaceTensionMethod(s.st_method);
        sim->setAdhesionMethod(s.adh_method);

        fm = sim->addFluidModel(pos, vel);
        // emitters as importScene adds them, before the fluid's forces
        // (src/Simulation.cpp:403-418, SceneLoader.cpp:123-139)
        for (auto& e : s.emitters)
            fm->addEmitter((unsigned)e[0], (unsigned)e[1], Vector3r(e[2], e[3], e[4]), e[5], Quat4r(e[6], e[7], e[8], e[9]),
                           e[10], e[11], e[12], e[13]);
        fm->setRefDensity(s.density0);
        if (s.visc_method > -1 && s.visc != 0.0) fm->setViscosityForce(s.visc, s.bvisc);
        if (s.st_method > -1 && s.st != 0.0) fm->setSurfaceTensionForce(s.st);
        if (s.adh_method > -1 && s.adh != 0.0) fm->setAdhesionForce(s.adh);

        if (s.boundary == Simulation::AKINCI_BOUNDARY_METHOD) {
            AkinciBoundaryModel* bm = new AkinciBoundaryModel();
            for (auto& b : s.boxes) bm->addCube(Vector3r(b[0], b[1], b[2]), Vector3r(b[3], b[4], b[5]));
            for (auto& b : s.spheres) bm->addSphere(Vector3r(b[0], b[1], b[2]), b[3]);
            // as importScene (src/Simulation.cpp:441-442): maximum sample distance spacing * 2r
            for (auto& gm : s.geometries) bm->addGeometry(gm.first, gm.second * s.radius * 2.0);
            sim->addBoundaryModel(bm);
        } else if (s.boundary == Simulation::PCISPH_BOUNDARY_METHOD) {
            // as Simulation::importScene builds it (src/Simulation.cpp:459-484)
            PCISPHBoundaryModel* bm = new PCISPHBoundaryModel();
            Real density0 = fm->getRefDensity();
            Real particleVolume = pow(2.0 * sim->getParticleRadius(), 3.0);
            bm->setMass(density0 * particleVolume);
            bm->setRefDensity(density0);
            bm->setNormalFct(s.bh_normal_fct);
            bm->setTangentialFct(s.bh_tang_fct);
            for (auto& b : s.bh_boxes) bm->addCube(Vector3r(b[0], b[1], b[2]), Vector3r(b[3], b[4], b[5]), b[6] != 0);
            for (auto& b : s.bh_spheres) bm->addSphere(Vector3r(b[0], b[1], b[2]), b[3], b[4] != 0);
            sim->addBoundaryModel(bm);
        } else if (s.boundary == Simulation::CUBE_BOUNDARY_METHOD && s.has_cube) {
            // importScene never creates a CubeBoundaryModel; it is added the way
            // CubeBoundaryModel::init expects: two points, min then max.
            CubeBoundaryModel* cbm = new CubeBoundaryModel();
            std::vector<Vector3r> pts = {Vector3r(s.cube[0], s.cube[1], s.cube[2]),
                                         Vector3r(s.cube[3], s.cube[4], s.cube[5])};
            cbm->init(pts);
            sim->addBoundaryModel(cbm);
        }

        sim->init();
    }

    if (s.boundary == Simulation::AKINCI_BOUNDARY_METHOD && sim->numberBoundaryModels() > 0) {
        AkinciBoundaryModel* bm = static_cast<AkinciBoundaryModel*>(sim->getBoundaryModel(0));
        std::vector<double> psi(bm->size());
        for (unsigned i = 0; i < bm->size(); ++i) psi[i] = bm->getVolume(i);
        putd("b.x", flat(bm->getPosition(), bm->size()));
        putd("b.psi", psi);
    }
    if (s.boundary == Simulation::PCISPH_BOUNDARY_METHOD && sim->numberBoundaryModels() > 0) {
        PCISPHBoundaryModel* bm = static_cast<PCISPHBoundaryModel*>(sim->getBoundaryModel(0));
        putd("b.x", flat(bm->getPosition(), bm->size()));
    }
    putscalar("h", sim->getSupportRadius());
    putscalar("mass", fm->getMass(0));
    dump_state("init", sim, s);
    if (s.dump_neighbors) dump_neighbors("init", sim);

    std::vector<double> step_seconds;
    for (int st = 1; st <= s.steps; ++st) {
        const double t0 = omp_get_wtime();
        sim->step();
        step_seconds.push_back(omp_get_wtime() - t0);
        const bool dump = (s.dump_every > 0 && st % s.dump_every == 0) || st == s.steps;
        if (dump) dump_state("s" + std::to_string(st), sim, s);
        if (st == 1 && s.dump_neighbors) dump_neighbors("s1", sim);
    }
    putd("step_seconds", step_seconds);
    std::fclose(g_out);
    return 0;
}
