/* CPU restatement of josemanuel28v/SPH's per-step particle loop.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path (tests, smoke check,
 * benchmark CPU-baseline leg).  Nothing in the product links it.
 *
 * Pinning: tests/test_oracle_pin.py runs this file and the reference's own
 * sources (compiled headless from the reference tree by `make ref`, with the
 * project's GLM shim) on the same inputs and requires identical bits for the
 * fields checked; tests/golden/ holds fixtures produced by the reference
 * build, which this oracle must reproduce when the reference tree is absent.
 *
 * Every function cites the reference function it restates (paths relative to
 * the reference repository).  Expressions are written in the reference's
 * evaluation order (C++ left-to-right, GLM component-wise vector ops), and
 * the file is compiled with -ffp-contract=off, so that sums and products
 * round exactly as the reference's parity build rounds them.
 */
#define _GNU_SOURCE
#include "sph_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* 3-vectors with GLM's component-wise semantics                             */
/* ------------------------------------------------------------------------ */
typedef struct { double x, y, z; } v3;
typedef struct { int x, y, z; } i3;

static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, double s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 smul(double s, v3 a) { return V(s * a.x, s * a.y, s * a.z); }
static inline v3 vdiv(v3 a, double s) { return V(a.x / s, a.y / s, a.z / s); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
/* glm::dot: (x*x' + y*y') + z*z' */
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vlen(v3 a) { return sqrt(vdot(a, a)); }
static inline double dmax(double a, double b) { return a < b ? b : a; }
static inline double dmin(double a, double b) { return b < a ? b : a; }

/* ------------------------------------------------------------------------ */
/* Smoothing kernels (src/CubicSpline.h, Poly6.h, Spiky.h, ViscoK.h,        */
/* Cohesion.h, Adhesion.h).  Coefficients as in each setSupportRadius.      */
/* ------------------------------------------------------------------------ */
typedef struct {
    double h;
    double cs_k, cs_l;                    /* CubicSpline.h:18-26 */
    double p6_h2, p6_value, p6_grad;      /* Poly6.h:19-28 */
    double sp_value, sp_grad;             /* Spiky.h:18-27 */
    double vk_lapl;                       /* ViscoK.h:18-26 */
    double co_c1, co_c2;                  /* Cohesion.h:20-27 */
} kernels;

static void kernels_init(kernels* k, double sr)
{
    const double pi = M_PI;
    const double h3 = sr * sr * sr;
    const double h6 = sr * sr * sr * sr * sr * sr;
    const double h9 = sr * sr * sr * sr * sr * sr * sr * sr * sr;
    k->h = sr;
    k->cs_k = 8.0 / (pi * h3);
    k->cs_l = 48.0 / (pi * h3);
    k->p6_h2 = sr * sr;
    k->p6_value = 315.0 / (64.0 * M_PI * h9);
    k->p6_grad = 945.0 / (32.0 * M_PI * h9);
    k->sp_value = 15.0 / (M_PI * h6);
    k->sp_grad = 45.0 / (M_PI * h6);
    k->vk_lapl = 45 / (M_PI * h6);
    k->co_c1 = 32.0 / (M_PI * h9);
    k->co_c2 = h6 / 64.0;
}

/* CubicSpline::W(Real) CubicSpline.h:28-46 */
static inline double cubic_W(const kernels* k, double r)
{
    double res = 0.0;
    const double q = r / k->h;
    if (q <= 1.0) {
        if (q <= 0.5) {
            const double q2 = q * q;
            const double q3 = q2 * q;
            res = k->cs_k * (6.0 * q3 - 6.0 * q2 + 1.0);
        } else {
            res = k->cs_k * (2.0 * pow(1.0 - q, 3.0));
        }
    }
    return res;
}
static inline double cubic_Wv(const kernels* k, v3 r) { return cubic_W(k, vlen(r)); }

/* CubicSpline::gradW CubicSpline.h:53-73 */
static inline v3 cubic_gradW(const kernels* k, v3 r)
{
    v3 res = V(0.0, 0.0, 0.0);
    const double rl = vlen(r);
    const double q = rl / k->h;
    if ((rl > 1.0e-5) && (q <= 1.0)) {
        const v3 gradq = vmul(r, 1.0 / (rl * k->h));
        if (q <= 0.5) {
            res = smul(k->cs_l * q * (3.0 * q - 2.0), gradq);
        } else {
            const double factor = 1.0 - q;
            res = smul(k->cs_l * (-factor * factor), gradq);
        }
    }
    return res;
}

/* Poly6::W Poly6.h:30-43 */
static inline double poly6_W(const kernels* k, v3 r)
{
    const double mod_r = vlen(r);
    const double mod_r2 = mod_r * mod_r;
    if (mod_r2 <= k->p6_h2) {
        const double diff = k->p6_h2 - mod_r2;
        return k->p6_value * diff * diff * diff;
    }
    return 0.0;
}
/* Poly6::gradW Poly6.h:45-57 */
static inline v3 poly6_gradW(const kernels* k, v3 r)
{
    const double mod_r = vlen(r);
    const double mod_r2 = mod_r * mod_r;
    if (mod_r2 <= k->p6_h2) {
        const double diff = k->p6_h2 - mod_r2;
        return smul(-diff * diff * k->p6_grad, r);
    }
    return V(0.0, 0.0, 0.0);
}
/* Spiky::gradW Spiky.h:43-55 */
static inline v3 spiky_gradW(const kernels* k, v3 r)
{
    const double mod_r = vlen(r);
    if (mod_r != 0 && mod_r <= k->h) {
        const double diff = k->h - mod_r;
        return smul(-k->sp_grad * diff * diff / mod_r, r);
    }
    return V(0.0, 0.0, 0.0);
}
/* ViscoK::laplW ViscoK.h:27-35 */
static inline double visc_laplW(const kernels* k, v3 r)
{
    const double mod_r = vlen(r);
    if (mod_r <= k->h) return k->vk_lapl * (k->h - mod_r);
    return 0.0;
}
/* Cohesion::W Cohesion.h:29-40 */
static inline double cohesion_W(const kernels* k, v3 r)
{
    double value = 0;
    const double mod_r = vlen(r);
    const double sr = k->h;
    if ((2.0 * mod_r > sr) && (mod_r <= sr))
        value = k->co_c1 * pow(sr - mod_r, 3.0) * pow(mod_r, 3.0);
    else if ((mod_r > 0) && (2.0 * mod_r <= sr))
        value = k->co_c1 * 2.0 * pow(sr - mod_r, 3.0) * pow(mod_r, 3.0) - k->co_c2;
    return value;
}
/* Adhesion::W Adhesion.h:23-35 (its valueCoef is computed but never applied) */
static inline double adhesion_W(const kernels* k, v3 r)
{
    const double mod_r = vlen(r);
    const double sr = k->h;
    if ((2.0 * mod_r > sr) && (mod_r <= sr)) {
        const double value = -4.0 * mod_r * mod_r / sr + 6 * mod_r - 2 * sr;
        return pow(value, 1.0 / 4.0);
    }
    return 0.0;
}

/* ------------------------------------------------------------------------ */
/* Spatial hash grid (src/HashTable.h).  Cells are floor(x / h); each cell   */
/* holds its fluid and boundary points in insertion (= index) order and the  */
/* candidate lists built by concatenating the 27 surrounding cells in        */
/* x -> y -> z offset order (HashTable.h:136-170).                            */
/* ------------------------------------------------------------------------ */
typedef struct {
    unsigned cap;        /* hash slots (power of two) */
    int* slot;           /* cell index or -1 */
    i3* key;             /* per cell */
    unsigned ncells, maxcells;
    unsigned *fstart, *fpts;  /* fluid points CSR */
    unsigned *bstart, *bpts;  /* boundary points CSR */
    unsigned *cstart, *cand;  /* fluid candidates CSR */
    unsigned *bcstart, *bcand;/* boundary candidates CSR */
    size_t cand_cap, bcand_cap;
    unsigned* fcell;     /* cell of each fluid particle at insertion */
    unsigned* bcell;
    unsigned nbuilt;     /* cells that have candidate lists (the last build's) */
} grid;

/* HashTable.h:26-29 (computed in int, as the reference does) */
static inline size_t cell_hash(i3 c)
{
    return (size_t)(unsigned)((unsigned)c.x * 73856093u + (unsigned)c.y * 19349663u + (unsigned)c.z * 83492791u);
}

static inline i3 cell_of(double x, double y, double z, double h)
{
    i3 c = {(int)floor(x / h), (int)floor(y / h), (int)floor(z / h)};
    return c;
}

static int grid_find(const grid* g, i3 c)
{
    if (!g->cap) return -1;
    size_t m = g->cap - 1, p = cell_hash(c) & m;
    for (;;) {
        int s = g->slot[p];
        if (s < 0) return -1;
        if (g->key[s].x == c.x && g->key[s].y == c.y && g->key[s].z == c.z) return s;
        p = (p + 1) & m;
    }
}

static void grid_rehash(grid* g, unsigned cap)
{
    free(g->slot);
    g->cap = cap;
    g->slot = (int*)malloc(cap * sizeof(int));
    for (unsigned i = 0; i < cap; ++i) g->slot[i] = -1;
    for (unsigned c = 0; c < g->ncells; ++c) {
        size_t m = cap - 1, p = cell_hash(g->key[c]) & m;
        while (g->slot[p] >= 0) p = (p + 1) & m;
        g->slot[p] = (int)c;
    }
}

/* unordered_map::operator[]: find or create (cells are never erased,
 * HashTable.h:176-196) */
static int grid_insert(grid* g, i3 c)
{
    int f = grid_find(g, c);
    if (f >= 0) return f;
    if (g->ncells + 1 > g->maxcells) {
        unsigned mc = g->maxcells ? 2 * g->maxcells : 4096;
        g->key = (i3*)realloc(g->key, mc * sizeof(i3));
        g->maxcells = mc;
    }
    if (2 * (g->ncells + 1) > g->cap) grid_rehash(g, g->cap ? 2 * g->cap : 8192);
    const int s = (int)g->ncells++;
    g->key[s] = c;
    size_t m = g->cap - 1, p = cell_hash(c) & m;
    while (g->slot[p] >= 0) p = (p + 1) & m;
    g->slot[p] = s;
    return s;
}

struct orc_scene {
    orc_params prm;
    double h, mass;
    kernels K;
    /* fluid (FluidModel.h:14-27), one fluid model */
    unsigned n;
    v3 *x, *v, *a;
    double *rho, *p;
    /* DFSPH (DFSPHSolver.h:12-31) */
    double *alpha, *div, *pred, *k, *kv;
    double avgDensError, avgDivError, eps;
    unsigned iterations, iterationsV, steps, sumIterations, sumIterationsV;
    unsigned min_it, max_it, min_it_v, max_it_v;
    double maxError, maxErrorV, cflFactor;
    /* PCISPH (PCISPHSolver.h:12-17) */
    v3 *predR, *predV, *pacc;
    double scaling, maxDensityError;
    /* surface tension normals (SurfaceTensionAkinci.h:23) */
    v3* normal;
    /* Akinci boundary (AkinciBoundaryModel.h:13-15) */
    unsigned nb, nb_cap;
    v3* bx;
    double* psi;
    /* solver weight of each boundary particle: rho0 psi_b (Akinci) or the
     * PCISPH model's mass (PCISPHBoundaryModel.h:13-24, Simulation.cpp:464-468) */
    double* bw;
    /* PCISPH boundary model: normals, densities, pressures */
    v3* bn;
    double *bdens, *bpress;
    double bmass;
    /* TimeManager (TimeManager.h:20-33) */
    double time, ts, minTs, maxTs;
    double maxVel;
    grid g;
    int inited;
    /* emitters (FluidModel.h:28, Emitter.h:9-40): n is numActiveParticles,
     * cap is numParticles (initial fluid plus every emitter's reservation) */
    unsigned cap;
    unsigned nem;
    struct orc_emitter {
        int type;
        unsigned numParticles;
        v3 r;
        double v, rot[4];            /* rot: w, x, y, z */
        double nextTimeEmit, spacing;
        int pause;
        v3* group;
        unsigned ng;
    } em[64];
};

static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

static void grid_free(grid* g)
{
    free(g->slot); free(g->key); free(g->fstart); free(g->fpts); free(g->bstart); free(g->bpts);
    free(g->cstart); free(g->cand); free(g->bcstart); free(g->bcand); free(g->fcell); free(g->bcell);
    memset(g, 0, sizeof *g);
}

/* SPHSolver::insertFluidParticles + insertBoundaryParticles + HashTable::
 * neighborhoodSearch (SPHSolver.cpp:172-221, HashTable.h:79-102,136-170).
 * Every cell ever created stays in the table with its point lists refilled
 * from the current points, and every cell gets its candidate lists, as the
 * reference's clear()-but-never-erase table does. */
static void grid_build(orc_scene* s)
{
    grid* g = &s->g;
    const double h = s->h;
    free(g->fcell); free(g->bcell); free(g->fpts); free(g->bpts);
    g->fcell = (unsigned*)xcalloc(s->n, sizeof(unsigned));
    g->bcell = (unsigned*)xcalloc(s->nb, sizeof(unsigned));
    g->fpts = (unsigned*)xcalloc(s->n, sizeof(unsigned));
    g->bpts = (unsigned*)xcalloc(s->nb, sizeof(unsigned));
    for (unsigned b = 0; b < s->nb; ++b)
        g->bcell[b] = (unsigned)grid_insert(g, cell_of(s->bx[b].x, s->bx[b].y, s->bx[b].z, h));
    for (unsigned i = 0; i < s->n; ++i)
        g->fcell[i] = (unsigned)grid_insert(g, cell_of(s->x[i].x, s->x[i].y, s->x[i].z, h));
    const unsigned nc = g->ncells;
    free(g->fstart); free(g->bstart); free(g->cstart); free(g->bcstart);
    g->fstart = (unsigned*)xcalloc(nc + 1, sizeof(unsigned));
    g->bstart = (unsigned*)xcalloc(nc + 1, sizeof(unsigned));
    g->cstart = (unsigned*)xcalloc(nc + 1, sizeof(unsigned));
    g->bcstart = (unsigned*)xcalloc(nc + 1, sizeof(unsigned));
    for (unsigned i = 0; i < s->n; ++i) g->fstart[g->fcell[i] + 1]++;
    for (unsigned b = 0; b < s->nb; ++b) g->bstart[g->bcell[b] + 1]++;
    for (unsigned c = 0; c < nc; ++c) { g->fstart[c + 1] += g->fstart[c]; g->bstart[c + 1] += g->bstart[c]; }
    {
        unsigned* fill = (unsigned*)xcalloc(nc, sizeof(unsigned));
        for (unsigned i = 0; i < s->n; ++i) { unsigned c = g->fcell[i]; g->fpts[g->fstart[c] + fill[c]++] = i; }
        memset(fill, 0, nc * sizeof(unsigned));
        for (unsigned b = 0; b < s->nb; ++b) { unsigned c = g->bcell[b]; g->bpts[g->bstart[c] + fill[c]++] = b; }
        free(fill);
    }
    /* candidate counts */
    #pragma omp parallel for schedule(static)
    for (unsigned c = 0; c < nc; ++c) {
        unsigned fc = 0, bc = 0;
        const i3 k = g->key[c];
        for (int dx = -1; dx <= 1; dx++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dz = -1; dz <= 1; dz++) {
                    i3 nk = {k.x + dx, k.y + dy, k.z + dz};
                    int nc2 = grid_find(g, nk);
                    if (nc2 >= 0) {
                        fc += g->fstart[nc2 + 1] - g->fstart[nc2];
                        bc += g->bstart[nc2 + 1] - g->bstart[nc2];
                    }
                }
        g->cstart[c + 1] = fc;
        g->bcstart[c + 1] = bc;
    }
    for (unsigned c = 0; c < nc; ++c) { g->cstart[c + 1] += g->cstart[c]; g->bcstart[c + 1] += g->bcstart[c]; }
    g->nbuilt = nc;
    if (g->cstart[nc] > g->cand_cap) { free(g->cand); g->cand_cap = g->cstart[nc]; g->cand = (unsigned*)xcalloc(g->cand_cap, sizeof(unsigned)); }
    if (g->bcstart[nc] > g->bcand_cap) { free(g->bcand); g->bcand_cap = g->bcstart[nc]; g->bcand = (unsigned*)xcalloc(g->bcand_cap, sizeof(unsigned)); }
    #pragma omp parallel for schedule(static)
    for (unsigned c = 0; c < nc; ++c) {
        unsigned fo = g->cstart[c], bo = g->bcstart[c];
        const i3 k = g->key[c];
        for (int dx = -1; dx <= 1; dx++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dz = -1; dz <= 1; dz++) {
                    i3 nk = {k.x + dx, k.y + dy, k.z + dz};
                    int nc2 = grid_find(g, nk);
                    if (nc2 >= 0) {
                        for (unsigned q = g->fstart[nc2]; q < g->fstart[nc2 + 1]; ++q) g->cand[fo++] = g->fpts[q];
                        for (unsigned q = g->bstart[nc2]; q < g->bstart[nc2 + 1]; ++q) g->bcand[bo++] = g->bpts[q];
                    }
                }
    }
}

/* The candidate lists of the cell holding position p, looked up at walk time
 * as `grid->table[cellId]` does (Simulation.h:15-44): a cell with no points
 * has no candidates. */
typedef struct { const unsigned *f, *b; unsigned nf, nbn; } cands;
static inline cands cands_at(const orc_scene* s, v3 p)
{
    cands r = {0, 0, 0, 0};
    int c = grid_find(&s->g, cell_of(p.x, p.y, p.z, s->h));
    if (c >= 0 && (unsigned)c < s->g.nbuilt) {
        r.f = s->g.cand + s->g.cstart[c];
        r.nf = s->g.cstart[c + 1] - s->g.cstart[c];
        r.b = s->g.bcand + s->g.bcstart[c];
        r.nbn = s->g.bcstart[c + 1] - s->g.bcstart[c];
    }
    return r;
}

static int akinci(const orc_scene* s) { return s->prm.boundary == 2; }
/* PCISPH boundary model (Simulation::PCISPH_BOUNDARY_METHOD) */
static int bh(const orc_scene* s) { return s->prm.boundary == 1; }
/* boundary particles take part in the solver sums (Akinci: weight rho0 psi_b,
 * PCISPH model: the model's mass) */
static int hasb(const orc_scene* s) { return s->prm.boundary == 1 || s->prm.boundary == 2; }

/* grid->table[cellId] as a lookup that creates the cell when missing
 * (unordered_map::operator[]): a cell created since the last neighbour
 * search has no candidates. */
static cands cands_at_create(orc_scene* s, v3 p)
{
    const i3 k = cell_of(p.x, p.y, p.z, s->h);
    if (grid_find(&s->g, k) < 0) grid_insert(&s->g, k);
    return cands_at(s, p);
}

/* ------------------------------------------------------------------------ */
/* Shared solver passes (src/SPHSolver.cpp)                                  */
/* ------------------------------------------------------------------------ */

/* SPHSolver::computeFluidDensities SPHSolver.cpp:44-91 */
static void compute_densities(orc_scene* s)
{
    const int hb = hasb(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i];
        cands c = cands_at(s, ri);
        double density = 0;
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            density += s->mass * cubic_Wv(&s->K, vsub(ri, s->x[j]));
        }
        if (hb)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                density += s->bw[b] * cubic_Wv(&s->K, vsub(ri, s->bx[b]));
            }
        s->rho[i] = density;
    }
}

/* AkinciBoundaryModel::computeVolume AkinciBoundayModel.cpp:11-40 */
static void compute_volume(orc_scene* s)
{
    #pragma omp parallel for
    for (unsigned i = 0; i < s->nb; ++i) {
        const v3 ri = s->bx[i];
        cands c = cands_at(s, ri);
        double delta = 0.0;
        for (unsigned q = 0; q < c.nbn; ++q) delta += cubic_Wv(&s->K, vsub(ri, s->bx[c.b[q]]));
        s->psi[i] = 1.0 / delta;
    }
}

/* SPHSolver::integrate SPHSolver.cpp:141-170 */
static void integrate_symplectic(orc_scene* s)
{
    const double ts = s->ts;
    const v3 g = V(s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2]);
    double maxVel = 0.0;
    for (unsigned i = 0; i < s->n; ++i) {
        s->a[i] = vadd(s->a[i], g);
        s->v[i] = vadd(s->v[i], vmul(s->a[i], ts));
        s->x[i] = vadd(s->x[i], vmul(s->v[i], ts));
        s->a[i] = V(0, 0, 0);
        maxVel = dmax(maxVel, vlen(s->v[i]));
    }
    s->maxVel = maxVel;
}

/* CubeBoundaryModel::correctPositionAndVelocity CubeBoundaryModel.cpp:16-94
 * with the factors CubeBoundaryModel::init sets (normal 0, tangential 1). */
static void cube_correct(orc_scene* s)
{
    const double normalFct = 0.0, tangentialFct = 1.0;
    const double* mn = s->prm.cube_min;
    const double* mx = s->prm.cube_max;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; i++) {
        v3 pos = s->x[i], vel = s->v[i];
        if (pos.x < mn[0]) { pos.x = mn[0]; if (vel.x < 0.f) vel.x *= -normalFct; vel.y *= tangentialFct; vel.z *= tangentialFct; }
        else if (pos.x > mx[0]) { pos.x = mx[0]; if (vel.x > 0.f) vel.x *= -normalFct; vel.y *= tangentialFct; vel.z *= tangentialFct; }
        if (pos.y < mn[1]) { pos.y = mn[1]; if (vel.y < 0.f) vel.y *= -normalFct; vel.x *= tangentialFct; vel.z *= tangentialFct; }
        else if (pos.y > mx[1]) { pos.y = mx[1]; if (vel.y > 0.f) vel.y *= -normalFct; vel.x *= tangentialFct; vel.z *= tangentialFct; }
        if (pos.z < mn[2]) { pos.z = mn[2]; if (vel.z < 0.f) vel.z *= -normalFct; vel.x *= tangentialFct; vel.y *= tangentialFct; }
        else if (pos.z > mx[2]) { pos.z = mx[2]; if (vel.z > 0.f) vel.z *= -normalFct; vel.x *= tangentialFct; vel.y *= tangentialFct; }
        s->x[i] = pos; s->v[i] = vel;
    }
}

/* ------------------------------------------------------------------------ */
/* Non-pressure forces (Simulation::computeNonPressureForces                 */
/* Simulation.cpp:313-323; created in the order viscosity, surface tension,  */
/* adhesion, FluidModel.cpp:73-122 via Simulation.cpp:423-430)               */
/* ------------------------------------------------------------------------ */

/* XSPHViscosity::step XSPHViscosity.h:32-69 */
static void force_xsph(orc_scene* s)
{
    const double density0 = s->prm.density0, visc = s->prm.visc, bvisc = s->prm.bvisc, ts = s->ts;
    const int ak = akinci(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; i++) {
        const v3 ri = s->x[i], vi = s->v[i];
        v3 ai = s->a[i];
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const v3 rj = s->x[j], vj = s->v[j];
            ai = vadd(ai, vdiv(vmul(smul(visc * (s->mass / s->rho[j]), vsub(vj, vi)), cubic_Wv(&s->K, vsub(ri, rj))), ts));
        }
        if (bvisc != 0.0 && ak)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                ai = vadd(ai, vdiv(vmul(smul(bvisc * (density0 * s->psi[b] / s->rho[i]), vneg(vi)),
                                        cubic_Wv(&s->K, vsub(ri, s->bx[b]))), ts));
            }
        s->a[i] = ai;
    }
}

/* StandardViscosityForce::step StandardViscosityForce.h:29-79 */
static void force_standard_viscosity(orc_scene* s)
{
    const double density0 = s->prm.density0, visc = s->prm.visc, bvisc = s->prm.bvisc;
    const int ak = akinci(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i], vi = s->v[i];
        v3 ai = s->a[i];
        v3 viscoForce = V(0.0, 0.0, 0.0);
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            viscoForce = vadd(viscoForce, vmul(vdiv(smul(s->mass, vsub(s->v[j], vi)), s->rho[j]),
                                               visc_laplW(&s->K, vsub(ri, s->x[j]))));
        }
        double kinematicVisco = visc / density0;
        viscoForce = vmul(viscoForce, kinematicVisco);
        ai = vadd(ai, viscoForce);
        viscoForce = V(0.0, 0.0, 0.0);
        if (bvisc != 0.0 && ak) {
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                viscoForce = vadd(viscoForce, vmul(vdiv(smul(density0 * s->psi[b], vneg(vi)), s->rho[i]),
                                                   visc_laplW(&s->K, vsub(ri, s->bx[b]))));
            }
            kinematicVisco = bvisc / density0;
            viscoForce = vmul(viscoForce, kinematicVisco);
            ai = vadd(ai, viscoForce);
        }
        s->a[i] = ai;
    }
}

/* ArtificialViscosity::step ArtificialViscosity.h:31-83 */
static void force_artificial_viscosity(orc_scene* s)
{
    const double density0 = s->prm.density0, visc = s->prm.visc, bvisc = s->prm.bvisc;
    const double h2 = s->h * s->h;
    const int ak = akinci(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; i++) {
        const v3 ri = s->x[i], vi = s->v[i];
        v3 ai = s->a[i];
        const double dens_i = s->rho[i];
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const v3 rirj = vsub(ri, s->x[j]);
            const double dotProd = vdot(vsub(vi, s->v[j]), rirj);
            const double dens_j = s->rho[j];
            const double sqDist = vlen(rirj) * vlen(rirj);
            const double kij = 2 * density0 / (dens_i + dens_j);
            ai = vadd(ai, smul(kij * 10.0 * 0.1 * visc * (s->mass / dens_j) * dotProd / (sqDist + 0.01 * h2),
                               cubic_gradW(&s->K, rirj)));
        }
        if (bvisc != 0.0 && ak)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                const v3 rirb = vsub(ri, s->bx[b]);
                const double dotProd = vdot(vi, rirb);
                const double sqDist = vlen(rirb) * vlen(rirb);
                ai = vadd(ai, smul(10.0 * 0.1 * bvisc * (density0 * s->psi[b] / dens_i) * dotProd / (sqDist + 0.01 * h2),
                                   cubic_gradW(&s->K, rirb)));
            }
        s->a[i] = ai;
    }
}

/* SurfaceTensionAkinci::step SurfaceTensionAkinci.h:34-98 */
static void force_surface_tension(orc_scene* s)
{
    const double density0 = s->prm.density0, stCoef = s->prm.st, sr = s->h;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; i++) {
        const v3 ri = s->x[i];
        v3 ni = V(0.0, 0.0, 0.0);
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const double vol = s->mass / s->rho[j];
            ni = vadd(ni, smul(vol, cubic_gradW(&s->K, vsub(ri, s->x[j]))));
        }
        ni = vmul(ni, 1.0 * sr);
        s->normal[i] = ni;
    }
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; i++) {
        const v3 ri = s->x[i], ni = s->normal[i];
        v3 ai = s->a[i];
        const double dens_i = s->rho[i];
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const v3 rj = s->x[j], nj = s->normal[j];
            const double dens_j = s->rho[j];
            const v3 rij = vsub(ri, rj);
            const double rijMag = vlen(rij);
            const double kij = 2.0 * density0 / (dens_i + dens_j);
            if (rijMag > 0.0 && rijMag <= sr) {
                const v3 cohesion = vdiv(smul(-s->mass * cohesion_W(&s->K, rij), rij), rijMag);
                const v3 curvature = smul(-1.0, vsub(ni, nj));
                ai = vadd(ai, smul(stCoef * kij, vadd(cohesion, curvature)));
            }
        }
        s->a[i] = ai;
    }
}

/* AdhesionForce::step AdhesionForce.h:30-62 */
static void force_adhesion(orc_scene* s)
{
    const double density0 = s->prm.density0, beta = s->prm.adh;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; i++) {
        const v3 ri = s->x[i];
        v3 ai = s->a[i];
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nbn; ++q) {
            unsigned b = c.b[q];
            const v3 rib = vsub(ri, s->bx[b]);
            const double mod_rib = vlen(rib);
            if (mod_rib > 0.0)
                ai = vsub(ai, vdiv(smul(beta * density0 * s->psi[b] * adhesion_W(&s->K, rib), rib), mod_rib));
        }
        s->a[i] = ai;
    }
}

static void non_pressure_forces(orc_scene* s)
{
    const orc_params* p = &s->prm;
    if (p->visc_method > -1 && p->visc != 0.0) {
        if (p->visc_method == 0) force_standard_viscosity(s);
        else if (p->visc_method == 1) force_artificial_viscosity(s);
        else if (p->visc_method == 2) force_xsph(s);
    }
    if (p->st_method == 3 && p->st != 0.0) force_surface_tension(s);
    if (p->adh_method == 4 && p->adh != 0.0) force_adhesion(s);
}

/* ------------------------------------------------------------------------ */
/* DFSPH (src/DFSPHSolver.cpp)                                               */
/* ------------------------------------------------------------------------ */

/* ------------------------------------------------------------------------ */
/* PCISPH boundary model (src/PCISPHBoundaryModel.cpp, SPHSolver.cpp)         */
/* ------------------------------------------------------------------------ */

/* SPHSolver::computeBoundaryDensities SPHSolver.cpp:94-127 */
static void bh_boundary_densities(orc_scene* s)
{
    #pragma omp parallel for
    for (unsigned i = 0; i < s->nb; ++i) {
        const v3 ri = s->bx[i];
        cands c = cands_at(s, ri);
        double density = 0;
        for (unsigned q = 0; q < c.nf; ++q) density += s->mass * cubic_Wv(&s->K, vsub(ri, s->x[c.f[q]]));
        for (unsigned q = 0; q < c.nbn; ++q) density += s->bmass * cubic_Wv(&s->K, vsub(ri, s->bx[c.b[q]]));
        s->bdens[i] = density;
    }
}

/* Collision weights of fluid particle i against the boundary points within
 * restRadius = h/2 of `ri` (PCISPHBoundaryModel.cpp:219-316, 394-448): the
 * weight uses the distance from `rw` (the current or the predicted position).
 * Returns 1 and the correction displacement when some weight is positive;
 * always writes the particle's normal (normalize of the weighted normal sum,
 * NaN when no point is within restRadius). */
static int bh_collide(orc_scene* s, unsigned i, v3 ri, v3 rw, v3* disp)
{
    const double restRadius = 0.5 * s->h;
    v3 avg_normal = V(0, 0, 0);
    double w_sum = 0, w2_sum = 0;
    /* the loops run serially in the reference: cells are created in order */
    cands c = cands_at_create(s, ri);
    for (unsigned q = 0; q < c.nbn; ++q) {
        const unsigned b = c.b[q];
        const v3 rb = s->bx[b];
        const v3 prib = vsub(rw, rb);
        if (vlen(vsub(ri, rb)) < restRadius) {
            const double w = dmax(0.0, (restRadius - vlen(prib)) / restRadius);
            w_sum += w;
            w2_sum += w * (restRadius - vlen(prib));
            avg_normal = vadd(avg_normal, smul(w, s->bn[b]));
        }
    }
    const v3 ni = vmul(avg_normal, 1.0 / sqrt(vdot(avg_normal, avg_normal)));
    s->normal[i] = ni;
    if (w_sum > 0) {
        *disp = smul(1.0 / w_sum * w2_sum, ni);
        return 1;
    }
    return 0;
}

/* PCISPHBoundaryModel::correctPositions :219-316 (pred: the PCISPH form,
 * weights from the predicted positions) */
static void bh_correct_positions(orc_scene* s, int pred)
{
    for (unsigned i = 0; i < s->n; ++i) {
        v3 d;
        if (bh_collide(s, i, s->x[i], pred ? s->predR[i] : s->x[i], &d)) s->x[i] = vadd(s->x[i], d);
    }
}

/* PCISPHBoundaryModel::correctPredPositions :394-448 */
static void bh_correct_pred_positions(orc_scene* s)
{
    for (unsigned i = 0; i < s->n; ++i) {
        v3 d;
        if (bh_collide(s, i, s->x[i], s->predR[i], &d)) s->predR[i] = vadd(s->predR[i], d);
    }
}

/* PCISPHBoundaryModel::correctVelocities :318-392: reflect the normal part
 * of the velocity (PCISPH: of the predicted velocity) for particles whose
 * normal is valid */
static void bh_correct_velocities(orc_scene* s, int pred)
{
    const double nf = s->prm.bh_normal_fct, tf = s->prm.bh_tang_fct;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ni = s->normal[i];
        if (vlen(ni) > 0) {
            const v3 u = pred ? s->predV[i] : s->v[i];
            const v3 nVel = smul(vdot(u, ni), ni);
            const v3 tVel = vsub(u, nVel);
            s->v[i] = vsub(smul(tf, tVel), smul(nf, nVel));
        }
    }
}

/* DFSPHSolver::computeAlpha DFSPHSolver.cpp:114-189 */
static void dfsph_alpha(orc_scene* s)
{
    const int hb = hasb(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i];
        cands c = cands_at(s, ri);
        v3 sumGrad = V(0.0, 0.0, 0.0);
        double sumSqGrad = 0.0;
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const v3 massGrad = smul(s->mass, cubic_gradW(&s->K, vsub(ri, s->x[j])));
            const double massGradMag = vlen(massGrad);
            sumGrad = vadd(sumGrad, massGrad);
            sumSqGrad += massGradMag * massGradMag;
        }
        if (hb)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                const v3 massGrad = smul(s->bw[b], cubic_gradW(&s->K, vsub(ri, s->bx[b])));
                sumGrad = vadd(sumGrad, massGrad);
            }
        const double sumGradMag = vlen(sumGrad);
        const double denominator = sumGradMag * sumGradMag + sumSqGrad;
        if (fabs(denominator) > s->eps) s->alpha[i] = s->rho[i] / denominator;
        else s->alpha[i] = 0.0;
    }
}

/* DFSPHSolver::predictVelocities DFSPHSolver.cpp:191-214 */
static void dfsph_predict_velocities(orc_scene* s)
{
    const double ts = s->ts;
    const v3 g = V(s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2]);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 acc = vadd(s->a[i], g);
        s->v[i] = vadd(s->v[i], vmul(acc, ts));
        s->a[i] = V(0.0, 0.0, 0.0);
    }
}

/* DFSPHSolver::updatePositions DFSPHSolver.cpp:216-236 */
static void dfsph_update_positions(orc_scene* s)
{
    const double ts = s->ts;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) s->x[i] = vadd(s->x[i], vmul(s->v[i], ts));
}

/* DFSPHSolver::predictDensities DFSPHSolver.cpp:238-309 */
static void dfsph_predict_densities(orc_scene* s)
{
    const double density0 = s->prm.density0, ts = s->ts;
    const int hb = hasb(s);
    double avgDensError = 0.0;
    #pragma omp parallel for reduction(+ : avgDensError)
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i], vi = s->v[i];
        double densityChange = 0;
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            densityChange += s->mass * vdot(vsub(vi, s->v[j]), cubic_gradW(&s->K, vsub(ri, s->x[j])));
        }
        if (hb)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                densityChange += s->bw[b] * vdot(vi, cubic_gradW(&s->K, vsub(ri, s->bx[b])));
            }
        double pred = s->rho[i] + densityChange * ts;
        pred = dmax(pred, density0);
        s->pred[i] = pred;
        avgDensError += (pred - density0) / density0;
    }
    if (s->n == 0) avgDensError = 0;
    else avgDensError /= s->n;
    s->avgDensError = avgDensError;
}

/* DFSPHSolver::densityWarmStart DFSPHSolver.cpp:592-690 */
static void dfsph_density_warm_start(orc_scene* s)
{
    const double ts = s->ts, ts2 = ts * ts;
    const int hb = hasb(s);
    const int bhm = bh(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const double dens_i = s->rho[i];
        s->k[i] = -dmax(-s->k[i] / dens_i, -0.000000001) / ts2;
    }
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i];
        v3 sum = V(0.0, 0.0, 0.0);
        const double ki = s->k[i];
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const double kSum = (ki + s->k[j]);
            if (fabs(kSum) > s->eps) sum = vadd(sum, smul(s->mass * kSum, cubic_gradW(&s->K, vsub(ri, s->x[j]))));
        }
        if (hb)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                const double kSum = bhm ? ki : 2.0 * ki;   /* DFSPHSolver.cpp:646-672 */
                if (fabs(kSum) > s->eps)
                    sum = vadd(sum, smul(s->bw[b] * kSum, cubic_gradW(&s->K, vsub(ri, s->bx[b]))));
            }
        s->v[i] = vsub(s->v[i], vmul(sum, ts));
    }
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) s->k[i] = 0.0;
}

/* DFSPHSolver::correctDensityError DFSPHSolver.cpp:311-406 */
static void dfsph_correct_density_error(orc_scene* s)
{
    const double density0 = s->prm.density0, ts = s->ts, ts2 = ts * ts;
    const int hb = hasb(s);
    dfsph_density_warm_start(s);
    dfsph_predict_densities(s);
    s->iterations = 0;
    s->avgDensError = 0;
    while (((s->avgDensError > s->maxError) || (s->iterations < s->min_it)) && s->iterations < s->max_it) {
        #pragma omp parallel for
        for (unsigned i = 0; i < s->n; ++i) {
            const v3 ri = s->x[i];
            const double dens_i = s->rho[i], predDens_i = s->pred[i], alpha_i = s->alpha[i];
            v3 sum = V(0.0, 0.0, 0.0);
            const double ki = (predDens_i - density0) * alpha_i / (ts2 * dens_i);
            s->k[i] += (predDens_i - density0) * alpha_i;
            cands c = cands_at(s, ri);
            for (unsigned q = 0; q < c.nf; ++q) {
                unsigned j = c.f[q];
                const double kj = (s->pred[j] - density0) * s->alpha[j] / (ts2 * s->rho[j]);
                const double kSum = (ki + kj);
                if (fabs(kSum) > s->eps) sum = vadd(sum, smul(s->mass * kSum, cubic_gradW(&s->K, vsub(ri, s->x[j]))));
            }
            if (fabs(ki) > s->eps && hb)
                for (unsigned q = 0; q < c.nbn; ++q) {
                    unsigned b = c.b[q];
                    sum = vadd(sum, smul(s->bw[b] * ki, cubic_gradW(&s->K, vsub(ri, s->bx[b]))));
                }
            s->v[i] = vsub(s->v[i], smul(ts, sum));
        }
        dfsph_predict_densities(s);
        ++s->iterations;
    }
    s->sumIterations += s->iterations;
}

/* DFSPHSolver::computeDivergenceError DFSPHSolver.cpp:408-492 */
static void dfsph_divergence_error(orc_scene* s)
{
    const double density0 = s->prm.density0;
    const int hb = hasb(s);
    double avgDivError = 0;
    #pragma omp parallel for reduction(+ : avgDivError)
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i], vi = s->v[i];
        double divError = 0;
        unsigned numNeighbors = 0;
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            const v3 grad = cubic_gradW(&s->K, vsub(ri, s->x[j]));
            divError += s->mass * vdot(vsub(vi, s->v[j]), grad);
            if (vlen(grad) > 0.0) numNeighbors++;
        }
        if (hb)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                const v3 grad = cubic_gradW(&s->K, vsub(ri, s->bx[b]));
                divError += s->bw[b] * vdot(vi, grad);
            }
        if (numNeighbors < 20) divError = 0.0;
        else divError = dmax(divError, 0.0);
        s->div[i] = divError;
        avgDivError += divError / density0;
    }
    avgDivError /= s->n;
    s->avgDivError = avgDivError;
}

/* DFSPHSolver::correctDivergenceError DFSPHSolver.cpp:494-590 (the loop is
 * bounded by maxIterations, not maxIterationsV, as the reference writes it) */
static void dfsph_correct_divergence_error(orc_scene* s)
{
    const double ts = s->ts;
    const int hb = hasb(s);
    dfsph_divergence_error(s);
    s->iterationsV = 0;
    s->avgDivError = 0;
    while (((s->avgDivError > s->maxErrorV / ts) || (s->iterationsV < s->min_it_v)) && s->iterationsV < s->max_it) {
        #pragma omp parallel for
        for (unsigned i = 0; i < s->n; ++i) {
            const v3 ri = s->x[i];
            const double dens_i = s->rho[i], divError_i = s->div[i], alpha_i = s->alpha[i];
            v3 sum = V(0.0, 0.0, 0.0);
            const double kiv = divError_i * alpha_i / (ts * dens_i);
            s->kv[i] += divError_i * alpha_i;
            cands c = cands_at(s, ri);
            for (unsigned q = 0; q < c.nf; ++q) {
                unsigned j = c.f[q];
                const double kjv = s->div[j] * s->alpha[j] / (ts * s->rho[j]);
                const double kSumV = (kiv + kjv);
                if (fabs(kSumV) > s->eps) sum = vadd(sum, smul(s->mass * kSumV, cubic_gradW(&s->K, vsub(ri, s->x[j]))));
            }
            if (fabs(kiv) > s->eps && hb)
                for (unsigned q = 0; q < c.nbn; ++q) {
                    unsigned b = c.b[q];
                    sum = vadd(sum, smul(s->bw[b] * kiv, cubic_gradW(&s->K, vsub(ri, s->bx[b]))));
                }
            s->v[i] = vsub(s->v[i], smul(ts, sum));
        }
        dfsph_divergence_error(s);
        ++s->iterationsV;
    }
    s->sumIterationsV += s->iterationsV;
}

/* DFSPHSolver::updateTimeStep DFSPHSolver.cpp:827-870 */
static void dfsph_update_time_step(orc_scene* s)
{
    const double ts = s->ts;
    const v3 g = V(s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2]);
    double maxVel = 0.1;
    #pragma omp parallel for reduction(max : maxVel)
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 acc = vadd(s->a[i], g);
        const v3 current_vi = vadd(s->v[i], vmul(acc, ts));
        maxVel = dmax(maxVel, sqrt(vlen(current_vi)));
    }
    s->maxVel = maxVel;
    double newTs;
    const double cflTs = s->cflFactor * 0.4 * 2.0 * s->prm.radius / maxVel;
    if (cflTs < ts) newTs = cflTs;
    else if (s->iterations > 3) newTs = ts * 0.99;
    else newTs = ts * 1.001;
    newTs = dmax(newTs, s->minTs);
    newTs = dmin(newTs, s->maxTs);
    s->ts = newTs;
}

/* ------------------------------------------------------------------------ */
/* Emitters (src/Emitter.cpp)                                                */
/* ------------------------------------------------------------------------ */

/* GLM's quat * vec3 for a unit quaternion (w, u): v + ((u x v) w + u x (u x v)) 2 */
static v3 vcross(v3 a, v3 b) { return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
static v3 quat_rotate(const double q[4], v3 v)
{
    const v3 u = V(q[1], q[2], q[3]);
    const v3 uv = vcross(u, v);
    const v3 uuv = vcross(u, uv);
    return vadd(v, vmul(vadd(vmul(uv, q[0]), uuv), 2.0));
}

/* Emitter::emitSquare / emitCircle Emitter.cpp:99-161 (identical bodies) */
static void emitter_emit(orc_scene* s, struct orc_emitter* e, double timeOffset)
{
    const double dist = 2.0 * s->prm.radius;
    const unsigned numActiveParticles = s->n;
    unsigned id = numActiveParticles;
    if (numActiveParticles + e->ng <= numActiveParticles + e->numParticles) {
        for (unsigned i = 0; i < e->ng; ++i) {
            v3 velocity = V(0, 0, e->v);
            const v3 g = V(s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2]);
            v3 position = vadd(e->group[i], smul(timeOffset, vadd(velocity, vmul(g, timeOffset))));
            position = quat_rotate(e->rot, position);
            velocity = quat_rotate(e->rot, velocity);
            position = vadd(position, e->r);
            s->x[id] = position;
            s->v[id] = velocity;
            ++id;
        }
        s->n = numActiveParticles + e->ng;   /* FluidModel::setNumActiveParticles */
        e->numParticles -= e->ng;
        e->nextTimeEmit += e->spacing * 1.105 * dist / e->v;
    }
}

/* Simulation::emitParticles -> FluidModel::emitParticles -> Emitter::
 * emitParticles (Simulation.cpp:325-329, FluidModel.cpp:145-149,
 * Emitter.cpp:85-97) */
static void emit_particles(orc_scene* s)
{
    const double time = s->time;
    for (unsigned k = 0; k < s->nem; ++k) {
        struct orc_emitter* e = &s->em[k];
        if (time >= e->nextTimeEmit && !e->pause) emitter_emit(s, e, time - e->nextTimeEmit);
    }
}

/* DFSPHSolver::step DFSPHSolver.cpp:38-112 */
static void dfsph_step(orc_scene* s)
{
    s->steps++;
    non_pressure_forces(s);
    dfsph_update_time_step(s);
    dfsph_predict_velocities(s);
    if (bh(s)) bh_correct_velocities(s, 0);      /* DFSPHSolver.cpp:51-57 */
    dfsph_correct_density_error(s);
    dfsph_update_positions(s);
    if (bh(s)) bh_correct_positions(s, 0);       /* :65-75 */
    emit_particles(s);                           /* :77 */
    grid_build(s);
    compute_densities(s);
    if (bh(s)) bh_boundary_densities(s);         /* SPHSolver::computeDensities :129-139 */
    dfsph_alpha(s);
    dfsph_correct_divergence_error(s);
    if (s->prm.boundary == 0 && s->prm.has_cube) cube_correct(s);
    s->time = s->time + s->ts;
}

/* ------------------------------------------------------------------------ */
/* WCSPH (src/WCSPHSolver.cpp)                                               */
/* ------------------------------------------------------------------------ */

/* WCSPHSolver::computeFluidPressures WCSPHSolver.cpp:80-95 */
static void wcsph_pressures(orc_scene* s)
{
    const double density0 = s->prm.density0, stiffness = s->prm.stiffness, gamma = s->prm.gamma;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i)
        s->p[i] = dmax(0.0, stiffness * density0 / gamma * (pow(s->rho[i] / density0, gamma) - 1));
}

/* WCSPHSolver::computeBoundaryPressures WCSPHSolver.cpp:97-114 */
static void wcsph_boundary_pressures(orc_scene* s)
{
    const double density0 = s->prm.density0, stiffness = s->prm.stiffness, gamma = s->prm.gamma;
    #pragma omp parallel for
    for (unsigned i = 0; i < s->nb; ++i)
        s->bpress[i] = dmax(0.0, stiffness * density0 / gamma * (pow(s->bdens[i] / density0, gamma) - 1));
}

/* WCSPHSolver::computePressureForce WCSPHSolver.cpp:132-188 */
static void wcsph_pressure_force(orc_scene* s)
{
    const int ak = akinci(s), bhm = bh(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i];
        v3 ai = s->a[i];
        const double densPress_i = s->p[i] / (s->rho[i] * s->rho[i]);
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            ai = vsub(ai, smul(s->mass * (densPress_i + s->p[j] / (s->rho[j] * s->rho[j])),
                               cubic_gradW(&s->K, vsub(ri, s->x[j]))));
        }
        if (ak)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                ai = vsub(ai, smul(s->bw[b] * (densPress_i * 1.0), cubic_gradW(&s->K, vsub(ri, s->bx[b]))));
            }
        else if (bhm)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                ai = vsub(ai, smul(s->bmass * (densPress_i + s->bpress[b] / (s->bdens[b] * s->bdens[b])),
                                   cubic_gradW(&s->K, vsub(ri, s->bx[b]))));
            }
        s->a[i] = ai;
    }
}

/* WCSPHSolver::step WCSPHSolver.cpp:14-78 */
static void wcsph_step(orc_scene* s)
{
    ++s->steps;
    grid_build(s);
    compute_densities(s);
    if (bh(s)) bh_boundary_densities(s);
    wcsph_pressures(s);
    if (bh(s)) wcsph_boundary_pressures(s);
    wcsph_pressure_force(s);
    non_pressure_forces(s);
    integrate_symplectic(s);
    if (s->prm.boundary == 0 && s->prm.has_cube) cube_correct(s);
    if (bh(s)) {                                 /* WCSPHSolver.cpp:62-72 */
        bh_correct_positions(s, 0);
        bh_correct_velocities(s, 0);
    }
    emit_particles(s);                           /* :75 */
    s->time = s->time + s->ts;
}

/* ------------------------------------------------------------------------ */
/* PCISPH (src/PCISPHSolver.cpp)                                             */
/* ------------------------------------------------------------------------ */

/* PCISPHSolver::computeScalingFactor PCISPHSolver.cpp:389-421 */
static void pcisph_scaling_factor(orc_scene* s)
{
    const double ts = s->ts;
    const double dist = 2.0 * s->prm.radius;
    v3 sumGrad = V(0, 0, 0);
    double sumSqGrad = 0;
    for (int i = -1; i <= 1; i++)
        for (int j = -1; j <= 1; j++)
            for (int k = -1; k <= 1; k++) {
                v3 rij = V(-i, -j, -k);
                rij = vmul(rij, dist);
                const v3 grad = poly6_gradW(&s->K, rij);
                sumGrad = vadd(sumGrad, grad);
                sumSqGrad += vdot(grad, grad);
            }
    const double beta = 2 * pow(s->mass * ts / s->prm.density0, 2);
    const double dotSumGrad = vdot(sumGrad, sumGrad);
    s->scaling = -1.0 / (beta * (-dotSumGrad - sumSqGrad));
}

/* PCISPHSolver::predictVelocityAndPosition PCISPHSolver.cpp:122-149 */
static void pcisph_predict(orc_scene* s)
{
    const double ts = s->ts;
    const v3 g = V(s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2]);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 acc = vadd(vadd(s->a[i], s->pacc[i]), g);
        s->predV[i] = vadd(s->v[i], vmul(acc, ts));
        s->predR[i] = vadd(s->x[i], vmul(s->predV[i], ts));
    }
}

/* PCISPHSolver::predictFluidDensities PCISPHSolver.cpp:164-212: predicted
 * positions, candidate lists of the current positions' cells. */
static void pcisph_predict_densities(orc_scene* s)
{
    const int hb = hasb(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->predR[i];
        cands c = cands_at(s, s->x[i]);
        double density = 0;
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            density += s->mass * cubic_Wv(&s->K, vsub(ri, s->predR[j]));
        }
        if (hb)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                density += s->bw[b] * cubic_Wv(&s->K, vsub(ri, s->bx[b]));
            }
        s->rho[i] = density;
    }
}

/* PCISPHSolver::predictBoundaryDensities PCISPHSolver.cpp:214-247 (Poly6,
 * predicted fluid positions) */
static void pcisph_predict_boundary_densities(orc_scene* s)
{
    #pragma omp parallel for
    for (unsigned i = 0; i < s->nb; ++i) {
        const v3 ri = s->bx[i];
        cands c = cands_at(s, ri);
        double density = 0;
        for (unsigned q = 0; q < c.nf; ++q) density += s->mass * poly6_W(&s->K, vsub(ri, s->predR[c.f[q]]));
        for (unsigned q = 0; q < c.nbn; ++q) density += s->bmass * poly6_W(&s->K, vsub(ri, s->bx[c.b[q]]));
        s->bdens[i] = density;
    }
}

/* PCISPHSolver::updatePressure PCISPHSolver.cpp:249-295 (the reference's
 * unsynchronised max becomes a max reduction) */
static void pcisph_update_pressure(orc_scene* s)
{
    const double density0 = s->prm.density0;
    double maxDensityError = 0;
    #pragma omp parallel for reduction(max : maxDensityError)
    for (unsigned i = 0; i < s->n; ++i) {
        const double error = dmax(0.0, s->rho[i] - density0);
        s->p[i] += s->scaling * error;
        maxDensityError = dmax(maxDensityError, error / density0);
    }
    s->maxDensityError = maxDensityError;
    if (bh(s)) {
        #pragma omp parallel for
        for (unsigned i = 0; i < s->nb; ++i) s->bpress[i] += s->scaling * dmax(0.0, s->bdens[i] - density0);
    }
}

/* PCISPHSolver::computePressureAcc PCISPHSolver.cpp:297-358 */
static void pcisph_pressure_acc(orc_scene* s)
{
    const int ak = akinci(s), bhm = bh(s);
    #pragma omp parallel for
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i];
        v3 pacc = V(0.0, 0.0, 0.0);
        const double densPress_i = s->p[i] / (s->rho[i] * s->rho[i]);
        cands c = cands_at(s, ri);
        for (unsigned q = 0; q < c.nf; ++q) {
            unsigned j = c.f[q];
            pacc = vsub(pacc, smul(s->mass * (densPress_i + s->p[j] / (s->rho[j] * s->rho[j])),
                                   spiky_gradW(&s->K, vsub(ri, s->x[j]))));
        }
        if (ak)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                pacc = vsub(pacc, smul(s->bw[b] * (densPress_i), spiky_gradW(&s->K, vsub(ri, s->bx[b]))));
            }
        else if (bhm)
            for (unsigned q = 0; q < c.nbn; ++q) {
                unsigned b = c.b[q];
                pacc = vsub(pacc, smul(s->bmass * (densPress_i + s->bpress[b] / (s->bdens[b] * s->bdens[b])),
                                       spiky_gradW(&s->K, vsub(ri, s->bx[b]))));
            }
        s->pacc[i] = pacc;
    }
}

/* PCISPHSolver::pressureSolver PCISPHSolver.cpp:360-387 (maxDensityError is
 * not reset before the first test, as in the reference) */
static void pcisph_pressure_solver(orc_scene* s)
{
    s->iterations = 0;
    while ((s->maxDensityError > s->maxError || s->iterations < s->min_it) && s->iterations < s->max_it) {
        pcisph_predict(s);
        if (bh(s)) bh_correct_pred_positions(s);    /* PCISPHSolver.cpp:367-377 */
        pcisph_predict_densities(s);
        if (bh(s)) pcisph_predict_boundary_densities(s);
        pcisph_update_pressure(s);
        pcisph_pressure_acc(s);
        ++s->iterations;
    }
}

/* PCISPHSolver::integrate PCISPHSolver.cpp:444-473 */
static void pcisph_integrate(orc_scene* s)
{
    const double ts = s->ts;
    const v3 g = V(s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2]);
    double maxVel = 0;
    for (unsigned i = 0; i < s->n; ++i) {
        s->a[i] = vadd(s->a[i], vadd(g, s->pacc[i]));
        s->v[i] = vadd(s->v[i], vmul(s->a[i], ts));
        s->x[i] = vadd(s->x[i], vmul(s->v[i], ts));
        s->a[i] = V(0, 0, 0);
        maxVel = dmax(maxVel, vlen(s->v[i]));
    }
    s->maxVel = maxVel;
}

/* PCISPHSolver::step PCISPHSolver.cpp:21-81 */
static void pcisph_step(orc_scene* s)
{
    ++s->steps;
    grid_build(s);
    compute_densities(s);
    if (bh(s)) bh_boundary_densities(s);
    non_pressure_forces(s);
    /* initPressure PCISPHSolver.cpp:83-120 */
    for (unsigned i = 0; i < s->n; ++i) { s->p[i] = 0.0; s->pacc[i] = V(0.0, 0.0, 0.0); }
    if (bh(s))
        for (unsigned i = 0; i < s->nb; ++i) s->bpress[i] = 0.0;
    pcisph_pressure_solver(s);
    pcisph_integrate(s);
    if (s->prm.boundary == 0 && s->prm.has_cube) cube_correct(s);
    if (bh(s)) {                                 /* PCISPHSolver.cpp:65-75 */
        bh_correct_positions(s, 1);
        bh_correct_velocities(s, 1);
    }
    emit_particles(s);                           /* :78 */
    s->time = s->time + s->ts;
}

/* ------------------------------------------------------------------------ */
/* Scene construction                                                         */
/* ------------------------------------------------------------------------ */

static void boundary_append(orc_scene* s, const double* pts, long long m);

orc_scene* orc_create(const orc_params* p)
{
    if (!p || p->method < 0 || p->method > 2) return NULL;
    orc_scene* s = (orc_scene*)calloc(1, sizeof(orc_scene));
    s->prm = *p;
    s->h = 4.0 * p->radius;              /* Simulation::setParticleRadius Simulation.cpp:192-199 */
    kernels_init(&s->K, s->h);           /* Simulation::initKernels :124-132 */
    {
        const double diameter = 2.0 * p->radius;       /* Simulation::initMasses :134-146 */
        const double particleVolume = pow(diameter, 3.0);
        s->mass = p->density0 * particleVolume;
    }
    /* PCISPH boundary model mass: density0 * (2r)^3, as the fluid's
     * (Simulation.cpp:464-468) */
    s->bmass = s->mass;
    s->ts = p->dt;
    /* TimeManager::setMinTimeStep stores min(minTs, 1/fps) (TimeManager.h:55) */
    {
        const double minFPSTimeStep = 1.0 / p->fps;
        s->minTs = minFPSTimeStep < p->min_dt ? minFPSTimeStep : p->min_dt;
    }
    s->maxTs = p->max_dt;
    s->eps = 1e-5;                        /* DFSPHSolver::init :26 */
    /* solver defaults: SPHSolver.cpp:12-19, DFSPHSolver.cpp:10-22 */
    s->min_it = 3; s->max_it = 100; s->maxError = 0.01;
    s->min_it_v = 1; s->max_it_v = 100; s->maxErrorV = 0.001; s->cflFactor = 1.0;
    if (p->method == 2) { s->min_it = 2; s->max_it = 100; }
    if (p->method != 0) s->maxError = p->eta;
    if (p->method == 2) { s->maxErrorV = p->eta_v; s->cflFactor = p->cfl; }
    if (p->min_it >= 0) s->min_it = (unsigned)p->min_it;
    if (p->max_it >= 0) s->max_it = (unsigned)p->max_it;
    if (p->min_it_v >= 0) s->min_it_v = (unsigned)p->min_it_v;
    if (p->max_it_v >= 0) s->max_it_v = (unsigned)p->max_it_v;
    if (p->boundary == 0 && p->has_cube) {
        /* CubeBoundaryModel::init keeps min and max as its two "particles"
         * (CubeBoundaryModel.cpp:5-14); insertBoundaryParticles puts them in
         * the grid like any boundary point (SPHSolver.cpp:195-213). */
        const double pts[6] = {p->cube_min[0], p->cube_min[1], p->cube_min[2],
                               p->cube_max[0], p->cube_max[1], p->cube_max[2]};
        boundary_append(s, pts, 2);
    }
    return s;
}

void orc_destroy(orc_scene* s)
{
    if (!s) return;
    free(s->x); free(s->v); free(s->a); free(s->rho); free(s->p);
    free(s->alpha); free(s->div); free(s->pred); free(s->k); free(s->kv);
    free(s->predR); free(s->predV); free(s->pacc); free(s->normal);
    free(s->bx); free(s->psi); free(s->bw); free(s->bn); free(s->bdens); free(s->bpress);
    for (unsigned k = 0; k < s->nem; ++k) free(s->em[k].group);
    grid_free(&s->g);
    free(s);
}

/* FluidModel::resizeFluid + solver resizeData (FluidModel.cpp:51-60,
 * DFSPHSolver.cpp:802-823, PCISPHSolver.cpp:423-441): per-particle arrays
 * of `cap` entries, new entries zero (std::vector::resize). */
static void* grow(void* p, size_t old, size_t nw, size_t sz)
{
    char* q = (char*)realloc(p, (nw ? nw : 1) * sz);
    if (q && nw > old) memset(q + old * sz, 0, (nw - old) * sz);
    return q;
}
static void fluid_resize(orc_scene* s, unsigned cap)
{
    const unsigned o = s->cap;
    s->x = (v3*)grow(s->x, o, cap, sizeof(v3)); s->v = (v3*)grow(s->v, o, cap, sizeof(v3));
    s->a = (v3*)grow(s->a, o, cap, sizeof(v3));
    s->rho = (double*)grow(s->rho, o, cap, 8); s->p = (double*)grow(s->p, o, cap, 8);
    s->alpha = (double*)grow(s->alpha, o, cap, 8); s->div = (double*)grow(s->div, o, cap, 8);
    s->pred = (double*)grow(s->pred, o, cap, 8); s->k = (double*)grow(s->k, o, cap, 8); s->kv = (double*)grow(s->kv, o, cap, 8);
    s->predR = (v3*)grow(s->predR, o, cap, sizeof(v3)); s->predV = (v3*)grow(s->predV, o, cap, sizeof(v3));
    s->pacc = (v3*)grow(s->pacc, o, cap, sizeof(v3)); s->normal = (v3*)grow(s->normal, o, cap, sizeof(v3));
    s->cap = cap;
}

int orc_set_fluid(orc_scene* s, const double* x, const double* v, unsigned n)
{
    if (!s || s->inited || s->n || s->nem) return -1;
    fluid_resize(s, n);
    s->n = n;
    for (unsigned i = 0; i < n; ++i) {
        s->x[i] = V(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        s->v[i] = v ? V(v[3 * i], v[3 * i + 1], v[3 * i + 2]) : V(0, 0, 0);
    }
    return 0;
}

static void boundary_append_n(orc_scene* s, const double* pts, const double* nrm, long long m)
{
    if (s->nb + m > s->nb_cap) {
        unsigned cap = s->nb_cap ? s->nb_cap : 1024;
        while (cap < s->nb + m) cap *= 2;
        s->bx = (v3*)realloc(s->bx, cap * sizeof(v3));
        s->bn = (v3*)realloc(s->bn, cap * sizeof(v3));
        s->psi = (double*)realloc(s->psi, cap * sizeof(double));
        s->bw = (double*)realloc(s->bw, cap * sizeof(double));
        s->bdens = (double*)realloc(s->bdens, cap * sizeof(double));
        s->bpress = (double*)realloc(s->bpress, cap * sizeof(double));
        s->nb_cap = cap;
    }
    for (long long q = 0; q < m; ++q) {
        s->bx[s->nb] = V(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
        s->bn[s->nb] = nrm ? V(nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]) : V(0, 0, 0);
        s->psi[s->nb] = 0.0;
        s->bw[s->nb] = 0.0;
        s->bdens[s->nb] = 0.0;
        s->bpress[s->nb] = 0.0;
        s->nb++;
    }
}

static void boundary_append(orc_scene* s, const double* pts, long long m) { boundary_append_n(s, pts, NULL, m); }

/* AkinciBoundaryModel::sampleCube AkinciBoundayModel.cpp:100-134 */
long long orc_sample_box(double supportRadius, const double mn[3], const double mx[3], double* out)
{
    const double lx = fabs(mn[0] - mx[0]);
    const double ly = fabs(mn[1] - mx[1]);
    const double lz = fabs(mn[2] - mx[2]);
    const unsigned nx = (unsigned)ceil(lx / (0.5 * supportRadius));
    const unsigned ny = (unsigned)ceil(ly / (0.5 * supportRadius));
    const unsigned nz = (unsigned)ceil(lz / (0.5 * supportRadius));
    const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
    long long count = 0;
    for (unsigned i = 0; i <= nx; i++)
        for (unsigned j = 0; j <= ny; j++)
            for (unsigned k = 0; k <= nz; k++)
                if ((i == 0 || i == nx) || (j == 0 || j == ny) || (k == 0 || k == nz)) {
                    if (out) {
                        out[3 * count] = i * dx + mn[0];
                        out[3 * count + 1] = j * dy + mn[1];
                        out[3 * count + 2] = k * dz + mn[2];
                    }
                    count++;
                }
    return count;
}

/* AkinciBoundaryModel::sampleSphere AkinciBoundayModel.cpp:136-164 */
long long orc_sample_sphere(double particleRadius, const double c[3], double radius, double* out)
{
    const double separacion = 1.5;
    const unsigned num_parts = (unsigned)floor(4.0 * M_PI * radius * radius / (M_PI * particleRadius * particleRadius) * separacion);
    const double a = 4.0 * M_PI / num_parts;
    const double d = sqrt(a);
    const int m_theta = (int)round(M_PI / d);
    const double d_theta = M_PI / m_theta;
    const double d_phi = a / d_theta;
    long long count = 0;
    for (int m = 0; m < m_theta; ++m) {
        const double theta = M_PI * (m + 0.5) / m_theta;
        const int m_phi = (int)round(2.0 * M_PI * sin(theta) / d_phi);
        for (int n = 0; n < m_phi; ++n) {
            const double phi = 2.0 * M_PI * n / m_phi;
            const double x = sin(theta) * cos(phi);
            const double y = sin(theta) * sin(phi);
            const double z = cos(theta);
            if (out) {
                out[3 * count] = radius * x + c[0];
                out[3 * count + 1] = radius * y + c[1];
                out[3 * count + 2] = radius * z + c[2];
            }
            count++;
        }
    }
    return count;
}

/* Simulation::buildFluidBlock Simulation.cpp:512-539 */
long long orc_fluid_block(double r, const double mn[3], const double mx[3], double* out)
{
    const double dist = 2.0 * r;
    const int px = (int)floor((mx[0] - mn[0]) / dist + 1e-5);
    const int py = (int)floor((mx[1] - mn[1]) / dist + 1e-5);
    const int pz = (int)floor((mx[2] - mn[2]) / dist + 1e-5);
    long long count = 0;
    for (int i = 0; i < px; ++i)
        for (int j = 0; j < py; ++j)
            for (int k = 0; k < pz; ++k) {
                if (out) {
                    out[3 * count] = i * dist + (mn[0] + r);
                    out[3 * count + 1] = j * dist + (mn[1] + r);
                    out[3 * count + 2] = k * dist + (mn[2] + r);
                }
                count++;
            }
    return count;
}

int orc_add_box(orc_scene* s, const double mn[3], const double mx[3])
{
    if (!s || s->inited) return -1;
    long long m = orc_sample_box(s->h, mn, mx, NULL);
    double* pts = (double*)xcalloc((size_t)(3 * m), 8);
    orc_sample_box(s->h, mn, mx, pts);
    boundary_append(s, pts, m);
    free(pts);
    return 0;
}

int orc_add_sphere(orc_scene* s, const double c[3], double radius)
{
    if (!s || s->inited) return -1;
    long long m = orc_sample_sphere(s->prm.radius, c, radius, NULL);
    double* pts = (double*)xcalloc((size_t)(3 * m), 8);
    orc_sample_sphere(s->prm.radius, c, radius, pts);
    boundary_append(s, pts, m);
    free(pts);
    return 0;
}

/* Pre-sampled points appended to the boundary model, as the reference's
 * BoundaryModel::addPoints-style setup fills its position vector directly
 * (AkinciBoundaryModel.h:13-31 keeps positions in one vector per model). */
int orc_add_points(orc_scene* s, const double* pts, unsigned m)
{
    if (!s || s->inited || (m && !pts)) return -1;
    boundary_append(s, pts, (long long)m);
    return 0;
}

static v3 unit(v3 a) { return vmul(a, 1.0 / sqrt(vdot(a, a))); }

/* PCISPHBoundaryModel::sampleCube PCISPHBoundaryModel.cpp:56-184: points on
 * the faces of the box at a spacing of at most 0.45 h, each with the normal of
 * its face, edge or corner (mean of the faces' normals, normalised), pointing
 * into the box; `inverted` 0 flips them outwards (addCube :7-30). */
long long orc_sample_bh_box(double supportRadius, const double mn[3], const double mx[3], int inverted, double* pts,
                            double* normals)
{
    const double lx = fabs(mn[0] - mx[0]), ly = fabs(mn[1] - mx[1]), lz = fabs(mn[2] - mx[2]);
    const unsigned nx = (unsigned)ceil(lx / (0.45 * supportRadius));
    const unsigned ny = (unsigned)ceil(ly / (0.45 * supportRadius));
    const unsigned nz = (unsigned)ceil(lz / (0.45 * supportRadius));
    const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
    const v3 L = V(1, 0, 0), R = V(-1, 0, 0), T = V(0, -1, 0), B = V(0, 1, 0), F = V(0, 0, -1), K = V(0, 0, 1);
    const double inv = inverted ? 1.0 : -1;
    long long count = 0;
    for (unsigned i = 0; i <= nx; i++)
        for (unsigned j = 0; j <= ny; j++)
            for (unsigned k = 0; k <= nz; k++) {
                const int xi0 = i == 0, xi1 = i == nx, yj0 = j == 0, yj1 = j == ny, zk0 = k == 0, zk1 = k == nz;
                if (!(xi0 || xi1 || yj0 || yj1 || zk0 || zk1)) continue;
                const int xin = !xi0 && !xi1, yin = !yj0 && !yj1, zin = !zk0 && !zk1;
                v3 n;
                if (!xin && !yin && !zin) {  /* corner: three faces */
                    n = unit(vdiv(vadd(vadd(xi0 ? L : R, zk0 ? K : F), yj0 ? B : T), 3.0));
                } else if (xin + yin + zin == 1) {  /* edge: two faces */
                    v3 a, b;
                    if (zin) { a = xi0 ? L : R; b = yj0 ? B : T; }
                    else if (xin) { a = zk0 ? K : F; b = yj0 ? B : T; }
                    else { a = xi0 ? L : R; b = zk0 ? K : F; }
                    n = unit(vmul(vadd(a, b), 0.5));
                } else {  /* face */
                    n = !xin ? (xi0 ? L : R) : !yin ? (yj0 ? B : T) : (zk0 ? K : F);
                }
                if (pts) {
                    pts[3 * count] = i * dx + mn[0];
                    pts[3 * count + 1] = j * dy + mn[1];
                    pts[3 * count + 2] = k * dz + mn[2];
                    const v3 o = smul(inv, n);
                    normals[3 * count] = o.x;
                    normals[3 * count + 1] = o.y;
                    normals[3 * count + 2] = o.z;
                }
                count++;
            }
    return count;
}

/* PCISPHBoundaryModel::addCube :7-30 */
int orc_add_bh_box(orc_scene* s, const double mn[3], const double mx[3], int inverted)
{
    if (!s || s->inited || !bh(s)) return -1;
    const long long m = orc_sample_bh_box(s->h, mn, mx, inverted, NULL, NULL);
    double* pts = (double*)xcalloc((size_t)(3 * m), 8);
    double* nrm = (double*)xcalloc((size_t)(3 * m), 8);
    orc_sample_bh_box(s->h, mn, mx, inverted, pts, nrm);
    boundary_append_n(s, pts, nrm, m);
    free(pts);
    free(nrm);
    return 0;
}

/* PCISPHBoundaryModel::addSphere :32-54 (normals inv * (centre - point), not
 * normalised; the Akinci sphere sampler) */
int orc_add_bh_sphere(orc_scene* s, const double c[3], double radius, int inverted)
{
    if (!s || s->inited || !bh(s)) return -1;
    const long long m = orc_sample_sphere(s->prm.radius, c, radius, NULL);
    double* pts = (double*)xcalloc((size_t)(3 * m), 8);
    double* nrm = (double*)xcalloc((size_t)(3 * m), 8);
    orc_sample_sphere(s->prm.radius, c, radius, pts);
    const double inv = inverted ? 1.0 : -1;
    for (long long q = 0; q < m; ++q) {
        const v3 n = smul(inv, vsub(V(c[0], c[1], c[2]), V(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2])));
        nrm[3 * q] = n.x; nrm[3 * q + 1] = n.y; nrm[3 * q + 2] = n.z;
    }
    boundary_append_n(s, pts, nrm, m);
    free(pts);
    free(nrm);
    return 0;
}

/* Emitter::buildCircleGroup / buildSquareGroup Emitter.cpp:31-79 (a
 * negative level count, converted to unsigned unchecked by the reference,
 * is taken as zero) */
long long orc_emitter_group(int type, double particleRadius, double width, double height, double* out)
{
    long long count = 0;
#define PUT(px, py) do { if (out) { out[3 * count] = (px); out[3 * count + 1] = (py); out[3 * count + 2] = 0.0; } ++count; } while (0)
    if (type == 1) {
        const double dist = 2.0 * particleRadius;
        const double lv = floor((width - 0.5 * dist) / dist);
        const unsigned numLevels = lv > 0.0 ? (unsigned)lv : 0u;
        PUT(0.0, 0.0);
        for (unsigned i = 0; i < numLevels; ++i) {
            const double radius = (i + 1) * dist;
            const double l = 2.0 * M_PI * radius;
            const unsigned nParts = (unsigned)floor(l / dist);
            const double inc = 2 * M_PI / nParts;
            for (unsigned j = 0; j < nParts; ++j) {
                const double angle = j * inc;
                PUT(radius * sin(angle), radius * cos(angle));
            }
        }
    } else {
        const double dist = particleRadius * 2.0;
        const double fx = floor(width / dist), fy = floor(height / dist);
        const unsigned numX = fx > 0.0 ? (unsigned)fx : 0u, numY = fy > 0.0 ? (unsigned)fy : 0u;
        const double realWidth = (numX - 1) * dist;
        const double realHeight = (numY - 1) * dist;
        for (unsigned i = 0; i < numX; ++i)
            for (unsigned j = 0; j < numY; ++j) PUT(realWidth * 0.5 - i * dist, realHeight * 0.5 - j * dist);
    }
#undef PUT
    return count;
}

/* FluidModel::addEmitter FluidModel.cpp:124-143 and the Emitter
 * constructor Emitter.cpp:10-29 */
int orc_add_emitter(orc_scene* s, int type, unsigned numParticles, const double r[3], double v, const double rot[4],
                    double startTime, double w, double h, double spacing)
{
    if (!s || s->inited || s->nem >= 64 || (type != 0 && type != 1)) return -1;
    struct orc_emitter* e = &s->em[s->nem];
    memset(e, 0, sizeof *e);
    e->type = type;
    e->numParticles = numParticles;
    e->r = V(r[0], r[1], r[2]);
    e->v = v;
    for (int k = 0; k < 4; ++k) e->rot[k] = rot[k];
    e->nextTimeEmit = startTime;
    e->spacing = spacing;
    const long long m = orc_emitter_group(type, s->prm.radius, w, h, NULL);
    double* buf = (double*)xcalloc((size_t)m * 3, 8);
    orc_emitter_group(type, s->prm.radius, w, h, buf);
    e->group = (v3*)xcalloc((size_t)m, sizeof(v3));
    for (long long i = 0; i < m; ++i) e->group[i] = V(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]);
    free(buf);
    e->ng = (unsigned)m;
    s->nem++;
    fluid_resize(s, s->cap + numParticles);
    return 0;
}

/* Simulation::setEmittersPause -> Emitter::setPause (Simulation.h:316,
 * Emitter.cpp:80-84) */
int orc_pause_emitters(orc_scene* s, int pause)
{
    if (!s) return -1;
    for (unsigned k = 0; k < s->nem; ++k) {
        s->em[k].pause = pause != 0;
        s->em[k].nextTimeEmit = s->time;
    }
    return 0;
}

/* Simulation::init -> solver->init (Simulation.cpp:102-110; SPHSolver.cpp:
 * 22-39; DFSPHSolver.cpp:24-36; PCISPHSolver.cpp:12-19; WCSPHSolver.cpp:9) */
int orc_init(orc_scene* s)
{
    if (!s || s->inited) return -1;
    if (s->prm.method == 1) pcisph_scaling_factor(s);
    if (akinci(s)) {
        /* boundary points inserted first, candidates, then psi */
        unsigned n = s->n;
        s->n = 0;
        grid_build(s);
        s->n = n;
        compute_volume(s);
        for (unsigned b = 0; b < s->nb; ++b) s->bw[b] = s->prm.density0 * s->psi[b];
    }
    if (bh(s))
        for (unsigned b = 0; b < s->nb; ++b) s->bw[b] = s->bmass;
    if (s->prm.method == 2) {
        grid_build(s);
        compute_densities(s);
        if (bh(s)) bh_boundary_densities(s);
        dfsph_alpha(s);
    }
    s->inited = 1;
    return 0;
}

/* Simulation::step Simulation.cpp:148-182 -> solver->step() */
int orc_step(orc_scene* s, int nsteps)
{
    if (!s || !s->inited) return -1;
    for (int q = 0; q < nsteps; ++q) {
        if (s->prm.method == 0) wcsph_step(s);
        else if (s->prm.method == 1) pcisph_step(s);
        else dfsph_step(s);
    }
    return 0;
}

/* Test instrument, not part of the reference: adds U(-dx, dx) to every
 * position component and U(-dv, dv) to every velocity component (splitmix64
 * stream from `seed`).  Used to measure how far the reference's own
 * trajectories spread under rounding-sized noise injected every step. */
static double orc_unit(uint64_t* st)
{
    uint64_t z = (*st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

int orc_perturb(orc_scene* s, double dx, double dv, unsigned long long seed)
{
    if (!s || !s->inited) return -1;
    uint64_t st = seed;
    for (unsigned i = 0; i < s->n; ++i) {
        s->x[i].x += dx * orc_unit(&st); s->x[i].y += dx * orc_unit(&st); s->x[i].z += dx * orc_unit(&st);
        s->v[i].x += dv * orc_unit(&st); s->v[i].y += dv * orc_unit(&st); s->v[i].z += dv * orc_unit(&st);
    }
    return 0;
}

unsigned orc_num_fluid(const orc_scene* s) { return s ? s->n : 0; }
unsigned orc_num_boundary(const orc_scene* s) { return s ? s->nb : 0; }

static void put_v3(const v3* a, unsigned n, double* out)
{
    for (unsigned i = 0; i < n; ++i) { out[3 * i] = a[i].x; out[3 * i + 1] = a[i].y; out[3 * i + 2] = a[i].z; }
}

int orc_get(const orc_scene* s, const char* f, double* out)
{
    if (!s || !f || !out) return -1;
    const unsigned n = s->n;
    if (!strcmp(f, "x")) put_v3(s->x, n, out);
    else if (!strcmp(f, "v")) put_v3(s->v, n, out);
    else if (!strcmp(f, "a")) put_v3(s->a, n, out);
    else if (!strcmp(f, "pacc")) put_v3(s->pacc, n, out);
    else if (!strcmp(f, "normal")) put_v3(s->normal, n, out);
    else if (!strcmp(f, "bx")) put_v3(s->bx, s->nb, out);
    else if (!strcmp(f, "rho")) memcpy(out, s->rho, n * 8);
    else if (!strcmp(f, "p")) memcpy(out, s->p, n * 8);
    else if (!strcmp(f, "alpha")) memcpy(out, s->alpha, n * 8);
    else if (!strcmp(f, "div")) memcpy(out, s->div, n * 8);
    else if (!strcmp(f, "pred")) memcpy(out, s->pred, n * 8);
    else if (!strcmp(f, "k")) memcpy(out, s->k, n * 8);
    else if (!strcmp(f, "kv")) memcpy(out, s->kv, n * 8);
    else if (!strcmp(f, "psi")) memcpy(out, s->psi, s->nb * 8);
    else if (!strcmp(f, "bn")) put_v3(s->bn, s->nb, out);
    else if (!strcmp(f, "bdens")) memcpy(out, s->bdens, s->nb * 8);
    else if (!strcmp(f, "bpress")) memcpy(out, s->bpress, s->nb * 8);
    else return -2;
    return 0;
}

int orc_get_scalar(const orc_scene* s, const char* f, double* out)
{
    if (!s || !f || !out) return -1;
    if (!strcmp(f, "time")) *out = s->time;
    else if (!strcmp(f, "dt")) *out = s->ts;
    else if (!strcmp(f, "iterations")) *out = s->iterations;
    else if (!strcmp(f, "iterationsV")) *out = s->iterationsV;
    else if (!strcmp(f, "avgDensError")) *out = s->avgDensError;
    else if (!strcmp(f, "avgDivError")) *out = s->avgDivError;
    else if (!strcmp(f, "maxDensityError")) *out = s->maxDensityError;
    else if (!strcmp(f, "scaling")) *out = s->scaling;
    else if (!strcmp(f, "mass")) *out = s->mass;
    else if (!strcmp(f, "h")) *out = s->h;
    else if (!strcmp(f, "steps")) *out = s->steps;
    else if (!strcmp(f, "sumIterations")) *out = s->sumIterations;
    else return -2;
    return 0;
}

int orc_neighbors(orc_scene* s, int* cells, int* cell_rank, int* nbr_off, int* nbr, int* bnbr_off, int* bnbr,
                  long long* totals)
{
    if (!s) return -1;
    long long nf = 0, nbt = 0;
    const double h = s->h;
    for (unsigned i = 0; i < s->n; ++i) {
        const v3 ri = s->x[i];
        i3 ck = cell_of(ri.x, ri.y, ri.z, h);
        int c = grid_find(&s->g, ck);
        if (cells) { cells[3 * i] = ck.x; cells[3 * i + 1] = ck.y; cells[3 * i + 2] = ck.z; }
        if (cell_rank) {
            int r = -1;
            if (c >= 0)
                for (unsigned q = s->g.fstart[c]; q < s->g.fstart[c + 1]; ++q)
                    if (s->g.fpts[q] == i) { r = (int)(q - s->g.fstart[c]); break; }
            cell_rank[i] = r;
        }
        if (nbr_off) nbr_off[i] = (int)nf;
        if (bnbr_off) bnbr_off[i] = (int)nbt;
        cands cd = cands_at(s, ri);
        for (unsigned q = 0; q < cd.nf; ++q) {
            unsigned j = cd.f[q];
            if (vlen(vsub(ri, s->x[j])) / h <= 1.0) { if (nbr) nbr[nf] = (int)j; nf++; }
        }
        for (unsigned q = 0; q < cd.nbn; ++q) {
            unsigned b = cd.b[q];
            if (vlen(vsub(ri, s->bx[b])) / h <= 1.0) { if (bnbr) bnbr[nbt] = (int)b; nbt++; }
        }
    }
    if (nbr_off) nbr_off[s->n] = (int)nf;
    if (bnbr_off) bnbr_off[s->n] = (int)nbt;
    if (totals) { totals[0] = nf; totals[1] = nbt; }
    return 0;
}
