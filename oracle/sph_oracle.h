/* CPU restatement of the reference simulator's per-step particle loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path:
 * only the tests, the smoke check and the benchmark's CPU-baseline leg load
 * it.  The product (sph_gb300) never links or calls it.
 *
 * FP64 throughout, with each expression evaluated in the order the reference
 * writes it (and no FMA contraction), so that on the same inputs it
 * reproduces the reference's own results; see sph_oracle.c for the
 * per-function citations into josemanuel28v/SPH.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int method;            /* 0 WCSPH, 1 PCISPH, 2 DFSPH (src/Simulation.cpp:21-23) */
    int boundary;          /* 0 cube, 1 PCISPH particles, 2 Akinci (:25-27) */
    double radius;         /* particle radius r; support radius h = 4 r */
    double gravity[3];
    double dt, min_dt, max_dt, fps;
    double density0;
    double stiffness, gamma;              /* WCSPH */
    double eta, eta_v, cfl;               /* PCISPH / DFSPH */
    int min_it, max_it, min_it_v, max_it_v; /* < 0: keep the solver's default */
    int visc_method;       /* 0 standard, 1 artificial, 2 XSPH, -1 none */
    double visc, bvisc;
    int st_method;         /* 3 Akinci surface tension, -1 none */
    double st;
    int adh_method;        /* 4 Akinci adhesion, -1 none */
    double adh;
    double cube_min[3], cube_max[3];      /* cube boundary (boundary == 0) */
    int has_cube;
    double bh_normal_fct, bh_tang_fct;    /* PCISPH boundary model (boundary == 1) */
} orc_params;

typedef struct orc_scene orc_scene;

orc_scene* orc_create(const orc_params* p);
void orc_destroy(orc_scene* s);
int orc_set_fluid(orc_scene* s, const double* x, const double* v, unsigned n);
int orc_add_box(orc_scene* s, const double mn[3], const double mx[3]);
int orc_add_sphere(orc_scene* s, const double c[3], double radius);
int orc_add_points(orc_scene* s, const double* pts, unsigned m);
/* PCISPH boundary model (boundary == 1): sampled cube / sphere with normals */
int orc_add_bh_box(orc_scene* s, const double mn[3], const double mx[3], int inverted);
int orc_add_bh_sphere(orc_scene* s, const double c[3], double radius, int inverted);
long long orc_sample_bh_box(double supportRadius, const double mn[3], const double mx[3], int inverted, double* pts,
                            double* normals);
/* emitters: type 0 square, 1 circle; rot = (w, x, y, z).  After
 * orc_set_fluid (which may pass n = 0). */
int orc_add_emitter(orc_scene* s, int type, unsigned numParticles, const double r[3], double v, const double rot[4],
                    double startTime, double w, double h, double spacing);
int orc_pause_emitters(orc_scene* s, int pause);
long long orc_emitter_group(int type, double particleRadius, double width, double height, double* out);
int orc_init(orc_scene* s);
int orc_step(orc_scene* s, int nsteps);
/* test instrument: uniform noise on positions and velocities */
int orc_perturb(orc_scene* s, double dx, double dv, unsigned long long seed);
unsigned orc_num_fluid(const orc_scene* s);
unsigned orc_num_boundary(const orc_scene* s);
/* field: x v a rho p alpha div pred k kv pacc normal bx psi */
int orc_get(const orc_scene* s, const char* field, double* out);
/* name: time dt iterations iterationsV avgDensError avgDivError
 *       maxDensityError scaling mass h steps sumIterations */
int orc_get_scalar(const orc_scene* s, const char* name, double* out);
/* Neighbour sets of every fluid particle as the reference's walks see them:
 * candidates of the particle's current cell within the cubic spline's
 * support (q <= 1).  Pass NULL arrays to get the totals first. */
int orc_neighbors(orc_scene* s, int* cells, int* cell_rank, int* nbr_off, int* nbr, int* bnbr_off,
                  int* bnbr, long long* totals);
/* Sampling helpers (Akinci box / sphere, fluid block) for callers that want
 * the points without a scene. Return the number of points; out may be NULL. */
long long orc_sample_box(double h, const double mn[3], const double mx[3], double* out);
long long orc_sample_sphere(double r, const double c[3], double radius, double* out);
long long orc_fluid_block(double r, const double mn[3], const double mx[3], double* out);

#ifdef __cplusplus
}
#endif
#endif
