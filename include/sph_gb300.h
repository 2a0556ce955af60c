/* sph_gb300: GB300 (sm_103a) implementation of the per-step particle loop of
 * josemanuel28v/SPH, behind a plain C ABI.
 *
 * One context (sph_ctx) holds one scene: one fluid model and one boundary
 * model, the way the reference's Simulation singleton holds them, but with
 * explicit handles instead of a process-global (src/Simulation.cpp:84-90), so
 * contexts are independent and many can live in one process.  All state is
 * device-resident; host buffers are touched only by the upload/download
 * calls.  Every function returns SPH_OK (0) or a negative SPH_ERR_* code and
 * never throws; sph_ctx_last_error() describes the last failure.
 *
 * Reference interfaces replaced (paths in the reference repository):
 *   SPHSolver::init/step/resizeData            src/SPHSolver.h:37-39
 *   Simulation::init / step                    src/Simulation.cpp:102-182
 *   WCSPHSolver / PCISPHSolver / DFSPHSolver    src/*Solver.{h,cpp}
 *   NonPressureForce::step (the five plugins)  src/NonPressureForce.h:17
 *   AkinciBoundaryModel::addCube/addSphere/computeVolume
 *                                              src/AkinciBoundayModel.cpp:11-164
 *   CubeBoundaryModel::correctPositionAndVelocity src/CubeBoundaryModel.cpp:16-94
 *   HashTable insert / neighborhoodSearch      src/HashTable.h:79-170
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_OK 0
#define SPH_ERR_INVALID -1      /* bad argument or call order */
#define SPH_ERR_CUDA -2         /* a CUDA call failed */
#define SPH_ERR_UNSUPPORTED -3  /* feature not available in this build */
#define SPH_ERR_CAPACITY -4     /* grid or particle capacity exceeded */

/* Method ids, identical to the reference's (src/Simulation.cpp:21-43). */
#define SPH_WCSPH 0
#define SPH_PCISPH 1
#define SPH_DFSPH 2
#define SPH_BOUNDARY_CUBE 0
#define SPH_BOUNDARY_PCISPH 1
#define SPH_BOUNDARY_AKINCI 2
#define SPH_VISCOSITY_STANDARD 0
#define SPH_VISCOSITY_ARTIFICIAL 1
#define SPH_VISCOSITY_XSPH 2
#define SPH_SURFACE_TENSION_AKINCI 3
#define SPH_ADHESION_AKINCI 4

/* Arithmetic of the device path. */
#define SPH_PRECISION_F32 0   /* production: FP32 bulk, cell-relative positions, FP64 reductions */
#define SPH_PRECISION_F64 1   /* parity: FP64 throughout, the reference's expression order */

/* Fields for sph_ctx_download (original particle order, FP64). */
#define SPH_FIELD_POSITION 0        /* 3 per fluid particle */
#define SPH_FIELD_VELOCITY 1        /* 3 */
#define SPH_FIELD_ACCELERATION 2    /* 3, non-pressure acceleration */
#define SPH_FIELD_DENSITY 3         /* 1 */
#define SPH_FIELD_PRESSURE 4        /* 1 (WCSPH / PCISPH) */
#define SPH_FIELD_ALPHA 5           /* 1 (DFSPH) */
#define SPH_FIELD_PRED_DENSITY 6    /* 1 (DFSPH) */
#define SPH_FIELD_DIV_ERROR 7       /* 1 (DFSPH) */
#define SPH_FIELD_KAPPA 8           /* 1 (DFSPH k) */
#define SPH_FIELD_KAPPA_V 9         /* 1 (DFSPH kv) */
#define SPH_FIELD_PRESSURE_ACC 10   /* 3 (PCISPH) */
#define SPH_FIELD_NORMAL 11         /* 3 (surface tension) */
#define SPH_FIELD_BOUNDARY_POSITION 12 /* 3 per boundary particle */
#define SPH_FIELD_BOUNDARY_VOLUME 13   /* 1 per boundary particle (psi) */
#define SPH_FIELD_BOUNDARY_DENSITY 14  /* 1 per boundary particle (PCISPH boundary model) */
#define SPH_FIELD_BOUNDARY_PRESSURE 15 /* 1 per boundary particle (PCISPH boundary model) */

/* Device status bits (sph_stats.status). */
#define SPH_STATUS_OUT_OF_GRID 1u   /* a particle left the grid box; it was kept in the border cell */
#define SPH_STATUS_NONFINITE 2u     /* a position or velocity (checked at every grid build) or a solver
                                       reduction is NaN/Inf */
#define SPH_STATUS_ITER_CAP 4u      /* density / pressure solve stopped at maxIterations */
#define SPH_STATUS_ITER_CAP_V 8u    /* divergence solve stopped at the iteration cap */
#define SPH_STATUS_DIVERGED 16u     /* pool: a particle's relative solver error exceeded 6e10 / n (n the
                                       scene's particles; 15,000 at 4M): the scene has blown up, its average
                                       error reads +Inf and its loop runs to the cap */
#define SPH_STATUS_BOUNDS 32u       /* bounds-checked build only (libsph_gb300_checked.so, -DSPH_BOUNDS_CHECK):
                                       a neighbour index read from a pair record or candidate list was out
                                       of range and skipped (a pool reports it with every scene) */

typedef struct sph_ctx sph_ctx;

/* Scene description: the fields of the reference's SceneInfo / Fluid /
 * Boundary structs (src/Simulation.h:47-131) that the particle loop uses,
 * plus device-path settings.  Fill with sph_scene_desc_init first. */
typedef struct sph_scene_desc {
    int simulation_method;        /* SPH_WCSPH / SPH_PCISPH / SPH_DFSPH */
    int boundary_method;          /* SPH_BOUNDARY_* */
    int precision;                /* SPH_PRECISION_* */
    double particle_radius;       /* r; support radius h = 4 r (Simulation.cpp:197) */
    double gravity[3];
    double time_step;             /* initial dt */
    double min_time_step, max_time_step, fps; /* min dt is min(min_time_step, 1/fps) (TimeManager.h:55) */
    double density0;
    double stiffness, gamma;      /* WCSPH */
    double max_error;             /* eta: PCISPH max / DFSPH average density error */
    double max_error_v;           /* DFSPH etaV */
    double cfl_factor;            /* DFSPH */
    int min_iterations, max_iterations;     /* < 0: solver default */
    int min_iterations_v, max_iterations_v; /* < 0: solver default */
    int viscosity_method;         /* SPH_VISCOSITY_* or -1 */
    double viscosity, boundary_viscosity;
    int surface_tension_method;   /* SPH_SURFACE_TENSION_AKINCI or -1 */
    double surface_tension;
    int adhesion_method;          /* SPH_ADHESION_AKINCI or -1 */
    double adhesion;
    int has_cube;                 /* cube boundary present (boundary_method 0) */
    double cube_min[3], cube_max[3];
    double domain_min[3], domain_max[3]; /* grid box; equal min/max: derive from the points */
    int threads_per_particle;     /* lanes per particle in the FP32 cell walks: 1, 2, 4, 8; 0 (default):
                                     8 below 20k fluid particles, 4 below 40k, 2 below 160k, else 1 */
    int neighbor_list_max;        /* DFSPH: > 0 builds per-particle pair lists with this many
                                     slots after each grid build and runs the solver walks over
                                     them; 0 walks the 27 cells in every pass */
    double bh_normal_fct;         /* PCISPH boundary model: normal and tangential velocity */
    double bh_tangential_fct;     /* factors of its collisions (scene "normalFct", "tangFct") */
} sph_scene_desc;

typedef struct sph_stats {
    double time;                  /* simulated time */
    double dt;                    /* current time step */
    double avg_density_error;     /* DFSPH: last predicted average density error */
    double avg_divergence_error;  /* DFSPH: last average divergence error */
    double max_density_error;     /* PCISPH: last maximum density error */
    double max_velocity;          /* DFSPH: max(0.1, sqrt(|v|)) of the last CFL step */
    unsigned iterations;          /* density / pressure iterations of the last step */
    unsigned iterations_v;        /* divergence iterations of the last step */
    unsigned steps;
    unsigned status;              /* SPH_STATUS_* bits, sticky */
    unsigned long long sum_iterations, sum_iterations_v;
    unsigned num_fluid, num_boundary;
    unsigned long long list_pairs; /* DFSPH pair lists: stored pairs (0 without lists) */
    unsigned list_overflow;       /* particles whose neighbours exceed neighbor_list_max */
    unsigned num_fluid_total;     /* FluidModel::getNumParticles: active + slots reserved by emitters;
                                     num_fluid is getNumActiveParticles */
    unsigned grid_growths;        /* times the grid box grew to take in particles that left it */
} sph_stats;

/* Defaults of the reference (SPHSolver.cpp:12-19, DFSPHSolver.cpp:10-22,
 * TimeManager.h:43-47, FluidModel.cpp:98). */
int sph_scene_desc_init(sph_scene_desc* desc);

/* Simulation::setSimulationMethod + setters (Simulation.cpp:207-231). */
int sph_ctx_create(const sph_scene_desc* desc, sph_ctx** out);
int sph_ctx_destroy(sph_ctx* ctx);

/* FluidModel::init (FluidModel.cpp:37-49): positions/velocities, xyz per
 * particle, FP64.  v may be NULL (zero). */
int sph_ctx_set_fluid(sph_ctx* ctx, const double* x, const double* v, unsigned n);
/* Simulation::buildFluidBlock (Simulation.cpp:512-539); appends. */
int sph_ctx_add_fluid_block(sph_ctx* ctx, const double min[3], const double max[3]);
/* AkinciBoundaryModel::addCube / addSphere (AkinciBoundayModel.cpp:42-98,
 * sampling :100-164); appends to the scene's boundary model. */
int sph_ctx_add_boundary_box(sph_ctx* ctx, const double min[3], const double max[3]);
int sph_ctx_add_boundary_sphere(sph_ctx* ctx, const double center[3], double radius);
/* Raw boundary points (xyz, FP64). */
int sph_ctx_add_boundary_points(sph_ctx* ctx, const double* x, unsigned n);
/* PCISPHBoundaryModel::addCube / ::addSphere (src/PCISPHBoundaryModel.cpp:7-54)
 * for boundary_method SPH_BOUNDARY_PCISPH: points with normals; `inverted`
 * non-zero points the normals into the box (a container) or towards the
 * sphere's centre.  sph_ctx_add_boundary_box / _sphere with this boundary
 * method add an inverted box and a solid sphere.  Boundary points without
 * normals (sph_ctx_add_boundary_points) are rejected for this model. */
int sph_ctx_add_pcisph_box(sph_ctx* ctx, const double mn[3], const double mx[3], int inverted);
int sph_ctx_add_pcisph_sphere(sph_ctx* ctx, const double c[3], double radius, int inverted);
/* PCISPHBoundaryModel points with their normals (xyz each, FP64) as the
 * model holds them (src/PCISPHBoundaryModel.h:12-16): for a caller that built
 * the model itself. */
int sph_ctx_add_pcisph_points(sph_ctx* ctx, const double* x, const double* normals, unsigned n);
/* AkinciBoundaryModel::addGeometry (AkinciBoundayModel.cpp:78-98,166-221):
 * the surface of a triangulated OBJ mesh sampled at most max_distance apart
 * (vertices, edges, then lines across each face; the scene file's
 * "geometry" entry passes spacing * 2r), rotated by pi/2 about x as the
 * reference places every mesh: (x, y, z) -> (x, -z, y).  Akinci boundary
 * model only. */
int sph_ctx_add_boundary_mesh(sph_ctx* ctx, const char* obj_path, double max_distance);

/* FluidModel::addEmitter (FluidModel.cpp:124-143, Emitter.cpp:10-29), before
 * sph_ctx_init: an emitter of num_particles particles, square (type
 * SPH_EMITTER_SQUARE, width x height) or circular (SPH_EMITTER_CIRCLE, radius
 * width), at position, rotated by the unit quaternion rotation = (w, x, y, z)
 * (the scene file's "rotation" array, SceneLoader.cpp:128-131), emitting along
 * its local z at speed velocity from start_time on, one group every
 * spacing * 1.105 * 2r / velocity seconds (Emitter.cpp:85-161).  Emitted
 * particles take the next original indices; sph_ctx_num_particles and the
 * downloads cover the active ones.  At most 64 emitters per scene; the
 * fluid set by sph_ctx_set_fluid may be empty when a scene has emitters. */
#define SPH_EMITTER_SQUARE 0
#define SPH_EMITTER_CIRCLE 1
int sph_ctx_add_emitter(sph_ctx* ctx, int type, unsigned num_particles, const double position[3], double velocity,
                        const double rotation[4], double start_time, double width, double height, double spacing);
/* Simulation::setEmittersPause (Simulation.h:316, Emitter.cpp:80-84): pause
 * (1) or resume (0) every emitter; both restart its clock at the current
 * time.  After sph_ctx_init. */
int sph_ctx_pause_emitters(sph_ctx* ctx, int pause);

/* Scene files (SceneLoader::readConfiguration SceneLoader.cpp:9-198 and
 * Simulation::importScene Simulation.cpp:331-494).  sph_ctx_load_scene reads
 * the JSON scene file and creates a context holding its fluid blocks,
 * emitters and boundary shapes, not yet initialised; sph_ctx_import_scene
 * also initialises it, as importScene does.  The reference's settings come
 * from the file; base (may be NULL for the defaults) supplies this
 * library's own: precision, threads_per_particle, neighbor_list_max and the
 * grid box.  The scene must have one fluid model and at most one Boundary
 * entry.  Mesh files ("geometry") are read relative to the working
 * directory, as the reference reads them, and sampled for the Akinci model
 * only; as in importScene, boundaryMethod 0 creates no boundary and the
 * PCISPH boundary model takes boxes and spheres only.  The context steps
 * only while Configuration.startTime <= time <= endTime and names frame
 * files after json_path (sph_ctx_set_frame_output).  On failure
 * sph_scene_load_error() describes the problem. */
int sph_ctx_load_scene(const char* json_path, const sph_scene_desc* base, sph_ctx** out);
int sph_ctx_import_scene(const char* json_path, const sph_scene_desc* base, sph_ctx** out);
const char* sph_scene_load_error(void);

/* Simulation::init -> solver->init (Simulation.cpp:102-110,
 * SPHSolver.cpp:22-39, DFSPHSolver.cpp:24-36, PCISPHSolver.cpp:12-19):
 * uploads, builds the grids, boundary volumes, and DFSPH densities/alpha. */
int sph_ctx_init(sph_ctx* ctx);

/* nsteps calls of Simulation::step -> solver->step (Simulation.cpp:148-182).
 * Asynchronous on the context's stream except where a solver loop needs a
 * convergence test read back (see sph_ctx_set_graph). */
int sph_ctx_step(sph_ctx* ctx, int nsteps);
/* sph_ctx_step bracketed by CUDA events on the context's stream; waits for
 * the steps and returns their device time in *elapsed_ms. */
int sph_ctx_step_timed(sph_ctx* ctx, int nsteps, float* elapsed_ms);
/* Wait for the context's stream. */
int sph_ctx_synchronize(sph_ctx* ctx);

/* Run whole steps as one CUDA graph with device-side solver loops
 * (conditional WHILE nodes): no host round trip per iteration.  1 = on. */
int sph_ctx_set_graph(sph_ctx* ctx, int enable);

/* The reference hashes cells without bounds (src/HashTable.h:79-102); the
 * dense grid box here grows instead.  Every 16 steps a context reads, without
 * waiting, whether a step kept a particle in a border cell (SPH_STATUS_OUT_OF_GRID);
 * if so, before its next step it re-plans the box around every point with a
 * 25 % margin (results unchanged; sph_stats.grid_growths counts it).  On by
 * default; 0 keeps the box fixed: particles outside it stay in the border cells,
 * neighbour sets still exact, walks slower.  The PCISPH boundary model keeps its
 * box (SPH_ERR_UNSUPPORTED for 1). */
int sph_ctx_set_grid_growth(sph_ctx* ctx, int enable);

/* Simulation::step / run (Simulation.cpp:148-190) and the frame export
 * (SceneLoader::writeFluid SceneLoader.cpp:200-264, TimeManager::hasToSave
 * TimeManager.h:101-110).  With a time window set (scene files set it) or
 * frame output on, sph_ctx_step reads the simulated time around every step:
 * it steps only while start <= time <= end, and after each step, once
 * 1/fps has passed since the last frame time, counts a frame and (output
 * on) writes it to scene_path with "_NNNN" (the frame number, first frame 1)
 * inserted before its last five characters (".json").  A frame file holds
 * numActiveParticles, numParticles (active plus emitter slots not yet
 * used), positions and velocities of every slot (unused ones zero), time
 * and timeStep.  sph_ctx_run steps until the time leaves the window or
 * max_steps have run; without frame output it steps in unchecked runs that
 * provably stay inside the window (the frame count then stands still).
 * Frame files are written by a host thread while the next steps run (the
 * state is captured on the device when the frame is due); they are complete
 * when sph_ctx_synchronize, sph_ctx_run or sph_ctx_destroy returns, which
 * also report a failed write.  sph_ctx_write_frame writes the current state
 * to any path, synchronously. */
int sph_ctx_set_time_window(sph_ctx* ctx, double start_time, double end_time);
int sph_ctx_set_frame_output(sph_ctx* ctx, const char* scene_path, int active);
int sph_ctx_get_frame(const sph_ctx* ctx, unsigned* frame);
int sph_ctx_write_frame(sph_ctx* ctx, const char* path);
int sph_ctx_run(sph_ctx* ctx, unsigned long long max_steps, unsigned long long* steps_done);

int sph_ctx_num_particles(const sph_ctx* ctx, unsigned* num_fluid, unsigned* num_boundary);
/* The descriptor the context was created with (for a loaded scene file:
 * the settings read from it). */
int sph_ctx_get_desc(const sph_ctx* ctx, sph_scene_desc* out);
/* Copy a field to host memory in original particle order (FP64). */
int sph_ctx_download(sph_ctx* ctx, int field, double* out);
/* Same result as sph_ctx_download, without allocating device memory.  It has
 * no counterpart in the reference (which keeps its fields in host vectors).
 * For callers that cannot allocate on the device: a frame-export hook in a
 * long-running serving process whose device memory is fully reserved for
 * resident scenes, or a real-time driver that must not call cudaFree (it
 * waits for the whole device).  sph_ctx_download allocates a staging buffer
 * per call; this variant stages through one fixed 4 MiB device array inside
 * the library instead.
 *   - Limit: a field of at most 524,288 values (174,762 particles for
 *     3-component fields); larger fields return SPH_ERR_CAPACITY.
 *   - The array is held by every GPU that loads the library until exit.
 *   - The first call on a device looks up the array's device address (with
 *     the context's device current); make that first call before any stream
 *     capture.  The address is kept until exit: after a cudaDeviceReset of
 *     a device, do not call this entry point on that device again.
 *   - All calls share the array: calls that overlap on the GPU (contexts used
 *     from several host threads at once) race.  Each call writes every value
 *     it returns, so nothing needs clearing between calls. */
int sph_ctx_download_noalloc(sph_ctx* ctx, int field, double* out);
int sph_ctx_get_stats(sph_ctx* ctx, sph_stats* out);
const char* sph_ctx_last_error(const sph_ctx* ctx);

/* Test hook: per fluid particle (original order) its cell floor(x/h)
 * (3 ints), its rank inside the cell, and the neighbour lists the solver
 * walks (fluid and boundary candidates with |xi - xj| / h <= 1, in walk
 * order).  Call with NULL arrays to get totals[0] (fluid pairs) and
 * totals[1] (boundary pairs) first. */
int sph_ctx_neighbors(sph_ctx* ctx, int* cells, int* cell_rank, int* nbr_off, int* nbr, int* bnbr_off, int* bnbr,
                      long long* totals);

/* Test hook: the DFSPH pair lists (neighbor_list_max > 0) that the solver
 * passes sum over, as the last grid build stored them: per fluid particle
 * (original order) every neighbour with a non-zero kernel gradient, in walk
 * order, as original indices.  These are the neighbourhoods of
 * HashTable::neighborhoodSearch (src/HashTable.h:136-170) that the
 * reference's DFSPH sums (DFSPHSolver.cpp:114-590): its candidates j != i
 * with 1e-5 < |xi - xj| < h.  count[i] is the particle's neighbour count; a
 * count above neighbor_list_max means the list overflowed and was not stored
 * (the passes walk that particle's cells instead) and contributes no entries.
 * Each array may be NULL; off has n + 1 entries (CSR), nbr needs off and
 * *total entries (the stored pairs, returned in any case). */
int sph_ctx_pair_lists(sph_ctx* ctx, int* count, int* off, int* nbr, long long* total);

/* Number of kernels of this library the context has launched (graph steps
 * counted from the captured graph and the iterations its loops ran). */
int sph_ctx_get_launch_count(sph_ctx* ctx, unsigned long long* out);
/* Per-kernel CUDA-event timing of host-driven steps (no effect in graph
 * mode).  sph_ctx_get_profile writes "name launches total_ms" lines for the
 * launches since the previous call and returns the text length. */
int sph_ctx_set_profiling(sph_ctx* ctx, int enable);
int sph_ctx_get_profile(sph_ctx* ctx, char* buf, unsigned long long len);
/* Step phases under the reference's phase-timer names
 * (Simulation::startCounting/stopCounting: DFSPHSolver.cpp:43-101,
 * PCISPHSolver.cpp:26-67, WCSPHSolver.cpp:20-64, "Step computation"
 * Simulation.cpp:158; fused phases join the names with '+').  Every phase is
 * an NVTX range; with profiling on, sph_ctx_get_phase_profile writes
 * "name<TAB>count<TAB>total_ms" lines for the phases timed (CUDA events)
 * since the previous call and returns the text length.  A graph step is one
 * "Step computation" phase. */
int sph_ctx_get_phase_profile(sph_ctx* ctx, char* buf, unsigned long long len);

/* cudaSetDevice for the calling thread; contexts created afterwards live on
 * that device. */
int sph_select_device(int device);

/* ------------------------------------------------------------------------
 * Batched pool: many independent DFSPH scenes (Akinci boundaries, FP32, pair
 * lists) resident on one GPU and advanced together.  No counterpart in the
 * reference, which holds one scene per process (Simulation singleton,
 * src/Simulation.cpp:84-90); each pooled scene runs the same per-step loop as
 * sph_ctx_step, and its results do not depend on which other scenes share
 * the pool.  Scenes are admitted and removed between steps.  A pool may be
 * shared by several host threads (a thread submitting scenes while another
 * steps and polls): calls on one pool are serialised, and each runs on the
 * device the pool was created on.
 * ------------------------------------------------------------------------ */
typedef struct sph_pool sph_pool;

typedef struct sph_pool_desc {
    unsigned long long max_particles;   /* fluid particles resident at once */
    unsigned long long max_boundary;    /* boundary particles resident at once */
    unsigned long long max_keys;        /* total grid key space of resident scenes */
    unsigned max_scenes;
    int neighbor_list_max;              /* pair-list slots per particle */
} sph_pool_desc;

/* Capacities that fit a device-memory budget in bytes. */
int sph_pool_desc_from_budget(unsigned long long hbm_bytes, int neighbor_list_max, sph_pool_desc* out);
int sph_pool_create(const sph_pool_desc* desc, sph_pool** out);
int sph_pool_destroy(sph_pool* pool);
/* Queue a scene (fluid x/v and Akinci boundary points, xyz FP64) to run for
 * `steps` steps; it becomes resident at the next sph_pool_step.  Returns
 * SPH_ERR_CAPACITY when it does not fit beside the resident and queued
 * scenes (admission control). */
int sph_pool_add_scene(sph_pool* pool, const sph_scene_desc* desc, const double* x, const double* v, unsigned n,
                       const double* boundary_x, unsigned nb, unsigned steps, int* scene_id);
/* Release a scene (finished or not) at the next step. */
int sph_pool_remove_scene(sph_pool* pool, int scene_id);
/* nsteps steps of every resident scene that still has steps to run;
 * nsteps = 0 only applies pending admissions and removals (new scenes
 * become resident with their initial densities, alpha factors and pair
 * lists, DFSPHSolver::init). */
int sph_pool_step(sph_pool* pool, int nsteps);
/* Whole pool steps as one CUDA graph with device-side solver loops. */
int sph_pool_set_graph(sph_pool* pool, int enable);
int sph_pool_synchronize(sph_pool* pool);
/* Statistics of one scene; *done = 1 once its steps have completed.  A
 * scene whose solver reductions turned NaN / Inf (SPH_STATUS_NONFINITE) is
 * retired after that step: done, with fewer steps than it asked for. */
int sph_pool_query(sph_pool* pool, int scene_id, sph_stats* out, int* done);
/* Ids of resident scenes whose steps have completed (up to max_ids). */
int sph_pool_poll(sph_pool* pool, int* done_ids, int max_ids, int* num_done);
/* A field of one resident scene (original particle order, FP64). */
int sph_pool_download(sph_pool* pool, int scene_id, int field, double* out);
int sph_pool_usage(sph_pool* pool, unsigned long long* particles, unsigned long long* boundary,
                   unsigned long long* keys, unsigned* scenes);
int sph_pool_get_launch_count(sph_pool* pool, unsigned long long* out);
/* sph_pool_step bracketed by CUDA events on the pool's stream (admissions are
 * applied before the first event); returns the device time in *elapsed_ms. */
int sph_pool_step_timed(sph_pool* pool, int nsteps, float* elapsed_ms);
/* Per-kernel CUDA-event timing of host-driven pool steps, reported as
 * "name launches total_ms" lines (as sph_ctx_get_profile). */
int sph_pool_set_profiling(sph_pool* pool, int enable);
int sph_pool_get_profile(sph_pool* pool, char* buf, unsigned long long len);
/* As sph_ctx_get_phase_profile, for the pool's steps (relayouts excluded). */
int sph_pool_get_phase_profile(sph_pool* pool, char* buf, unsigned long long len);
/* Launch shapes of the pool's hot kernels.  Results do not depend on them. */
typedef struct sph_pool_tuning {
    int build_block;      /* pair-list build: threads per block and threads per SM */
    int build_occupancy;  /* the register budget allows: (128, 896), (128, 1024), (256, 768), (256, 1024) */
    int queue_depth;      /* candidates staged per particle in shared memory by the build: 8..64, multiple of 8 */
    int solver_block;     /* solver passes: threads per block (128 or 256) and threads per SM */
    int solver_occupancy; /* the register budget allows (1024, 1536 or 2048) */
    int scan_width;       /* grid keys per thread of the cell-count scan (sort width): 4, 8 or 16 */
    int source;           /* 0 defaults or set by the caller, 1 tuning cache, 2 measured */
    int steps_left;       /* tuning steps still to run (read only) */
} sph_pool_tuning;
/* Autotuner (no reference counterpart): mode 0 off (keep the current
 * shapes), 1 (default) after each re-layout use the cached shapes for this
 * GPU model / particle-count bucket / list width or measure them over the
 * next 24 steps (ordinary steps of every resident scene, host-driven), 2 as 1
 * but measure again.  The cache is a text file (SPH_GB300_TUNE_FILE, default
 * ~/.cache/sph_gb300_tune.txt). */
int sph_pool_set_autotune(sph_pool* pool, int mode);
int sph_pool_get_tuning(sph_pool* pool, sph_pool_tuning* out);
/* Fixed shapes (turns the autotuner off); values outside the sets above are
 * rejected with SPH_ERR_INVALID. */
int sph_pool_set_tuning(sph_pool* pool, const sph_pool_tuning* tuning);
/* The last measurement, one "candidate: ms" line per candidate. */
int sph_pool_get_tuning_log(sph_pool* pool, char* buf, unsigned long long len);
/* Checkpoint / resume of one pooled scene.  The reference keeps no resumable
 * state (its frame files, SceneLoader::writeFluid src/SceneLoader.cpp:200-264,
 * hold positions and velocities only, without the time step, the DFSPH
 * warm-start k / kv or the iteration history).  A snapshot holds the scene's
 * device state as stored (cell-relative FP32 positions with their cells,
 * velocities, k, kv, predicted densities, boundary points), its grid box, its
 * solver scalars (time, dt, steps, iteration counts and sums, status) and the
 * steps it has left; a scene restored from it, on this pool or another one of
 * the same library version, continues bit for bit as if never interrupted.
 * sph_pool_snapshot with buf NULL returns the size in *size; it waits for the
 * pool's stream.  sph_pool_restore admits the scene (resident at the next
 * step) with `steps` more steps to run, 0 for the steps it had left. */
int sph_pool_snapshot(sph_pool* pool, int scene_id, void* buf, unsigned long long capacity, unsigned long long* size);
int sph_pool_restore(sph_pool* pool, const void* buf, unsigned long long size, unsigned steps, int* scene_id);
/* A resident scene's pair lists, as sph_ctx_pair_lists (original indices
 * within the scene). */
int sph_pool_pair_lists(sph_pool* pool, int scene_id, int* count, int* off, int* nbr, long long* total);
/* Pair-list occupancy: stored pairs and particles whose neighbours overflow. */
int sph_pool_list_pairs(sph_pool* pool, unsigned long long* pairs, unsigned* overflow);
/* The list build's work at the current positions (a diagnostic pass, for its
 * FP32 roofline): out[0..3] = fluid candidates its walks visit (27 cells,
 * trimmed), fluid pairs within h, boundary candidates, boundary pairs. */
int sph_pool_count_work(sph_pool* pool, unsigned long long out[4]);
const char* sph_pool_last_error(const sph_pool* pool);

/* ------------------------------------------------------------------------
 * Request loop over a pool (no counterpart in the reference): clients submit
 * scenes from any thread; one driver thread steps the pool in epochs of
 * epoch_steps, admits queued scenes between epochs as capacity frees up (in
 * arrival order, trying the first `lookahead`, so a scene that does not fit
 * does not block smaller ones behind it), and retires completed scenes.
 * Admission's host work overlaps the epoch running on the device.  While a
 * server exists, only its driver steps the pool.  Latency is measured from
 * sph_server_submit to the poll that found the scene complete.
 * ------------------------------------------------------------------------ */
typedef struct sph_server sph_server;
typedef struct sph_server_desc {
    unsigned epoch_steps;   /* pool steps between admission passes (default 10) */
    unsigned lookahead;     /* queued requests tried per admission pass (default 8) */
    int keep_results;       /* keep each completed scene's final positions and velocities (sph_server_fetch) */
    unsigned long long max_queued_bytes;  /* host bytes of queued (not yet admitted) requests; a submission
                                           * beyond it is rejected with SPH_ERR_CAPACITY (0: no bound) */
} sph_server_desc;
#define SPH_REQUEST_QUEUED 0
#define SPH_REQUEST_RESIDENT 1
#define SPH_REQUEST_DONE 2
#define SPH_REQUEST_FAILED 3   /* rejected by the pool (not capacity): sph_pool_last_error */
typedef struct sph_request_info {
    long long id;
    int state;              /* SPH_REQUEST_* */
    unsigned num_fluid, steps, steps_done, status;  /* status: SPH_STATUS_* bits of the scene */
    double latency_s;       /* submission to completion (SPH_REQUEST_DONE) */
} sph_request_info;
typedef struct sph_server_stats {
    unsigned long long submitted, admitted, completed, failed, queued, resident, epochs;
    double wall_s;                    /* since sph_server_create */
    double particle_steps;            /* completed scenes' plus resident scenes' steps so far, x particles */
    double particle_steps_per_s;
    double p50_latency_s, p99_latency_s, mean_latency_s;  /* over completed requests */
    unsigned long long rejected;      /* submissions refused by max_queued_bytes */
    unsigned long long queued_bytes;  /* host bytes held by queued requests */
} sph_server_stats;
int sph_server_desc_init(sph_server_desc* desc);
int sph_server_create(sph_pool* pool, const sph_server_desc* desc, sph_server** out);
/* Stops the driver after its current epoch (resident scenes stay in the pool). */
int sph_server_destroy(sph_server* server);
/* Queue a scene (the arrays are copied; the call does not wait for the GPU).
 * SPH_ERR_CAPACITY: the queue holds max_queued_bytes already (nothing
 * queued, no request id). */
int sph_server_submit(sph_server* server, const sph_scene_desc* desc, const double* x, const double* v, unsigned n,
                      const double* boundary_x, unsigned nb, unsigned steps, long long* request_id);
/* Requests completed (or failed) since the previous call, up to max. */
int sph_server_completed(sph_server* server, sph_request_info* out, int max, int* num);
int sph_server_query(sph_server* server, long long request_id, sph_request_info* out);
/* A completed request's final SPH_FIELD_POSITION or SPH_FIELD_VELOCITY
 * (keep_results), original particle order, 3 doubles per particle. */
int sph_server_fetch(sph_server* server, long long request_id, int field, double* out);
int sph_server_release(sph_server* server, long long request_id);
/* Wait until nothing is queued or resident, at most timeout_s seconds. */
int sph_server_drain(sph_server* server, double timeout_s, int* idle);
int sph_server_get_stats(sph_server* server, sph_server_stats* out);
const char* sph_server_last_error(const sph_server* server);

/* Sampling helpers with the reference's point sets, usable without a
 * context; out may be NULL to query the count.  Return the point count. */
long long sph_sample_box(double support_radius, const double min[3], const double max[3], double* out);
/* PCISPHBoundaryModel::sampleCube: points and normals (out, normals may be
 * NULL to count). */
long long sph_sample_pcisph_box(double support_radius, const double mn[3], const double mx[3], int inverted,
                                double* out, double* normals);
long long sph_sample_sphere(double particle_radius, const double center[3], double radius, double* out);
long long sph_fluid_block(double particle_radius, const double min[3], const double max[3], double* out);
/* Emitter::buildSquareGroup / buildCircleGroup (Emitter.cpp:31-79): the
 * group an emitter emits each time, in its local frame (out may be NULL). */
long long sph_emitter_group(int type, double particle_radius, double width, double height, double* out);
/* The points sph_ctx_add_boundary_mesh adds (out may be NULL to count; -1
 * when the file cannot be read or is malformed). */
long long sph_sample_mesh(const char* obj_path, double max_distance, double* out);

/* Build identification string. */
const char* sph_version(void);

#ifdef __cplusplus
}
#endif
#endif
