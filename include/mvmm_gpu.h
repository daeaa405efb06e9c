/*
 * mvmm_gpu: GB300 (sm_103a) implementation of mvmm_hydro's per-face
 * finite-volume update, behind a plain C ABI.
 *
 * This header is the drop-in boundary.  Each entry point names the reference
 * interface it replaces (paths inside the mvmm_hydro source tree).  Every
 * function returns 0 on success or a negative MVMM_E* code; the text of the
 * last error is available from mvmm_last_error().  Soft numerical failures
 * that the reference reports by panicking (a stuck Newton iteration, negative
 * mass, ...) are returned as MVMM_E_NUMERIC with the bits of mvmm_error_bits().
 *
 * Memory: all device memory is owned by the context; callers pass host
 * pointers (pageable or pinned) and sizes only.  A context is used by one host
 * thread at a time and orders all its work on one CUDA stream (mvmm_step_cells
 * adds a second stream for overlapped copies and joins it before returning).
 */
#ifndef MVMM_GPU_H
#define MVMM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- enums ---------------------------------------------------------- */
/* Riemann solver kind: riemann_solver.rs:28-44 and bin/main.rs:625-642
 * ("HLLC", "Exact", "PVRS", "AIRS", "TSRS", "TRRS", "LinearAdvection"). */
enum {
    MVMM_RIEMANN_HLLC = 0,
    MVMM_RIEMANN_EXACT = 1,
    MVMM_RIEMANN_PVRS = 2,
    MVMM_RIEMANN_AIRS = 3,            /* airs.rs:18-38, needs airs_threshold */
    MVMM_RIEMANN_TSRS = 4,            /* tsrs.rs:25-51 */
    MVMM_RIEMANN_TRRS = 5,            /* trrs.rs:14-32 */
    MVMM_RIEMANN_LINEAR_ADVECTION = 6 /* linear_advection.rs:17-34, needs advection_velocity */
};
/* Runner: bin/main.rs:667-673 ("OptimalOrder", "Godunov"). */
enum { MVMM_RUNNER_OPTIMAL_ORDER = 0, MVMM_RUNNER_GODUNOV = 1 };
/* Boundary: space.rs:26-32. */
enum { MVMM_BOUNDARY_PERIODIC = 0, MVMM_BOUNDARY_REFLECTIVE = 1, MVMM_BOUNDARY_OPEN = 2, MVMM_BOUNDARY_VACUUM = 3 };
/* Equation of state: gas_law.rs:66-70. */
enum { MVMM_EOS_IDEAL = 0, MVMM_EOS_ISOTHERMAL = 1 };
/* Arithmetic form of the face stage. */
enum {
    MVMM_PRECISION_FP64 = 0,    /* plain: everything FP64, reference evaluation order */
    MVMM_PRECISION_FP32FACE = 1 /* reconstruction, limiter, gradients, Riemann solve and
                                   face fluxes FP32 (face geometry formed in FP64 and
                                   rounded once; the exact solver's Newton sum FP64);
                                   conserved state, flux accumulation, timesteps and the
                                   integer timeline FP64 */
};
/* Particle motion: engine.rs:7-13, Particle::set_particle_velocity
 * (part.rs:328-372).  For the moving modes the host rebuilds the Voronoi mesh
 * from the drifted generators (mvmm_drift, mvmm_get_positions, mvmm_set_mesh)
 * before each step; in an open or vacuum box it also removes the generators
 * that left (space.rs:840-853) and creates a context over the others. */
enum { MVMM_MOTION_FIXED = 0, MVMM_MOTION_STEER = 1, MVMM_MOTION_STEER_PAKMOR = 2, MVMM_MOTION_FLUID = 3 };

/* ---- status codes / error bits --------------------------------------- */
enum {
    MVMM_OK = 0,
    MVMM_E_INVALID = -1,  /* bad argument / size / state */
    MVMM_E_CUDA = -2,     /* CUDA runtime error */
    MVMM_E_NUMERIC = -3,  /* see mvmm_error_bits */
    MVMM_E_NOMEM = -4,
    MVMM_E_UNSUPPORTED = -5
};
enum {
    MVMM_ERR_NEWTON_CAP = 1u << 0,    /* exact.rs:272-274 (panic in the reference) */
    MVMM_ERR_BRENT_BRACKET = 1u << 1, /* exact.rs:132-134 */
    MVMM_ERR_NEG_MASS = 1u << 2,      /* part.rs:220 */
    MVMM_ERR_NEG_ENERGY = 1u << 3,    /* part.rs:221-224, 227-231 */
    MVMM_ERR_NONFINITE = 1u << 4,     /* part.rs:180-182, 249-260 */
    MVMM_ERR_NEG_PRIM = 1u << 5,      /* part.rs:246-247, physical_quantities.rs:220-221 */
    MVMM_ERR_ZERO_DTI = 1u << 6,      /* timeline.rs:397 */
    MVMM_ERR_BOUNDS = 1u << 7         /* a mesh index outside its array (checked on upload) */
};

/* ---- plain structs ---------------------------------------------------- */
/* EulerEqnsFvs::new(riemann_solver, cfl, gas_law) (euler_eqns_fvs.rs:13-17)
 * plus the engine/space settings the per-face update reads. */
typedef struct mvmm_params {
    double gamma;                      /* GasLaw::new(gamma, ..) */
    int eos;                           /* MVMM_EOS_* */
    double isothermal_internal_energy; /* EquationOfState::Isothermal payload */
    double cfl;                        /* cfl_criterion */
    int riemann;                       /* MVMM_RIEMANN_* */
    int boundary;                      /* MVMM_BOUNDARY_* */
    int dimensionality;                /* 1, 2, 3 */
    int sync_all;                      /* time_integration.sync_timesteps */
    double t_end;                      /* defines time_base = t_end / 2^57 (engine.rs:118) */
    int max_newton_iter;               /* exact solver cap, 1000 in the reference */
    int precision;                     /* MVMM_PRECISION_* */
    int particle_motion;               /* MVMM_MOTION_* */
    int runner;                        /* MVMM_RUNNER_*: OptimalOrderRunner or GodunovHydroRunner */
    double airs_threshold;             /* AIRiemannSolver::new(threshold); NaN = missing */
    double advection_velocity[3];      /* LinearAdvectionRiemannSover::new(velocity) */
    double box_size[3];                /* Space::box_size; periodic wrap of drifted generators */
    /* The gravity solver (bin/main.rs:643-662, gravity.rs).  The runners take
     * its timestep per cell where smaller (optimal_order.rs:47-50,
     * godunov.rs:41-44).  They never compute accelerations (the "TODO: gravity"
     * at optimal_order.rs:33), so a_grav stays zero and the kicks kick2 / kick1
     * add nothing; gravity_accelerations = 1 computes the accelerations at
     * that point instead (the external potential's, or self-gravity's direct
     * sum over j > i, gravity.rs:22-43), and the kicks apply them
     * (Particle::grav_kick, part.rs:303-312). */
    int gravity;                     /* MVMM_GRAVITY_* */
    double gravity_softening;        /* SelfGravity / KeplerianPotential softening_length */
    double gravity_acceleration[3];  /* Potential::Constant acceleration */
    double gravity_position[3];      /* KeplerianPotential position */
    int gravity_accelerations;       /* 0: as the reference; 1: the accelerations kick (not
                                        through mvmm_step_cells) */
    /* The cell-wise limiter's extrapolation to a face.  0 (the reference,
     * runner/hydrodynamics.rs:119): face centroid - centroid - shift for the
     * left cell, + shift for the right one.  flux_exchange puts the face
     * centroid in the left cell's frame (flux.rs:33-35), so across a periodic
     * seam those offsets are a box length long and the limiter misbehaves
     * there (a shear layer stops advancing its time).  1: the offsets in
     * flux_exchange's frame, face centroid - centroid (left) and face centroid
     * - shift - centroid (right); not the reference's arithmetic. */
    int limiter_frame;
} mvmm_params;
/* Gravity solver kind (bin/main.rs:643-662). */
enum { MVMM_GRAVITY_NONE = 0, MVMM_GRAVITY_SELF = 1, MVMM_GRAVITY_CONSTANT = 2, MVMM_GRAVITY_KEPLERIAN = 3 };

/* Cell state, SoA, n cells.  Row layout [components][n]; grad row 3*q+k is
 * d(quantity q)/d(axis k).  Mirrors Particle (part.rs:10-39). */
typedef struct mvmm_cells {
    int64_t n;
    double *cons, *prim, *grad, *gc, *extrap, *facc;
    double *volume, *loc, *centroid, *v, *v_rel;
    double *max_a_over_r, *max_signal_velocity, *dt;
    int8_t *timebin;
} mvmm_cells;

/* Face list + cell->face CSR: Vec<VoronoiFace> + voronoi_cell_face_connections
 * (space.rs:70-81).  right < 0 encodes face.right() == None; shift is zero
 * where face.shift() is None.  normal/centroid/shift are [3][n_faces]. */
typedef struct mvmm_mesh {
    int64_t n_cells, n_faces;
    const int32_t *left, *right;
    const double *area, *normal, *centroid, *shift;
    const int32_t *csr_off, *csr_face; /* [n_cells+1], [csr_off[n_cells]] */
} mvmm_mesh;

typedef struct mvmm_ctx mvmm_ctx;

/* ---- context ---------------------------------------------------------- */
/* Builds the solver: replaces `EulerEqnsFvs::<R>::new` (euler_eqns_fvs.rs:13-17)
 * as constructed in bin/main.rs:625-642, and takes ownership of a device copy
 * of the mesh produced by Space::initialize (space.rs:88-211). */
int mvmm_ctx_create(const mvmm_params *params, const mvmm_mesh *mesh, mvmm_ctx **out);
int mvmm_ctx_destroy(mvmm_ctx *ctx);
/* Batched context (no counterpart in the reference, which runs one simulation
 * per process): n_instances independent simulations packed into one mesh.
 * Cells of instance k are cell_offsets[k] .. cell_offsets[k+1]-1 and no face
 * may join two instances; each instance has its own integer timeline with
 * time_base = t_end[k] / 2^57, all share params (gamma, solver, boundary, ...).
 * Every stage of a step is one launch over all instances; finished instances
 * are skipped.  mvmm_step / mvmm_run / mvmm_enqueue_steps step every unfinished
 * instance from its own device timeline (their ti arguments are ignored for a
 * batch); mvmm_run returns when all are finished. */
int mvmm_ctx_create_batched(const mvmm_params *params, const mvmm_mesh *mesh, int64_t n_instances,
                            const int64_t *cell_offsets, const double *t_end, mvmm_ctx **out);
/* Per-instance timeline state, arrays of n_instances (any may be NULL). */
int mvmm_batch_state(mvmm_ctx *ctx, uint64_t *ti_current, uint64_t *ti_old, int64_t *steps, int64_t *active_faces,
                     uint32_t *err_bits, int *finished);
/* Runs all work of this context on the given cudaStream_t (NULL = own stream). */
int mvmm_ctx_set_stream(mvmm_ctx *ctx, void *cuda_stream);
/* Host <-> device copies of the whole cell state (the &mut [Particle] the
 * FiniteVolumeSolver trait passes on every call, finite_volume_solver.rs:9-17). */
int mvmm_upload_cells(mvmm_ctx *ctx, const mvmm_cells *cells);
int mvmm_download_cells(mvmm_ctx *ctx, mvmm_cells *cells);
uint32_t mvmm_error_bits(mvmm_ctx *ctx);
const char *mvmm_last_error(void);

/* ---- FiniteVolumeSolver trait (finite_volume_solver.rs:9-17) ------------ */
/* predict(&self, particles, dt)  (euler_eqns_fvs.rs:20-24) */
int mvmm_predict(mvmm_ctx *ctx, double dt);
/* compute_fluxes(&self, faces, particles, part_is_active, boundary) -> Vec<FluxInfo>
 * (euler_eqns_fvs.rs:26-48).  active: host uint8[n]; fluxes_out: host
 * double[10][n_faces] = (fluxes 5, mflux 3, v_max, a_over_r) (flux.rs:10-21). */
int mvmm_compute_fluxes(mvmm_ctx *ctx, const uint8_t *active, double *fluxes_out, int64_t *n_active_faces);
/* convert_conserved_to_primitive(&self, particles, part_is_active) (euler_eqns_fvs.rs:63-69) */
int mvmm_convert_conserved_to_primitive(mvmm_ctx *ctx, const uint8_t *active);
/* compute_timesteps(&self, particles, part_is_active, motion, dim) -> Vec<f64>
 * (euler_eqns_fvs.rs:50-61); dt_out: host double[n] (INFINITY if inactive). */
int mvmm_compute_timesteps(mvmm_ctx *ctx, const uint8_t *active, double *dt_out);

/* ---- GravitySolver trait (gravity.rs:6-10) ----------------------------- */
/* compute_timesteps(&self, particles) -> Vec<f64> (gravity.rs:45-53, 71-73,
 * 90-95, 119-123): dt_out host double[n]; INFINITY where the solver sets no
 * limit (self-gravity with zero accelerations, a constant potential). */
int mvmm_gravity_timesteps(mvmm_ctx *ctx, double *dt_out);
/* compute_accelerations(&self, particles) (gravity.rs:22-43, 67-70, 81-86,
 * 110-136): a_out host double[3][n].  Self-gravity sums over the current
 * masses and positions and, as the reference's &mut form does, replaces the
 * stored a_grav the self-gravity timestep and kicks read. */
int mvmm_gravity_accelerations(mvmm_ctx *ctx, double *a_out);

/* ---- runner free functions (runner/hydrodynamics.rs) ----------------- */
/* apply_fluxes + kick2 (runner/hydrodynamics.rs:13-39, 51-57); fluxes: host double[10][n_faces]. */
int mvmm_apply_fluxes(mvmm_ctx *ctx, const double *fluxes, const uint8_t *active);
/* gradient_estimate + gradient_limit + gradient_apply (runner/hydrodynamics.rs:67-143). */
int mvmm_gradients(mvmm_ctx *ctx, const uint8_t *active);

/* ---- Runner::step / Engine::run --------------------------------------- */
/* OptimalOrderRunner::step (runner/hydrodynamics/optimal_order.rs:15-64) at
 * integer time ti_current with the previous sync point ti_old; returns ti_next
 * and the number of faces that reached flux_exchange*. */
int mvmm_step(mvmm_ctx *ctx, uint64_t ti_current, uint64_t ti_old, uint64_t *ti_next, int64_t *n_active_faces);
/* ---- moving meshes ------------------------------------------------------ */
/* Space::drift (space.rs:833-854, part.rs:107-119): every cell's generator,
 * centroid and gradients centroid move by v*dt; generators that leave a
 * periodic box are wrapped (part.rs:449-455), those that leave a reflective
 * box are mirrored back with their primitive velocity and gradients reflected
 * (Particle::box_reflect, part.rs:457-469); in an open or vacuum box they stay
 * outside for the host to remove.  Engine::run calls it between sync points
 * (engine.rs:164-176). */
int mvmm_drift(mvmm_ctx *ctx, double dt);
/* The generator positions loc [3][n] (what Space::volume_calculation feeds the
 * Voronoi builder, space.rs:236-263). */
int mvmm_get_positions(mvmm_ctx *ctx, double *loc);
/* Space::volume_calculation's result (space.rs:236-263): the new face list and
 * cell->face CSR replace the mesh now; volume and centroid [3][n] of the new
 * cells are applied to the active cells of the next step after its predict
 * stage (Particle::update_geometry, part.rs:151-158). */
int mvmm_set_mesh(mvmm_ctx *ctx, const mvmm_mesh *mesh, const double *volume, const double *centroid);
/* Page-locked host memory (cudaHostAlloc) for arrays a host hands to the
 * copying calls (mvmm_set_mesh, mvmm_step_cells, the uploads and downloads):
 * copies from and to it run at the link's speed instead of through a staging
 * buffer.  No counterpart in the reference (its state lives on the host). */
int mvmm_host_alloc(size_t bytes, void **ptr);
int mvmm_host_free(void *ptr);

/* Runner::step(&mut Space, ..) on host-resident state (runner.rs:6-22): uploads
 * `in`, runs one step (OptimalOrderRunner or GodunovHydroRunner) of a fixed
 * mesh and writes the new state to `out` (which may be `in`, wholly or field by
 * field) in one call.  Copies of the rows the update alone reads and of the
 * rows final after it overlap the other stages.  Where the device can address
 * the host arrays (pinned memory, or pageable memory on systems whose GPU uses
 * the host page tables) the copies run as kernels; arrays `out` shares with
 * `in` then receive only the 8 KB chunks the step changed.  volume, loc and
 * centroid, which the step does not change, are not copied back.  Single
 * simulations only. */
int mvmm_step_cells(mvmm_ctx *ctx, const mvmm_cells *in, mvmm_cells *out, uint64_t ti_current, uint64_t ti_old,
                    uint64_t *ti_next, int64_t *n_active_faces);
/* Runner::step(&mut Space, ..) on host-resident state (runner.rs:6-22) that
 * moves only what changed.  The context keeps a device mirror of `cells`:
 * `cells` must hold what the previous call left in it, except for the
 * n_changed cells listed in `changed`, whose rows (every field and the time
 * bin) the caller may have rewritten; those are read from the host, one step
 * runs, and the cells the step rewrote are written back into `cells` in place,
 * 32 consecutive cells at a time: all rows but volume, loc and centroid (which
 * a fixed mesh keeps) where one of them changed more than its extrapolations
 * (a hierarchical step: the active cells and their neighbours), else the
 * extrapolation rows where those moved.  changed = NULL uploads every
 * cell: the first call, and any call whose arrays the previous call did not
 * leave.  The device must address the arrays (pinned memory, or pageable
 * memory where the GPU uses the host page tables); else MVMM_E_UNSUPPORTED.
 * *bytes_stored (or NULL): the bytes this call wrote into `cells`.  Single
 * simulations of a fixed mesh. */
int mvmm_step_cells_changed(mvmm_ctx *ctx, mvmm_cells *cells, const int32_t *changed, int64_t n_changed,
                            uint64_t ti_current, uint64_t ti_old, uint64_t *ti_next, int64_t *n_active_faces,
                            int64_t *bytes_stored);
/* Engine::run (engine.rs:152-199) from the given sync point, device resident:
 * runs at most max_steps steps (<= 0: to t_end).  On return *ti_current /
 * *ti_old are the next sync point; *steps_done and *n_active_faces count the
 * work done; *finished is 1 once the step at t_end has run. */
int mvmm_run(mvmm_ctx *ctx, int64_t max_steps, uint64_t *ti_current, uint64_t *ti_old, int64_t *steps_done,
             int64_t *n_active_faces, int *finished);
/* Enqueues n steps on the context stream without synchronising (for timing
 * with events recorded on the same stream); state advances on the device. */
int mvmm_enqueue_steps(mvmm_ctx *ctx, int64_t n_steps);
/* Hierarchical steps of one simulation on a fixed mesh defer the time
 * extrapolation of inactive cells (Particle::extrapolate_state, part.rs:123-132)
 * until a step reads the cell; the state on the device is complete once this
 * call's work has run.  Enqueued on the context stream without synchronising
 * (timing with events); mvmm_download_cells and the per-stage calls do it
 * themselves.  No counterpart in the reference, which extrapolates every cell
 * each step. */
int mvmm_flush_deferred(mvmm_ctx *ctx);
/* Sets the device timeline to (ti_current, ti_old) before mvmm_enqueue_steps. */
int mvmm_set_time(mvmm_ctx *ctx, uint64_t ti_current, uint64_t ti_old);
/* Reads the device timeline and counters (synchronises the stream). */
int mvmm_get_time(mvmm_ctx *ctx, uint64_t *ti_current, uint64_t *ti_old, int64_t *steps, int64_t *active_faces,
                  int *finished);
/* Counters of the device timeline since the context was created: steps run,
 * faces that reached flux_exchange*, active cells, and (FP32-face form with
 * the exact solver) faces whose pressure came from the full FP64 iteration
 * instead of the FP32 search + FP64 Newton polish.  Synchronises the stream.
 * No counterpart in the reference (its status line prints step counts only). */
typedef struct mvmm_stats {
    int64_t steps, active_faces, active_cells, fp64_fallback_faces;
    /* bytes moved between host arrays and the device by the cell copies
     * (mvmm_upload_cells, mvmm_download_cells, mvmm_step_cells) */
    int64_t host_bytes_in, host_bytes_out;
} mvmm_stats;
int mvmm_get_stats(mvmm_ctx *ctx, mvmm_stats *out);
/* Autotuner (no counterpart in the reference): times `steps` steps of this
 * context's own workload for each thread-block size of the face kernel and of
 * the cell kernels (64, 128, 256), keeps the fastest pair and restores the
 * state it started from (it allocates a temporary device copy of the cell
 * state).  Returns the chosen sizes. */
int mvmm_autotune(mvmm_ctx *ctx, int steps, int *blk_face, int *blk_cell);
/* Per-kernel timing of the step (events around each kernel on the context
 * stream): enable, then read the accumulated milliseconds and launch counts
 * of the MVMM_NUM_KERNELS kernels in the order predict, face_flux, update,
 * gradient_timestep, limiter, end. */
#define MVMM_NUM_KERNELS 6
int mvmm_profile_enable(mvmm_ctx *ctx, int enable);
int mvmm_profile_read(mvmm_ctx *ctx, double *ms, int64_t *launches);

/* ---- RiemannFluxSolver (riemann_solver.rs:78-87) ---------------------- */
/* solve_for_flux over arrays: left/right [5][n] primitive states, v_face and
 * normal [3][n], out [5][n]; host pointers.  precision selects the FP64 or
 * FP32 arithmetic form. */
int mvmm_riemann_flux(int kind, int precision, double gamma, int64_t n, const double *left, const double *right,
                      const double *v_face, const double *normal, double *out);
/* RiemannStarSolver::sample preceded by the vacuum test of the blanket
 * solve_for_flux (riemann_solver.rs:224-287): half state at x/t = 0.
 * HLLC and LinearAdvection, which are not star solvers, sample the exact
 * solution.  These two kind-only forms reject AIRS and LinearAdvection, whose
 * settings they cannot carry. */
int mvmm_riemann_sample(int kind, int precision, double gamma, int64_t n, const double *left, const double *right,
                        const double *normal, double *out);
/* The same two calls configured like a context: riemann, precision, gamma,
 * airs_threshold and advection_velocity are read from params (ideal gas). */
int mvmm_riemann_flux_p(const mvmm_params *params, int64_t n, const double *left, const double *right,
                        const double *v_face, const double *normal, double *out);
int mvmm_riemann_sample_p(const mvmm_params *params, int64_t n, const double *left, const double *right,
                          const double *normal, double *out);

/* ---- allocation-free variant ------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a host that owns the device memory budget and hands out slices of it, code
 * running while its own CUDA graph is captured, or code that must avoid the
 * implicit device synchronisation of cudaMalloc/cudaFree.  Runs the flux
 * exchange and scatter of one step (mvmm_compute_fluxes, then
 * mvmm_apply_fluxes with kick2, then mvmm_convert_conserved_to_primitive for
 * the active cells) in the plain FP64 form on DEVICE arrays owned by the
 * caller: device_mesh and device_cells hold device pointers with the layouts
 * documented above, device_active is a device uint8[n] mask, device_err a
 * device uint32 the call ORs MVMM_ERR_* bits into (the caller clears it; may be
 * NULL).  The cell state is updated in place.  Asynchronous on cuda_stream.
 * Solvers: HLLC, exact and PVRS (AIRS, TSRS, TRRS and LinearAdvection return
 * MVMM_E_UNSUPPORTED, as does the FP32-face precision).  The mesh indices are
 * not validated on the host (the arrays are on the device): the kernels skip
 * a face or CSR entry whose index lies outside its array and OR
 * MVMM_ERR_BOUNDS into *device_err instead of reading out of bounds.
 *
 * The per-face intermediate results live in one static device array of
 * MVMM_NOALLOC_MAX_FACES faces (7 doubles each, 3.5 MiB) that every GPU which
 * loads this library keeps until the process exits.  Meshes with more faces
 * are rejected with MVMM_E_INVALID.  The array is shared by all calls and
 * keeps the last call's contents; each call overwrites every entry it reads,
 * so nothing needs clearing, but calls that overlap on the GPU (different
 * streams or threads) race on it and must be serialised by the caller.  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  No cudaMalloc, cudaFree or allocating library
 * routine is called. */
#define MVMM_NOALLOC_MAX_FACES 65536
int mvmm_flux_update_noalloc(const mvmm_params *params, const mvmm_mesh *device_mesh, mvmm_cells *device_cells,
                             const uint8_t *device_active, uint32_t *device_err, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
