/*
 * CPU oracle for the mvmm_hydro per-face finite-volume update.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it to produce the
 * reference answer.  The GPU product never links, loads or calls it.
 *
 * It restates, in plain C with FP contraction disabled, the reference's CPU
 * path (mvmm_hydro, Rust):  OptimalOrderRunner::step and everything it calls.
 * Every function cites the reference file:line it follows.  Data is kept as an
 * array of Particle structs exactly like the reference; the host API below
 * converts from / to the SoA layout shared with the GPU library.
 */
#ifndef MVMM_ORACLE_H
#define MVMM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Riemann solver kinds (riemann_solver.rs:28-44; LinearAdvection from
 * bin/main.rs:637-640). */
enum { ORC_HLLC = 0, ORC_EXACT = 1, ORC_PVRS = 2, ORC_AIRS = 3, ORC_TSRS = 4, ORC_TRRS = 5,
       ORC_LINEAR_ADVECTION = 6 };
/* Particle motion (engine.rs:7-13). */
enum { ORC_MOTION_FIXED = 0, ORC_MOTION_STEER = 1, ORC_MOTION_STEER_PAKMOR = 2, ORC_MOTION_FLUID = 3 };
/* Runner (bin/main.rs:667-673). */
enum { ORC_RUNNER_OPTIMAL_ORDER = 0, ORC_RUNNER_GODUNOV = 1 };
/* Boundary (space.rs:26-32). */
enum { ORC_PERIODIC = 0, ORC_REFLECTIVE = 1, ORC_OPEN = 2, ORC_VACUUM = 3 };
/* Equation of state (gas_law.rs:66-70). */
enum { ORC_EOS_IDEAL = 0, ORC_EOS_ISOTHERMAL = 1 };

/* Error bits, set where the reference panics / asserts. */
enum {
    ORC_ERR_NEWTON_CAP = 1u << 0,    /* exact.rs:272-274 */
    ORC_ERR_BRENT_BRACKET = 1u << 1, /* exact.rs:132-134 */
    ORC_ERR_NEG_MASS = 1u << 2,      /* part.rs:220 */
    ORC_ERR_NEG_ENERGY = 1u << 3,    /* part.rs:221-224 */
    ORC_ERR_NONFINITE = 1u << 4,     /* part.rs:180-182, 249-260 */
    ORC_ERR_NEG_PRIM = 1u << 5,      /* part.rs:246-247 */
    ORC_ERR_ZERO_DTI = 1u << 6,      /* timeline.rs:397 */
    ORC_ERR_MOTION = 1u << 7         /* unsupported particle motion */
};

typedef struct orc_params {
    double gamma;
    int eos;
    double isothermal_internal_energy;
    double cfl;
    int riemann;
    int boundary;
    int dimensionality;
    int sync_all;
    double t_end;
    int max_newton_iter; /* 1000 in the reference (exact.rs:272) */
    int n_threads;       /* OpenMP threads (0 = runtime default) */
    int runner;          /* ORC_RUNNER_* */
    double airs_threshold;        /* AIRiemannSolver::new(threshold) */
    double advection_velocity[3]; /* LinearAdvectionRiemannSover::new(velocity) */
    int particle_motion;          /* ORC_MOTION_* (engine.rs:7-13) */
    double box_size[3];           /* Space::box_size (periodic wrap after a drift) */
    /* gravity solver (bin/main.rs:643-662, gravity.rs) */
    int gravity;                     /* ORC_GRAVITY_* */
    double gravity_softening;        /* SelfGravity / KeplerianPotential softening_length */
    double gravity_acceleration[3];  /* Potential::Constant acceleration */
    double gravity_position[3];      /* KeplerianPotential position */
    int gravity_accelerations;       /* 1: compute_accelerations at the runner's "TODO: gravity"
                                        point (external potentials), 0: never (the reference) */
    int limiter_frame;               /* 0: the reference's cell-wise limiter offsets; 1: flux_exchange's frame */
} orc_params;

enum { ORC_GRAVITY_NONE = 0, ORC_GRAVITY_SELF = 1, ORC_GRAVITY_CONSTANT = 2, ORC_GRAVITY_KEPLERIAN = 3 };

/* SoA views; identical field meaning to the GPU library's mvmm_cells /
 * mvmm_mesh.  grad is [15][n] with row 3*q+k = d(quantity q)/d(axis k). */
typedef struct orc_cells {
    int64_t n;
    double *cons, *prim, *grad, *gc, *extrap, *facc;
    double *volume, *loc, *centroid, *v, *v_rel;
    double *max_a_over_r, *max_signal_velocity, *dt;
    int8_t *timebin;
} orc_cells;

typedef struct orc_mesh {
    int64_t n_cells, n_faces;
    const int32_t *left, *right; /* right < 0: boundary face */
    const double *area, *normal, *centroid, *shift; /* [F], [3][F] ... */
    const int32_t *csr_off, *csr_face;
} orc_mesh;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_params *p, const orc_mesh *m);
/* GravitySolver::compute_timesteps / compute_accelerations (gravity.rs):
 * dt_out [n]; a_out [3][n] (also stored as the cells' accelerations). */
void orc_gravity_timesteps(orc_ctx *c, double *dt_out);
void orc_gravity_accelerations(orc_ctx *c, double *a_out);
void orc_destroy(orc_ctx *c);
void orc_set_cells(orc_ctx *c, const orc_cells *in);
void orc_get_cells(const orc_ctx *c, orc_cells *out);
uint32_t orc_error(const orc_ctx *c);

/* One OptimalOrderRunner::step; returns ti_next. *n_active_faces gets the
 * number of faces that reached flux_exchange*. */
uint64_t orc_step(orc_ctx *c, uint64_t ti_current, uint64_t ti_old, int64_t *n_active_faces);
/* Engine::run with a Step sync point per step (engine.rs:152-199).  Runs at
 * most max_steps steps (<=0: unbounded); returns the number of steps run. */
int64_t orc_run(orc_ctx *c, int64_t max_steps, uint64_t *ti_current, uint64_t *ti_old,
                int64_t *n_active_faces);

/* Moving meshes.  Space::drift (space.rs:833-854) of every generator,
 * centroid and gradients centroid by v*dt with the periodic wrap; and
 * Space::volume_calculation's result (space.rs:236-263): the new faces and CSR
 * replace the mesh, volume and centroid [3][n] are applied to the active
 * cells of the next step after its predict (Particle::update_geometry). */
void orc_drift(orc_ctx *c, double dt);
void orc_set_mesh(orc_ctx *c, const orc_mesh *m, const double *volume, const double *centroid);

/* Per-stage entry points (FiniteVolumeSolver trait + runner free functions). */
void orc_predict(orc_ctx *c, double dt);
/* fluxes: [10][F] SoA (5 fluxes, 3 mflux, v_max, a_over_r) */
int64_t orc_compute_fluxes(orc_ctx *c, const uint8_t *active, double *fluxes);
void orc_apply_fluxes(orc_ctx *c, const double *fluxes, const uint8_t *active);
void orc_convert_conserved_to_primitive(orc_ctx *c, const uint8_t *active);
void orc_gradients(orc_ctx *c, const uint8_t *active);
void orc_compute_timesteps(orc_ctx *c, const uint8_t *active, double *dt_out);

/* Riemann solver over arrays; states are [5][n] SoA primitive vectors,
 * v_face and normal [3][n], output [5][n] conserved flux. */
void orc_riemann_flux(int kind, double gamma, int64_t n, const double *left, const double *right,
                      const double *v_face, const double *normal, double *out, uint32_t *err);
/* The same with the AIRS threshold and the LinearAdvection velocity (adv[3],
 * NULL = zero); the plain forms use threshold 2 and zero velocity. */
void orc_riemann_flux_ex(int kind, double gamma, double airs_threshold, const double *adv, int64_t n,
                         const double *left, const double *right, const double *v_face, const double *normal,
                         double *out, uint32_t *err);
void orc_riemann_sample_ex(int kind, double gamma, double airs_threshold, int64_t n, const double *left,
                           const double *right, const double *normal, double *out, uint32_t *err);
/* Half state sampled at x/t = 0 (RiemannStarSolver::sample, vacuum-aware as
 * in the blanket solve_for_flux); output [5][n] primitive. */
void orc_riemann_sample(int kind, double gamma, int64_t n, const double *left, const double *right,
                        const double *normal, double *out, uint32_t *err);
/* ExactRiemannSolver::solve_for_star_state with explicit inputs; out[4] =
 * (rho_l, rho_r, u, p) (exact.rs:241-291). */
void orc_exact_star(double gamma, double rho_l, double p_l, double a_l, double rho_r, double p_r, double a_r,
                    double v_l, double v_r, double *out, uint32_t *err);
/* State conversions (physical_quantities.rs:213-226, 294-304). */
void orc_cons_from_primitives(double gamma, const double *prim5, double volume, double *cons5);
void orc_prim_from_conserved(double gamma, const double *cons5, double volume, double *prim5);
/* Timeline helpers (timeline.rs). */
uint64_t orc_get_integer_timestep(int bin);
int orc_get_time_bin(uint64_t dti);
int orc_get_max_active_bin(uint64_t ti);
uint64_t orc_make_integer_timestep(double dt, int old_bin, int min_ngb_bin, uint64_t ti_current,
                                   double time_base_inv, uint32_t *err);

#ifdef __cplusplus
}
#endif
#endif
