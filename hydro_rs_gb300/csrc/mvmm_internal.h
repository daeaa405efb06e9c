// Internal declarations shared by the kernels and the host side of the library.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mvmm {

// Run-time solver settings: kind (SOLVER_*), AIRiemannSolver threshold
// (airs.rs:8-16) and LinearAdvectionRiemannSover velocity (linear_advection.rs:7-15).
struct RSx {
    int kind;
    double airs_threshold;
    double adv[3];
};

// Gas-law constants (AdiabaticIndex::from, gas_law.rs:9-18) evaluated once on
// the host, so that kernels do not repeat the divisions per thread.
struct GasK {
    double gamma, gamma_inv, odgm1, odgp1, iso_u, inv_m;
    int eos, rm;
};

// Cell state on the device: one float64 block of kCellFields * n doubles,
// field f of cell i at cd[f * n + i] (SoA; rows as in mvmm_cells).
enum CellField : int {
    F_CONS = 0,     // 5
    F_PRIM = 5,     // 5
    F_GRAD = 10,    // 15, row 3q+k
    F_GC = 25,      // 3
    F_EXTRAP = 28,  // 5
    F_FACC = 33,    // 5
    F_VOL = 38,
    F_LOC = 39,     // 3
    F_CEN = 42,     // 3
    F_V = 45,       // 3
    F_VREL = 48,    // 3
    F_MAOR = 51,
    F_MSV = 52,
    F_DT = 53,
    F_SRC = 54,     // 5: time-extrapolation source of the face stage (derived)
    F_CS = 59,      // sound speed of the face stage, 0 where rho <= 0 (derived)
    kCellFields = 60
};

// FP32 copies read by the FP32-face form (float block, field g of cell i at cf[g*n+i]).
enum CellField32 : int {
    G_PRIM = 0,    // 5
    G_GRAD = 5,    // 15
    G_EXTRAP = 20, // 5
    G_SRC = 25,    // 5
    G_CS = 30,
    G_DGC = 31,    // 3: gradients_centroid - loc
    G_DCEN = 34,   // 3: (unused)
    G_V = 37,      // 3: mesh velocity
    kCellFields32 = 40
};

// Static face geometry of the FP32-face form (float block, quantity g of face
// f at geo[g * nf + f]).  Formed in FP64 from the face data and the cells'
// positions and centroids whenever cells are uploaded (both are fixed on the
// device for a fixed mesh), then rounded once.  s is the face shift, n the
// normal; boundary faces (right < 0) use the reflected position / centroid.
enum FaceGeom32 : int {
    GE_RL = 0,    // 3: fc - loc_l
    GE_RR = 3,    // 3: (fc - loc_r) - s                       (interior)
    GE_DX = 6,    // 3: (loc_r + s) - loc_l; boundary: reflect(loc_l) - loc_l
    GE_FCM = 9,   // 3: fc - 0.5 ((loc_l + loc_r) + s)         (interior)
    GE_N = 12,    // 3: n
    GE_DS = 15,   // 3: (cen_r + s) - cen_l; boundary: reflect(cen_l) - cen_l
    GE_DL = 18,   // 3: (fc - cen_l) - s   (limiter extrapolation, left cell; fc - cen_l with limiter_frame)
    GE_DR = 21,   // 3: (fc - cen_r) + s   (limiter extrapolation, right cell; (fc - cen_r) - s with limiter_frame)
    GE_W = 24,    // area / |ds|^2         (WLS weight)
    GE_A = 25,    // area
    kFaceGeom32 = 26
};

// Device timeline + counters of one simulation (TimestepInfo, engine.rs:33-41).
struct DevTimeline {
    unsigned long long ti_current;
    unsigned long long ti_old;
    unsigned long long min_dti;       // reduction target of timesteps_apply
    int min_timebin;                  // reduction target of timestep_sync
    int done;                         // 1 once the step at t_end has run
    unsigned int err;                 // MVMM_ERR_* bits
    unsigned int n_alist;             // hierarchical steps: the first n_alist cells of the list are active
    unsigned long long steps;
    unsigned long long active_faces;  // cumulative faces that reached flux_exchange*
    unsigned long long active_cells;
    unsigned long long fallback_faces;  // FP32-face form: faces solved by the full FP64 iteration
    unsigned int n_list;                // length of this step's active-face list (hierarchical steps)
    unsigned int n_clist;               // length of this step's cell list (hierarchical steps)
    unsigned long long faces_mark;      // active_faces when the time was last set on the device
    unsigned long long host_stored;     // bytes the current mvmm_step_cells_changed call stored into host arrays
};

// Steps of dt kept for the deferred extrapolations of hierarchical steps; every
// kDtLog / 2 steps all cells are brought up to date, so none lags further.
constexpr int kDtLog = 4096;

// Job queues of the plain form's exact solver (KP::brent_jobs): Brent
// searches, Newton searches, and faces whose star pressure is the guess; each
// holds brent_cap jobs.
constexpr int kExactQueues = 3;

// KP::dirty marks: the cell's extrapolation rows changed, or any of its rows.
constexpr uint8_t kDirtyExtrap = 1, kDirtyAll = 2;

// Internal (not exported) flag a face's Riemann solve sets when the FP32-face
// form's split exact solver fell back to the full FP64 iteration.
constexpr unsigned int kInfoFallback = 1u << 16;

// Kernel parameters (passed by value).
struct KP {
    int n, nf;
    const int* left;
    const int* right;
    const double* area;
    const double* normal;    // [3][nf]
    const double* fcen;      // [3][nf]
    const double* shift;     // [3][nf]
    const int* csr_off;
    const int* csr_face;
    double* cd;              // cell fields
    float* cf;               // FP32 copies (FP32 form)
    int8_t* timebin;
    int8_t* tb_tmp;
    uint8_t* active;
    double* flux;            // face results, rows of nf
    float* flux32;           // FP32 form face results of a step, rows of nf: 5 fluxes, v_max, a_over_r
    float* geo;              // FP32 form static face geometry (FaceGeom32)
    unsigned long long* geo_pos;  // FP32 form: bits of loc and centroid [6][n] the geometry was built from
    uint8_t* geo_changed;    // FP32 form: 1 for cells whose loc or centroid bits changed since
    int geo_check;           // 1: k_geom32 rebuilds only the faces of changed cells
    int fp32;                // 1: FP32-face form
    int flux_rows;           // 7 (step) or 10 (stage, with mflux)
    DevTimeline* tl;
    double gamma, iso_u;
    int eos;
    double cfl;
    int boundary;
    int dim;
    int sync_all;
    int max_iter;
    double time_base, time_base_inv;
    int stage;               // 1: per-stage call (explicit dt / mask from the host)
    int stale_all;           // 1: every cell's state came from the host this step (fresh flags void)
    double* snap_late;       // or null: the update keeps the rows it reads first (cons, facc, max_signal_velocity,
                             //   max_a_over_r) as uploaded, at their field offsets (steps over all cells)
    double stage_dt;
    // batches: many independent simulations packed into one mesh; each has its
    // own device timeline tl[k] (k = inst[cell]) and time base
    const int* inst;         // per-cell instance index, nullptr for a single simulation
    int n_inst;
    const double* inst_tb;   // per-instance time_base (nullptr: time_base)
    const double* inst_tbi;  // per-instance 1 / time_base (nullptr: time_base_inv)
    int blk_face, blk_cell;  // thread-block sizes (chosen by mvmm_autotune)
    int n_sms;               // streaming multiprocessors of the context's device (grid sizing)
    // gravity solver (gravity.rs): MVMM_GRAVITY_* kind, whether the external
    // potential's accelerations kick (grav_acc), softening, Constant
    // acceleration, Keplerian position
    int grav, grav_acc;
    double grav_soft, grav_avec[3], grav_pos[3];
    double* agrav;           // self-gravity: a_grav [3][n] (SelfGravity::compute_accelerations), or null
    const int* inst_end;     // batches with self-gravity: each instance's cell end, or null
    int limiter_frame;       // 1: the cell-wise limiter's face offsets in flux_exchange's frame
    uint8_t* dirty;          // or null: 1 for cells whose host rows a kernel rewrote since the
                             //   last mvmm_step_cells_changed stored them (that call's copies back)
    GasK gk;                 // gas-law constants
    RSx rsx;                 // Riemann solver kind and its settings
    int godunov;             // 1: GodunovHydroRunner (no gradients), 0: OptimalOrderRunner
    int motion;              // MVMM_MOTION_*
    double box[3];           // periodic box (moving meshes)
    const double* new_vol;   // moving meshes: volume [n] and centroid [3][n] of the
    const double* new_cen;   //   rebuilt cells, applied to active cells after predict
    int use_list;            // 1: face kernel walks the compacted active-face list
    unsigned int* face_stamp;  // hierarchical steps: steps + 1 for faces active in this step
    unsigned int* extrap_step;  // hierarchical steps: the steps whose predict contribution a cell's
                                //   extrapolation includes (deferred for inactive cells, see k_predict)
    double* dt_log;             //   the dt of step s at [s % kDtLog]
    void* brent_jobs;          // plain form, exact solver: the face kernel's queued jobs (kExactQueues
    unsigned int* brent_count;  //   queues of brent_cap) and their counts this launch
    int brent_cap;
    unsigned int* blocks_done;  // k_limit blocks finished this step (the last one ends the step)
    unsigned int* touch;     // hierarchical steps: 1 for cells on this step's cell list
    uint8_t* fresh;          // 1: the cell's derived face-stage rows match its prim, grad and v_rel
    uint8_t* cf_fresh;       // FP32-face form: 1 where the FP32 copies of the gradients and of
                             //   gradients_centroid - loc were written with the FP64 rows (or null)
    int* cell_list;          // hierarchical steps: active cells and the cells next to an active face
    int* face_list;          // compacted active faces
};

// Sets the text mvmm_last_error() returns on this host thread and returns code
// (implemented in mvmm_api.cu).
int report_error(int code, const char* msg);

// launchers (implemented in step_fp64.cu / step_fp32.cu)
void launch_predict(const KP& p, cudaStream_t s);
void launch_derive(const KP& p, cudaStream_t s);
void launch_face_flux(const KP& p, int solver, int precision, cudaStream_t s);
void launch_update(const KP& p, int do_c2p, cudaStream_t s);
void launch_c2p(const KP& p, cudaStream_t s);
void launch_gradients(const KP& p, int do_timestep, cudaStream_t s);
void launch_timesteps(const KP& p, double* dt_out, cudaStream_t s);
void launch_gravity(const KP& p, int what, double* out, cudaStream_t s);
// k_self_gravity's shared memory (over the default 48 KB); once per process, before a launch
cudaError_t setup_self_gravity();
void launch_self_gravity(const KP& p, int kick, int do_c2p, cudaStream_t s);
void launch_limit(const KP& p, cudaStream_t s);
void launch_compact(const KP& p, cudaStream_t s);
void launch_end(const KP& p, cudaStream_t s);
int cell_grid(const KP& p);
void launch_set_time(const KP& p, unsigned long long ti_current, unsigned long long ti_old, cudaStream_t s);
void launch_drift(const KP& p, double dt, cudaStream_t s);
void launch_geometry(const KP& p, cudaStream_t s);
// FP32 form helpers
void launch_prep32(const KP& p, cudaStream_t s);

}  // namespace mvmm
