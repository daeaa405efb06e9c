// Host side of mvmm_gpu: context, device buffers, CUDA-graph step, C ABI.
//
// The engine loop (Engine::run, engine.rs:152-199) runs on the device: every
// step is one CUDA graph of six kernels that reads and advances a device
// timeline, so a run of many steps needs no host round trip per step.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mvmm_gpu.h"
#include "mvmm_internal.h"
#include "mvmm_device.cuh"

namespace mvmm {
void launch_face_flux_fp64(const KP& p, int solver, cudaStream_t s);
size_t brent_job_bytes();
void launch_extrap_flush(const KP& p, bool reset, cudaStream_t s);
void launch_riemann_fp64(int kind, int sample, double gamma, int64_t n, const double* l, const double* r,
                         const double* vf, const double* nrm, double* out, unsigned int* err, const RSx& x,
                         cudaStream_t s);
void launch_face_flux_fp32(const KP& p, int solver, cudaStream_t s);
void launch_gradients32(const KP& p, cudaStream_t s);
void launch_geom32(const KP& p, bool check, cudaStream_t s);
void launch_predict32(const KP& p, cudaStream_t s);
void launch_riemann_fp32(int kind, int sample, double gamma, int64_t n, const double* l, const double* r,
                         const double* vf, const double* nrm, double* out, unsigned int* err, const RSx& x,
                         cudaStream_t s);
}  // namespace mvmm

using namespace mvmm;

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
#define CUDA_TRY(expr)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(MVMM_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));               \
    } while (0)

constexpr unsigned long long kMax = 1ull << 57;
}  // namespace

namespace mvmm {
int report_error(int code, const char* msg) { return fail(code, msg ? msg : ""); }
}  // namespace mvmm

struct mvmm_ctx {
    mvmm_params prm{};
    int n = 0, nf = 0;
    int64_t ncsr = 0;
    int *left = nullptr, *right = nullptr, *csr_off = nullptr, *csr_face = nullptr;
    double *area = nullptr, *normal = nullptr, *fcen = nullptr, *shift = nullptr;
    double* cd = nullptr;
    float* cf = nullptr;
    int8_t *timebin = nullptr, *tb_tmp = nullptr;
    uint8_t* active = nullptr;
    double* flux = nullptr;
    float* flux32 = nullptr;
    float* geo = nullptr;
    unsigned long long* geo_pos = nullptr;  // FP32 form: loc and centroid bits of the last geometry build
    uint8_t* geo_changed = nullptr;
    bool geo_built = false;  // the FP32 geometry matches the current face arrays
    double* dtmp = nullptr;
    int n_inst = 1;
    int* inst = nullptr;       // per-cell instance (batches only)
    double* inst_tb = nullptr;  // per-instance time_base, 1/time_base (batches only)
    double* inst_tbi = nullptr;
    int* inst_end = nullptr;    // per-instance cell end (batches with self-gravity accelerations)
    double* agrav = nullptr;    // self-gravity: a_grav [3][n]
    unsigned int* face_stamp = nullptr;
    // moving meshes: face capacity, pending geometry of the rebuilt cells
    int nf_cap = 0;
    unsigned int* extrap_step = nullptr;  // hierarchical steps: deferred extrapolations (KP::extrap_step)
    double* dt_log = nullptr;
    void* brent_jobs = nullptr;  // plain form, exact solver: the queued jobs of a face launch
    unsigned int* brent_count = nullptr;
    int brent_cap = 0;
    int64_t ncsr_cap = 0;
    double *pend_vol = nullptr, *pend_cen = nullptr;
    bool pending_geometry = false;
    unsigned int* touch = nullptr;
    unsigned int* blocks_done = nullptr;
    uint8_t* fresh = nullptr;
    uint8_t* cf_fresh = nullptr;
    int* cell_list = nullptr;
    int* face_list = nullptr;
    int blk_face = 128, blk_cell = 128;
    DevTimeline* tl = nullptr;       // [n_inst]
    DevTimeline* tl_host = nullptr;  // pinned [n_inst]
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraphExec_t step_exec = nullptr;
    cudaGraphExec_t prof_exec = nullptr;  // the step graph with the per-kernel timing events
    bool prof = false;
    cudaEvent_t ev[MVMM_NUM_KERNELS + 1] = {};
    cudaStream_t side = nullptr;              // copies of mvmm_step_cells that overlap the step
    cudaStream_t geo_side = nullptr;          // its FP32 face-geometry refresh, beside predict
    cudaEvent_t ev_pred = nullptr, ev_in = nullptr, ev_upd = nullptr, ev_grad = nullptr, ev_out = nullptr,
                ev_geo = nullptr;
    double prof_ms[MVMM_NUM_KERNELS] = {};
    int64_t prof_n[MVMM_NUM_KERNELS] = {};
    double time_base = 0, time_base_inv = 0;
    uint32_t err_bits = 0;
    int device = 0, n_sms = 1;
    bool pageable_access = false;  // the device reads and writes pageable host memory
    // mvmm_step_cells: the uploaded rows as they arrived ([54][n] in the block's
    // field order, and the time bins), and bytes moved between host and device
    double* snap = nullptr;
    int8_t* snap_tb = nullptr;
    unsigned long long* xfer_stored = nullptr;  // device: bytes stored by copies that skip unchanged chunks
    int64_t host_bytes_in = 0, host_bytes_out = 0;
    // mvmm_step_cells_changed: 1 for cells a kernel rewrote since their rows
    // were last stored (KP::dirty), and the listed cells' indices
    uint8_t* dirty = nullptr;
    int* chg_list = nullptr;
};

namespace {

RSx solver_settings(const mvmm_params& prm) {
    RSx x;
    x.kind = prm.riemann;
    x.airs_threshold = prm.airs_threshold;
    for (int k = 0; k < 3; k++) x.adv[k] = prm.advection_velocity[k];
    return x;
}

// Settings each solver kind needs (MissingAIRSThreshold, errors.rs; the
// velocity check of bin/main.rs:637-640).
int check_solver(int kind, double airs_threshold, const double* adv) {
    if (kind < MVMM_RIEMANN_HLLC || kind > MVMM_RIEMANN_LINEAR_ADVECTION)
        return fail(MVMM_E_INVALID, "unknown Riemann solver");
    if (kind == MVMM_RIEMANN_AIRS && std::isnan(airs_threshold))
        return fail(MVMM_E_INVALID, "AIRS needs a threshold (airs_threshold is NaN)");
    if (kind == MVMM_RIEMANN_LINEAR_ADVECTION &&
        (!adv || !std::isfinite(adv[0]) || !std::isfinite(adv[1]) || !std::isfinite(adv[2])))
        return fail(MVMM_E_INVALID, "LinearAdvection needs a finite advection_velocity");
    return MVMM_OK;
}

KP make_kp(mvmm_ctx* c, int stage, int flux_rows) {
    KP p{};
    p.n = c->n;
    p.nf = c->nf;
    p.left = c->left;
    p.right = c->right;
    p.area = c->area;
    p.normal = c->normal;
    p.fcen = c->fcen;
    p.shift = c->shift;
    p.csr_off = c->csr_off;
    p.csr_face = c->csr_face;
    p.cd = c->cd;
    p.cf = c->cf;
    p.timebin = c->timebin;
    p.tb_tmp = c->tb_tmp;
    p.active = c->active;
    p.flux = c->flux;
    p.flux32 = c->flux32;
    p.geo = c->geo;
    p.geo_pos = c->geo_pos;
    p.geo_changed = c->geo_changed;
    p.fp32 = c->prm.precision == MVMM_PRECISION_FP32FACE ? 1 : 0;
    p.flux_rows = flux_rows;
    p.tl = c->tl;
    p.gamma = c->prm.gamma;
    p.iso_u = c->prm.isothermal_internal_energy;
    p.eos = c->prm.eos;
    p.cfl = c->prm.cfl;
    p.boundary = c->prm.boundary;
    p.dim = c->prm.dimensionality;
    p.sync_all = c->prm.sync_all;
    p.max_iter = c->prm.max_newton_iter > 0 ? c->prm.max_newton_iter : 1000;
    p.time_base = c->time_base;
    p.time_base_inv = c->time_base_inv;
    p.stage = stage;
    p.inst = c->inst;
    p.n_inst = c->n_inst;
    p.inst_tb = c->inst_tb;
    p.inst_tbi = c->inst_tbi;
    p.inst_end = c->inst_end;
    p.agrav = c->agrav;
    // hierarchical steps of a single simulation walk a compacted active-face
    // list; synchronised steps, batches and per-stage calls sweep all faces
    p.use_list = (!stage && !c->prm.sync_all && c->n_inst == 1) ? 1 : 0;
    p.face_stamp = c->face_stamp;
    p.extrap_step = c->extrap_step;
    p.dt_log = c->dt_log;
    p.brent_jobs = c->brent_jobs;
    p.brent_count = c->brent_count;
    p.brent_cap = c->brent_cap;
    p.touch = c->touch;
    p.blocks_done = c->blocks_done;
    p.fresh = c->fresh;
    p.cf_fresh = c->cf_fresh;
    p.cell_list = c->cell_list;
    p.face_list = c->face_list;
    p.blk_face = c->blk_face;
    p.n_sms = c->n_sms > 0 ? c->n_sms : 1;
    p.grav = c->prm.gravity;
    p.grav_acc = c->prm.gravity_accelerations ? 1 : 0;
    p.limiter_frame = c->prm.limiter_frame ? 1 : 0;
    p.dirty = c->dirty;
    p.grav_soft = c->prm.gravity_softening;
    for (int a = 0; a < 3; a++) {
        p.grav_avec[a] = c->prm.gravity_acceleration[a];
        p.grav_pos[a] = c->prm.gravity_position[a];
    }
    p.blk_cell = c->blk_cell;
    p.rsx = solver_settings(c->prm);
    const Gas<double> g = make_gas<double>(c->prm.gamma, c->prm.eos, c->prm.isothermal_internal_energy);
    p.gk.gamma = g.gamma;
    p.gk.gamma_inv = g.gamma_inv;
    p.gk.odgm1 = g.odgm1_;
    p.gk.odgp1 = g.odgp1_;
    p.gk.iso_u = g.iso_u;
    p.gk.inv_m = g.inv_m;
    p.gk.eos = g.eos;
    p.gk.rm = g.rm;
    // a stage call to mvmm_gradients always estimates gradients
    p.godunov = (!stage && c->prm.runner == MVMM_RUNNER_GODUNOV) ? 1 : 0;
    p.motion = c->prm.particle_motion;
    for (int a = 0; a < 3; a++) p.box[a] = c->prm.box_size[a];
    p.new_vol = c->pend_vol;
    p.new_cen = c->pend_cen;
    return p;
}

// Brings the FP32 face geometry up to date with the cells' positions and
// centroids.  A fixed mesh whose geometry was built before rebuilds only the
// faces of cells whose loc or centroid bits changed; a moving mesh (whose
// face arrays change) and the first build rebuild every face.
void update_geom32(mvmm_ctx* c, const KP& p, cudaStream_t s) {
    if (c->prm.precision != MVMM_PRECISION_FP32FACE) return;
    launch_geom32(p, c->geo_built && c->prm.particle_motion == MVMM_MOTION_FIXED, s);
    c->geo_built = true;
}

// prepped: the FP32 copies of the cells were written by k_predict32
void launch_face(mvmm_ctx* c, const KP& p, bool prepped = false) {
    if (c->prm.precision == MVMM_PRECISION_FP32FACE) {
        if (!prepped) launch_prep32(p, c->stream);
        launch_face_flux_fp32(p, c->prm.riemann, c->stream);
    } else {
        launch_face_flux_fp64(p, c->prm.riemann, c->stream);
    }
}

// The six kernels of one OptimalOrderRunner step, optionally bracketed by events.
// A step on cells uploaded with it (mvmm_step_cells): predict recomputes every
// derived row, the face stage waits for an event (the FP32 geometry refreshed
// on a side stream), the update for another (the rows only it reads), and
// events are recorded after
// the update and after the gradient stage for the copies back.
struct StepHooks {
    bool stale_all = false;
    double* snap_late = nullptr;
    cudaEvent_t wait_before_face = nullptr;
    cudaEvent_t wait_before_update = nullptr;
    cudaEvent_t after_update = nullptr;
    cudaEvent_t after_gradients = nullptr;
};

// The per-kernel timing events; recorded as event nodes when the step is
// captured into the profiling graph.
void record_ev(mvmm_ctx* c, int j, cudaStream_t s) { cudaEventRecordWithFlags(c->ev[j], s, cudaEventRecordExternal); }

// Self-gravity accelerations kick: kick2 and cons->prim follow k_self_gravity.
bool self_gravity_kicks(const mvmm_ctx* c) {
    return c->prm.gravity == MVMM_GRAVITY_SELF && c->prm.gravity_accelerations;
}

void enqueue_step_kernels(mvmm_ctx* c, bool with_events, const StepHooks& h = StepHooks()) {
    KP p = make_kp(c, 0, 7);
    p.stale_all = h.stale_all ? 1 : 0;
    p.snap_late = h.snap_late;
    cudaStream_t s = c->stream;
    if (with_events) record_ev(c, 0, s);
    // steps over all cells of the FP32-face form: predict and the FP32 copies in one kernel
    const bool fused = c->prm.precision == MVMM_PRECISION_FP32FACE && !p.use_list;
    if (fused) launch_predict32(p, s);
    else launch_predict(p, s);
    if (c->pending_geometry) launch_geometry(p, s);  // after predict, as volume_calculation
    if (c->prm.particle_motion != MVMM_MOTION_FIXED) update_geom32(c, p, s);  // generators drifted, centroids updated
    if (h.wait_before_face) cudaStreamWaitEvent(s, h.wait_before_face, 0);
    if (p.use_list) launch_compact(p, s);
    if (with_events) record_ev(c, 1, s);
    launch_face(c, p, fused);
    if (with_events) record_ev(c, 2, s);
    if (h.wait_before_update) cudaStreamWaitEvent(s, h.wait_before_update, 0);
    launch_update(p, 1, s);
    if (self_gravity_kicks(c)) launch_self_gravity(p, 1, 1, s);  // kick2 and cons->prim after the accelerations
    if (h.after_update) cudaEventRecord(h.after_update, s);
    if (with_events) record_ev(c, 3, s);
    if (c->prm.precision == MVMM_PRECISION_FP32FACE) launch_gradients32(p, s);
    else launch_gradients(p, 1, s);
    if (h.after_gradients) cudaEventRecord(h.after_gradients, s);
    if (with_events) record_ev(c, 4, s);
    launch_limit(p, s);
    if (with_events) record_ev(c, 5, s);
    launch_end(p, s);
    if (with_events) record_ev(c, 6, s);
}

// The step as a CUDA graph; with_events: the profiling variant, with the
// per-kernel timing events as event-record nodes.
int build_graph(mvmm_ctx* c, bool with_events = false) {
    cudaGraphExec_t* exec = with_events ? &c->prof_exec : &c->step_exec;
    if (*exec) return MVMM_OK;
    cudaGraph_t g;
    CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step_kernels(c, with_events);
    CUDA_TRY(cudaStreamEndCapture(c->stream, &g));
    cudaError_t e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(MVMM_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return MVMM_OK;
}

// Kernel parameters hold the face count, the buffers and the block sizes:
// whatever changes them drops the captured step graphs.
void drop_graphs(mvmm_ctx* c) {
    for (cudaGraphExec_t* e : {&c->step_exec, &c->prof_exec})
        if (*e) {
            cudaGraphExecDestroy(*e);
            *e = nullptr;
        }
}

int enqueue_steps_impl(mvmm_ctx* c, int64_t n) {
    if (c->prof) {
        // per-kernel timing: a fixed mesh runs the step as the profiling graph,
        // so that the events time the kernels, not the host's launches
        const bool fixed = c->prm.particle_motion == MVMM_MOTION_FIXED;
        if (fixed) {
            int rc = build_graph(c, true);
            if (rc) return rc;
        }
        for (int64_t k = 0; k < n; k++) {
            if (fixed) {
                CUDA_TRY(cudaGraphLaunch(c->prof_exec, c->stream));
            } else {
                enqueue_step_kernels(c, true);
                c->pending_geometry = false;
            }
            CUDA_TRY(cudaEventSynchronize(c->ev[MVMM_NUM_KERNELS]));
            for (int j = 0; j < MVMM_NUM_KERNELS; j++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, c->ev[j], c->ev[j + 1]);
                c->prof_ms[j] += ms;
                c->prof_n[j] += 1;
            }
        }
        CUDA_TRY(cudaGetLastError());
        return MVMM_OK;
    }
    if (c->prm.particle_motion != MVMM_MOTION_FIXED) {
        // the mesh changes between steps: direct launches, the pending geometry once
        for (int64_t k = 0; k < n; k++) {
            enqueue_step_kernels(c, false);
            c->pending_geometry = false;
        }
        CUDA_TRY(cudaGetLastError());
        return MVMM_OK;
    }
    int rc = build_graph(c);
    if (rc) return rc;
    for (int64_t k = 0; k < n; k++) CUDA_TRY(cudaGraphLaunch(c->step_exec, c->stream));
    return MVMM_OK;
}

int read_tl(mvmm_ctx* c) {
    CUDA_TRY(cudaMemcpyAsync(c->tl_host, c->tl, sizeof(DevTimeline) * c->n_inst, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MVMM_OK;
}

int write_tl(mvmm_ctx* c) {
    CUDA_TRY(cudaMemcpyAsync(c->tl, c->tl_host, sizeof(DevTimeline) * c->n_inst, cudaMemcpyHostToDevice, c->stream));
    return MVMM_OK;
}

bool all_done(const mvmm_ctx* c) {
    for (int k = 0; k < c->n_inst; k++)
        if (!c->tl_host[k].done) return false;
    return true;
}
unsigned long long sum_field(const mvmm_ctx* c, unsigned long long DevTimeline::*f) {
    unsigned long long s = 0;
    for (int k = 0; k < c->n_inst; k++) s += c->tl_host[k].*f;
    return s;
}

// Host-side checks standing in for device bounds checks: every index the
// kernels dereference is validated once here.
int check_mesh(const mvmm_mesh* m, int boundary) {
    if (!m || m->n_cells <= 0 || m->n_faces < 0) return fail(MVMM_E_INVALID, "mesh: empty or negative sizes");
    if (m->n_cells > (1ll << 30) || m->n_faces > (1ll << 30)) return fail(MVMM_E_INVALID, "mesh: too large");
    if (!m->left || !m->right || !m->area || !m->normal || !m->centroid || !m->shift || !m->csr_off || !m->csr_face)
        return fail(MVMM_E_INVALID, "mesh: null pointer");
    int64_t n = m->n_cells, nf = m->n_faces;
    if (m->csr_off[0] != 0) return fail(MVMM_E_INVALID, "mesh: csr_off[0] != 0");
    // every index is checked before anything reads through it; the checks run
    // over the host's cores (a moving mesh passes every step)
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t f = 0; f < nf; f++) {
        const int32_t l = m->left[f], r = m->right[f];
        if (l < 0 || l >= n) bad |= 1;
        if (r >= n || r < -1) bad |= 2;
        if (r < 0 && boundary == MVMM_BOUNDARY_PERIODIC) bad |= 4;
    }
    if (bad & 1) return fail(MVMM_E_INVALID, "mesh: face left index out of range");
    if (bad & 2) return fail(MVMM_E_INVALID, "mesh: face right index out of range");
    if (bad & 4) return fail(MVMM_E_INVALID, "mesh: boundary face with periodic boundary conditions");
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t i = 0; i < n; i++)
        if (m->csr_off[i + 1] < m->csr_off[i]) bad |= 8;
    if (bad & 8) return fail(MVMM_E_INVALID, "mesh: csr_off not monotone");
    const int64_t ncsr = m->csr_off[n];
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t k = 0; k < ncsr; k++) {
        const int32_t f = m->csr_face[k];
        if (f < 0 || f >= nf) bad |= 16;
    }
    if (bad & 16) return fail(MVMM_E_INVALID, "mesh: csr face index out of range");
    // each cell lists exactly the faces that touch it: every listed face
    // touches the cell, and the list lengths add up to the faces' ends
    std::vector<int32_t> deg(n, 0);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < nf; f++) {
#pragma omp atomic
        deg[m->left[f]]++;
        if (m->right[f] >= 0) {
#pragma omp atomic
            deg[m->right[f]]++;
        }
    }
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t i = 0; i < n; i++) {
        if (m->csr_off[i + 1] - m->csr_off[i] != deg[i]) bad |= 32;
        for (int32_t k = m->csr_off[i]; k < m->csr_off[i + 1]; k++) {
            const int32_t f = m->csr_face[k];
            if (m->left[f] != i && m->right[f] != i) bad |= 64;
        }
    }
    if (bad & 32) return fail(MVMM_E_INVALID, "mesh: csr does not match faces");
    if (bad & 64) return fail(MVMM_E_INVALID, "mesh: csr lists a face not touching the cell");
    return MVMM_OK;
}

int finish(mvmm_ctx* c) {
    int rc = read_tl(c);
    if (rc) return rc;
    uint32_t bits = 0;
    for (int k = 0; k < c->n_inst; k++) bits |= c->tl_host[k].err;
    if (bits & ~c->err_bits) {
        c->err_bits |= bits;
        char buf[96];
        snprintf(buf, sizeof(buf), "numerical failure, error bits 0x%x", bits);
        return fail(MVMM_E_NUMERIC, buf);
    }
    c->err_bits |= bits;
    return MVMM_OK;
}

}  // namespace

extern "C" {

const char* mvmm_last_error(void) { return g_last_error.c_str(); }

static int create_impl(const mvmm_params* prm, const mvmm_mesh* m, int64_t n_inst, const int64_t* cell_off,
                       const double* t_end, mvmm_ctx** out) {
    if (!prm || !out) return fail(MVMM_E_INVALID, "null argument");
    *out = nullptr;
    if (!(prm->gamma > 1.0)) return fail(MVMM_E_INVALID, "gamma must be > 1");
    if (prm->dimensionality < 1 || prm->dimensionality > 3) return fail(MVMM_E_INVALID, "dimensionality must be 1..3");
    int rs = check_solver(prm->riemann, prm->airs_threshold, prm->advection_velocity);
    if (rs) return rs;
    if (prm->runner != MVMM_RUNNER_OPTIMAL_ORDER && prm->runner != MVMM_RUNNER_GODUNOV)
        return fail(MVMM_E_INVALID, "unknown runner");
    if (prm->boundary < 0 || prm->boundary > 3) return fail(MVMM_E_INVALID, "unknown boundary");
    if (prm->precision < 0 || prm->precision > 1) return fail(MVMM_E_INVALID, "unknown precision");
    if (prm->eos < 0 || prm->eos > 1) return fail(MVMM_E_INVALID, "unknown equation of state");
    if (prm->particle_motion < MVMM_MOTION_FIXED || prm->particle_motion > MVMM_MOTION_FLUID)
        return fail(MVMM_E_INVALID, "unknown particle motion");
    if (prm->particle_motion != MVMM_MOTION_FIXED) {
        if (n_inst > 1) return fail(MVMM_E_UNSUPPORTED, "moving meshes are stepped one simulation at a time");
        for (int a = 0; a < prm->dimensionality; a++)
            if (!(prm->box_size[a] > 0.)) return fail(MVMM_E_INVALID, "moving meshes need box_size > 0");
    }
    if (prm->gravity < MVMM_GRAVITY_NONE || prm->gravity > MVMM_GRAVITY_KEPLERIAN)
        return fail(MVMM_E_INVALID, "unknown gravity solver");
    if ((prm->gravity == MVMM_GRAVITY_SELF || prm->gravity == MVMM_GRAVITY_KEPLERIAN) &&
        !(prm->gravity_softening >= 0.))
        return fail(MVMM_E_INVALID, "gravity needs a softening_length >= 0");
    if (!(prm->t_end > 0.0)) return fail(MVMM_E_INVALID, "t_end must be > 0");
    int rc = check_mesh(m, prm->boundary);
    if (rc) return rc;
    std::vector<int32_t> inst_h;
    if (n_inst > 1) {
        if (!cell_off || !t_end) return fail(MVMM_E_INVALID, "batch: null offsets or t_end");
        if (n_inst > (1 << 24)) return fail(MVMM_E_INVALID, "batch: too many instances");
        if (cell_off[0] != 0 || cell_off[n_inst] != m->n_cells) return fail(MVMM_E_INVALID, "batch: offsets must span the cells");
        inst_h.resize(m->n_cells);
        for (int64_t k = 0; k < n_inst; k++) {
            if (cell_off[k + 1] < cell_off[k]) return fail(MVMM_E_INVALID, "batch: offsets not monotone");
            if (!(t_end[k] > 0.0)) return fail(MVMM_E_INVALID, "batch: t_end must be > 0");
            for (int64_t i = cell_off[k]; i < cell_off[k + 1]; i++) inst_h[i] = (int32_t)k;
        }
        for (int64_t f = 0; f < m->n_faces; f++)
            if (m->right[f] >= 0 && inst_h[m->left[f]] != inst_h[m->right[f]])
                return fail(MVMM_E_INVALID, "batch: a face joins two instances");
    } else {
        n_inst = 1;
    }
    mvmm_ctx* c = new mvmm_ctx();
    c->prm = *prm;
    c->n_inst = (int)n_inst;
    c->n = (int)m->n_cells;
    c->nf = (int)m->n_faces;
    c->ncsr = m->csr_off[m->n_cells];
    c->time_base = prm->t_end / (double)kMax;  // Engine::new (engine.rs:118-119)
    c->time_base_inv = 1. / c->time_base;
    size_t n = c->n, nf = c->nf > 0 ? c->nf : 1;
    auto cleanup = [&](int code, const std::string& msg) {
        mvmm_ctx_destroy(c);
        return fail(code, msg);
    };
#define ALLOC(ptr, bytes)                                                                  \
    do {                                                                                   \
        cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));                              \
        if (e_ != cudaSuccess) return cleanup(MVMM_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e_)); \
    } while (0)
    ALLOC(c->left, nf * 4);
    ALLOC(c->right, nf * 4);
    ALLOC(c->area, nf * 8);
    ALLOC(c->normal, 3 * nf * 8);
    ALLOC(c->fcen, 3 * nf * 8);
    ALLOC(c->shift, 3 * nf * 8);
    ALLOC(c->csr_off, (n + 1) * 4);
    ALLOC(c->csr_face, (c->ncsr > 0 ? c->ncsr : 1) * 4);
    ALLOC(c->cd, (size_t)kCellFields * n * 8);
    c->nf_cap = (int)nf;
    c->ncsr_cap = c->ncsr > 0 ? c->ncsr : 1;
    if (prm->particle_motion != MVMM_MOTION_FIXED) {
        ALLOC(c->pend_vol, n * 8);
        ALLOC(c->pend_cen, 3 * n * 8);
    }
    if (prm->precision == MVMM_PRECISION_FP32FACE) {
        ALLOC(c->cf, (size_t)kCellFields32 * n * 4);
        ALLOC(c->flux32, 7 * nf * 4);
        ALLOC(c->geo, (size_t)kFaceGeom32 * nf * 4);
        ALLOC(c->geo_pos, 6 * n * 8);
        ALLOC(c->geo_changed, n);
    }
    ALLOC(c->timebin, n);
    ALLOC(c->tb_tmp, n);
    ALLOC(c->active, n);
    ALLOC(c->flux, 10 * nf * 8);
    if (prm->precision == MVMM_PRECISION_FP64 && prm->riemann == MVMM_RIEMANN_EXACT && nf > 0) {
        // kExactQueues queues of brent_cap jobs (Brent searches, Newton searches,
        // faces to finish) and their counts; a job per face in each, so that
        // the face kernel never runs a search or a flux itself
        c->brent_cap = (int)nf;
        ALLOC(c->brent_jobs, kExactQueues * (size_t)c->brent_cap * brent_job_bytes());
        ALLOC(c->brent_count, (kExactQueues + 1) * sizeof(unsigned int));  // + k_face_search's job counter
    }
    ALLOC(c->dtmp, n * 8);
    if (!prm->sync_all && c->n_inst == 1 && prm->particle_motion == MVMM_MOTION_FIXED) {  // hierarchical steps
        ALLOC(c->extrap_step, n * 4);
        ALLOC(c->dt_log, (size_t)kDtLog * 8);
    }
    ALLOC(c->face_stamp, nf * 4);
    ALLOC(c->touch, n * 4);
    ALLOC(c->blocks_done, 4);
    ALLOC(c->xfer_stored, 8);
    ALLOC(c->fresh, n);
    if (prm->precision == MVMM_PRECISION_FP32FACE && prm->particle_motion == MVMM_MOTION_FIXED)
        ALLOC(c->cf_fresh, n);
    ALLOC(c->cell_list, n * 4);
    ALLOC(c->face_list, nf * 4);
    ALLOC(c->tl, sizeof(DevTimeline) * c->n_inst);
    if (c->n_inst > 1) {
        ALLOC(c->inst, n * 4);
        ALLOC(c->inst_tb, c->n_inst * 8);
        ALLOC(c->inst_tbi, c->n_inst * 8);
        if (prm->gravity == MVMM_GRAVITY_SELF) ALLOC(c->inst_end, c->n_inst * 4);
    }
    if (prm->gravity == MVMM_GRAVITY_SELF) ALLOC(c->agrav, 3 * n * 8);
#undef ALLOC
    if (cudaMallocHost((void**)&c->tl_host, sizeof(DevTimeline) * c->n_inst) != cudaSuccess)
        return cleanup(MVMM_E_NOMEM, "cudaMallocHost failed");
    if (prm->gravity == MVMM_GRAVITY_SELF) {
        cudaError_t e = setup_self_gravity();
        if (e != cudaSuccess) return cleanup(MVMM_E_CUDA, std::string("self-gravity kernel: ") + cudaGetErrorString(e));
    }
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return cleanup(MVMM_E_CUDA, "cudaStreamCreate failed");
    c->own_stream = true;
    for (int k = 0; k <= MVMM_NUM_KERNELS; k++) cudaEventCreate(&c->ev[k]);
    {
        int pa = 0;
        if (cudaGetDevice(&c->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&c->n_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, c->device) != cudaSuccess)
            return cleanup(MVMM_E_CUDA, "device query failed");
        c->pageable_access = pa != 0;
    }
    cudaStream_t s = c->stream;
    if (c->nf > 0) {
        cudaMemcpyAsync(c->left, m->left, nf * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->right, m->right, nf * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->area, m->area, nf * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->normal, m->normal, 3 * nf * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->fcen, m->centroid, 3 * nf * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->shift, m->shift, 3 * nf * 8, cudaMemcpyHostToDevice, s);
    }
    cudaMemcpyAsync(c->csr_off, m->csr_off, (n + 1) * 4, cudaMemcpyHostToDevice, s);
    if (c->ncsr > 0) cudaMemcpyAsync(c->csr_face, m->csr_face, c->ncsr * 4, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(c->cd, 0, (size_t)kCellFields * n * 8, s);
    cudaMemsetAsync(c->timebin, 0, n, s);
    cudaMemsetAsync(c->tb_tmp, 0, n, s);
    cudaMemsetAsync(c->active, 0, n, s);
    cudaMemsetAsync(c->flux, 0, 10 * nf * 8, s);
    cudaMemsetAsync(c->face_stamp, 0, nf * 4, s);
    cudaMemsetAsync(c->touch, 0, n * 4, s);
    cudaMemsetAsync(c->blocks_done, 0, 4, s);
    cudaMemsetAsync(c->fresh, 0, n, s);
    if (c->cf_fresh) cudaMemsetAsync(c->cf_fresh, 0, n, s);
    if (c->extrap_step) cudaMemsetAsync(c->extrap_step, 0, n * 4, s);  // current at step 0
    if (c->agrav) cudaMemsetAsync(c->agrav, 0, 3 * n * 8, s);  // Particle::new: a_grav = 0
    std::memset(c->tl_host, 0, sizeof(DevTimeline) * c->n_inst);
    for (int k = 0; k < c->n_inst; k++) {
        c->tl_host[k].min_dti = kMax;
        c->tl_host[k].min_timebin = 127;
    }
    cudaMemcpyAsync(c->tl, c->tl_host, sizeof(DevTimeline) * c->n_inst, cudaMemcpyHostToDevice, s);
    std::vector<double> tb, tbi;
    std::vector<int32_t> inst_end_h;
    if (c->n_inst > 1) {
        tb.resize(c->n_inst);
        tbi.resize(c->n_inst);
        for (int k = 0; k < c->n_inst; k++) {
            tb[k] = t_end[k] / (double)kMax;  // Engine::new per simulation (engine.rs:118-119)
            tbi[k] = 1. / tb[k];
        }
        cudaMemcpyAsync(c->inst, inst_h.data(), n * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->inst_tb, tb.data(), c->n_inst * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(c->inst_tbi, tbi.data(), c->n_inst * 8, cudaMemcpyHostToDevice, s);
        if (c->inst_end) {
            inst_end_h.resize(c->n_inst);
            for (int k = 0; k < c->n_inst; k++) inst_end_h[k] = (int32_t)cell_off[k + 1];
            cudaMemcpyAsync(c->inst_end, inst_end_h.data(), c->n_inst * 4, cudaMemcpyHostToDevice, s);
        }
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cleanup(MVMM_E_CUDA, std::string("mesh upload: ") + cudaGetErrorString(e));
    *out = c;
    return MVMM_OK;
}

int mvmm_ctx_create(const mvmm_params* prm, const mvmm_mesh* m, mvmm_ctx** out) {
    return create_impl(prm, m, 1, nullptr, nullptr, out);
}

int mvmm_ctx_create_batched(const mvmm_params* prm, const mvmm_mesh* m, int64_t n_instances,
                            const int64_t* cell_offsets, const double* t_end, mvmm_ctx** out) {
    if (n_instances < 1) return fail(MVMM_E_INVALID, "batch: n_instances must be >= 1");
    if (n_instances == 1) {
        mvmm_params q = *prm;
        if (t_end) q.t_end = t_end[0];
        return create_impl(&q, m, 1, nullptr, nullptr, out);
    }
    return create_impl(prm, m, n_instances, cell_offsets, t_end, out);
}

int mvmm_batch_state(mvmm_ctx* c, uint64_t* ti_current, uint64_t* ti_old, int64_t* steps, int64_t* active_faces,
                     uint32_t* err_bits, int* finished) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rc = read_tl(c);
    if (rc) return rc;
    for (int k = 0; k < c->n_inst; k++) {
        const DevTimeline& t = c->tl_host[k];
        if (ti_current) ti_current[k] = t.ti_current;
        if (ti_old) ti_old[k] = t.ti_old;
        if (steps) steps[k] = (int64_t)t.steps;
        if (active_faces) active_faces[k] = (int64_t)t.active_faces;
        if (err_bits) err_bits[k] = t.err;
        if (finished) finished[k] = t.done;
    }
    return MVMM_OK;
}

int mvmm_ctx_destroy(mvmm_ctx* c) {
    if (!c) return MVMM_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    void* ptrs[] = {c->left, c->right, c->csr_off, c->csr_face, c->area, c->normal, c->fcen, c->shift, c->cd,
                    c->cf, c->timebin, c->tb_tmp, c->active, c->flux, c->flux32, c->geo, c->geo_pos, c->geo_changed, c->snap, c->snap_tb, c->xfer_stored, c->brent_jobs, c->brent_count, c->extrap_step, c->dt_log, c->dtmp, c->face_stamp, c->touch, c->blocks_done, c->cell_list, c->fresh, c->cf_fresh,
                    c->pend_vol, c->pend_cen, c->dirty, c->chg_list,
                    c->face_list, c->tl,
                    c->inst, c->inst_tb, c->inst_tbi, c->inst_end, c->agrav};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->tl_host) cudaFreeHost(c->tl_host);
    for (int k = 0; k <= MVMM_NUM_KERNELS; k++)
        if (c->ev[k]) cudaEventDestroy(c->ev[k]);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->geo_side) cudaStreamDestroy(c->geo_side);
    for (cudaEvent_t e : {c->ev_pred, c->ev_in, c->ev_upd, c->ev_grad, c->ev_out, c->ev_geo})
        if (e) cudaEventDestroy(e);
    delete c;
    return MVMM_OK;
}

int mvmm_ctx_set_stream(mvmm_ctx* c, void* stream) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (stream) {
        c->stream = (cudaStream_t)stream;
        c->own_stream = false;
    } else {
        CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    return MVMM_OK;
}

uint32_t mvmm_error_bits(mvmm_ctx* c) { return c ? c->err_bits : 0u; }

}  // extern "C"

namespace {
// One host array of cell rows and its place in the device block.
struct RowCopy {
    double* host;
    int field, rows;
};
// The rows of mvmm_cells in the device's field order; subset: a bit per entry.
constexpr unsigned kAllRows = 0x3fffu;
// mvmm_step_cells moves the rows in three groups each way, each as soon as the
// step can use it or has finished with it.
constexpr unsigned kRowsPredictIn = 0x0416u;  // prim, grad, extrap, v_rel (+ timebin): what predict reads
constexpr unsigned kRowsFaceIn = 0x2388u;     // gc, loc, centroid, v, dt: read from the face stage on
constexpr unsigned kRowsLateIn = 0x1861u;     // cons, facc, volume, max_a_over_r, max_signal_velocity: from the update on
constexpr unsigned kRowsEarlyOut = 0x0023u;   // cons, prim, facc: final once the update has run
constexpr unsigned kRowsMidOut = 0x1E0Cu;     // grad, gc, v, v_rel, max_a_over_r, max_signal_velocity: after gradients
constexpr unsigned kRowsLateOut = 0x2010u;    // extrap, dt (+ timebin): after the limiter
// volume, loc, centroid: a step of a fixed mesh reads them and never writes them
// (the geometry only changes through mvmm_drift / mvmm_set_mesh, which take
// moving meshes, and mvmm_step_cells steps fixed ones)
constexpr unsigned kRowsPassThrough = 0x01C0u;
int row_map(const mvmm_cells* h, unsigned subset, RowCopy* out, size_t* m) {
    const RowCopy all[14] = {{h->cons, F_CONS, 5},         {h->prim, F_PRIM, 5},     {h->grad, F_GRAD, 15},
                             {h->gc, F_GC, 3},             {h->extrap, F_EXTRAP, 5}, {h->facc, F_FACC, 5},
                             {h->volume, F_VOL, 1},        {h->loc, F_LOC, 3},       {h->centroid, F_CEN, 3},
                             {h->v, F_V, 3},               {h->v_rel, F_VREL, 3},    {h->max_a_over_r, F_MAOR, 1},
                             {h->max_signal_velocity, F_MSV, 1}, {h->dt, F_DT, 1}};
    *m = 0;
    for (int k = 0; k < 14; k++) {
        if (!all[k].host) return fail(MVMM_E_INVALID, "null cell field");
        if (subset & (1u << k)) out[(*m)++] = all[k];
    }
    if (!h->timebin) return fail(MVMM_E_INVALID, "null timebin");
    return MVMM_OK;
}
// Host <-> device transfers of cell rows.  A cudaMemcpyAsync costs a few
// microseconds of copy-engine setup on top of its bytes (and from pageable
// memory runs at well under the link's rate), and a row group is up to a dozen
// separate host arrays, so a group can move in ONE kernel that loads (or
// stores) the host rows through their device-visible address: the mapping of
// pinned memory, or the host address itself where the device reads pageable
// memory through the host page tables.  That kernel holds SM slots for the
// whole transfer, so pinned rows whose copy overlaps the step's kernels go by
// the copy engines instead.  Host arrays the device cannot address always go
// by cudaMemcpyAsync.
struct Xfer {
    const char* src;
    char* dst;
    long long bytes;
    char* dst2 = nullptr;        // host -> device: a second device copy (the snapshot), or null
    const char* ref = nullptr;   // device -> host: a device copy of the host's current content, or null
};
constexpr int kMaxXfer = 16;
constexpr long long kXferChunk = 8192;  // bytes a block moves (or compares) at a time
struct XferSet {
    Xfer x[kMaxXfer];
    long long chunk_off[kMaxXfer + 1];  // prefix sums of the transfers' chunk counts
    int m;
    unsigned long long* stored;  // bytes stored by transfers with a ref
};

__device__ __forceinline__ bool differs(uint4 a, uint4 b) { return a.x != b.x || a.y != b.y || a.z != b.z || a.w != b.w; }
__device__ __forceinline__ bool differs(unsigned long long a, unsigned long long b) { return a != b; }
__device__ __forceinline__ bool differs(char a, char b) { return a != b; }

// One chunk in units of U (16, 8 or 1 bytes).  With ref the chunk is stored
// only if it differs from ref somewhere (the host already holds ref's bytes),
// and the stored bytes are counted; with d2 it is written twice.  Up to four
// loads in flight per thread cover the link's latency.
template <typename U>
__device__ __forceinline__ void xfer_chunk(const U* __restrict__ s, U* __restrict__ d, U* __restrict__ d2,
                                           const U* __restrict__ ref, long long nv, unsigned long long* stored) {
    if (ref) {
        bool diff = false;
        for (long long k = threadIdx.x; k < nv; k += blockDim.x) diff = diff || differs(s[k], ref[k]);
        if (!__syncthreads_or(diff)) return;
        if (threadIdx.x == 0) atomicAdd(stored, (unsigned long long)(nv * (long long)sizeof(U)));
    }
    for (long long k0 = threadIdx.x; k0 < nv; k0 += 4 * (long long)blockDim.x) {
        U v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long k = k0 + (long long)u * blockDim.x;
            if (k < nv) v[u] = s[k];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long k = k0 + (long long)u * blockDim.x;
            if (k < nv) {
                d[k] = v[u];
                if (d2) d2[k] = v[u];
            }
        }
    }
}
__global__ void __launch_bounds__(256) k_xfer(XferSet t) {
    const long long total = t.chunk_off[t.m];
    for (long long ch = blockIdx.x; ch < total; ch += gridDim.x) {
        int j = 0;
        while (j + 1 < t.m && t.chunk_off[j + 1] <= ch) j++;
        const Xfer& x = t.x[j];
        const long long b0 = (ch - t.chunk_off[j]) * kXferChunk;
        const long long len = x.bytes - b0 < kXferChunk ? x.bytes - b0 : kXferChunk;
        const char* src = x.src + b0;
        char* dst = x.dst + b0;
        char* dst2 = x.dst2 ? x.dst2 + b0 : nullptr;
        const char* ref = x.ref ? x.ref + b0 : nullptr;
        const unsigned long long a = (unsigned long long)(uintptr_t)src | (uintptr_t)dst | (uintptr_t)dst2 |
                                     (uintptr_t)ref | (unsigned long long)len;
        if ((a & 15) == 0)
            xfer_chunk((const uint4*)src, (uint4*)dst, (uint4*)dst2, (const uint4*)ref, len >> 4, t.stored);
        else if ((a & 7) == 0)
            xfer_chunk((const unsigned long long*)src, (unsigned long long*)dst, (unsigned long long*)dst2,
                       (const unsigned long long*)ref, len >> 3, t.stored);
        else
            xfer_chunk(src, dst, dst2, ref, len, t.stored);
    }
}

// The address at which the device reaches host array p, or null; *pinned:
// page-locked host memory (which the copy engines move at the link's rate).
const void* device_view(mvmm_ctx* c, const void* p, bool* pinned) {
    *pinned = false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    switch (a.type) {
        case cudaMemoryTypeHost:  // pinned / registered: mapped on a UVA system
            *pinned = true;
            return a.devicePointer;
        case cudaMemoryTypeDevice:
        case cudaMemoryTypeManaged:
            return a.device == c->device ? a.devicePointer : nullptr;
        default:  // unregistered (pageable)
            return c->pageable_access ? p : nullptr;
    }
}

// Moves m (host array, device row) pairs on stream s.  Pairs go in one kernel
// except, by cudaMemcpyAsync, those whose host array the device cannot
// address and, with overlap (the copy runs beside the step's kernels), plain
// copies of pinned memory.  A pair with a ref always takes the kernel where
// the device can address its host array (its bytes mostly need no storing).
// max_blocks caps the kernel's grid (0: four blocks per SM), so that beside a
// kernel on the critical path it holds few SM slots.
int transfer(mvmm_ctx* c, const Xfer* pairs, int m, bool h2d, bool overlap, int max_blocks, cudaStream_t s) {
    XferSet t{};
    t.m = 0;
    t.stored = c->xfer_stored;
    long long chunks = 0;
    for (int k = 0; k < m; k++) {
        const Xfer& x = pairs[k];
        if (x.bytes <= 0) continue;
        const char* host = h2d ? x.src : (const char*)x.dst;
        bool pinned = false, pinned_end = false;
        const char* view = (const char*)device_view(c, host, &pinned);
        // rows merged from separate arrays must lie in one mapping
        if (view && (const char*)device_view(c, host + x.bytes - 1, &pinned_end) != view + x.bytes - 1)
            view = nullptr;
        if (!view || (overlap && pinned && !x.ref)) {
            const cudaMemcpyKind kind = h2d ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
            CUDA_TRY(cudaMemcpyAsync(x.dst, x.src, (size_t)x.bytes, kind, s));
            if (x.dst2) CUDA_TRY(cudaMemcpyAsync(x.dst2, x.dst, (size_t)x.bytes, cudaMemcpyDeviceToDevice, s));
            if (h2d) c->host_bytes_in += x.bytes;
            else c->host_bytes_out += x.bytes;
            continue;
        }
        Xfer v = x;
        if (h2d) v.src = view;
        else v.dst = (char*)view;
        if (h2d) c->host_bytes_in += x.bytes;
        else if (!x.ref) c->host_bytes_out += x.bytes;  // with a ref the kernel counts what it stores
        t.x[t.m] = v;
        t.chunk_off[t.m] = chunks;
        chunks += (x.bytes + kXferChunk - 1) / kXferChunk;
        t.m++;
    }
    if (t.m == 0) return MVMM_OK;
    t.chunk_off[t.m] = chunks;
    const long long cap = max_blocks > 0 ? max_blocks : 4LL * c->n_sms;
    k_xfer<<<(unsigned)(chunks < cap ? chunks : cap), 256, 0, s>>>(t);
    CUDA_TRY(cudaGetLastError());
    return MVMM_OK;
}

// Options of a row copy.  overlap: it runs beside the step's kernels;
// max_blocks: the copy kernel's grid cap (0: four blocks per SM).
// snapshot (host -> device): the rows also go to the snapshot block.
// in_place (device -> host): the host arrays of `in_place` that `h` shares
// still hold the bytes of the snapshot, so only what differs is stored;
// diff_rows: the rows (row_map bits) whose snapshot is current.
struct CopyOpts {
    bool overlap = false;
    int max_blocks = 0;
    bool snapshot = false;
    const mvmm_cells* in_place = nullptr;
    unsigned diff_rows = 0x3fffu;
};

// The host array of field k (row_map order) of h.
const void* field_ptr(const mvmm_cells* h, int k) {
    const void* f[14] = {h->cons, h->prim, h->grad, h->gc, h->extrap, h->facc, h->volume,
                         h->loc, h->centroid, h->v, h->v_rel, h->max_a_over_r, h->max_signal_velocity, h->dt};
    return f[k];
}

// Copies rows between the host arrays and the device block; rows that lie
// back to back on the host in the device's field order form one transfer.
int copy_rows(mvmm_ctx* c, const mvmm_cells* h, const RowCopy* map, const int* idx, size_t m, bool timebin,
              cudaMemcpyKind kind, const CopyOpts& o, cudaStream_t s) {
    const size_t n = c->n;
    const bool h2d = kind == cudaMemcpyHostToDevice;
    auto diffable = [&](size_t a) {
        return !h2d && o.in_place && c->snap && ((o.diff_rows >> idx[a]) & 1u) &&
               field_ptr(h, idx[a]) == field_ptr(o.in_place, idx[a]);
    };
    Xfer x[kMaxXfer];
    int nx = 0;
    for (size_t a = 0; a < m;) {
        size_t b = a + 1;
        int rows = map[a].rows;
        const bool dif = diffable(a);
        while (b < m && map[b].host == map[a].host + (size_t)rows * n && map[b].field == map[a].field + rows &&
               diffable(b) == dif)
            rows += map[b++].rows;
        char* dev = (char*)(c->cd + (size_t)map[a].field * n);
        char* snap = c->snap ? (char*)(c->snap + (size_t)map[a].field * n) : nullptr;
        char* host = (char*)map[a].host;
        Xfer t{h2d ? host : dev, h2d ? dev : host, (long long)rows * (long long)n * 8};
        if (h2d && o.snapshot) t.dst2 = snap;
        if (dif) t.ref = snap;
        x[nx++] = t;
        a = b;
    }
    if (timebin) {
        Xfer t{h2d ? (const char*)h->timebin : (const char*)c->timebin, h2d ? (char*)c->timebin : (char*)h->timebin,
               (long long)n};
        if (h2d && o.snapshot) t.dst2 = (char*)c->snap_tb;
        if (!h2d && o.in_place && c->snap && h->timebin == o.in_place->timebin) t.ref = (const char*)c->snap_tb;
        x[nx++] = t;
    }
    return transfer(c, x, nx, h2d, o.overlap, o.max_blocks, s);
}
// Device copy of the rows of `subset` (and the time bins) into the snapshot
// block, on stream s.
int snapshot_rows(mvmm_ctx* c, unsigned subset, bool timebin, cudaStream_t s) {
    static const int first[14] = {F_CONS, F_PRIM, F_GRAD, F_GC, F_EXTRAP, F_FACC, F_VOL,
                                  F_LOC, F_CEN, F_V, F_VREL, F_MAOR, F_MSV, F_DT};
    static const int rows[14] = {5, 5, 15, 3, 5, 5, 1, 3, 3, 3, 3, 1, 1, 1};
    const long long n = c->n;
    XferSet t{};
    t.stored = c->xfer_stored;
    long long chunks = 0;
    auto add = [&](const char* src, char* dst, long long bytes) {
        t.x[t.m] = Xfer{src, dst, bytes};
        t.chunk_off[t.m++] = chunks;
        chunks += (bytes + kXferChunk - 1) / kXferChunk;
    };
    for (int k = 0; k < 14; k++) {
        if (!(subset & (1u << k))) continue;
        add((const char*)(c->cd + first[k] * n), (char*)(c->snap + first[k] * n), rows[k] * n * 8);
    }
    if (timebin) add((const char*)c->timebin, (char*)c->snap_tb, n);
    if (t.m == 0 || chunks == 0) return MVMM_OK;
    t.chunk_off[t.m] = chunks;
    const long long cap = 4LL * c->n_sms;
    k_xfer<<<(unsigned)(chunks < cap ? chunks : cap), 256, 0, s>>>(t);
    CUDA_TRY(cudaGetLastError());
    return MVMM_OK;
}
int copy_cells(mvmm_ctx* c, const mvmm_cells* h, unsigned subset, bool timebin, cudaMemcpyKind kind,
               cudaStream_t s, const CopyOpts& o = CopyOpts()) {
    if (h->n != c->n) return fail(MVMM_E_INVALID, "cell count does not match the mesh");
    RowCopy map[14];
    int idx[14];
    size_t m = 0;
    int rc = row_map(h, subset, map, &m);
    if (rc) return rc;
    for (int k = 0, j = 0; k < 14; k++)
        if (subset & (1u << k)) idx[j++] = k;
    return copy_rows(c, h, map, idx, m, timebin, kind, o, s);
}
// Hierarchical steps defer the extrapolation of inactive cells: every cell's
// is made before the state is read or changed as a whole; reset: the state was
// replaced (uploaded or restored), none is pending.
int sync_extrap(mvmm_ctx* c, bool reset, cudaStream_t s) {
    if (!c->extrap_step) return MVMM_OK;
    launch_extrap_flush(make_kp(c, 0, 7), reset, s);
    CUDA_TRY(cudaGetLastError());
    return MVMM_OK;
}
// The cell state changed outside a step: every cell's derived face-stage rows
// are recomputed by the next predict.
int mark_stale(mvmm_ctx* c, cudaStream_t s) {
    CUDA_TRY(cudaMemsetAsync(c->fresh, 0, c->n, s));
    if (c->cf_fresh) CUDA_TRY(cudaMemsetAsync(c->cf_fresh, 0, c->n, s));
    return MVMM_OK;
}
// positions and centroids may have changed: refresh the FP32 face geometry
int refresh_geometry(mvmm_ctx* c, cudaStream_t s) {
    int rc = mark_stale(c, s);
    if (rc) return rc;
    update_geom32(c, make_kp(c, 0, 7), s);
    CUDA_TRY(cudaGetLastError());
    return MVMM_OK;
}
}  // namespace

extern "C" {

int mvmm_upload_cells(mvmm_ctx* c, const mvmm_cells* h) {
    if (!c || !h) return fail(MVMM_E_INVALID, "null argument");
    int rc = copy_cells(c, h, kAllRows, true, cudaMemcpyHostToDevice, c->stream);
    if (rc) return rc;
    rc = sync_extrap(c, true, c->stream);
    if (rc) return rc;
    return refresh_geometry(c, c->stream);
}

int mvmm_download_cells(mvmm_ctx* c, mvmm_cells* h) {
    if (!c || !h) return fail(MVMM_E_INVALID, "null argument");
    int rc = sync_extrap(c, false, c->stream);
    if (rc) return rc;
    rc = copy_cells(c, h, kAllRows, true, cudaMemcpyDeviceToHost, c->stream);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MVMM_OK;
}

int mvmm_step_cells(mvmm_ctx* c, const mvmm_cells* in, mvmm_cells* out, uint64_t ti_current, uint64_t ti_old,
                    uint64_t* ti_next, int64_t* n_active_faces) {
    if (!c || !in || !out) return fail(MVMM_E_INVALID, "null argument");
    if (c->n_inst != 1) return fail(MVMM_E_UNSUPPORTED, "mvmm_step_cells steps a single simulation");
    if (c->prm.particle_motion != MVMM_MOTION_FIXED)
        return fail(MVMM_E_UNSUPPORTED, "mvmm_step_cells steps a fixed mesh");
    if (c->prm.gravity_accelerations)  // kick1 rewrites the conserved rows after their copy back has begun
        return fail(MVMM_E_UNSUPPORTED, "mvmm_step_cells does not apply gravity accelerations");
    if (!c->side) {
        CUDA_TRY(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
        CUDA_TRY(cudaStreamCreateWithFlags(&c->geo_side, cudaStreamNonBlocking));
        for (cudaEvent_t* e : {&c->ev_pred, &c->ev_in, &c->ev_upd, &c->ev_grad, &c->ev_out, &c->ev_geo})
            CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    if (!c->snap) {
        if (cudaMalloc((void**)&c->snap, (size_t)F_SRC * c->n * 8) != cudaSuccess ||
            cudaMalloc((void**)&c->snap_tb, (size_t)c->n) != cudaSuccess)
            return fail(MVMM_E_NOMEM, "mvmm_step_cells: cudaMalloc failed");
    }
    cudaStream_t s = c->stream, s2 = c->side;
    launch_set_time(make_kp(c, 0, 7), ti_current, ti_old, s);
    // host -> device: the rows predict and the face stage read in one transfer
    // on the step's own stream, then (copies in one direction share the link)
    // the rows the update alone reads on the side stream, which land while the
    // face stage runs
    CopyOpts up;
    up.snapshot = true;  // the uploaded bytes, against which the copies back skip unchanged chunks
    int rc = copy_cells(c, in, kRowsPredictIn | kRowsFaceIn, true, cudaMemcpyHostToDevice, s, up);
    if (rc) return rc;
    rc = sync_extrap(c, true, s);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(c->ev_pred, s));
    CUDA_TRY(cudaStreamWaitEvent(s2, c->ev_pred, 0));
    // the FP32 face geometry follows the uploaded positions and centroids, on a
    // stream of its own while predict runs (predict does not read it)
    const bool fp32_geom = c->prm.precision == MVMM_PRECISION_FP32FACE;
    if (fp32_geom) {
        CUDA_TRY(cudaStreamWaitEvent(c->geo_side, c->ev_pred, 0));
        update_geom32(c, make_kp(c, 0, 7), c->geo_side);
        CUDA_TRY(cudaEventRecord(c->ev_geo, c->geo_side));
    }
    up.overlap = true;
    up.snapshot = false;  // taken on the device once the rows have landed (below)
    rc = copy_cells(c, in, kRowsLateIn, false, cudaMemcpyHostToDevice, s2, up);
    if (rc) return rc;
    // their snapshot: with every cell updated every step the update kernel
    // keeps the bytes it reads; else a device copy, which the update waits for
    const unsigned late_snap = kRowsLateIn & ~kRowsPassThrough;
    if (!c->prm.sync_all) {
        rc = snapshot_rows(c, late_snap, false, s2);
        if (rc) return rc;
    }
    CUDA_TRY(cudaEventRecord(c->ev_in, s2));
    StepHooks h;
    h.stale_all = true;
    if (c->prm.sync_all) h.snap_late = c->snap;
    h.wait_before_face = fp32_geom ? c->ev_geo : nullptr;
    h.wait_before_update = c->ev_in;
    h.after_update = c->ev_upd;
    h.after_gradients = c->ev_grad;
    enqueue_step_kernels(c, false, h);
    // device -> host on the side stream: the rows final after the update while
    // the gradient stage runs, those final after it while the limiter runs.
    // Arrays that `out` shares with `in` still hold the uploaded bytes: only
    // the chunks the step changed are stored.
    CopyOpts back;
    back.overlap = true;
    back.max_blocks = 64;  // beside the gradient stage
    back.in_place = in;
    back.diff_rows = kRowsPredictIn | kRowsFaceIn | late_snap;
    CUDA_TRY(cudaStreamWaitEvent(s2, c->ev_upd, 0));
    rc = copy_cells(c, out, kRowsEarlyOut, false, cudaMemcpyDeviceToHost, s2, back);
    if (rc) return rc;
    CUDA_TRY(cudaStreamWaitEvent(s2, c->ev_grad, 0));
    back.max_blocks = 128;  // beside the limiter (which the copies after it wait for)
    rc = copy_cells(c, out, kRowsMidOut, false, cudaMemcpyDeviceToHost, s2, back);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(c->ev_out, s2));
    back.overlap = false;
    back.max_blocks = 0;
    rc = copy_cells(c, out, kRowsLateOut, true, cudaMemcpyDeviceToHost, s, back);
    if (rc) return rc;
    CUDA_TRY(cudaStreamWaitEvent(s, c->ev_out, 0));
    CUDA_TRY(cudaGetLastError());
    // the rows the step leaves unchanged do not cross the link back: nothing to
    // do in place, else a host copy from `in` while the step runs (after the
    // uploads, so that an `out` row that overlaps an `in` row is read first)
    const size_t n = (size_t)c->n;
    const struct {
        const double* src;
        double* dst;
        size_t len;
    } pass[3] = {{in->volume, out->volume, n}, {in->loc, out->loc, 3 * n}, {in->centroid, out->centroid, 3 * n}};
    static_assert(kRowsPassThrough == ((1u << 6) | (1u << 7) | (1u << 8)), "volume, loc, centroid");
    bool waited = false;
    for (const auto& r : pass) {
        if (r.src == r.dst) continue;
        if (!waited) CUDA_TRY(cudaEventSynchronize(c->ev_in));
        waited = true;
        std::memmove(r.dst, r.src, r.len * sizeof(double));
    }
    rc = finish(c);
    if (ti_next) *ti_next = c->tl_host->ti_current;
    if (n_active_faces) *n_active_faces = (int64_t)(c->tl_host->active_faces - c->tl_host->faces_mark);
    return rc;
}

}  // extern "C"

namespace {
// ---- host-resident state moved where it changes -------------------------
// The host rows of mvmm_cells at the addresses the device reaches them by:
// row r of the device block (r < F_SRC, the block's field order) and the
// time bins.
struct HostRows {
    double* row[F_SRC];
    int8_t* tb;
};
// volume, loc and centroid: a step of a fixed mesh never writes them
constexpr int kKeptFirst = F_VOL, kKeptEnd = F_V;
constexpr long long kStoredCellBytes = (long long)(F_SRC - (kKeptEnd - kKeptFirst)) * 8 + 1;

int host_rows(mvmm_ctx* c, const mvmm_cells* h, HostRows* out) {
    RowCopy map[14];
    size_t m = 0;
    int rc = row_map(h, kAllRows, map, &m);
    if (rc) return rc;
    const size_t n = (size_t)c->n;
    auto view = [&](const void* p, size_t bytes) -> char* {
        bool pinned = false, pinned_end = false;
        const char* v = (const char*)device_view(c, p, &pinned);
        if (v && (const char*)device_view(c, (const char*)p + bytes - 1, &pinned_end) != v + bytes - 1) v = nullptr;
        return (char*)v;
    };
    const char* why = "mvmm_step_cells_changed: the device cannot address a cell array (pin it)";
    for (size_t k = 0; k < m; k++) {
        double* v = (double*)view(map[k].host, (size_t)map[k].rows * n * 8);
        if (!v) return fail(MVMM_E_UNSUPPORTED, why);
        for (int j = 0; j < map[k].rows; j++) out->row[map[k].field + j] = v + (size_t)j * n;
    }
    out->tb = (int8_t*)view(h->timebin, n);
    if (!out->tb) return fail(MVMM_E_UNSUPPORTED, why);
    return MVMM_OK;
}

// The listed cells' rows (blockIdx.y: the row, F_SRC the time bin) from the
// host arrays.  Their derived rows are recomputed by the next predict, and no
// deferred extrapolation is pending for them.  Indices were checked on the host.
__global__ void __launch_bounds__(256) k_gather_cells(HostRows h, const int* __restrict__ list, int m, KP p) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int i = list[j];
    const int r = blockIdx.y;
    if (r < F_SRC) {
        p.cd[(size_t)r * p.n + i] = h.row[r][i];
    } else {
        p.timebin[i] = h.tb[i];
        p.fresh[i] = 0;
        if (p.cf_fresh) p.cf_fresh[i] = 0;
        if (p.extrap_step) p.extrap_step[i] = (unsigned int)p.tl[0].steps;
    }
}

// Rows [A, B) of cell i to the host, eight loads in flight before their stores.
template <int A, int B>
__device__ __forceinline__ void store_rows(const HostRows& h, const double* __restrict__ cd, size_t n, int i) {
#pragma unroll
    for (int r0 = A; r0 < B; r0 += 8) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (r0 + u < B) v[u] = cd[(size_t)(r0 + u) * n + i];
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (r0 + u < B) h.row[r0 + u][i] = v[u];
    }
}

// Stores the rows of the cells a kernel marked since the last store, a warp
// per 32 consecutive cells (whole 256-byte segments of each row): all their
// rows wherever one of them is marked kDirtyAll, else their extrapolation rows
// wherever one is marked kDirtyExtrap (inactive cells of a hierarchical step
// whose time extrapolation moved).  Clears the marks; counts the bytes into
// the timeline.
__global__ void __launch_bounds__(256) k_store_dirty(HostRows h, KP p) {
    const int lane = threadIdx.x & 31;
    const int n_warps = (int)((gridDim.x * blockDim.x) >> 5);
    const int groups = (p.n + 31) >> 5;
    for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < groups; w += n_warps) {
        const int i = (w << 5) + lane;
        const bool in = i < p.n;
        const uint8_t d = in ? p.dirty[i] : 0;
        const bool all = __any_sync(0xffffffffu, (d & kDirtyAll) != 0);
        if (!__any_sync(0xffffffffu, d != 0)) continue;
        if (in) {
            if (all) {
                store_rows<0, kKeptFirst>(h, p.cd, (size_t)p.n, i);
                store_rows<kKeptEnd, F_SRC>(h, p.cd, (size_t)p.n, i);
                h.tb[i] = p.timebin[i];
            } else {
                store_rows<F_EXTRAP, F_EXTRAP + 5>(h, p.cd, (size_t)p.n, i);
            }
            p.dirty[i] = 0;
        }
        if (lane == 0) {
            const int cells = min(32, p.n - (w << 5));
            const unsigned long long per = all ? (unsigned long long)kStoredCellBytes : 5ull * 8ull;
            atomicAdd(&p.tl[0].host_stored, (unsigned long long)cells * per);
        }
    }
}
}  // namespace

extern "C" {

int mvmm_step_cells_changed(mvmm_ctx* c, mvmm_cells* cells, const int32_t* changed, int64_t n_changed,
                            uint64_t ti_current, uint64_t ti_old, uint64_t* ti_next, int64_t* n_active_faces,
                            int64_t* bytes_stored) {
    if (!c || !cells) return fail(MVMM_E_INVALID, "null argument");
    if (c->n_inst != 1) return fail(MVMM_E_UNSUPPORTED, "mvmm_step_cells_changed steps a single simulation");
    if (c->prm.particle_motion != MVMM_MOTION_FIXED)
        return fail(MVMM_E_UNSUPPORTED, "mvmm_step_cells_changed steps a fixed mesh");
    if (cells->n != c->n) return fail(MVMM_E_INVALID, "cell count does not match the mesh");
    if (changed && (n_changed < 0 || n_changed > c->n))
        return fail(MVMM_E_INVALID, "n_changed must lie in [0, n_cells]");
    if (changed)
        for (int64_t k = 0; k < n_changed; k++)
            if (changed[k] < 0 || changed[k] >= c->n) return fail(MVMM_E_INVALID, "changed: cell index out of range");
    HostRows h;
    int rc = host_rows(c, cells, &h);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    if (!c->dirty) {
        if (cudaMalloc((void**)&c->dirty, (size_t)c->n) != cudaSuccess ||
            cudaMalloc((void**)&c->chg_list, (size_t)c->n * 4) != cudaSuccess)
            return fail(MVMM_E_NOMEM, "mvmm_step_cells_changed: cudaMalloc failed");
        CUDA_TRY(cudaMemsetAsync(c->dirty, 0, (size_t)c->n, s));
        drop_graphs(c);  // the captured kernels' parameters now carry the marks
    }
    launch_set_time(make_kp(c, 0, 7), ti_current, ti_old, s);
    CUDA_TRY(cudaMemsetAsync(&c->tl->host_stored, 0, sizeof(unsigned long long), s));
    if (!changed) {
        // every cell: the arrays become the device's mirror
        rc = copy_cells(c, cells, kAllRows, true, cudaMemcpyHostToDevice, s);
        if (rc) return rc;
        rc = sync_extrap(c, true, s);
        if (rc) return rc;
        rc = refresh_geometry(c, s);
        if (rc) return rc;
        CUDA_TRY(cudaMemsetAsync(c->dirty, 0, (size_t)c->n, s));
    } else if (n_changed > 0) {
        CUDA_TRY(cudaMemcpyAsync(c->chg_list, changed, (size_t)n_changed * 4, cudaMemcpyHostToDevice, s));
        const KP p = make_kp(c, 0, 7);
        k_gather_cells<<<dim3((unsigned)((n_changed + 255) / 256), F_SRC + 1), 256, 0, s>>>(h, c->chg_list,
                                                                                          (int)n_changed, p);
        CUDA_TRY(cudaGetLastError());
        update_geom32(c, p, s);  // the faces of cells whose position or centroid changed
        CUDA_TRY(cudaGetLastError());
        c->host_bytes_in += n_changed * ((int64_t)F_SRC * 8 + 1);
    }
    rc = enqueue_steps_impl(c, 1);
    if (rc) return rc;
    // the deferred extrapolations are made (and marked where their bits change),
    // so that the host rows hold the state after the step
    rc = sync_extrap(c, false, s);
    if (rc) return rc;
    const long long blocks = std::min<long long>(((long long)c->n + 255) / 256, 16LL * c->n_sms);
    k_store_dirty<<<(unsigned)blocks, 256, 0, s>>>(h, make_kp(c, 0, 7));
    CUDA_TRY(cudaGetLastError());
    rc = finish(c);
    const unsigned long long stored = c->tl_host->host_stored;
    c->host_bytes_out += (int64_t)stored;
    if (bytes_stored) *bytes_stored = (int64_t)stored;
    if (ti_next) *ti_next = c->tl_host->ti_current;
    if (n_active_faces) *n_active_faces = (int64_t)(c->tl_host->active_faces - c->tl_host->faces_mark);
    return rc;
}

// ---- per-stage --------------------------------------------------------
static int upload_mask(mvmm_ctx* c, const uint8_t* active) {
    if (!active) return fail(MVMM_E_INVALID, "null active mask");
    int rc = sync_extrap(c, false, c->stream);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->active, active, c->n, cudaMemcpyHostToDevice, c->stream));
    return mark_stale(c, c->stream);
}

int mvmm_predict(mvmm_ctx* c, double dt) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rs = sync_extrap(c, false, c->stream);
    if (rs) return rs;
    rs = mark_stale(c, c->stream);
    if (rs) return rs;
    KP p = make_kp(c, 1, 10);
    p.stage_dt = dt;
    launch_predict(p, c->stream);
    CUDA_TRY(cudaGetLastError());
    return finish(c);
}

int mvmm_compute_fluxes(mvmm_ctx* c, const uint8_t* active, double* out, int64_t* n_active) {
    if (!c || !out) return fail(MVMM_E_INVALID, "null argument");
    int rc = upload_mask(c, active);
    if (rc) return rc;
    rc = read_tl(c);
    if (rc) return rc;
    unsigned long long before = sum_field(c, &DevTimeline::active_faces);
    KP p = make_kp(c, 1, 10);
    launch_derive(p, c->stream);
    launch_face(c, p);
    CUDA_TRY(cudaGetLastError());
    if (c->nf > 0)
        CUDA_TRY(cudaMemcpyAsync(out, c->flux, (size_t)10 * c->nf * 8, cudaMemcpyDeviceToHost, c->stream));
    rc = finish(c);
    if (n_active) *n_active = (int64_t)(sum_field(c, &DevTimeline::active_faces) - before);
    return rc;
}

int mvmm_apply_fluxes(mvmm_ctx* c, const double* fluxes, const uint8_t* active) {
    if (!c || !fluxes) return fail(MVMM_E_INVALID, "null argument");
    int rc = upload_mask(c, active);
    if (rc) return rc;
    if (c->nf > 0)
        CUDA_TRY(cudaMemcpyAsync(c->flux, fluxes, (size_t)10 * c->nf * 8, cudaMemcpyHostToDevice, c->stream));
    KP p = make_kp(c, 1, 10);
    launch_update(p, 0, c->stream);
    if (self_gravity_kicks(c)) launch_self_gravity(p, 1, 0, c->stream);
    CUDA_TRY(cudaGetLastError());
    return finish(c);
}

int mvmm_convert_conserved_to_primitive(mvmm_ctx* c, const uint8_t* active) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rc = upload_mask(c, active);
    if (rc) return rc;
    launch_c2p(make_kp(c, 1, 10), c->stream);
    CUDA_TRY(cudaGetLastError());
    return finish(c);
}

int mvmm_gradients(mvmm_ctx* c, const uint8_t* active) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rc = upload_mask(c, active);
    if (rc) return rc;
    launch_gradients(make_kp(c, 1, 10), 0, c->stream);
    CUDA_TRY(cudaGetLastError());
    return finish(c);
}

int mvmm_compute_timesteps(mvmm_ctx* c, const uint8_t* active, double* dt_out) {
    if (!c || !dt_out) return fail(MVMM_E_INVALID, "null argument");
    int rc = upload_mask(c, active);
    if (rc) return rc;
    launch_timesteps(make_kp(c, 1, 10), c->dtmp, c->stream);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(dt_out, c->dtmp, (size_t)c->n * 8, cudaMemcpyDeviceToHost, c->stream));
    return finish(c);
}

// ---- GravitySolver trait -----------------------------------------------
int mvmm_gravity_timesteps(mvmm_ctx* c, double* dt_out) {
    if (!c || !dt_out) return fail(MVMM_E_INVALID, "null argument");
    launch_gravity(make_kp(c, 1, 10), -1, c->dtmp, c->stream);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(dt_out, c->dtmp, (size_t)c->n * 8, cudaMemcpyDeviceToHost, c->stream));
    return finish(c);
}

int mvmm_gravity_accelerations(mvmm_ctx* c, double* a_out) {
    if (!c || !a_out) return fail(MVMM_E_INVALID, "null argument");
    const KP p = make_kp(c, 1, 10);
    if (c->prm.gravity == MVMM_GRAVITY_SELF) {  // SelfGravity::compute_accelerations sets every a_grav
        launch_self_gravity(p, 0, 0, c->stream);
        CUDA_TRY(cudaGetLastError());
        if (c->n > 0)
            CUDA_TRY(cudaMemcpyAsync(a_out, c->agrav, (size_t)3 * c->n * 8, cudaMemcpyDeviceToHost, c->stream));
        return finish(c);
    }
    for (int a = 0; a < 3; a++) {
        if (c->prm.gravity == MVMM_GRAVITY_NONE) {
            CUDA_TRY(cudaMemsetAsync(c->dtmp, 0, (size_t)c->n * 8, c->stream));
        } else {
            launch_gravity(p, a, c->dtmp, c->stream);
            CUDA_TRY(cudaGetLastError());
        }
        CUDA_TRY(cudaMemcpyAsync(a_out + (size_t)a * c->n, c->dtmp, (size_t)c->n * 8, cudaMemcpyDeviceToHost,
                                 c->stream));
    }
    return finish(c);
}

// ---- step / run --------------------------------------------------------
int mvmm_set_time(mvmm_ctx* c, uint64_t ti_current, uint64_t ti_old) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rc = read_tl(c);
    if (rc) return rc;
    for (int k = 0; k < c->n_inst; k++) {  // a batch restarts every simulation at the same point
        c->tl_host[k].ti_current = ti_current;
        c->tl_host[k].ti_old = ti_old;
        c->tl_host[k].min_dti = kMax;
        c->tl_host[k].min_timebin = 127;
        c->tl_host[k].done = 0;
    }
    rc = write_tl(c);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MVMM_OK;
}

int mvmm_get_time(mvmm_ctx* c, uint64_t* ti_current, uint64_t* ti_old, int64_t* steps, int64_t* active_faces,
                  int* finished) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rc = read_tl(c);
    if (rc) return rc;
    if (ti_current) *ti_current = c->tl_host->ti_current;
    if (ti_old) *ti_old = c->tl_host->ti_old;
    if (steps) *steps = (int64_t)c->tl_host->steps;
    if (active_faces) *active_faces = (int64_t)sum_field(c, &DevTimeline::active_faces);
    if (finished) *finished = all_done(c) ? 1 : 0;
    return MVMM_OK;
}

int mvmm_get_stats(mvmm_ctx* c, mvmm_stats* out) {
    if (!c || !out) return fail(MVMM_E_INVALID, "null argument");
    int rc = read_tl(c);
    if (rc) return rc;
    out->steps = (int64_t)sum_field(c, &DevTimeline::steps);
    out->active_faces = (int64_t)sum_field(c, &DevTimeline::active_faces);
    out->active_cells = (int64_t)sum_field(c, &DevTimeline::active_cells);
    out->fp64_fallback_faces = (int64_t)sum_field(c, &DevTimeline::fallback_faces);
    unsigned long long stored = 0;
    CUDA_TRY(cudaMemcpy(&stored, c->xfer_stored, 8, cudaMemcpyDeviceToHost));
    out->host_bytes_in = c->host_bytes_in;
    out->host_bytes_out = c->host_bytes_out + (int64_t)stored;
    return MVMM_OK;
}

int mvmm_step(mvmm_ctx* c, uint64_t ti_current, uint64_t ti_old, uint64_t* ti_next, int64_t* n_active_faces) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    // a batch continues every simulation from its own device timeline
    int rc = c->n_inst == 1 ? mvmm_set_time(c, ti_current, ti_old) : read_tl(c);
    if (rc) return rc;
    unsigned long long before = sum_field(c, &DevTimeline::active_faces);
    rc = enqueue_steps_impl(c, 1);
    if (rc) return rc;
    rc = finish(c);
    if (ti_next) *ti_next = c->tl_host->ti_current;
    if (n_active_faces) *n_active_faces = (int64_t)(sum_field(c, &DevTimeline::active_faces) - before);
    return rc;
}

static int reject_moving(mvmm_ctx* c) {
    if (c->prm.particle_motion != MVMM_MOTION_FIXED)
        return fail(MVMM_E_UNSUPPORTED, "a moving mesh is stepped from the host: mvmm_drift, mvmm_set_mesh, mvmm_step");
    return MVMM_OK;
}

int mvmm_enqueue_steps(mvmm_ctx* c, int64_t n_steps) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    int rc = reject_moving(c);
    if (rc) return rc;
    return enqueue_steps_impl(c, n_steps);
}

int mvmm_flush_deferred(mvmm_ctx* c) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    return sync_extrap(c, false, c->stream);
}

int mvmm_drift(mvmm_ctx* c, double dt) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    if (c->prm.particle_motion == MVMM_MOTION_FIXED) return MVMM_OK;  // v = 0: nothing moves
    if (!(dt >= 0.)) return fail(MVMM_E_INVALID, "drift: dt must be >= 0");
    launch_drift(make_kp(c, 0, 7), dt, c->stream);
    CUDA_TRY(cudaGetLastError());
    return finish(c);
}

int mvmm_get_positions(mvmm_ctx* c, double* loc) {
    if (!c || !loc) return fail(MVMM_E_INVALID, "null argument");
    CUDA_TRY(cudaMemcpyAsync(loc, c->cd + (size_t)F_LOC * c->n, (size_t)3 * c->n * 8, cudaMemcpyDeviceToHost,
                             c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MVMM_OK;
}

int mvmm_set_mesh(mvmm_ctx* c, const mvmm_mesh* m, const double* volume, const double* centroid) {
    if (!c || !m || !volume || !centroid) return fail(MVMM_E_INVALID, "null argument");
    if (c->prm.particle_motion == MVMM_MOTION_FIXED)
        return fail(MVMM_E_INVALID, "set_mesh: the context was created for a fixed mesh");
    if (m->n_cells != c->n) return fail(MVMM_E_INVALID, "set_mesh: cell count changed");
    int rc = check_mesh(m, c->prm.boundary);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaStreamSynchronize(s));
    int nf = (int)m->n_faces;
    int64_t ncsr = m->csr_off[m->n_cells];
    if (nf > c->nf_cap || ncsr > c->ncsr_cap) {
        // grow with headroom; every face-sized buffer is reallocated
        int cap = nf > c->nf_cap ? nf + nf / 4 + 16 : c->nf_cap;
        int64_t ccap = ncsr > c->ncsr_cap ? ncsr + ncsr / 4 + 16 : c->ncsr_cap;
        struct Buf {
            void** ptr;
            size_t bytes;
        } bufs[] = {{(void**)&c->left, (size_t)cap * 4},       {(void**)&c->right, (size_t)cap * 4},
                    {(void**)&c->area, (size_t)cap * 8},       {(void**)&c->normal, (size_t)cap * 24},
                    {(void**)&c->fcen, (size_t)cap * 24},      {(void**)&c->shift, (size_t)cap * 24},
                    {(void**)&c->flux, (size_t)cap * 80},      {(void**)&c->face_stamp, (size_t)cap * 4},
                    {(void**)&c->face_list, (size_t)cap * 4},  {(void**)&c->csr_face, (size_t)ccap * 4},
                    {(void**)&c->flux32, c->flux32 ? (size_t)cap * 28 : 0},
                    {(void**)&c->geo, c->geo ? (size_t)cap * 4 * kFaceGeom32 : 0}};
        for (auto& b : bufs) {
            if (!b.bytes) continue;
            cudaFree(*b.ptr);
            *b.ptr = nullptr;
            if (cudaMalloc(b.ptr, b.bytes) != cudaSuccess) return fail(MVMM_E_NOMEM, "set_mesh: cudaMalloc failed");
        }
        CUDA_TRY(cudaMemsetAsync(c->face_stamp, 0, (size_t)cap * 4, s));
        if (c->brent_jobs) {
            const int bcap = (int)cap;
            cudaFree(c->brent_jobs);
            c->brent_jobs = nullptr;
            if (cudaMalloc(&c->brent_jobs, kExactQueues * (size_t)bcap * brent_job_bytes()) != cudaSuccess)
                return fail(MVMM_E_NOMEM, "set_mesh: cudaMalloc failed");
            c->brent_cap = bcap;
        }
        c->nf_cap = cap;
        c->ncsr_cap = ccap;
    }
    // face rows are [3][nf]: the row stride changes with the face count
    c->nf = nf;
    c->ncsr = ncsr;
    if (nf > 0) {
        CUDA_TRY(cudaMemcpyAsync(c->left, m->left, (size_t)nf * 4, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(c->right, m->right, (size_t)nf * 4, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(c->area, m->area, (size_t)nf * 8, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(c->normal, m->normal, (size_t)nf * 24, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(c->fcen, m->centroid, (size_t)nf * 24, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(c->shift, m->shift, (size_t)nf * 24, cudaMemcpyHostToDevice, s));
    }
    CUDA_TRY(cudaMemcpyAsync(c->csr_off, m->csr_off, (size_t)(c->n + 1) * 4, cudaMemcpyHostToDevice, s));
    if (ncsr > 0) CUDA_TRY(cudaMemcpyAsync(c->csr_face, m->csr_face, (size_t)ncsr * 4, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->pend_vol, volume, (size_t)c->n * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->pend_cen, centroid, (size_t)c->n * 24, cudaMemcpyHostToDevice, s));
    c->pending_geometry = true;
    c->geo_built = false;  // new face arrays
    drop_graphs(c);  // kernel parameters hold the face count and pointers
    CUDA_TRY(cudaStreamSynchronize(s));
    return MVMM_OK;
}

int mvmm_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(MVMM_E_INVALID, "null argument");
    *ptr = nullptr;
    if (bytes == 0) return MVMM_OK;
    cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(MVMM_E_NOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    return MVMM_OK;
}

int mvmm_host_free(void* ptr) {
    if (ptr) CUDA_TRY(cudaFreeHost(ptr));
    return MVMM_OK;
}

int mvmm_run(mvmm_ctx* c, int64_t max_steps, uint64_t* ti_current, uint64_t* ti_old, int64_t* steps_done,
             int64_t* n_active_faces, int* finished) {
    if (!c || !ti_current || !ti_old) return fail(MVMM_E_INVALID, "null argument");
    int rm = reject_moving(c);
    if (rm) return rm;
    int rc = c->n_inst == 1 ? mvmm_set_time(c, *ti_current, *ti_old) : read_tl(c);
    if (rc) return rc;
    unsigned long long s0 = c->tl_host->steps, f0 = sum_field(c, &DevTimeline::active_faces);
    const int64_t chunk = 64;
    int64_t launched = 0;
    int numeric = MVMM_OK;
    for (;;) {
        int64_t k = chunk;
        if (max_steps > 0 && launched + k > max_steps) k = max_steps - launched;
        if (k <= 0) break;
        rc = enqueue_steps_impl(c, k);
        if (rc) return rc;
        launched += k;
        rc = finish(c);
        // a batch runs on when one simulation fails (it stops, see k_end);
        // the failure is returned at the end, per-simulation bits in mvmm_batch_state
        if (rc == MVMM_E_NUMERIC && c->n_inst > 1) {
            numeric = rc;
            rc = MVMM_OK;
        }
        if (rc) break;
        if (all_done(c)) break;
    }
    if (!rc && numeric) rc = fail(numeric, "numerical failure in at least one simulation of the batch");
    int rc2 = read_tl(c);
    if (rc2) return rc2;
    *ti_current = c->tl_host->ti_current;
    *ti_old = c->tl_host->ti_old;
    if (steps_done) *steps_done = (int64_t)(c->tl_host->steps - s0);
    if (n_active_faces) *n_active_faces = (int64_t)(sum_field(c, &DevTimeline::active_faces) - f0);
    if (finished) *finished = all_done(c) ? 1 : 0;
    return rc;
}

// Chooses the thread-block sizes of the face kernel and of the cell kernels by
// timing steps of this context's own workload, then puts the state back: the
// cell state, time bins and timelines are saved to a device copy first.
int mvmm_autotune(mvmm_ctx* c, int steps, int* blk_face, int* blk_cell) {
    if (!c || steps < 1) return fail(MVMM_E_INVALID, "bad arguments");
    int rc = read_tl(c);
    if (rc) return rc;
    size_t n = c->n;
    size_t bytes = (size_t)kCellFields * n * 8;
    double* save = nullptr;
    int8_t* save_tb = nullptr;
    CUDA_TRY(cudaMalloc((void**)&save, bytes));
    if (cudaMalloc((void**)&save_tb, n) != cudaSuccess) {
        cudaFree(save);
        return fail(MVMM_E_NOMEM, "cudaMalloc failed");
    }
    std::vector<DevTimeline> tl0(c->tl_host, c->tl_host + c->n_inst);
    sync_extrap(c, false, c->stream);
    cudaMemcpyAsync(save, c->cd, bytes, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(save_tb, c->timebin, n, cudaMemcpyDeviceToDevice, c->stream);
    const int cand[3] = {64, 128, 256};
    float best = 1e30f;
    int bf = c->blk_face, bc = c->blk_cell;
    bool prof = c->prof;
    c->prof = false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            c->blk_face = cand[i];
            c->blk_cell = cand[j];
            drop_graphs(c);
            // restore, warm once, time `steps` steps
            cudaMemcpyAsync(c->cd, save, bytes, cudaMemcpyDeviceToDevice, c->stream);
            cudaMemcpyAsync(c->timebin, save_tb, n, cudaMemcpyDeviceToDevice, c->stream);
            mark_stale(c, c->stream);
            // the restored step counter repeats: clear the face stamps it keys
            cudaMemsetAsync(c->face_stamp, 0, (size_t)(c->nf > 0 ? c->nf : 1) * 4, c->stream);
            std::copy(tl0.begin(), tl0.end(), c->tl_host);
            write_tl(c);
            sync_extrap(c, true, c->stream);
            rc = enqueue_steps_impl(c, 1);
            if (rc) break;
            cudaEventRecord(e0, c->stream);
            rc = enqueue_steps_impl(c, steps);
            if (rc) break;
            cudaEventRecord(e1, c->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                bf = cand[i];
                bc = cand[j];
            }
        }
    c->blk_face = bf;
    c->blk_cell = bc;
    drop_graphs(c);
    cudaMemcpyAsync(c->cd, save, bytes, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->timebin, save_tb, n, cudaMemcpyDeviceToDevice, c->stream);
    mark_stale(c, c->stream);
    cudaMemsetAsync(c->face_stamp, 0, (size_t)(c->nf > 0 ? c->nf : 1) * 4, c->stream);
    std::copy(tl0.begin(), tl0.end(), c->tl_host);
    write_tl(c);
    sync_extrap(c, true, c->stream);
    cudaStreamSynchronize(c->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(save);
    cudaFree(save_tb);
    c->prof = prof;
    if (rc) return rc;
    if (blk_face) *blk_face = bf;
    if (blk_cell) *blk_cell = bc;
    return MVMM_OK;
}

int mvmm_profile_enable(mvmm_ctx* c, int enable) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    c->prof = enable != 0;
    for (int j = 0; j < MVMM_NUM_KERNELS; j++) {
        c->prof_ms[j] = 0;
        c->prof_n[j] = 0;
    }
    return MVMM_OK;
}

int mvmm_profile_read(mvmm_ctx* c, double* ms, int64_t* launches) {
    if (!c) return fail(MVMM_E_INVALID, "null context");
    for (int j = 0; j < MVMM_NUM_KERNELS; j++) {
        if (ms) ms[j] = c->prof_ms[j];
        if (launches) launches[j] = c->prof_n[j];
    }
    return MVMM_OK;
}

// ---- Riemann over arrays ----------------------------------------------
static int riemann_common(int kind, int precision, int sample, double gamma, int64_t n, const double* l,
                          const double* r, const double* vf, const double* nrm, double* out, const RSx& x) {
    int rs = check_solver(kind, x.airs_threshold, x.adv);
    if (rs) return rs;
    if (precision < 0 || precision > 1) return fail(MVMM_E_INVALID, "unknown precision");
    if (!(gamma > 1.0)) return fail(MVMM_E_INVALID, "gamma must be > 1");
    if (n < 0 || (n > 0 && (!l || !r || !nrm || !out || (!sample && !vf)))) return fail(MVMM_E_INVALID, "bad arrays");
    if (n == 0) return MVMM_OK;
    double* d = nullptr;
    unsigned int* derr = nullptr;
    size_t tot = (size_t)n * (5 + 5 + 3 + 3 + 5);
    CUDA_TRY(cudaMalloc((void**)&d, tot * 8));
    if (cudaMalloc((void**)&derr, 4) != cudaSuccess) {
        cudaFree(d);
        return fail(MVMM_E_NOMEM, "cudaMalloc failed");
    }
    double *dl = d, *dr = d + 5 * n, *dv = d + 10 * n, *dn = d + 13 * n, *dout = d + 16 * n;
    cudaMemcpy(dl, l, (size_t)n * 5 * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dr, r, (size_t)n * 5 * 8, cudaMemcpyHostToDevice);
    if (!sample) cudaMemcpy(dv, vf, (size_t)n * 3 * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dn, nrm, (size_t)n * 3 * 8, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, 4);
    if (precision == MVMM_PRECISION_FP32FACE)
        launch_riemann_fp32(kind, sample, gamma, n, dl, dr, dv, dn, dout, derr, x, 0);
    else
        launch_riemann_fp64(kind, sample, gamma, n, dl, dr, dv, dn, dout, derr, x, 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 5 * 8, cudaMemcpyDeviceToHost);
    unsigned int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaFree(derr);
    if (e != cudaSuccess) return fail(MVMM_E_CUDA, cudaGetErrorString(e));
    if (herr) return fail(MVMM_E_NUMERIC, "Riemann solver reported a numerical failure");
    return MVMM_OK;
}

// The kind-only forms carry no AIRS threshold or advection velocity.
static RSx no_settings(int kind) {
    RSx x;
    x.kind = kind;
    x.airs_threshold = NAN;
    x.adv[0] = x.adv[1] = x.adv[2] = NAN;
    return x;
}

int mvmm_riemann_flux(int kind, int precision, double gamma, int64_t n, const double* left, const double* right,
                      const double* v_face, const double* normal, double* out) {
    return riemann_common(kind, precision, 0, gamma, n, left, right, v_face, normal, out, no_settings(kind));
}

int mvmm_riemann_sample(int kind, int precision, double gamma, int64_t n, const double* left, const double* right,
                        const double* normal, double* out) {
    return riemann_common(kind, precision, 1, gamma, n, left, right, nullptr, normal, out, no_settings(kind));
}

int mvmm_riemann_flux_p(const mvmm_params* p, int64_t n, const double* left, const double* right,
                        const double* v_face, const double* normal, double* out) {
    if (!p) return fail(MVMM_E_INVALID, "null params");
    return riemann_common(p->riemann, p->precision, 0, p->gamma, n, left, right, v_face, normal, out,
                          solver_settings(*p));
}

int mvmm_riemann_sample_p(const mvmm_params* p, int64_t n, const double* left, const double* right,
                          const double* normal, double* out) {
    if (!p) return fail(MVMM_E_INVALID, "null params");
    return riemann_common(p->riemann, p->precision, 1, p->gamma, n, left, right, nullptr, normal, out,
                          solver_settings(*p));
}

}  // extern "C"
