// Plain FP64 form of the OptimalOrderRunner step (runner/hydrodynamics/optimal_order.rs:15-64).
//
// Compiled with -fmad=false: every expression is rounded exactly as the Rust
// reference evaluates it.  One CUDA thread per face for the flux stage, one per
// cell for the cell stages; the flux scatter is a deterministic CSR gather in
// the reference's face order (no atomics on floating-point data).
#include "cmp64.cuh"
#include "face64.cuh"
#include "mvmm_cellops.cuh"

namespace mvmm {

namespace {

// Particle::time_extrapolations body before the -dt factor (part.rs:134-149).
__device__ __forceinline__ St<double> extrap_source(const KP& p, int i, const St<double>& prim, double rho_inv) {
    V3<double> vr = C3(p, F_VREL, i);
    V3<double> g0 = C3(p, F_GRAD + 0, i);
    V3<double> g4 = C3(p, F_GRAD + 12, i);
    double div_v = C(p, F_GRAD + 3, i) + C(p, F_GRAD + 7, i) + C(p, F_GRAD + 11, i);
    St<double> s;
    s.q[0] = prim.q[0] * div_v + dot(vr, g0);
    s.q[1] = vr.x * div_v + rho_inv * g4.x;
    s.q[2] = vr.y * div_v + rho_inv * g4.y;
    s.q[3] = vr.z * div_v + rho_inv * g4.z;
    s.q[4] = p.gamma * prim.q[4] * div_v + dot(vr, g4);
    return s;
}

// Face-stage derived fields: extrapolation source and v_max sound speed.
__device__ __forceinline__ void write_derived(const KP& p, int i, const St<double>& prim, const St<double>& src,
                                              double rho_inv) {
    if (gt0_64(prim.q[0])) {
        W5(p, F_SRC, i, src);
        W(p, F_CS, i, gas(p).sound_speed(prim.q[4], rho_inv));
    } else {
        W5(p, F_SRC, i, st_zero<double>());
        W(p, F_CS, i, 0.);
    }
}

// ------------------------------------------------------------- predict --
// Hierarchical steps defer the extrapolation of inactive cells whose source
// row is current: the source, the density test and so each step's addition
// ex + (-dt) src are fixed until the cell changes, so they are made later, in
// step order, from the log of the steps' dt: for the cells a step reads (the
// cells next to its active faces), before a download, and every kDtLog / 2
// steps for all cells.  Brings cell i up to date before step `upto`.
// Consecutive steps of the same dt add the same rounded product, so it is
// formed once per run of equal dt; and an addition that leaves a component
// unchanged leaves it unchanged for the rest of that run (the same operation on
// the same bits), which ends the run early for that component: a cell whose
// source is zero (a uniform neighbourhood) catches up in one addition.
__device__ __forceinline__ void extrap_catch_up(const KP& p, int i, unsigned int upto) {
    const unsigned int from = p.extrap_step[i];
    if (from >= upto) return;
    St<double> ex = C5(p, F_EXTRAP, i);
    if (gt0_64(C(p, F_PRIM, i))) {
        const St<double> src = C5(p, F_SRC, i);
        unsigned int s = from;
        while (s < upto) {
            const double dt = p.dt_log[s % kDtLog];
            const long long dt_bits = __double_as_longlong(dt);
            unsigned int e = s + 1;
            while (e < upto && __double_as_longlong(p.dt_log[e % kDtLog]) == dt_bits) e++;
            const St<double> t = (-dt) * src;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                double x = ex.q[q];
                for (unsigned int k = s; k < e; k++) {
                    const double y = x + t.q[q];
                    if (__double_as_longlong(y) == __double_as_longlong(x)) break;
                    x = y;
                }
                ex.q[q] = x;
            }
            s = e;
        }
    } else {
        ex = ex + st_zero<double>();  // adding zero twice gives the bits of adding it once
    }
    if (p.dirty) {  // only a change of bits makes the host's copy stale
        bool changed = false;
#pragma unroll
        for (int q = 0; q < 5; q++)
            changed = changed || __double_as_longlong(ex.q[q]) != __double_as_longlong(C(p, F_EXTRAP + q, i));
        if (changed) p.dirty[i] |= kDirtyExtrap;
    }
    W5(p, F_EXTRAP, i, ex);
    p.extrap_step[i] = upto;
}

// EulerEqnsFvs::predict -> Particle::extrapolate_state (part.rs:123-132),
// plus the active mask bin_is_ending (engine.rs:63-65) in step mode.
__global__ void __launch_bounds__(kMaxBlock) k_predict(KP p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = false;
    int k = i < p.n ? inst_of(p, i) : -1;
    if (k >= 0 && p.tl[k].done) k = -1;  // a finished simulation of a batch is left untouched
    if (k >= 0) {
        unsigned long long tc = 0, to = 0;
        if (!p.stage) {
            tc = p.tl[k].ti_current;
            to = p.tl[k].ti_old;
            act = p.timebin[i] <= max_active_bin_bits(tc);
            p.active[i] = act;
        }
        // TimestepInfo::dt_from_dti; formed only where it is used, as the FP64
        // conversion and product cost every cell a hierarchical step defers
        auto step_dt = [&]() { return p.stage ? p.stage_dt : (double)(tc - to) * tbase(p, k); };
        // hierarchical steps: this step's number, for the deferred extrapolations
        const bool lazy = p.extrap_step != nullptr && !p.stage;
        const unsigned int s = lazy ? (unsigned int)p.tl[k].steps : 0u;
        if (lazy && i == 0) p.dt_log[s % kDtLog] = step_dt();
        const bool fresh = !p.stage && !p.stale_all && p.fresh[i];
        if (lazy && fresh && !act && s % (kDtLog / 2) != 0) {
            // deferred (extrap_catch_up)
        } else if (fresh) {
            const double dt = step_dt();
            // prim, grad and v_rel are unchanged since this cell's source row was
            // written (it was not active, nothing was uploaded): the same bits
            if (lazy) extrap_catch_up(p, i, s);
            St<double> ex = C5(p, F_EXTRAP, i);
            if (gt0_64(C(p, F_PRIM, i))) W5(p, F_EXTRAP, i, ex + (-dt) * C5(p, F_SRC, i));
            else W5(p, F_EXTRAP, i, ex + st_zero<double>());
            if (lazy) p.extrap_step[i] = s + 1;
            mark_dirty(p, i, kDirtyExtrap);
        } else {
            const double dt = step_dt();
            if (lazy) extrap_catch_up(p, i, s);
            mark_dirty(p, i, kDirtyExtrap);
            St<double> prim = C5(p, F_PRIM, i);
            double rho_inv = 1. / prim.q[0];
            St<double> src = extrap_source(p, i, prim, rho_inv);
            if (gt0_64(prim.q[0])) {
                St<double> ex = C5(p, F_EXTRAP, i);
                W5(p, F_EXTRAP, i, ex + (-dt) * src);
            } else {
                St<double> ex = C5(p, F_EXTRAP, i);
                W5(p, F_EXTRAP, i, ex + st_zero<double>());
            }
            // check_physical (physical_quantities.rs:245-254) zeroes the state
            // where density or pressure is negative; compared bitwise, so that
            // a NaN component also counts as reset, as the float comparison did
            St<double> chk = prim;
            if (lt0_64(prim.q[0]) || lt0_64(prim.q[4])) chk = st_zero<double>();
            bool reset = false;
#pragma unroll
            for (int q = 0; q < 5; q++)
                reset = reset || __double_as_longlong(chk.q[q]) != __double_as_longlong(prim.q[q]) ||
                        is_nan64(prim.q[q]);
            if (reset) {
                W5(p, F_PRIM, i, chk);
                mark_dirty(p, i);
            }
            // volume: dvdt is zero for a fixed mesh, so volume.clamp(..) leaves it unchanged
            write_derived(p, i, chk, src, rho_inv);
            // a reset prim no longer matches the source row (computed from the old one)
            if (!p.stage) p.fresh[i] = !reset;
            if (lazy) p.extrap_step[i] = s + 1;
        }
    }
    // active cells: counted per warp, or in a hierarchical step as the length
    // of the list's active head (added by k_end)
    if (p.use_list) list_cell_warp(p, act, i, true);
    else if (!p.stage) inst_count(p, k, act, CNT_CELLS);
}

// Recomputes the derived face-stage fields (per-stage flux calls).
__global__ void __launch_bounds__(kMaxBlock) k_derive(KP p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    St<double> prim = C5(p, F_PRIM, i);
    double rho_inv = 1. / prim.q[0];
    St<double> src = extrap_source(p, i, prim, rho_inv);
    write_derived(p, i, prim, src, rho_inv);
}

// ------------------------------------------------------------ face flux --
// The face physics (face64.cuh) reads the context's cell block: the derived
// rows predict wrote (time-extrapolation source, sound speed) included.
struct AccKP {
    const KP& p;
    __device__ __forceinline__ St<double> prim(int i) const { return C5(p, F_PRIM, i); }
    __device__ __forceinline__ V3<double> gc(int i) const { return C3(p, F_GC, i); }
    __device__ __forceinline__ V3<double> cen(int i) const { return C3(p, F_CEN, i); }
    __device__ __forceinline__ V3<double> loc(int i) const { return C3(p, F_LOC, i); }
    __device__ __forceinline__ V3<double> v(int i) const { return C3(p, F_V, i); }
    __device__ __forceinline__ double dt(int i) const { return C(p, F_DT, i); }
    __device__ __forceinline__ double cs(int i) const { return C(p, F_CS, i); }
    __device__ __forceinline__ double gdot(int i, int q, V3<double> dx) const { return mvmm::gdot(p, i, q, dx); }
    __device__ __forceinline__ double extrap(int i, int q) const { return C(p, F_EXTRAP + q, i); }
    __device__ __forceinline__ St<double> src(int i, const St<double>&) const { return C5(p, F_SRC, i); }
    __device__ __forceinline__ V3<double> fcen(int f) const { return F3(p.fcen, p.nf, f); }
    __device__ __forceinline__ V3<double> shift(int f) const { return F3(p.shift, p.nf, f); }
    __device__ __forceinline__ V3<double> normal(int f) const { return F3(p.normal, p.nf, f); }
    __device__ __forceinline__ double area(int f) const { return p.area[f]; }
    __device__ __forceinline__ int boundary() const { return p.boundary; }
};

// The face rows of a result: 5 fluxes and v_max, a_over_r (step), or the
// FluxInfo rows with mflux (per-stage calls).
__device__ __forceinline__ void write_face(const KP& p, int f, const FaceOut& o) {
    double* out = p.flux;
    size_t nf = (size_t)p.nf;
#pragma unroll
    for (int q = 0; q < 5; q++) out[q * nf + f] = o.fl.q[q];
    if (p.flux_rows == 10) {
        out[5 * nf + f] = o.mflux.x;
        out[6 * nf + f] = o.mflux.y;
        out[7 * nf + f] = o.mflux.z;
        out[8 * nf + f] = o.v_max;
        out[9 * nf + f] = o.a_over_r;
    } else {
        out[5 * nf + f] = o.v_max;
        out[6 * nf + f] = o.a_over_r;
    }
}

// The exact solver's searches and the rest of its faces leave the face kernel
// for kernels of their own.  Warps of the face kernel would run each with only
// the lanes whose guess took that path, holding the FP64 pipe for all 32;
// queued, they run with full warps.  A job holds the face's Riemann problem
// after the guess and what the face's result needs; p_guess becomes the star
// pressure once the search has run.
struct BrentJob {
    FacePre q;
    double vl, vr, al, ar, p_guess, fp_guess, fp0;  // fp0 = f(0)
    int f, k;
};
// The exact solver's flux from the star pressure on (riemann_solver.rs:258-284,
// exact.rs:214-238), as star_half_state + flux_from_half_state do.
// The two sides of sample_star are written once, for the side x/t = 0 falls
// on: that side's state, velocity and signed sound speed are selected, and its
// comparisons carry the side's sign, so the lanes of a warp run one code path
// whichever side each samples.  Every comparison and value is the one
// sample_star forms on that side, and only that side's middle density
// (star_state_from_pstar forms both; sample_star reads one) is formed.
__device__ __forceinline__ St<double> exact_flux_from_p(double pst, const FacePre& q, double vl, double vr, double al,
                                                        double ar, const Gas<double>& g) {
    const ExSide L = ex_side(q.l.q[0], q.l.q[4], al, g), R = ex_side(q.r.q[0], q.r.q[4], ar, g);
    // star_state_from_pstar's u, its two terms in ex_f's branch-coherent order
    const bool lo_left = L.p <= R.p;
    const double t_lo = ex_fb(pst, lo_left ? L : R, g);
    const double t_hi = ex_fb(pst, lo_left ? R : L, g);
    const double u = 0.5 * (vl + vr) + 0.5 * ((lo_left ? t_hi : t_lo) - (lo_left ? t_lo : t_hi));
    // sample_star (riemann_solver.rs:224-255): u < 0 samples the right side
    const bool right = u < 0.;
    const St<double> s = right ? q.r : q.l;
    const ExSide S = right ? R : L;
    const double v = right ? vr : vl;
    const double a = right ? -ar : al;  // the sampler's signed sound speed
    const double sg = right ? -1. : 1.;
    St<double> w;
    if (pst > s.q[4]) {  // shock
        const double sp = shock_speed(v, a, pst / s.q[4], g);
        w = sg * sp < 0. ? sample_middle(ex_middle_density(pst, S, g), u, pst, s, v, q.n) : s;
    } else if (sg * (v - a) < 0.) {  // rarefaction whose head lies on the other side of x/t = 0
        if (sg * rarefaction_tail_speed(u, a, pst / s.q[4], g) > 0.) w = sample_rarefaction_fan(s, a, v, q.n, g);
        else w = sample_middle(ex_middle_density(pst, S, g), u, pst, s, v, q.n);
    } else {
        w = s;
    }
    return flux_from_half_state(w, q.iv, q.n, g);
}

// EulerEqnsFvs::compute_fluxes (euler_eqns_fvs.rs:26-48): the active-face rule,
// dt = min(dt_l, dt_r), interior / boundary dispatch.
// QUEUE (the exact solver with its job queues): every face's solve is queued.
// (Register budgets of 128 and 168 for more resident warps measured slower
// than the compiler's own 170.)
template <int SOLVER, bool QUEUE = false>
__global__ void __launch_bounds__(kMaxBlock) k_face_flux(KP p) {
    if (p.use_list && p.tl[0].done) return;
    const Gas<double> g = gas(p);
    // all faces (one per thread), or the compacted active-face list (grid-stride)
    const int n_items = p.use_list ? (int)p.tl[0].n_list : p.nf;
    for (int base = blockIdx.x * blockDim.x; base < n_items; base += gridDim.x * blockDim.x) {
        int idx = base + threadIdx.x;
        int f = idx < n_items ? (p.use_list ? p.face_list[idx] : idx) : -1;
        int k = f >= 0 ? inst_of(p, p.left[f]) : -1;
        if (k >= 0 && p.tl[k].done) k = -1;
        bool counted = false;
        unsigned int err = 0;
        if (k >= 0) {
            int l = p.left[f], r = p.right[f];
            bool la = p.active[l] != 0;
            FacePre q;
            if (r >= 0) {
                bool ra = p.active[r] != 0;
                double dtl = C(p, F_DT, l), dtr = C(p, F_DT, r);
                if (interior_face_active(la, ra, dtl, dtr)) {
                    q = face_interior_pre(AccKP{p}, f, l, r, m_min(dtl, dtr));
                    counted = true;
                }
            } else if (la) {
                q = face_boundary_pre(AccKP{p}, f, l);
                counted = true;
            }
            FaceOut o;
            bool queued = false;
            if (!counted) {
                o = face_zero();
            } else if constexpr (QUEUE) {
                // star_half_state (riemann_solver.rs:258-284) with the exact
                // star solver: its Newton and Brent stages are queued, each for
                // a kernel of its own that finishes the face
                double vl = dot(vel(q.l), q.n);
                double vr = dot(vel(q.r), q.n);
                double al = g.sound_speed(q.l.q[4], 1. / q.l.q[0]);
                double ar = g.sound_speed(q.r.q[4], 1. / q.r.q[0]);
                double vrml = vr - vl;
                St<double> F;
                if (is_vacuum(q.l, q.r, al, ar, vrml, g)) {
                    F = flux_from_half_state(vacuum_sample(q.l, q.r, vl, vr, al, ar, q.n, g), q.iv, q.n, g);
                } else {
                    const ExSide L = ex_side(q.l.q[0], q.l.q[4], al, g), R = ex_side(q.r.q[0], q.r.q[4], ar, g);
                    double pg, fpg, fp0;
                    const int next = ex_star_start(L, R, vl, vr, g, &pg, &fpg, &fp0);
                    // queue 0: Brent searches; 1: Newton searches; 2: the guess is the pressure.
                    // Each queue holds a job per face (brent_cap >= nf): none overflows.
                    const int qi = next == EX_BRENT ? 0 : next == EX_NEWTON ? 1 : 2;
                    const unsigned int slot = atomicAdd(p.brent_count + qi, 1u);
                    BrentJob& J = reinterpret_cast<BrentJob*>(p.brent_jobs)[(size_t)qi * p.brent_cap + slot];
                    J.q = q;
                    J.vl = vl;
                    J.vr = vr;
                    J.al = al;
                    J.ar = ar;
                    J.p_guess = pg;
                    J.fp_guess = fpg;
                    J.fp0 = fp0;
                    J.f = f;
                    J.k = k;
                    queued = true;
                }
                if (!queued) o = face_finish(q, F);
            } else {
                o = face_finish(q, solve_for_flux<double, SOLVER>(q.l, q.r, q.iv, q.n, g, g, p.max_iter, &err, &p.rsx));
            }
            if (!queued) write_face(p, f, o);
            if (err) set_err(p, k, err);
        }
        if (!p.use_list) inst_count(p, k, counted, CNT_FACES);  // list mode counts the list in k_end
    }
}

// The queued jobs run a tile of kJobTile jobs per block at a time, the tile
// ordered by the branches the job's pressure (the guess in a search, the star
// pressure when the face is finished) takes: for each side whether it lies
// above the side's pressure (the shock branch of fb, fprimeb and the middle
// density, else the rarefaction branch with its power).  On the nearly uniform
// states of a smooth flow the guess, the star pressure and both side pressures
// differ in their last digits only, so which branches a face takes is close to
// random, and a warp of unsorted faces would run both branches of every
// evaluation.  A tile sorted by that key (a counting sort in shared memory)
// fills most warps with faces that take the same branches; each face's
// arithmetic is unchanged.
constexpr int kJobTile = 128;
// The branches of fb at the job's pressure (0: below both side pressures, 1:
// between them, 2: above both); between them, the sampler's side decides
// whether it meets the shock or the rarefaction, so key 1 splits by the side
// x/t = 0 is likely to fall on (u* ~ (v_l + v_r) / 2) against which side
// has the lower pressure: keys 0..3.
__device__ __forceinline__ int job_branch_key(const BrentJob& J) {
    const double pl = J.q.l.q[4], pr = J.q.r.q[4];
    const double lo = fmin(pl, pr), hi = fmax(pl, pr);
    const int pat = (J.p_guess > lo ? 1 : 0) + (J.p_guess > hi ? 1 : 0);
    if (pat != 1) return pat == 0 ? 0 : 3;
    return ((pl <= pr) != (J.vl + J.vr < 0.)) ? 1 : 2;
}
constexpr int kJobKeys = 4;
// The index of the job this thread runs in the tile starting at base (or -1);
// job(t) is job t of the n_jobs the kernel runs.
template <class Job>
__device__ __forceinline__ int sorted_job(const Job& job, unsigned int base, unsigned int n_jobs, int* s_count,
                                          int* s_order) {
    const unsigned int j = base + threadIdx.x;
    const int key = j < n_jobs ? job_branch_key(job(j)) : kJobKeys;
    if (threadIdx.x <= kJobKeys) s_count[threadIdx.x] = 0;
    __syncthreads();
    const int rank = atomicAdd(&s_count[key], 1);
    __syncthreads();
    int start = 0;
    for (int k = 0; k < key; k++) start += s_count[k];
    s_order[start + rank] = key < kJobKeys ? (int)j : -1;
    __syncthreads();
    const int mine = s_order[threadIdx.x];
    __syncthreads();  // the arrays are reused by the next tile
    return mine;
}
__device__ __forceinline__ BrentJob* queue_jobs(const KP& p, int qi) {
    return reinterpret_cast<BrentJob*>(p.brent_jobs) + (size_t)qi * p.brent_cap;
}
__device__ __forceinline__ unsigned int queue_count(const KP& p, int qi) {
    return min(p.brent_count[qi], (unsigned int)p.brent_cap);
}

// Both search queues in one pool: Newton jobs first, then Brent jobs.
// Searches end after different numbers of evaluations, so a warp that ran one
// search per lane would hold the FP64 pipe for all 32 lanes until its longest
// search ended.  Here a lane runs its search one evaluation of f at a time
// (NewtonMachine, then BrentMachine on [0, p] where the Newton loop ends above
// the root; or BrentMachine alone, from the guess and f(0) the face kernel
// formed) and, when it ends, takes the next job (a warp-aggregated fetch from a
// counter), so the warps stay full until both queues run dry.  Each job's star
// pressure goes back into its p_guess for k_face_finish.
struct SearchLane {
    int j = -1;        // job (index into the combined queue), or -1
    int k = 0;         // its simulation
    bool newton = false;
    unsigned int err = 0;
    ExSide L, R;
    double vl = 0., vr = 0., fp0 = 0.;
    NewtonMachine nm;
    BrentMachine bm;
};
__device__ __forceinline__ bool search_lane_done(const SearchLane& s) { return s.newton ? s.nm.done : s.bm.done; }
// Newton done: Brent follows where its loop ended above the root
__device__ __forceinline__ void search_after_newton(SearchLane& s, int max_iter) {
    s.err |= s.nm.err;
    if (s.nm.brent) {
        s.newton = false;
        s.bm.start(0., s.nm.pg, s.fp0, s.nm.fpg, 1e-6, max_iter);  // Brent on [0, p], f(0) as formed
    }
}
__device__ __forceinline__ double search_result(SearchLane& s) {
    if (s.newton) return s.nm.pg;
    s.err |= s.bm.err;
    return s.bm.b;
}
// The searches' evaluations of f are regrouped across the block: the lanes of
// a warp holding different jobs would take different branches of fb (shock or
// rarefaction on each side, depending on where x lies against the two side
// pressures) and run both.  Each round every lane with a search posts its x and
// its job's sides in shared memory, the block sorts the posts by that branch
// pattern (a counting sort), each thread evaluates ex_f for the post at its
// place, and the owner reads its value back: the same function on the same
// data, so the same bits, with most warps on one pattern.
constexpr int kSearchBlock = 256;
struct EvalPost {
    double x, vl, vr;
    ExSide L, R;
};
// (Only the grouping depends on it, so it compares bit patterns on the integer
// pipe, which order non-negative doubles as their values.)
__device__ __forceinline__ int ex_f_key(double x, const ExSide& L, const ExSide& R) {
    const long long a = __double_as_longlong(L.p), b = __double_as_longlong(R.p), k = __double_as_longlong(x);
    return (k > min(a, b) ? 1 : 0) + (k > max(a, b) ? 1 : 0);
}
// The index of the post this thread evaluates (key 3: no post), posts sorted by key.
__device__ __forceinline__ int block_sorted(int key, int* s_count, int* s_order) {
    if (threadIdx.x < 4) s_count[threadIdx.x] = 0;
    __syncthreads();
    const int rank = atomicAdd(&s_count[key], 1);
    __syncthreads();
    int start = 0;
    for (int k = 0; k < key; k++) start += s_count[k];
    s_order[start + rank] = key < 3 ? (int)threadIdx.x : -1;
    __syncthreads();
    return s_order[threadIdx.x];
}
// Four resident blocks per SM (64 registers, some spilled): the FP64 pipe's
// latency is hidden better than with two (126 registers) or three (80):
// 0.898, 0.865 and 0.843 ms for the face stage at 256^2.
__global__ void __launch_bounds__(kSearchBlock, 4) k_face_search(KP p) {
    __shared__ EvalPost s_post[kSearchBlock];
    __shared__ double s_res[kSearchBlock];
    __shared__ int s_count[4], s_order[kSearchBlock];
    const Gas<double> g = gas(p);
    const unsigned int n1 = queue_count(p, 1), n0 = queue_count(p, 0);
    const unsigned int n_jobs = n1 + n0;
    BrentJob* newton_jobs = queue_jobs(p, 1);
    BrentJob* brent_jobs = queue_jobs(p, 0);
    unsigned int* next = p.brent_count + kExactQueues;  // jobs handed out
    const unsigned int lane = threadIdx.x & 31;
    auto job = [&](unsigned int t) -> BrentJob& { return t < n1 ? newton_jobs[t] : brent_jobs[t - n1]; };
    SearchLane s;
    bool dry = false;
    auto retire = [&]() {
        job((unsigned int)s.j).p_guess = search_result(s);
        if (s.err) set_err(p, s.k, s.err);
        s.j = -1;
    };
    while (true) {
        // lanes without a search take jobs until each holds one that needs f, or the queues are dry
        while (true) {
            const unsigned int need = __ballot_sync(0xffffffffu, s.j < 0 && !dry);
            if (!need) break;
            const int leader = __ffs(need) - 1;
            unsigned int base = 0;
            if ((int)lane == leader) base = atomicAdd(next, (unsigned int)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need & (1u << lane)) {
                const unsigned int t = base + (unsigned int)__popc(need & ((1u << lane) - 1u));
                if (t < n_jobs) {
                    const BrentJob& J = job(t);
                    s.j = (int)t;
                    s.k = J.k;
                    s.err = 0;
                    s.L = ex_side(J.q.l.q[0], J.q.l.q[4], J.al, g);
                    s.R = ex_side(J.q.r.q[0], J.q.r.q[4], J.ar, g);
                    s.vl = J.vl;
                    s.vr = J.vr;
                    s.fp0 = J.fp0;
                    s.newton = t < n1;
                    if (s.newton) {
                        s.nm.start(J.p_guess, J.fp_guess, p.max_iter, s.L, s.R, g);
                        if (s.nm.done) search_after_newton(s, p.max_iter);
                    } else {
                        s.bm.start(0., J.p_guess, J.fp0, J.fp_guess, 1e-6, p.max_iter);  // on [0, guess]
                    }
                    if (search_lane_done(s)) retire();
                } else {
                    dry = true;
                }
            }
        }
        const bool has = s.j >= 0;
        if (!__syncthreads_or(has)) break;  // block-uniform: every lane's search has ended, the queues are dry
        int key = 3;
        if (has) {
            const double x = s.newton ? s.nm.x : s.bm.x;
            s_post[threadIdx.x] = EvalPost{x, s.vl, s.vr, s.L, s.R};
            key = ex_f_key(x, s.L, s.R);
        }
        const int o = block_sorted(key, s_count, s_order);
        if (o >= 0) {
            const EvalPost e = s_post[o];
            s_res[o] = ex_f(e.x, e.L, e.R, e.vl, e.vr, g);
        }
        __syncthreads();
        if (has) {
            const double fx = s_res[threadIdx.x];
            if (s.newton) {
                s.nm.step(fx, s.L, s.R, g);
                if (s.nm.done) search_after_newton(s, p.max_iter);
            } else {
                s.bm.step(fx);
            }
            if (search_lane_done(s)) retire();
        }
    }
}

// Every queued face from its star pressure on (star state, sample, flux), the
// three queues one after another: apart from the searches, the faces of a warp
// run the same code, where in the face kernel only its lanes whose guess was the
// pressure would have run it.
__global__ void __launch_bounds__(kJobTile) k_face_finish(KP p) {
    __shared__ int s_count[kJobKeys + 1], s_order[kJobTile];
    const Gas<double> g = gas(p);
    const unsigned int n0 = queue_count(p, 0), n1 = queue_count(p, 1), n2 = queue_count(p, 2);
    const unsigned int n_jobs = n0 + n1 + n2;
    const BrentJob* jobs = queue_jobs(p, 0);
    const size_t cap = (size_t)p.brent_cap;
    auto job = [&](unsigned int t) -> const BrentJob& {
        return t < n0 ? jobs[t] : t < n0 + n1 ? jobs[cap + (t - n0)] : jobs[2 * cap + (t - n0 - n1)];
    };
    for (unsigned int base = blockIdx.x * kJobTile; base < n_jobs; base += gridDim.x * kJobTile) {
        const int t = sorted_job(job, base, n_jobs, s_count, s_order);
        if (t < 0) continue;
        const BrentJob J = job((unsigned int)t);
        write_face(p, J.f, face_finish(J.q, exact_flux_from_p(J.p_guess, J.q, J.vl, J.vr, J.al, J.ar, g)));
    }
}

// Per-time-bin active-face list (hierarchical steps): walks the faces of the
// active cells (the head of the cell list, written by predict), applies the
// active-face rule of compute_fluxes (euler_eqns_fvs.rs:35-45), stamps each
// active face once and appends it to the face list, and puts the other cell of
// every face of an active cell on the cell list (its update and wake-up).  The
// work is O(faces of active cells); list orders are arbitrary, and each face
// writes only its own result rows, so results do not depend on them.
__global__ void __launch_bounds__(kMaxBlock) k_compact(KP p) {
    if (p.tl[0].done) return;
    const int n_act = (int)p.tl[0].n_alist;
    const unsigned int stamp = face_stamp_now(p);
    const int lane = threadIdx.x & 31;
    // one warp per active cell, its lanes over the cell's faces: the face
    // gathers of a cell are issued together instead of one after another
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_act; w += n_warps) {
        const int i = p.cell_list[w];
        const int k0 = p.csr_off[i];
        const int deg = p.csr_off[i + 1] - k0;
        for (int j0 = 0; j0 < deg; j0 += 32) {  // warp-uniform
            int j = j0 + lane;
            bool have = j < deg;
            int f = have ? p.csr_face[k0 + j] : 0;
            int o = -1;
            bool act = false;
            if (have) {
                int l = p.left[f], r = p.right[f];
                o = l == i ? r : l;
                bool la = p.active[l] != 0;
                if (r >= 0) {
                    bool ra = p.active[r] != 0;
                    double dtl = C(p, F_DT, l), dtr = C(p, F_DT, r);
                    act = interior_face_active(la, ra, dtl, dtr);
                } else {
                    act = la;
                }
            }
            // a face between two active cells is reached twice: the stamp lists it once
            bool first = act && atomicExch(&p.face_stamp[f], stamp) != stamp;
            unsigned int b = __ballot_sync(0xffffffffu, first);
            if (b) {
                int leader = __ffs(b) - 1;
                unsigned int start = 0;
                if (lane == leader) start = atomicAdd(&p.tl[0].n_list, (unsigned int)__popc(b));
                start = __shfl_sync(0xffffffffu, start, leader);
                if (first) p.face_list[start + __popc(b & ((1u << lane) - 1u))] = f;
            }
            // a cell newly on the list is read by this step (its faces, its update):
            // its deferred extrapolation is made now, this step's included
            if (list_cell_warp(p, o >= 0, o >= 0 ? o : 0) && p.extrap_step)
                extrap_catch_up(p, o, (unsigned int)p.tl[0].steps + 1u);
        }
    }
}

// Every cell's deferred extrapolation made (before the state is read as a
// whole); reset: none is pending (the cells were uploaded).
__global__ void __launch_bounds__(kMaxBlock) k_extrap_flush(KP p, int reset) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const unsigned int now = (unsigned int)p.tl[0].steps;
    if (reset) p.extrap_step[i] = now;
    else extrap_catch_up(p, i, now);
}

// ---------------------------------------------------- cons -> primitive --
// Particle::convert_conserved_to_primitive (part.rs:219-261)
__device__ __forceinline__ void c2p(const KP& p, int i, const St<double>& cons, unsigned int* err) {
    W5(p, F_PRIM, i, c2p64(cons, C(p, F_VOL, i), gas(p), err));
}

// ---------------------------------------------------- scatter + update --
// FP32 face fluxes are accumulated at FP64 accuracy in Sum2 pairs (TwoSum),
// without a per-face FP64 conversion.

// apply_fluxes (runner/hydrodynamics.rs:13-39): CSR gather of every face of
// the cell in CSR order; active cells fold the accumulator into the conserved
// state (Particle::apply_flux, part.rs:178-193), then kick2 and cons->prim.
// ROWS32: the FP32-face form's step rows (FP32 dt * area * F, v_max,
// a_over_r), summed per cell in FP32 two-sums and added to the FP64
// accumulator once; otherwise the FP64 rows are folded in face order.
__device__ __forceinline__ void update_finish(const KP& p, int i, int k, bool act, St<double> facc, double msv,
                                              double maor, int do_c2p);
template <bool ROWS32>
__device__ __forceinline__ void update_cell(const KP& p, int i, int do_c2p) {
    const int k = inst_of(p, i);
    if (p.tl[k].done) return;
    bool act = p.active[i] != 0;
    St<double> facc = C5(p, F_FACC, i);
    double msv = C(p, F_MSV, i), maor = C(p, F_MAOR, i);
    if (p.snap_late) {  // the uploaded bytes of the rows this kernel rewrites, for the copy back's comparison
        const size_t n = (size_t)p.n;
#pragma unroll
        for (int q = 0; q < 5; q++) {
            p.snap_late[(F_CONS + q) * n + i] = C(p, F_CONS + q, i);
            p.snap_late[(F_FACC + q) * n + i] = facc.q[q];
        }
        p.snap_late[F_MSV * n + i] = msv;
        p.snap_late[F_MAOR * n + i] = maor;
    }
    const size_t nf = (size_t)p.nf;
    int k0 = p.csr_off[i], k1 = p.csr_off[i + 1];
    const unsigned int stamp = p.use_list ? face_stamp_now(p) : 0u;
    if (ROWS32) {
        const float* fl = p.flux32;
        Sum2 acc[5];
#pragma unroll
        for (int q = 0; q < 5; q++) acc[q] = {0.f, 0.f};
        float vm = -INFINITY, ar = -INFINITY;
        // faces in batches of 4: a batch's loads are in flight together, and the
        // batch is then added in CSR order (the same sums as one face at a time)
        for (int kb = k0; kb < k1; kb += 4) {
            int ff[4];
            bool use[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                use[j] = kb + j < k1;
                ff[j] = use[j] ? p.csr_face[kb + j] : 0;
            }
            float x[4][7], sg[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (use[j] && p.use_list) use[j] = p.face_stamp[ff[j]] == stamp;
                sg[j] = use[j] && p.left[ff[j]] == i ? -1.f : 1.f;  // update_fluxes_left / _right (part.rs:160-176)
#pragma unroll
                for (int q = 0; q < 7; q++) x[j][q] = use[j] ? fl[q * nf + ff[j]] : 0.f;
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (!use[j]) continue;
#pragma unroll
                for (int q = 0; q < 5; q++) sum2_add(acc[q], sg[j] * x[j][q]);
                vm = fmaxf(vm, x[j][5]);
                ar = fmaxf(ar, x[j][6]);
            }
        }
#pragma unroll
        for (int q = 0; q < 5; q++) facc.q[q] = facc.q[q] + (f64(acc[q].hi) + f64(acc[q].lo));
        if (act && k1 > k0) {
            msv = m_max(f64(vm), msv);
            maor = m_max(maor, f64(ar));
        }
    } else {
        const int rv = p.flux_rows == 10 ? 8 : 5;
        const double* fl = p.flux;
        for (int k = k0; k < k1; k++) {
            int f = p.csr_face[k];
            // an inactive face carries FluxInfo::zero(): adding it changes nothing
            if (p.use_list && p.face_stamp[f] != stamp) continue;
            St<double> x;
#pragma unroll
            for (int q = 0; q < 5; q++) x.q[q] = fl[q * nf + f];
            if (p.left[f] == i) facc = facc - x;  // update_fluxes_left (part.rs:160-167)
            else facc = facc + x;                 // update_fluxes_right (part.rs:169-176)
            if (act) {
                msv = m_max(fl[rv * nf + f], msv);
                maor = m_max(maor, fl[(rv + 1) * nf + f]);
            }
        }
    }
    update_finish(p, i, k, act, facc, msv, maor, do_c2p);
}

// cons->prim of an updated cell, with the FP32 copies the FP32-face form's
// gradient stage reads.
__device__ __forceinline__ void c2p_with_copies(const KP& p, int i, const St<double>& cons, unsigned int* err) {
    c2p(p, i, cons, err);
    if (p.fp32) {
#pragma unroll
        for (int q = 0; q < 5; q++) p.cf[(size_t)(G_PRIM + q) * p.n + i] = f32(C(p, F_PRIM + q, i));
    }
}
// Self-gravity accelerations need every cell's updated mass, so kick2 and
// cons->prim of the active cells move to k_self_gravity.
__device__ __forceinline__ bool self_gravity_kicks(const KP& p) { return p.grav == MVMM_GRAVITY_SELF && p.grav_acc; }

// Particle::apply_flux, kick2 and cons->prim of one cell once its faces are summed.
__device__ __forceinline__ void update_finish(const KP& p, int i, int k, bool act, St<double> facc, double msv,
                                              double maor, int do_c2p) {
    unsigned int err = 0;
    mark_dirty(p, i);  // the pending fluxes at least
    if (act) {
        p.fresh[i] = 0;  // prim (here), grad and v_rel (gradient stage) change
        St<double> cons = apply_flux64(C5(p, F_CONS, i), facc, &err);
        facc = st_zero<double>();
        W(p, F_MSV, i, msv);
        W(p, F_MAOR, i, maor);
        if (self_gravity_kicks(p)) {
            W5(p, F_CONS, i, cons);
        } else {
            // kick2 (runner/hydrodynamics.rs:51-57); accelerations only where the
            // external potential's are computed (at the runner's "TODO: gravity")
            cons = p.grav_acc ? grav_kick64(cons, C(p, F_DT, i), grav_acceleration(p, C3(p, F_LOC, i)))
                              : zero_kick64(cons);
            W5(p, F_CONS, i, cons);
            if (do_c2p) c2p_with_copies(p, i, cons, &err);
        }
    }
    W5(p, F_FACC, i, facc);
    if (err) set_err(p, k, err);
}
// Hierarchical steps: a warp per listed cell.  The lanes gather the cell's
// faces together, and every lane then folds them into the accumulator in CSR
// order from the lanes' registers, so the sum is the one update_cell forms.
template <bool ROWS32>
__device__ __forceinline__ void update_cell_warp(const KP& p, int i, int do_c2p, int lane) {
    const int k = inst_of(p, i);
    if (p.tl[k].done) return;
    const bool act = p.active[i] != 0;
    St<double> facc = C5(p, F_FACC, i);
    double msv = C(p, F_MSV, i), maor = C(p, F_MAOR, i);
    const size_t nf = (size_t)p.nf;
    const int k0 = p.csr_off[i], deg = p.csr_off[i + 1] - k0;
    const unsigned int stamp = face_stamp_now(p);
    const int rv = p.flux_rows == 10 ? 8 : 5;
    Sum2 acc[5];
#pragma unroll
    for (int q = 0; q < 5; q++) acc[q] = {0.f, 0.f};
    float vm32 = -INFINITY, ar32 = -INFINITY;
    for (int j0 = 0; j0 < deg; j0 += 32) {  // warp-uniform
        const int j = j0 + lane;
        int use = 0, lft = 0;
        double x[7];
#pragma unroll
        for (int q = 0; q < 7; q++) x[q] = 0.;
        if (j < deg) {
            int f = p.csr_face[k0 + j];
            use = p.face_stamp[f] == stamp;
            if (use) {
                lft = p.left[f] == i;
                if (ROWS32) {
#pragma unroll
                    for (int q = 0; q < 7; q++) x[q] = (double)p.flux32[q * nf + f];
                } else {
#pragma unroll
                    for (int q = 0; q < 5; q++) x[q] = p.flux[q * nf + f];
                    x[5] = p.flux[rv * nf + f];
                    x[6] = p.flux[(rv + 1) * nf + f];
                }
            }
        }
        const int n = min(32, deg - j0);
        for (int t = 0; t < n; t++) {
            if (!__shfl_sync(0xffffffffu, use, t)) continue;  // warp-uniform
            const bool lt = __shfl_sync(0xffffffffu, lft, t) != 0;
            St<double> y;
#pragma unroll
            for (int q = 0; q < 5; q++) y.q[q] = __shfl_sync(0xffffffffu, x[q], t);
            const double vm = __shfl_sync(0xffffffffu, x[5], t), ar = __shfl_sync(0xffffffffu, x[6], t);
            if (ROWS32) {
                const float sg = lt ? -1.f : 1.f;
#pragma unroll
                for (int q = 0; q < 5; q++) sum2_add(acc[q], sg * (float)y.q[q]);
                vm32 = fmaxf(vm32, (float)vm);
                ar32 = fmaxf(ar32, (float)ar);
            } else {
                // a lane per sum: lanes 0-4 the accumulator rows, 5 max_signal_velocity,
                // 6 max_a_over_r, each folded face by face as the reference does
                if (lane < 5) {
                    double yq = y.q[0], fq = facc.q[0];
#pragma unroll
                    for (int q = 1; q < 5; q++)
                        if (lane == q) {
                            yq = y.q[q];
                            fq = facc.q[q];
                        }
                    fq = lt ? fq - yq : fq + yq;  // update_fluxes_left / _right (part.rs:160-176)
#pragma unroll
                    for (int q = 0; q < 5; q++)
                        if (lane == q) facc.q[q] = fq;
                } else if (act && lane == 5) {
                    msv = m_max(vm, msv);
                } else if (act && lane == 6) {
                    maor = m_max(maor, ar);
                }
            }
        }
    }
    if (!ROWS32) {  // the sums to every lane
#pragma unroll
        for (int q = 0; q < 5; q++) facc.q[q] = __shfl_sync(0xffffffffu, facc.q[q], q);
        msv = __shfl_sync(0xffffffffu, msv, 5);
        maor = __shfl_sync(0xffffffffu, maor, 6);
    }
    if (ROWS32) {
#pragma unroll
        for (int q = 0; q < 5; q++) facc.q[q] = facc.q[q] + (f64(acc[q].hi) + f64(acc[q].lo));
        if (act && deg > 0) {
            msv = m_max(f64(vm32), msv);
            maor = m_max(maor, f64(ar32));
        }
    }
    if (lane == 0) update_finish(p, i, k, act, facc, msv, maor, do_c2p);
}

// LIST: hierarchical step, a warp per listed cell (a separate instantiation
// from the all-cells kernel, which keeps its own register budget)
template <bool ROWS32, bool LIST>
__global__ void __launch_bounds__(kMaxBlock) k_update(KP p, int do_c2p) {
    const int n_items = cell_items(p);
    if (LIST) {
        const int lane = threadIdx.x & 31, n_warps = (gridDim.x * blockDim.x) >> 5;
        for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_items; w += n_warps)
            update_cell_warp<ROWS32>(p, p.cell_list[w], do_c2p, lane);
    } else {
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_items; idx += gridDim.x * blockDim.x)
            update_cell<ROWS32>(p, cell_at(p, idx), do_c2p);
    }
}

__global__ void __launch_bounds__(kMaxBlock) k_c2p(KP p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n || !p.active[i]) return;
    unsigned int err = 0;
    c2p(p, i, C5(p, F_CONS, i), &err);
    if (err) set_err(p, inst_of(p, i), err);
}

// ------------------------------------------------------------ gradients --
// The cell-wise limiter's extrapolation from cell i to face f (sh: the face
// shift as seen from i, other_side).  The reference's offset is face centroid -
// centroid - sh (runner/hydrodynamics.rs:119); with limiter_frame set it is taken
// in flux_exchange's frame (flux.rs:33-35), where the face centroid is the left
// cell's: face centroid - centroid for the left cell, + sh (that is, - shift)
// for the right one.
__device__ __forceinline__ V3<double> limiter_offset(const KP& p, int i, int f, V3<double> cen, V3<double> sh) {
    const V3<double> d = F3(p.fcen, p.nf, f) - cen;
    if (!p.limiter_frame) return d - sh;
    return i == p.left[f] ? d : d + sh;
}

// LimiterData::limit_single_quantity (gradients.rs:85-91):
// min(1, d_max / e_max, d_min / e_min), or 1 where an extrapolation bound is 0.
// A ratio that is at least 1 cannot lower the minimum with 1, so its IEEE
// division is skipped where that follows from a comparison (e_max > 0 and
// d_max >= e_max; e_min < 0 and d_min <= e_min): in a smooth flow most cells are
// not limited and take neither division.  The value is the same, NaN ratios
// (which fmin passes over) included.
__device__ __forceinline__ double limit_factor(double d_max, double d_min, double e_max, double e_min) {
    if (is_zero64(e_max) || is_zero64(e_min)) return 1.;  // comparisons on the integer pipe (cmp64.cuh)
    const bool max_ge1 = gt0_64(e_max) && cmp64::ge(d_max, e_max);
    const bool min_ge1 = lt0_64(e_min) && cmp64::le(d_min, e_min);
    if (max_ge1 && min_ge1) return 1.;
    if (max_ge1) return m_min(1.0, d_min / e_min);
    if (min_ge1) return m_min(1.0, d_max / e_max);
    return m_min(1.0, m_min(d_max / e_max, d_min / e_min));
}

// gradient_estimate + gradient_limit + gradient_apply (runner/hydrodynamics.rs:67-143)
// fused per cell; in step mode also compute_timesteps + timesteps_apply
// (euler_eqns_fvs.rs:50-61, runner/hydrodynamics.rs:145-158) with block-level
// min reductions of the integer timestep and the new time bins.
// The place in the block's tile (0 .. blockDim - 1) of the item this thread
// takes, items sorted by key (0 .. kDegKeys - 1; kDegKeys: no item, -1 back),
// by a counting sort in shared memory.
constexpr int kDegKeys = 32;
__device__ __forceinline__ int tile_sorted(int key, int* s_count, int* s_order) {
    for (int k = threadIdx.x; k <= kDegKeys; k += blockDim.x) s_count[k] = 0;
    __syncthreads();
    const int rank = atomicAdd(&s_count[key], 1);
    __syncthreads();
    int start = 0;
    for (int k = 0; k < key; k++) start += s_count[k];
    s_order[start + rank] = key < kDegKeys ? (int)threadIdx.x : -1;
    __syncthreads();
    const int mine = s_order[threadIdx.x];
    __syncthreads();  // the arrays are reused by the next tile
    return mine;
}
__device__ __forceinline__ void gradients_cell(const KP& p, int i, int do_timestep) {
    unsigned long long my_dti = MAX_NR_TIMESTEPS;
    int my_tb = 127;
    unsigned int err = 0;
    int k = i >= 0 ? inst_of(p, i) : -1;
    if (k >= 0 && p.tl[k].done) k = -1;
    if (k >= 0) {
        int tb = p.timebin[i];
        if (p.active[i]) {
            mark_dirty(p, i);
          if (!p.godunov) {  // GodunovHydroRunner::step has no gradient stage (godunov.rs:14-58)
            V3<double> cen = C3(p, F_CEN, i);
            St<double> prim = C5(p, F_PRIM, i);
            // GradientData::init (gradients.rs:14-33).  The WLS matrix is
            // symmetric term by term (ds.x*ds.y == ds.y*ds.x exactly), so its
            // six distinct entries are accumulated once: a00 a01 a02 / a11 a12 / a22.
            double a00 = 0., a01 = 0., a02 = 0., a11 = 0., a12 = 0., a22 = 0.;
            if (p.dim == 1) { a11 = 1.; a22 = 1.; }
            else if (p.dim == 2) { a22 = 1.; }
            V3<double> gr[5];
#pragma unroll
            for (int q = 0; q < 5; q++) gr[q] = v3(0., 0., 0.);
            int k0 = p.csr_off[i], k1 = p.csr_off[i + 1];
            for (int k = k0; k < k1; k++) {
                int f = p.csr_face[k];
                St<double> op;
                V3<double> oc, sh;
                other_side(p, i, f, prim, cen, op, oc, sh);
                V3<double> ds = (oc + sh) - cen;
                double w = p.area[f] / len2(ds);
                // GradientData::collect (gradients.rs:35-41).  When ds.z is
                // exactly zero (2D meshes) the z terms add +-0 to entries that
                // are +0 (or 1), which leaves them unchanged, so they are skipped.
                bool z = !is_zero64(ds.z);
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    double wdq = w * (op.q[q] - prim.q[q]);
                    gr[q].x = gr[q].x + wdq * ds.x;
                    gr[q].y = gr[q].y + wdq * ds.y;
                    if (z) gr[q].z = gr[q].z + wdq * ds.z;
                }
                a00 = a00 + w * (ds.x * ds.x);
                a01 = a01 + w * (ds.x * ds.y);
                a11 = a11 + w * (ds.y * ds.y);
                if (z) {
                    a02 = a02 + w * (ds.x * ds.z);
                    a12 = a12 + w * (ds.y * ds.z);
                    a22 = a22 + w * (ds.z * ds.z);
                }
            }
            V3<double> m0 = v3(a00, a01, a02), m1 = v3(a01, a11, a12), m2 = v3(a02, a12, a22);
            // GradientData::finalize with glam DMat3::inverse (gradients.rs:43-55)
            V3<double> t0 = cross(m1, m2), t1 = cross(m2, m0), t2 = cross(m0, m1);
            double det = dot(m2, t2);
            double inv_det = 1.0 / det;
            V3<double> r0 = inv_det * t0, r1 = inv_det * t1, r2 = inv_det * t2;
            V3<double> c0 = v3(r0.x, r1.x, r2.x), c1 = v3(r0.y, r1.y, r2.y), c2 = v3(r0.z, r1.z, r2.z);
            bool finite = true;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                V3<double> x = gr[q];
                V3<double> res = x.x * c0;
                res = res + x.y * c1;
                res = res + x.z * c2;
                gr[q] = res;
                finite = finite && is_finite64(res.x) && is_finite64(res.y) && is_finite64(res.z);
            }
            if (!finite) {
#pragma unroll
                for (int q = 0; q < 5; q++) gr[q] = v3(0., 0., 0.);
            }
            // LimiterData (gradients.rs:58-103)
            St<double> mn = prim, mx = prim, emn, emx;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                emn.q[q] = INFINITY;
                emx.q[q] = -INFINITY;
            }
            for (int k = k0; k < k1; k++) {
                int f = p.csr_face[k];
                St<double> op;
                V3<double> oc, sh;
                other_side(p, i, f, prim, cen, op, oc, sh);
                V3<double> d = limiter_offset(p, i, f, cen, sh);
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    double ex = dot(gr[q], d);
                    mn.q[q] = m_min(mn.q[q], op.q[q]);
                    mx.q[q] = m_max(mx.q[q], op.q[q]);
                    emn.q[q] = m_min(emn.q[q], ex);
                    emx.q[q] = m_max(emx.q[q], ex);
                }
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
                double d_max = mx.q[q] - prim.q[q];
                double d_min = mn.q[q] - prim.q[q];
                const double alpha = limit_factor(d_max, d_min, emx.q[q], emn.q[q]);
                gr[q] = alpha * gr[q];
                W3(p, F_GRAD + 3 * q, i, gr[q]);
            }
            W3(p, F_GC, i, cen);  // gradient_apply
          }
            if (do_timestep) {
                double dt_new = limit_by_gravity(p, i, particle_timestep(p, i));
                unsigned long long tc = p.tl[k].ti_current;
                unsigned long long dti = make_integer_timestep(dt_new, tb, NUM_TIME_BINS, tc, tbase_inv(p, k));
                if (dti == 0) err |= 1u << 6;
                W(p, F_DT, i, (double)dti * tbase(p, k));  // Particle::set_timestep
                tb = get_time_bin(dti);
                my_dti = dti;
            }
        }
        if (do_timestep) {
            p.tb_tmp[i] = (int8_t)tb;
            my_tb = tb;
        }
    }
    if (err) set_err(p, k, err);
    if (!do_timestep) return;
    inst_min_dti_tb(p, k, my_dti, my_tb);
}
__device__ __forceinline__ double warp_min_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = m_min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = m_max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Hierarchical steps: a warp per listed cell.  The lanes gather the cell's
// faces together; the WLS sums are folded in CSR order from the lanes'
// registers (the sums gradients_cell forms, bit for bit), and the limiter's
// minima and maxima are warp reductions (fmin / fmax do not depend on order).
__device__ __forceinline__ void gradients_cell_warp(const KP& p, int i, int do_timestep, int lane) {
    unsigned long long my_dti = MAX_NR_TIMESTEPS;
    int my_tb = 127;
    unsigned int err = 0;
    int k = inst_of(p, i);
    if (p.tl[k].done) k = -1;
    if (k >= 0) {
        int tb = p.timebin[i];
        if (p.active[i]) {
            mark_dirty(p, i);
          if (!p.godunov) {
            V3<double> cen = C3(p, F_CEN, i);
            St<double> prim = C5(p, F_PRIM, i);
            // GradientData::collect in CSR order, a lane per accumulator: lanes
            // 0-14 the 15 gradient sums (quantity lane / 3, axis lane % 3),
            // lanes 15-20 the six matrix entries a00 a01 a11 a02 a12 a22.  Every
            // lane forms its term as the reference does, t = (u v) x with
            // (u, v, x) = (w, dq, ds_axis) or (ds_a, ds_b, w) (w (ds_a ds_b) in the
            // reference: the same product), and adds it to its sum face by face,
            // so each sum is the reference's; one warp instruction then carries
            // all 21 sums instead of every lane forming all of them.
            const int k0 = p.csr_off[i], deg = p.csr_off[i + 1] - k0;
            const bool grad_lane = lane < 15;
            const int gq = lane / 3, gax = lane % 3;            // gradient lanes
            const int me = lane - 15;                            // matrix lanes: entry
            const int ma = me == 0 || me == 1 || me == 3 ? 0 : me == 5 ? 2 : 1;  // a00 a01 a11 a02 a12 a22:
            const int mb = me == 0 ? 0 : me == 1 || me == 2 ? 1 : 2;              //   first and second axis
            const bool zdep = grad_lane ? gax == 2 : me >= 3;    // a term the reference skips where ds.z == 0
            double acc = 0.;
            if (!grad_lane && ((p.dim == 1 && (me == 2 || me == 5)) || (p.dim == 2 && me == 5))) acc = 1.;
            for (int j0 = 0; j0 < deg; j0 += 32) {  // warp-uniform
                double w = 0., dq[5] = {0., 0., 0., 0., 0.};
                V3<double> ds = v3(0., 0., 0.);
                if (j0 + lane < deg) {
                    int f = p.csr_face[k0 + j0 + lane];
                    St<double> op;
                    V3<double> oc, sh;
                    other_side(p, i, f, prim, cen, op, oc, sh);
                    ds = (oc + sh) - cen;
                    w = p.area[f] / len2(ds);
#pragma unroll
                    for (int q = 0; q < 5; q++) dq[q] = op.q[q] - prim.q[q];
                }
                const int n = min(32, deg - j0);
                for (int t = 0; t < n; t++) {
                    const double wt = __shfl_sync(0xffffffffu, w, t);
                    const double dx = __shfl_sync(0xffffffffu, ds.x, t), dy = __shfl_sync(0xffffffffu, ds.y, t),
                                 dz = __shfl_sync(0xffffffffu, ds.z, t);
                    double dqt = 0.;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        const double v = __shfl_sync(0xffffffffu, dq[q], t);
                        if (q == gq) dqt = v;
                    }
                    const bool z = !is_zero64(dz);
                    const double da = ma == 0 ? dx : ma == 1 ? dy : dz, db = mb == 0 ? dx : mb == 1 ? dy : dz;
                    const double dax = gax == 0 ? dx : gax == 1 ? dy : dz;
                    const double u = grad_lane ? wt : da, v = grad_lane ? dqt : db, x = grad_lane ? dax : wt;
                    const double term = (u * v) * x;
                    if (lane < 21 && (z || !zdep)) acc = acc + term;
                }
            }
            V3<double> gr[5];
#pragma unroll
            for (int q = 0; q < 5; q++)
                gr[q] = v3(__shfl_sync(0xffffffffu, acc, 3 * q), __shfl_sync(0xffffffffu, acc, 3 * q + 1),
                           __shfl_sync(0xffffffffu, acc, 3 * q + 2));
            const double a00 = __shfl_sync(0xffffffffu, acc, 15), a01 = __shfl_sync(0xffffffffu, acc, 16),
                         a11 = __shfl_sync(0xffffffffu, acc, 17), a02 = __shfl_sync(0xffffffffu, acc, 18),
                         a12 = __shfl_sync(0xffffffffu, acc, 19), a22 = __shfl_sync(0xffffffffu, acc, 20);
            V3<double> m0 = v3(a00, a01, a02), m1 = v3(a01, a11, a12), m2 = v3(a02, a12, a22);
            V3<double> t0 = cross(m1, m2), t1 = cross(m2, m0), t2 = cross(m0, m1);
            double det = dot(m2, t2);
            double inv_det = 1.0 / det;
            V3<double> r0 = inv_det * t0, r1 = inv_det * t1, r2 = inv_det * t2;
            V3<double> c0 = v3(r0.x, r1.x, r2.x), c1 = v3(r0.y, r1.y, r2.y), c2 = v3(r0.z, r1.z, r2.z);
            bool finite = true;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                V3<double> x = gr[q];
                V3<double> res = x.x * c0;
                res = res + x.y * c1;
                res = res + x.z * c2;
                gr[q] = res;
                finite = finite && is_finite64(res.x) && is_finite64(res.y) && is_finite64(res.z);
            }
            if (!finite) {
#pragma unroll
                for (int q = 0; q < 5; q++) gr[q] = v3(0., 0., 0.);
            }
            St<double> mn = prim, mx = prim, emn, emx;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                emn.q[q] = INFINITY;
                emx.q[q] = -INFINITY;
            }
            for (int j = lane; j < deg; j += 32) {
                int f = p.csr_face[k0 + j];
                St<double> op;
                V3<double> oc, sh;
                other_side(p, i, f, prim, cen, op, oc, sh);
                V3<double> d = limiter_offset(p, i, f, cen, sh);
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    double ex = dot(gr[q], d);
                    mn.q[q] = m_min(mn.q[q], op.q[q]);
                    mx.q[q] = m_max(mx.q[q], op.q[q]);
                    emn.q[q] = m_min(emn.q[q], ex);
                    emx.q[q] = m_max(emx.q[q], ex);
                }
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
                mn.q[q] = warp_min_d(mn.q[q]);
                mx.q[q] = warp_max_d(mx.q[q]);
                emn.q[q] = warp_min_d(emn.q[q]);
                emx.q[q] = warp_max_d(emx.q[q]);
                double d_max = mx.q[q] - prim.q[q];
                double d_min = mn.q[q] - prim.q[q];
                const double alpha = limit_factor(d_max, d_min, emx.q[q], emn.q[q]);
                gr[q] = alpha * gr[q];
                if (lane == 0) W3(p, F_GRAD + 3 * q, i, gr[q]);
            }
            if (lane == 0) W3(p, F_GC, i, cen);  // gradient_apply
          }
            if (do_timestep && lane == 0) {
                double dt_new = limit_by_gravity(p, i, particle_timestep(p, i));
                unsigned long long tc = p.tl[k].ti_current;
                unsigned long long dti = make_integer_timestep(dt_new, tb, NUM_TIME_BINS, tc, tbase_inv(p, k));
                if (dti == 0) err |= 1u << 6;
                W(p, F_DT, i, (double)dti * tbase(p, k));  // Particle::set_timestep
                tb = get_time_bin(dti);
                my_dti = dti;
            }
        }
        if (do_timestep && lane == 0) {
            p.tb_tmp[i] = (int8_t)tb;
            my_tb = tb;
        }
    }
    if (err) set_err(p, k, err);
    if (!do_timestep) return;
    inst_min_dti_tb(p, lane == 0 ? k : -1, my_dti, my_tb);
}

template <bool LIST>
// Three resident 256-thread blocks per SM (85 registers): the gradient stage
// 0.206 -> 0.193 ms at 256^2 against the compiler's 128 registers.
__global__ void __launch_bounds__(kMaxBlock, 3) k_gradients(KP p, int do_timestep) {
    const int n_items = cell_items(p);
    if constexpr (LIST) {
        const int lane = threadIdx.x & 31, n_warps = (gridDim.x * blockDim.x) >> 5;
        for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_items; w += n_warps)
            gradients_cell_warp(p, cell_at(p, w), do_timestep, lane);
        return;
    }
    // The cells' loops over their faces have as many trips as the cell has
    // faces (5-8 on a 2D Voronoi mesh), and a warp runs until its cell with the
    // most faces is done: each tile of cells is ordered by face count (a
    // counting sort in shared memory), so that a warp's cells have about the
    // same number.  Each cell's arithmetic is unchanged.  Block-uniform trip
    // count: the per-instance reductions need every lane, the sort every thread.
    __shared__ int s_count[kDegKeys + 1], s_order[kMaxBlock];
    for (int base = blockIdx.x * blockDim.x; base < n_items; base += gridDim.x * blockDim.x) {
        const int idx = base + threadIdx.x;
        const int i = idx < n_items ? cell_at(p, idx) : -1;
        const int key = i < 0 ? kDegKeys : min(p.csr_off[i + 1] - p.csr_off[i], kDegKeys - 1);
        const int t = tile_sorted(key, s_count, s_order);
        gradients_cell(p, t < 0 ? -1 : cell_at(p, base + t), do_timestep);
    }
}

// compute_timesteps as a stage (euler_eqns_fvs.rs:50-61)
__global__ void __launch_bounds__(kMaxBlock) k_timesteps(KP p, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    out[i] = p.active[i] ? particle_timestep(p, i) : INFINITY;
}

// GravitySolver::compute_timesteps (what < 0) or one component of
// ExternalPotentialGravity::compute_accelerations (what = 0, 1, 2) for every
// cell (gravity.rs:45-53, 67-73, 81-95, 110-136).
__global__ void __launch_bounds__(kMaxBlock) k_gravity(KP p, int what, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    if (what < 0) {
        out[i] = grav_timestep(p, i);
    } else {
        const V3<double> a = grav_acceleration(p, C3(p, F_LOC, i));
        out[i] = what == 0 ? a.x : what == 1 ? a.y : a.z;
    }
}

// SelfGravity::compute_accelerations (gravity.rs:22-43): cell i sums, in index
// order, the pull of the cells after it in its simulation (j > i only, as the
// reference does):
//     r = |x_j - x_i| + softening,   a_i += (m_j (x_j - x_i)) / (r r r),
// with m_j the conserved mass after this step's update.  Each a_i is a
// sequential sum, so its rounding fixes the order of the additions; the terms
// are independent.  A block takes a row group of kGravRows cells (one per
// lane) and walks the cells after it in rounds of kGravRound: the round's
// positions and masses are staged in shared memory, each warp forms the terms
// of its 32 of them for the whole row group, and then three warps add the
// round's terms, one component each, in index order.  So the four warps share
// the FP64 work of the longest rows, which would otherwise run on one
// scheduler, and blocks over the first cells (the longest sums) start first.
// Where a displacement component is zero (every pair of a 2D or 1D problem)
// its term is +0, which leaves the sum as it is (a sum that starts at +0 is
// never -0), so the component's division and addition are skipped; r^2 skips
// its +0 square the same way.
// kick: then kick2 and cons->prim (do_c2p) of the active cells, which the
// update left to this kernel.
constexpr int kGravRows = 32, kGravWarps = 4, kGravRound = 32 * kGravWarps;
struct GravSmem {
    double x[kGravRound], y[kGravRound], z[kGravRound], m[kGravRound];
    double t[3][kGravRound][kGravRows];  // the round's terms, [component][j][row]
    double acc[3][kGravRows];
    int end;      // the row group's last j + 1
    int any[3];   // components with a term other than +0 in this round
};
__global__ void __launch_bounds__(kGravRound) k_self_gravity(KP p, int kick, int do_c2p) {
    extern __shared__ __align__(16) unsigned char grav_smem[];
    GravSmem& S = *reinterpret_cast<GravSmem*>(grav_smem);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = blockIdx.x * kGravRows, i = i0 + lane;
    const bool own = i < p.n;
    const int k = own ? inst_of(p, i) : 0;
    const int jend = own ? (p.inst_end ? p.inst_end[k] : p.n) : 0;
    if (threadIdx.x == 0) S.end = 0;
    __syncthreads();
    if (w == 0 && own) atomicMax(&S.end, jend);
    __syncthreads();
    const int block_end = S.end;
    const V3<double> xi = own ? C3(p, F_LOC, i) : v3(0., 0., 0.);
    const double eps = p.grav_soft;
    double acc = 0.;  // warps 0-2: component w of a_i
    for (int jr = i0 + 1; jr < block_end; jr += kGravRound) {
        const int jt = jr + threadIdx.x;
        if (jt < p.n) {
            S.x[threadIdx.x] = C(p, F_LOC, jt);
            S.y[threadIdx.x] = C(p, F_LOC + 1, jt);
            S.z[threadIdx.x] = C(p, F_LOC + 2, jt);
            S.m[threadIdx.x] = C(p, F_CONS, jt);
        }
        if (threadIdx.x < 3) S.any[threadIdx.x] = threadIdx.x == 0;
        __syncthreads();
        bool any_y = false, any_z = false;
        for (int u = 0; u < 32; u++) {
            const int t = 32 * w + u, j = jr + t;
            double tx = 0., ty = 0., tz = 0.;
            if (j > i && j < jend) {
                const double dx = S.x[t] - xi.x, dy = S.y[t] - xi.y, dz = S.z[t] - xi.z;
                // the tests on the integer pipe (cmp64): FP64 comparisons take FP64-pipe issue slots
                const bool ny = cmp64::ne(dy, 0.), nz = cmp64::ne(dz, 0.);
                double r2 = dx * dx;
                if (ny) r2 = r2 + dy * dy;
                if (nz) r2 = r2 + dz * dz;
                const double r = sqrt(r2) + eps;  // (x_j - x_i).length() + softening
                const double m = S.m[t], r3 = r * r * r;
                // m * 0 / r3 is a zero for a finite m and r3 > 0
                const bool zero_ok = (cmp64::bits(m) & cmp64::kMag) < cmp64::kInf && cmp64::gt(r3, 0.);
                tx = (m * dx) / r3;
                if (ny || !zero_ok) {
                    ty = (m * dy) / r3;
                    any_y = true;
                }
                if (nz || !zero_ok) {
                    tz = (m * dz) / r3;
                    any_z = true;
                }
            }
            S.t[0][t][lane] = tx;
            S.t[1][t][lane] = ty;
            S.t[2][t][lane] = tz;
        }
        if (any_y) S.any[1] = 1;
        if (any_z) S.any[2] = 1;
        __syncthreads();
        if (w < 3 && S.any[w]) {
            const int t0 = max(i + 1 - jr, 0), t1 = min(jend - jr, kGravRound);
            for (int t = t0; t < t1; t++) acc = acc + S.t[w][t][lane];
        }
        __syncthreads();  // the round's rows are consumed
    }
    if (w < 3) S.acc[w][lane] = acc;
    __syncthreads();
    if (w != 0 || !own) return;
    const double ax = S.acc[0][lane], ay = S.acc[1][lane], az = S.acc[2][lane];
    p.agrav[i] = ax;
    p.agrav[p.n + i] = ay;
    p.agrav[2 * p.n + i] = az;
    if (!kick || !p.active[i] || p.tl[k].done) return;
    // kick2 (runner/hydrodynamics.rs:51-57) and cons->prim
    unsigned int err = 0;
    const St<double> cons = grav_kick64(C5(p, F_CONS, i), C(p, F_DT, i), v3(ax, ay, az));
    // Other blocks may still be reading the mass row: grav_kick adds +0 to it,
    // which changes its bits only from -0 to +0, and a term m_j (x_j - x_i) / r^3
    // of either zero leaves every sum (which starts at +0) as it is.
    if (__double_as_longlong(cons.q[0]) != __double_as_longlong(C(p, F_CONS, i))) W(p, F_CONS, i, cons.q[0]);
#pragma unroll
    for (int q = 1; q < 5; q++) W(p, F_CONS + q, i, cons.q[q]);
    if (do_c2p) c2p_with_copies(p, i, cons, &err);
    if (err) set_err(p, k, err);
}

// ------------------------------------------------- limiter / sync / end --
// timestep_sync or timestep_limiter (runner/hydrodynamics.rs:160-191) with
// Particle::timestep_limit (part.rs:263-297); then reset_extrapolations and
// kick1 (runner/hydrodynamics.rs:41-49, 193-195).
// The neighbour wake-up bin of timestep_limiter (runner/hydrodynamics.rs:165-184):
// the smallest new bin of an active neighbour plus the allowed difference.
__device__ __forceinline__ int face_wakeup(const KP& p, int i, int f) {
    int l = p.left[f], r = p.right[f];
    int o = i == l ? r : l;
    if (o < 0 || !p.active[o]) return 1 << 20;
    return (int)p.tb_tmp[o] + TIME_BIN_NEIGHBOUR_MAX_DELTA_BIN;
}
// wakeup < 0: computed here (one thread per cell); else given (warp per cell)
__device__ __forceinline__ void limit_cell(const KP& p, int i, int wakeup = -1) {
    if (p.use_list) p.touch[i] = 0;  // the last stage that reads the cell list
    const int k = inst_of(p, i);
    if (p.tl[k].done) return;
    mark_dirty(p, i);  // time bin, dt, extrapolations
    const double time_base = tbase(p, k);
    int tb = p.tb_tmp[i];
    if (p.sync_all) {
        wakeup = p.tl[k].min_timebin;
    } else if (wakeup < 0) {
        wakeup = tb;
        int k0 = p.csr_off[i], k1 = p.csr_off[i + 1];
        for (int k = k0; k < k1; k++) wakeup = min(wakeup, face_wakeup(p, i, p.csr_face[k]));
    } else {
        wakeup = min(wakeup, tb);
    }
    if (wakeup < tb) {
        unsigned long long tc = p.tl[k].ti_current;
        double dt = C(p, F_DT, i);
        if (tb <= max_active_bin_bits(tc)) {  // bin_is_starting
            tb = wakeup;
            dt = (double)get_integer_timestep(tb) * time_base;
        } else {
            unsigned long long ti_end_old = get_integer_time_end(tc, tb);
            dt -= (double)(ti_end_old - tc) * time_base;
            tb = wakeup;
            unsigned long long dti_new = get_integer_timestep(tb);
            unsigned long long ti_end = get_integer_time_end(tc, tb);
            dt += (ti_end == tc) ? (double)dti_new * time_base : (double)(ti_end - tc) * time_base;
        }
        W(p, F_DT, i, dt);
    }
    p.timebin[i] = (int8_t)tb;
    if (p.active[i]) {
        W5(p, F_EXTRAP, i, st_zero<double>());
        if (p.motion != 0) {
            // Particle::hydro_kick1 (part.rs:87-104): half a kick of the particle
            // velocity with the pressure gradient over the new timestep
            double rho = C(p, F_PRIM, i);
            if (rho > 0.) {
                double kick_fac = 0.5 * C(p, F_DT, i) / rho;
                for (int a = 0; a < p.dim; a++) W(p, F_V + a, i, C(p, F_V + a, i) - kick_fac * C(p, F_GRAD + 12 + a, i));
            }
        }
        // kick1: grav_kick adds +0 to the momentum.  The update of this step
        // (kick2) already added +0 to it, and (x + 0) + 0 == x + 0 for every
        // double x, so the row is left as the update wrote it; only where
        // the external potential's accelerations are computed does it kick,
        // over the new dt.
        if (p.grav_acc) W5(p, F_CONS, i, grav_kick64(C5(p, F_CONS, i), C(p, F_DT, i), cell_acceleration(p, i)));
    }
}
__device__ __forceinline__ void end_instance(const KP& p, int k);
__global__ void __launch_bounds__(kMaxBlock) k_limit(KP p) {
    const int n_items = cell_items(p);
    if (p.use_list && !p.sync_all) {
        // hierarchical step: a warp per listed cell, its lanes over the faces,
        // the wake-up bin reduced across the warp (an integer minimum)
        const int lane = threadIdx.x & 31, n_warps = (gridDim.x * blockDim.x) >> 5;
        for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_items; w += n_warps) {
            const int i = p.cell_list[w];
            const int k0 = p.csr_off[i], deg = p.csr_off[i + 1] - k0;
            int wake = 1 << 20;
            for (int j = lane; j < deg; j += 32) wake = min(wake, face_wakeup(p, i, p.csr_face[k0 + j]));
            wake = __reduce_min_sync(0xffffffffu, wake);
            if (lane == 0) limit_cell(p, i, wake);
        }
    } else {
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_items; idx += gridDim.x * blockDim.x)
            limit_cell(p, cell_at(p, idx));
    }
    // the last block to finish does the engine's bookkeeping of the step
    // (end_instance); no cell data is read there, only the timelines
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(p.blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        for (int k = threadIdx.x; k < p.n_inst; k += blockDim.x) end_instance(p, k);
        if (threadIdx.x == 0) *p.blocks_done = 0;
    }
}

// Engine bookkeeping after a step (engine.rs:194-199, 258-268): advance the
// device timeline to the next sync point and reset the reductions.
__device__ __forceinline__ void end_instance(const KP& p, int k) {
    DevTimeline* tl = p.tl + k;
    if (tl->done) return;
    unsigned long long tc = tl->ti_current;
    unsigned long long tn = tc + tl->min_dti;
    tl->steps += 1;
    if (tc >= MAX_NR_TIMESTEPS) tl->done = 1;
    // a simulation whose step reported a failure stops here (the reference
    // panics); the other simulations of a batch carry on
    if (tl->err) tl->done = 1;
    tl->ti_old = tc;
    tl->ti_current = tn;
    tl->min_dti = MAX_NR_TIMESTEPS;
    tl->min_timebin = 127;
    tl->active_faces += tl->n_list;  // list mode: the list is this step's active faces
    tl->n_list = 0;
    tl->active_cells += tl->n_alist;  // list mode: the active head of the cell list
    tl->n_clist = 0;
    tl->n_alist = 0;
}

// Particle::reflect_quantities and reflect_gradients (part.rs:385-428) about
// the unit normal n, the reference's steps as they are: State::reflect of the
// primitive velocity (physical_quantities.rs:239-242); the density gradient
// reflected, the pressure gradient with the density gradient's reflected
// normal component; the velocity gradients first take the velocity's sign
// change, then are reflected themselves.  Gradient rows: F_GRAD + 3 q + axis.
__device__ void reflect_cell(const KP& p, int i, const V3<double> n) {
    V3<double> vel = C3(p, F_PRIM + 1, i);
    vel = vel - (2. * dot(vel, n)) * n;
    W(p, F_PRIM + 1, i, vel.x);
    W(p, F_PRIM + 2, i, vel.y);
    W(p, F_PRIM + 3, i, vel.z);
    V3<double> g[5];
#pragma unroll
    for (int q = 0; q < 5; q++) g[q] = C3(p, F_GRAD + 3 * q, i);
    g[0] = g[0] - (2. * dot(g[0], n)) * n;
    g[4] = g[4] - (2. * dot(g[0], n)) * n;
    const V3<double> twice = 2. * v3(dot(v3(g[1].x, g[2].x, g[3].x), n), dot(v3(g[1].y, g[2].y, g[3].y), n),
                                     dot(v3(g[1].z, g[2].z, g[3].z), n));
    g[1] = g[1] - n.x * twice;
    g[2] = g[2] - n.y * twice;
    g[3] = g[3] - n.z * twice;
#pragma unroll
    for (int q = 1; q <= 3; q++) g[q] = g[q] - (2. * dot(g[q], n)) * n;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        W(p, F_GRAD + 3 * q, i, g[q].x);
        W(p, F_GRAD + 3 * q + 1, i, g[q].y);
        W(p, F_GRAD + 3 * q + 2, i, g[q].z);
    }
}

// Space::drift (space.rs:833-854) with Particle::drift (part.rs:107-119): every
// generator by v dt; outside the box it is wrapped (Particle::box_wrap,
// part.rs:449-455, utils.rs:23-32) or reflected (reflective walls); in an open
// or vacuum box it stays where it drifted and the host removes it.
__global__ void __launch_bounds__(kMaxBlock) k_drift(KP p, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const int k = inst_of(p, i);
    if (p.tl[k].done) return;
    double loc[3], cen[3], gc[3];
    for (int a = 0; a < 3; a++) {
        loc[a] = C(p, F_LOC + a, i);
        cen[a] = C(p, F_CEN + a, i);
        gc[a] = C(p, F_GC + a, i);
    }
    for (int a = 0; a < p.dim; a++) {
        double v = C(p, F_V + a, i);
        loc[a] += v * dt;
        cen[a] += v * dt;
        gc[a] += v * dt;
    }
    if (!isfinite(loc[0]) || !isfinite(loc[1]) || !isfinite(loc[2])) {
        set_err(p, k, 1u << 4);  // "Infinite x after drift!"
    } else {
        bool inside = true;
        for (int a = 0; a < p.dim; a++) inside = inside && loc[a] >= 0. && loc[a] < p.box[a];
        if (!inside && p.boundary == MVMM_BOUNDARY_REFLECTIVE) {
            // Particle::box_reflect (part.rs:457-469), utils.rs box_reflect (:34-43):
            // mirrored into the box; loc alone moves
            const V3<double> old = v3(loc[0], loc[1], loc[2]);
            for (int a = 0; a < p.dim; a++) {
                if (loc[a] < 0.) loc[a] -= 2. * loc[a];
                if (loc[a] > p.box[a]) loc[a] -= 2. * (loc[a] - p.box[a]);
            }
            bool back = true;  // assert!(contains(..)) after the reflection
            for (int a = 0; a < p.dim; a++) back = back && loc[a] >= 0. && loc[a] < p.box[a];
            if (!back) set_err(p, k, 1u << 4);
            const V3<double> shift = v3(loc[0], loc[1], loc[2]) - old;
            if (len2(shift) > 0.) {
                reflect_cell(p, i, (1. / len(shift)) * shift);  // shift * shift.length_recip()
                p.fresh[i] = 0;  // prim and grad changed: the derived face-stage rows are stale
            }
        } else if (!inside && p.boundary == MVMM_BOUNDARY_PERIODIC) {
            double old[3] = {loc[0], loc[1], loc[2]};
            for (int a = 0; a < p.dim; a++) {
                // one box length per pass, as the reference's loops (bounded: a
                // generator moves less than a cell per step)
                for (int it = 0; it < 64 && loc[a] < 0.; it++) loc[a] += p.box[a];
                for (int it = 0; it < 64 && loc[a] >= p.box[a]; it++) loc[a] -= p.box[a];
            }
            for (int a = 0; a < 3; a++) {
                double shift = loc[a] - old[a];
                gc[a] += shift;
                cen[a] += shift;
            }
        }
    }
    for (int a = 0; a < 3; a++) {
        W(p, F_LOC + a, i, loc[a]);
        W(p, F_CEN + a, i, cen[a]);
        W(p, F_GC + a, i, gc[a]);
    }
}

// Particle::update_geometry (part.rs:151-158) of the active cells with the
// rebuilt mesh's volume and centroid (Space::volume_calculation, space.rs:236-263).
__global__ void __launch_bounds__(kMaxBlock) k_geometry(KP p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n || !p.active[i]) return;
    if (p.tl[inst_of(p, i)].done) return;
    double vol = p.new_vol[i];
    if (!(vol >= 0.)) set_err(p, inst_of(p, i), 1u << 4);  // assert!(self.volume >= 0.)
    W(p, F_VOL, i, vol);
    for (int a = 0; a < 3; a++) W(p, F_CEN + a, i, p.new_cen[(size_t)a * p.n + i]);
}

// Sets every simulation's integer time on the device (the counters stay);
// faces_mark remembers the face counter so the step's own count can be read.
__global__ void k_set_time(KP p, unsigned long long ti_current, unsigned long long ti_old) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= p.n_inst) return;
    DevTimeline* tl = p.tl + k;
    tl->ti_current = ti_current;
    tl->ti_old = ti_old;
    tl->min_dti = MAX_NR_TIMESTEPS;
    tl->min_timebin = 127;
    tl->done = 0;
    tl->faces_mark = tl->active_faces;
}

// ---------------------------------------------- Riemann over arrays --
template <int SOLVER, bool SAMPLE>
__global__ void k_riemann(double gamma, int64_t n, const double* l, const double* r, const double* vf,
                          const double* nrm, double* out, unsigned int* errp, RSx x) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Gas<double> g = make_gas<double>(gamma, 0, 0.);
    St<double> L, R;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        L.q[q] = l[q * n + i];
        R.q[q] = r[q * n + i];
    }
    V3<double> nn = v3(nrm[i], nrm[n + i], nrm[2 * n + i]);
    unsigned int err = 0;
    St<double> o;
    if (SAMPLE) {
        o = star_half_state<double, SOLVER>(L, R, nn, g, g, 1000, &err, &x);
    } else {
        V3<double> iv = v3(vf[i], vf[n + i], vf[2 * n + i]);
        o = solve_for_flux<double, SOLVER>(L, R, iv, nn, g, g, 1000, &err, &x);
    }
#pragma unroll
    for (int q = 0; q < 5; q++) out[q * n + i] = o.q[q];
    if (err) atomicOr(errp, err);
}

inline int grid(int n, int b = kBlock) { return (n + b - 1) / b; }

}  // namespace

// Blocks of a cell kernel: one thread per cell, or in a hierarchical step half
// a wave of resident blocks (the device's SMs x 1024 threads) striding over the cell
// list, whose length is known on the device only.
int cell_grid(const KP& p) {
    int g = grid(p.n, p.blk_cell);
    int wave = p.n_sms * 1024 / p.blk_cell;
    return p.use_list && g > wave ? wave : g;
}

void launch_predict(const KP& p, cudaStream_t s) {
    if (p.n > 0) k_predict<<<grid(p.n, p.blk_cell), p.blk_cell, 0, s>>>(p);
}
void launch_derive(const KP& p, cudaStream_t s) {
    if (p.n > 0) k_derive<<<grid(p.n, p.blk_cell), p.blk_cell, 0, s>>>(p);
}
// list mode: a grid of a few waves walks the list (its length is only known on the device)
inline int face_grid(const KP& p) {
    int g = grid(p.nf, p.blk_face), cap = p.n_sms * 512 / p.blk_face;
    return p.use_list && g > cap ? cap : g;
}

size_t brent_job_bytes() { return sizeof(BrentJob); }
// The pools' lanes draw jobs until the queues are dry: as many blocks as fit
// on the device at once
template <class K>
int pool_grid(const KP& p, K kernel, int block, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return p.n_sms * per_sm;
}
void launch_face_flux_fp64(const KP& p, int solver, cudaStream_t s) {
    if (p.nf <= 0) return;
    int g = face_grid(p);
    if (solver == SOLVER_HLLC) k_face_flux<SOLVER_HLLC><<<g, p.blk_face, 0, s>>>(p);
    else if (solver == SOLVER_EXACT && p.brent_jobs) {
        cudaMemsetAsync(p.brent_count, 0, (kExactQueues + 1) * sizeof(unsigned int), s);
        k_face_flux<SOLVER_EXACT, true><<<g, p.blk_face, 0, s>>>(p);
        k_face_search<<<pool_grid(p, k_face_search, kSearchBlock, 0), kSearchBlock, 0, s>>>(p);
        const int finish_grid =
            (int)std::min<long long>((kExactQueues * (long long)p.brent_cap + kJobTile - 1) / kJobTile, p.n_sms * 16LL);
        k_face_finish<<<finish_grid, kJobTile, 0, s>>>(p);
    } else if (solver == SOLVER_EXACT) k_face_flux<SOLVER_EXACT><<<g, p.blk_face, 0, s>>>(p);
    else if (solver == SOLVER_PVRS) k_face_flux<SOLVER_PVRS><<<g, p.blk_face, 0, s>>>(p);
    else k_face_flux<SOLVER_EXTRA><<<g, p.blk_face, 0, s>>>(p);
}
void launch_extrap_flush(const KP& p, bool reset, cudaStream_t s) {
    if (p.extrap_step && p.n > 0) k_extrap_flush<<<grid(p.n, kBlock), kBlock, 0, s>>>(p, reset ? 1 : 0);
}
void launch_compact(const KP& p, cudaStream_t s) {
    if (p.nf > 0) k_compact<<<cell_grid(p), p.blk_cell, 0, s>>>(p);
}
void launch_update(const KP& p, int do_c2p, cudaStream_t s) {
    if (p.n <= 0) return;
    const bool r32 = p.fp32 && p.flux_rows == 7;
    if (p.use_list) {
        if (r32) k_update<true, true><<<cell_grid(p), p.blk_cell, 0, s>>>(p, do_c2p);
        else k_update<false, true><<<cell_grid(p), p.blk_cell, 0, s>>>(p, do_c2p);
    } else {
        if (r32) k_update<true, false><<<cell_grid(p), p.blk_cell, 0, s>>>(p, do_c2p);
        else k_update<false, false><<<cell_grid(p), p.blk_cell, 0, s>>>(p, do_c2p);
    }
}
void launch_c2p(const KP& p, cudaStream_t s) {
    if (p.n > 0) k_c2p<<<grid(p.n, p.blk_cell), p.blk_cell, 0, s>>>(p);
}
void launch_gradients(const KP& p, int do_timestep, cudaStream_t s) {
    if (p.n <= 0) return;
    if (p.use_list) k_gradients<true><<<cell_grid(p), p.blk_cell, 0, s>>>(p, do_timestep);
    else k_gradients<false><<<cell_grid(p), p.blk_cell, 0, s>>>(p, do_timestep);
}
void launch_timesteps(const KP& p, double* dt_out, cudaStream_t s) {
    if (p.n > 0) k_timesteps<<<grid(p.n, p.blk_cell), p.blk_cell, 0, s>>>(p, dt_out);
}
cudaError_t setup_self_gravity() {
    return cudaFuncSetAttribute(k_self_gravity, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GravSmem));
}
void launch_self_gravity(const KP& p, int kick, int do_c2p, cudaStream_t s) {
    if (p.n > 0)
        k_self_gravity<<<(p.n + kGravRows - 1) / kGravRows, kGravRound, sizeof(GravSmem), s>>>(p, kick, do_c2p);
}
void launch_gravity(const KP& p, int what, double* out, cudaStream_t s) {
    if (p.n > 0) k_gravity<<<grid(p.n, p.blk_cell), p.blk_cell, 0, s>>>(p, what, out);
}
void launch_limit(const KP& p, cudaStream_t s) {
    if (p.n <= 0) return;
    // steps over all cells: few, full blocks striding over the cells, so that
    // few blocks take part in the last-block hand-off of the step's bookkeeping
    if (p.use_list) k_limit<<<cell_grid(p), p.blk_cell, 0, s>>>(p);
    else k_limit<<<std::min(grid(p.n, 256), p.n_sms * 8), 256, 0, s>>>(p);
}
// the engine bookkeeping runs in the last block of k_limit
void launch_end(const KP&, cudaStream_t) {}
void launch_drift(const KP& p, double dt, cudaStream_t s) {
    if (p.n > 0) k_drift<<<grid(p.n, kBlock), kBlock, 0, s>>>(p, dt);
}
void launch_geometry(const KP& p, cudaStream_t s) {
    if (p.n > 0) k_geometry<<<grid(p.n, kBlock), kBlock, 0, s>>>(p);
}
void launch_set_time(const KP& p, unsigned long long ti_current, unsigned long long ti_old, cudaStream_t s) {
    k_set_time<<<(p.n_inst + 127) / 128, 128, 0, s>>>(p, ti_current, ti_old);
}

// kind: SOLVER_*; sampling is defined for the star solvers, so HLLC and
// linear advection sample the exact solution.
void launch_riemann_fp64(int kind, int sample, double gamma, int64_t n, const double* l, const double* r,
                         const double* vf, const double* nrm, double* out, unsigned int* err, const RSx& x,
                         cudaStream_t s) {
    if (n <= 0) return;
    int g = (int)((n + kBlock - 1) / kBlock);
    if (sample) {
        if (kind == SOLVER_PVRS) k_riemann<SOLVER_PVRS, true><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else if (kind >= SOLVER_AIRS && kind <= SOLVER_TRRS)
            k_riemann<SOLVER_EXTRA, true><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else k_riemann<SOLVER_EXACT, true><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
    } else {
        if (kind == SOLVER_HLLC) k_riemann<SOLVER_HLLC, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else if (kind == SOLVER_EXACT) k_riemann<SOLVER_EXACT, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else if (kind == SOLVER_PVRS) k_riemann<SOLVER_PVRS, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else k_riemann<SOLVER_EXTRA, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
    }
}

}  // namespace mvmm
