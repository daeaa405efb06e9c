// FP32-face form of the flux stage (flux.rs:23-195 restated in FP32).
//
// Reconstruction, the pair-wise limiter, the Riemann solve and the face flux
// run in FP32 on a static FP32 face geometry (differences formed in FP64 once
// per upload, then rounded); the exact solver's last Newton step sums the
// cancelling terms without rounding (full FP64 iteration where the FP32 search
// does not converge).  A step
// writes FP32 face fluxes dt * area * F; the scatter and the conserved update
// accumulate them in FP64 (the update kernel is shared with the plain form),
// so every face flux leaves one cell and enters the other exactly.  Compiled
// with FMA contraction enabled.
#include "mvmm_cellops.cuh"

// Minimum resident 256-thread blocks of k_face_flux32 per SM, i.e. its register
// budget: 3 caps it at 80 registers (it needs 128 unconstrained); the extra
// occupancy outweighs the spills (face stage 15% faster at 256^2, 28% at 512^2).
// 4 (64 registers, ~10% more spill traffic) measured 29.5 us against 29.0 at 256^2.
#ifndef FACE32_MINB
#define FACE32_MINB 3
#endif

namespace mvmm {

namespace {

__device__ __forceinline__ float G(const KP& p, int f, int i) { return p.cf[(size_t)f * p.n + i]; }
__device__ __forceinline__ V3<float> G3(const KP& p, int f, int i) { return {G(p, f, i), G(p, f + 1, i), G(p, f + 2, i)}; }
__device__ __forceinline__ St<float> G5(const KP& p, int f, int i) {
    St<float> s;
#pragma unroll
    for (int q = 0; q < 5; q++) s.q[q] = G(p, f + q, i);
    return s;
}
__device__ __forceinline__ void prep32_cell(const KP& p, int i) {
    if (p.tl[inst_of(p, i)].done) return;
    size_t n = p.n;
    float* cf = p.cf;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        cf[(G_PRIM + q) * n + i] = f32(C(p, F_PRIM + q, i));
        cf[(G_EXTRAP + q) * n + i] = f32(C(p, F_EXTRAP + q, i));
        cf[(G_SRC + q) * n + i] = f32(C(p, F_SRC + q, i));
    }
#pragma unroll
    for (int q = 0; q < 15; q++) cf[(G_GRAD + q) * n + i] = f32(C(p, F_GRAD + q, i));
    cf[G_CS * n + i] = f32(C(p, F_CS, i));
    V3<double> loc = C3(p, F_LOC, i);
    V3<double> dgc = C3(p, F_GC, i) - loc;
    V3<double> v = C3(p, F_V, i);
    cf[(G_DGC + 0) * n + i] = f32(dgc.x);
    cf[(G_DGC + 1) * n + i] = f32(dgc.y);
    cf[(G_DGC + 2) * n + i] = f32(dgc.z);
    cf[(G_V + 0) * n + i] = f32(v.x);
    cf[(G_V + 1) * n + i] = f32(v.y);
    cf[(G_V + 2) * n + i] = f32(v.z);
}
// Steps over all cells (synchronised steps, batches): EulerEqnsFvs::predict
// (Particle::extrapolate_state, part.rs:123-132, with the active mask of
// engine.rs:63-65) fused with the FP32 copies the face stage reads.  The
// extrapolation source and the sound speed feed only FP32 arithmetic, so they
// are formed in FP32 from those copies; the extrapolation itself is state and
// accumulates in FP64.  Branches as the plain predict: the update of the
// extrapolation tests the density before check_physical, the face-stage rows
// the checked state.
__global__ void __launch_bounds__(kMaxBlock) k_predict32(KP p) {
    // two rows of blocks: row 0 forms the extrapolation (and the copies it
    // reads); row 1 converts the copies nothing here reads (six gradient rows,
    // gradients_centroid - loc, v), so twice the warps hide the loads' latency
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool main_row = blockIdx.y == 0;
    bool act = false;
    int k = i < p.n ? inst_of(p, i) : -1;
    if (k >= 0 && p.tl[k].done) k = -1;  // a finished simulation of a batch is left untouched
    const size_t n = (size_t)p.n;
    float* cf = p.cf;
    // the gradient and gradients_centroid - loc copies of a fixed mesh's cell are
    // current when the last gradient stage wrote them and nothing was uploaded since
    const bool cur = k >= 0 && p.cf_fresh && !p.stale_all && p.cf_fresh[i];
    if (k >= 0 && !main_row && !cur) {
#pragma unroll
        for (int q : {4, 5, 6, 8, 9, 10}) cf[(G_GRAD + q) * n + i] = f32(C(p, F_GRAD + q, i));
        const V3<double> dgc = C3(p, F_GC, i) - C3(p, F_LOC, i);
        const V3<double> v = C3(p, F_V, i);
        cf[(G_DGC + 0) * n + i] = f32(dgc.x);
        cf[(G_DGC + 1) * n + i] = f32(dgc.y);
        cf[(G_DGC + 2) * n + i] = f32(dgc.z);
        cf[(G_V + 0) * n + i] = f32(v.x);
        cf[(G_V + 1) * n + i] = f32(v.y);
        cf[(G_V + 2) * n + i] = f32(v.z);
    }
    if (!main_row) return;  // block-uniform
    if (k >= 0) {
        const unsigned long long tc = p.tl[k].ti_current, to = p.tl[k].ti_old;
        const double dt = (double)(tc - to) * tbase(p, k);  // TimestepInfo::dt_from_dti
        act = p.timebin[i] <= max_active_bin_bits(tc);
        p.active[i] = act;
        p.fresh[i] = 0;
        const St<double> prim = C5(p, F_PRIM, i);
        const bool pos = gt0_64(prim.q[0]);
        const bool reset = lt0_64(prim.q[0]) || lt0_64(prim.q[4]);  // check_physical zeroes the state
        St<float> w;
#pragma unroll
        for (int q = 0; q < 5; q++) w.q[q] = f32(prim.q[q]);
        // the gradient rows the source reads: d(rho), the velocity divergence, d(P)
        float gr[15];
#pragma unroll
        for (int q : {0, 1, 2, 3, 7, 11, 12, 13, 14}) gr[q] = cur ? G(p, G_GRAD + q, i) : f32(C(p, F_GRAD + q, i));
        const V3<float> vr = f32v(C3(p, F_VREL, i));
        const Gas<float> g = gas_t<float>(p);
        const float rho_inv = 1.f / w.q[0];
        const float div_v = gr[3] + gr[7] + gr[11];
        const V3<float> g0 = v3(gr[0], gr[1], gr[2]), g4 = v3(gr[12], gr[13], gr[14]);
        St<float> src;  // Particle::time_extrapolations before the -dt factor (part.rs:134-149)
        src.q[0] = w.q[0] * div_v + dot(vr, g0);
        src.q[1] = vr.x * div_v + rho_inv * g4.x;
        src.q[2] = vr.y * div_v + rho_inv * g4.y;
        src.q[3] = vr.z * div_v + rho_inv * g4.z;
        src.q[4] = g.gamma * w.q[4] * div_v + dot(vr, g4);
        St<double> ex = C5(p, F_EXTRAP, i);
#pragma unroll
        for (int q = 0; q < 5; q++) ex.q[q] = pos ? ex.q[q] + (-dt) * f64(src.q[q]) : ex.q[q] + 0.;
        W5(p, F_EXTRAP, i, ex);
        mark_dirty(p, i, reset ? kDirtyAll : kDirtyExtrap);
        if (reset) W5(p, F_PRIM, i, st_zero<double>());
        const bool live = pos && !reset;  // the checked density is positive
#pragma unroll
        for (int q = 0; q < 5; q++) {
            cf[(G_PRIM + q) * n + i] = reset ? 0.f : w.q[q];
            cf[(G_EXTRAP + q) * n + i] = f32(ex.q[q]);
            cf[(G_SRC + q) * n + i] = live ? src.q[q] : 0.f;
        }
        if (!cur) {
#pragma unroll
            for (int q : {0, 1, 2, 3, 7, 11, 12, 13, 14}) cf[(G_GRAD + q) * n + i] = gr[q];
        }
        cf[G_CS * n + i] = live ? g.sound_speed(w.q[4], rho_inv) : 0.f;
    }
    inst_count(p, k, act, CNT_CELLS);
}

// hierarchical steps convert only the cells on the step's cell list
__global__ void __launch_bounds__(kMaxBlock) k_prep32(KP p) {
    const int n_items = cell_items(p);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_items; idx += gridDim.x * blockDim.x)
        prep32_cell(p, cell_at(p, idx));
}

__device__ __forceinline__ V3<float> GE3(const KP& p, int g, int f) {
    const size_t nf = (size_t)p.nf;
    return {p.geo[g * nf + f], p.geo[(g + 1) * nf + f], p.geo[(g + 2) * nf + f]};
}

// Marks the cells whose position or centroid differs, bit for bit, from the
// one the FP32 face geometry was last built from, and records the new bits
// (integer compares: no FP64 pipe work).  force: every cell counts as changed.
__global__ void __launch_bounds__(kMaxBlock) k_geom_check(KP p, int force) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const size_t n = (size_t)p.n;
    const unsigned long long* cd = reinterpret_cast<const unsigned long long*>(p.cd);
    unsigned long long v[6];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        v[a] = cd[(F_LOC + a) * n + i];
        v[3 + a] = cd[(F_CEN + a) * n + i];
    }
    bool changed = force != 0;
#pragma unroll
    for (int k = 0; k < 6; k++) changed = changed || v[k] != p.geo_pos[k * n + i];
    if (changed) {
#pragma unroll
        for (int k = 0; k < 6; k++) p.geo_pos[k * n + i] = v[k];
    }
    p.geo_changed[i] = changed;
}

// Static face geometry (FaceGeom32), one thread per face.  With geo_check set
// only faces next to a changed cell are rebuilt (the face arrays themselves
// change only with the mesh, which rebuilds every face).
__global__ void __launch_bounds__(kMaxBlock) k_geom32(KP p) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= p.nf) return;
    int l = p.left[f], r = p.right[f];
    if (p.geo_check && !p.geo_changed[l] && (r < 0 || !p.geo_changed[r])) return;
    V3<double> fc = F3(p.fcen, p.nf, f), s = F3(p.shift, p.nf, f), n = F3(p.normal, p.nf, f);
    V3<double> locl = C3(p, F_LOC, l), cenl = C3(p, F_CEN, l);
    V3<double> z = v3(0., 0., 0.);
    V3<double> rr = z, fcm = z, dr = z, dx, ds;
    if (r >= 0) {
        V3<double> locr = C3(p, F_LOC, r), cenr = C3(p, F_CEN, r);
        rr = (fc - locr) - s;
        dx = (locr + s) - locl;
        fcm = fc - 0.5 * ((locl + locr) + s);
        ds = (cenr + s) - cenl;
        // the right cell's limiter offset: the reference's (fc - cen_r) + s, or with
        // limiter_frame flux_exchange's (fc - cen_r) - s
        dr = p.limiter_frame ? (fc - cenr) - s : (fc - cenr) + s;
    } else {
        // Particle::reflect (part.rs:374-383) of the cell's position and centroid
        dx = (2. * dot(fc - locl, n)) * n;
        ds = (2. * dot(fc - cenl, n)) * n;
    }
    const V3<double> dl = p.limiter_frame ? fc - cenl : (fc - cenl) - s;  // the left cell's
    V3<double> vals[8] = {fc - locl, rr, dx, fcm, n, ds, dl, dr};
    float* g = p.geo;
    const size_t nf = (size_t)p.nf;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        g[(3 * k + 0) * nf + f] = f32(vals[k].x);
        g[(3 * k + 1) * nf + f] = f32(vals[k].y);
        g[(3 * k + 2) * nf + f] = f32(vals[k].z);
    }
    g[GE_W * nf + f] = f32(p.area[f] / len2(ds));
    g[GE_A * nf + f] = f32(p.area[f]);
}

__device__ __forceinline__ St<float> reconstruct32(const KP& p, int i, const St<float>& prim, V3<float> dx, float td) {
    St<float> r;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        V3<float> g = G3(p, G_GRAD + 3 * q, i);
        r.q[q] = (prim.q[q] + dot(g, dx)) + G(p, G_EXTRAP + q, i);
    }
    if (prim.q[0] > 0.f) {
#pragma unroll
        for (int q = 0; q < 5; q++) r.q[q] += td * G(p, G_SRC + q, i);
    }
    return r;
}

struct Out32 {
    St<float> F;     // area-free face flux
    V3<float> dx;    // generator separation (mflux direction)
    float v_max, a_over_r;
};
// A face up to its Riemann solve: the two states handed to the solver (in the
// face frame), the face velocity and normal, and what the result needs.
struct Pre32 {
    St<float> l, r;
    V3<float> iv, n, dx;
    float v_max, a_over_r;
};

__device__ __forceinline__ Pre32 face_interior32_pre(const KP& p, int f, int l, int r, float dt) {
    V3<float> dx = GE3(p, GE_DX, f);
    V3<float> dx_left = GE3(p, GE_RL, f) - G3(p, G_DGC, l);
    V3<float> dx_right = GE3(p, GE_RR, f) - G3(p, G_DGC, r);
    float dx_gradients = len(dx_left - dx_right);
    V3<float> dx_centroid = GE3(p, GE_DS, f);
    St<float> pl = G5(p, G_PRIM, l), pr = G5(p, G_PRIM, r);
    float v_max = G(p, G_CS, l) + G(p, G_CS, r);
    v_max -= fminf(dot(vel(pr) - vel(pl), dx_centroid), 0.f);
    float td = 0.5f * dt;
    St<float> ldash = reconstruct32(p, l, pl, dx_left, td);
    St<float> rdash = reconstruct32(p, r, pr, dx_right, td);
    St<float> prim_left = pairwise_limiter(pl, pr, ldash, len(dx_left) / dx_gradients);
    St<float> prim_right = pairwise_limiter(pr, pl, rdash, len(dx_right) / dx_gradients);
    V3<float> vl = G3(p, G_V, l), vr = G3(p, G_V, r);
    float fac = dot(vr - vl, GE3(p, GE_FCM, f)) / len2(dx);
    V3<float> v_face = 0.5f * (vl + vr) - fac * dx;
    V3<float> mvf = neg(v_face);
    Pre32 q;
    q.l = boost(prim_left, mvf);
    q.r = boost(prim_right, mvf);
    q.iv = v_face;
    q.n = GE3(p, GE_N, f);
    q.dx = dx;
    q.v_max = v_max;
    q.a_over_r = p.geo[GE_A * (size_t)p.nf + f] / len(dx);  // feeds max_a_over_r only (mesh steering)
    return q;
}
__device__ __forceinline__ Pre32 face_boundary32_pre(const KP& p, int f, int i, float dt) {
    V3<float> n = GE3(p, GE_N, f);
    V3<float> dx_face = GE3(p, GE_RL, f) - G3(p, G_DGC, i);       // fc - gc
    float dx_gradients = len((2.f * dot(dx_face, n)) * n);        // |reflect(gc) - gc|
    V3<float> dx_centroid = GE3(p, GE_DS, f);
    V3<float> dx = GE3(p, GE_DX, f);
    St<float> prim = G5(p, G_PRIM, i);
    float v_max = G(p, G_CS, i);
    float td = 0.5f * dt;
    St<float> dash = reconstruct32(p, i, prim, dx_face, td);
    float dx_fac = len(dx_face) / dx_gradients;
    St<float> bnd;
    if (p.boundary == 1) {
        St<float> rprim = reflect(prim, n);
        dash = pairwise_limiter(prim, rprim, dash, dx_fac);
        v_max -= fminf(dot(vel(rprim) - vel(prim), dx_centroid), 0.f);
        bnd = reflect(dash, n);
    } else if (p.boundary == 2) {
        dash = pairwise_limiter(prim, prim, dash, dx_fac);
        bnd = dash;
    } else {
        St<float> vac = st_zero<float>();
        dash = pairwise_limiter(prim, vac, dash, dx_fac);
        v_max += fminf(dot(vel(prim), dx_centroid), 0.f);
        bnd = vac;
    }
    Pre32 q;
    q.l = dash;
    q.r = bnd;
    q.iv = v3(0.f, 0.f, 0.f);
    q.n = n;
    q.dx = dx;
    q.v_max = v_max;
    q.a_over_r = p.geo[GE_A * (size_t)p.nf + f] / len(dx);
    return q;
}
template <int SOLVER>
__device__ __forceinline__ Out32 face_solve32(const KP& p, const Pre32& q, const Gas<float>& g,
                                              const Gas<double>& g64, unsigned int* err) {
    Out32 o;
    o.F = solve_for_flux<float, SOLVER>(q.l, q.r, q.iv, q.n, g, g64, p.max_iter, err, &p.rsx);
    o.dx = q.dx;
    o.v_max = q.v_max;
    o.a_over_r = q.a_over_r;
    return o;
}
template <int SOLVER>
__global__ void __launch_bounds__(kMaxBlock, FACE32_MINB) k_face_flux32(KP p) {
    if (p.use_list && p.tl[0].done) return;
    const Gas<float> g = gas_t<float>(p);
    const Gas<double> g64 = gas_t<double>(p);
    const int n_items = p.use_list ? (int)p.tl[0].n_list : p.nf;
    const size_t nf = (size_t)p.nf;
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
            Out32 o;
            // The timesteps are non-negative doubles, which order as their bit
            // patterns (the sign bit cleared, so that -0 ties with +0): the
            // active-face rule and fmin(dt_l, dt_r) on the integer pipe, and dt
            // rounded to FP32 there too (to_f32_rn), keep this kernel off the
            // FP64 pipe.
            double dt = 0.;
            if (r >= 0) {
                bool ra = p.active[r] != 0;
                const double dtl = C(p, F_DT, l), dtr = C(p, F_DT, r);
                const long long kl = __double_as_longlong(dtl) & 0x7fffffffffffffffLL;
                const long long kr = __double_as_longlong(dtr) & 0x7fffffffffffffffLL;
                if (!((!la && !ra) || (kr < kl && !ra) || (kl < kr && !la))) {  // interior_face_active
                    dt = kl <= kr ? dtl : dtr;
                    o = face_solve32<SOLVER>(p, face_interior32_pre(p, f, l, r, f32(dt)), g, g64, &err);
                    counted = true;
                }
            } else if (la) {
                dt = C(p, F_DT, l);
                o = face_solve32<SOLVER>(p, face_boundary32_pre(p, f, l, f32(dt)), g, g64, &err);
                counted = true;
            }
            if (p.flux_rows == 7) {
                // step: FP32 rows dt * area * F, v_max, a_over_r (accumulated in FP64 by the update)
                float* out = p.flux32;
                float da = counted ? f32(dt) * p.geo[GE_A * nf + f] : 0.f;
#pragma unroll
                for (int q = 0; q < 5; q++) out[q * nf + f] = counted ? da * o.F.q[q] : 0.f;
                out[5 * nf + f] = counted ? o.v_max : 0.f;
                out[6 * nf + f] = counted ? o.a_over_r : 0.f;
            } else {
                // per-stage call: the FluxInfo rows in FP64, mflux included
                double area = p.area[f];
                double* out = p.flux;
#pragma unroll
                for (int q = 0; q < 5; q++) out[q * nf + f] = counted ? dt * (area * (double)o.F.q[q]) : 0.;
                double m = counted ? area * (double)o.F.q[0] : 0.;
                out[5 * nf + f] = m * (double)o.dx.x;
                out[6 * nf + f] = m * (double)o.dx.y;
                out[7 * nf + f] = m * (double)o.dx.z;
                out[8 * nf + f] = counted ? (double)o.v_max : 0.;
                out[9 * nf + f] = counted ? (double)o.a_over_r : 0.;
            }
            if (err & ~kInfoFallback) set_err(p, k, err & ~kInfoFallback);
        }
        inst_count(p, k, (err & kInfoFallback) != 0, CNT_FALLBACK);
        if (!p.use_list) inst_count(p, k, counted, CNT_FACES);
    }
}

// The other side of face f seen from cell i in the FP32-face form (the FP32
// counterpart of other_side): its primitive state, the centroid separation ds
// and the limiter's extrapolation vector, from the static face geometry.
__device__ __forceinline__ void other_side32(const KP& p, int i, int f, const St<float>& prim, St<float>& op,
                                             V3<float>& ds, V3<float>& d) {
    int l = p.left[f], r = p.right[f];
    if (i == l) {
        ds = GE3(p, GE_DS, f);
        d = GE3(p, GE_DL, f);
        if (r < 0) {  // Space::get_boundary_part (space.rs:213-229)
            V3<float> n = GE3(p, GE_N, f);
            if (p.boundary == 1) op = reflect(prim, n);
            else if (p.boundary == 2) op = prim;
            else op = st_zero<float>();
        } else {
            op = G5(p, G_PRIM, r);
        }
    } else {
        ds = neg(GE3(p, GE_DS, f));
        d = GE3(p, GE_DR, f);
        op = G5(p, G_PRIM, l);
    }
}

// gradient_estimate + gradient_limit + gradient_apply (runner/hydrodynamics.rs:67-143)
// for the FP32-face form: primitive differences from the FP32 copies (the
// update refreshes them for active cells), separations and WLS weights from
// the static face geometry, the WLS sums, the 3x3 inverse and the cell-wise
// limiter in FP32 (these slopes only feed the FP32 reconstruction); the
// timestep (Particle::timestep, timesteps_apply) stays FP64 as in the plain form.
// Particle::set_particle_velocity (part.rs:328-372) and Particle::timestep
// (part.rs:42-84) in the FP32-face form.  The thermal energy E - p.v/2 and the
// position differences are formed in FP64 (they cancel); the fluid velocity,
// sound speed, mesh velocity, |v_rel|, radius and the CFL ratio in FP32.  gr:
// the cell's (limited) gradients, rows q = 0..4; v and v_rel are stored in FP64.
__device__ __forceinline__ float radius32(float volume, int dim) {
    if (dim == 1) return 0.5f * volume;
    if (dim == 2) return sqrtf(0.31830988618379067154f * volume);
    return cbrtf(0.25f * 3.f * 0.31830988618379067154f * volume);
}
__device__ __forceinline__ V3<float> particle_velocity32(const KP& p, int i, V3<float> fluid_v, float sound_speed,
                                                         float vol, const V3<float>* gr) {
    if (p.motion == 0) return v3(0.f, 0.f, 0.f);  // Fixed
    if (p.motion == 3) return fluid_v;            // Fluid
    const V3<float> d = f32v(C3(p, F_CEN, i) - C3(p, F_LOC, i));
    if (p.motion == 1) {  // Steer
        const float abs_d = len(d);
        const float eta_r = 0.25f * radius32(vol, p.dim);
        if (abs_d > 0.9f * eta_r) {
            float fac = 0.99f * sound_speed / abs_d;
            if (abs_d < 1.1f * eta_r) fac *= 5.f * (abs_d - 0.9f * eta_r) / eta_r;
            return fluid_v + fac * d;
        }
        return fluid_v;
    }
    // SteerPakmor
    const float alpha = 2.f / (float)p.dim * f32(C(p, F_MAOR, i));
    const float beta = 2.25f;
    const float eta = fmaxf(0.f, fminf(0.5f, 2.f / beta * (alpha - 0.75f * beta)));
    const V3<float> dn = (1.f / len(d)) * d;
    // curl of the velocity gradient (physical_quantities.rs:149-155); gr[q] = d(quantity q)/d(x, y, z)
    const V3<float> curl = v3(gr[3].y - gr[2].z, gr[1].z - gr[3].x, gr[2].x - gr[1].y);
    const float v_reg = radius32(vol, p.dim) * len(curl);
    return fluid_v + (eta * fmaxf(sound_speed, v_reg)) * dn;
}
__device__ __forceinline__ double particle_timestep32(const KP& p, int i, const V3<float>* gr) {
    const St<double> cons = C5(p, F_CONS, i);
    if (is_zero64(cons.q[0])) {
        W3(p, F_V, i, v3(0., 0., 0.));
        return INFINITY;
    }
    const Gas<float> g = gas_t<float>(p);
    const float m_inv = 1.f / f32(cons.q[0]);
    const V3<float> dxg = f32v(C3(p, F_LOC, i) - C3(p, F_GC, i));
    const V3<float> d_v = v3(dot(gr[1], dxg), dot(gr[2], dxg), dot(gr[3], dxg));
    const V3<float> fluid_v = m_inv * f32v(vel(cons)) + d_v;
    const St<double> prim = C5(p, F_PRIM, i);
    const float u = f32(cons.q[4] - 0.5 * dot(vel(cons), vel(prim))) * m_inv;  // Particle::internal_energy
    const float vol = f32(C(p, F_VOL, i));
    const float c = g.sound_speed(g.pressure_from_internal_energy(u, f32(prim.q[0])), vol * m_inv);
    const V3<float> v = particle_velocity32(p, i, fluid_v, c, vol, gr);
    if (!isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z)) set_err(p, inst_of(p, i), 1u << 4);  // part.rs:366
    const V3<float> v_rel = fluid_v - v;
    W3(p, F_V, i, f64v(v));
    W3(p, F_VREL, i, f64v(v_rel));
    W(p, F_MAOR, i, 0.);
    const float v_max = fmaxf(f32(C(p, F_MSV, i)), len(v_rel) + c);
    W(p, F_MSV, i, 0.);
    if (v_max > 0.f) return f64(f32(p.cfl) * radius32(vol, p.dim) / v_max);
    return INFINITY;
}

// The cell's timestep for the integer timeline: FP32 (particle_timestep32),
// except where dt / time_base lies within ~1e-5 of a power of two, where the
// FP32 error could move it into the neighbouring time bin: there the FP64
// particle_timestep decides, as in the plain form.  max_signal_velocity,
// which the timestep consumes and resets, is put back first.
__device__ __forceinline__ double cell_timestep32(const KP& p, int i, int k, const V3<float>* gr) {
    const double msv = C(p, F_MSV, i);
    const double dt = particle_timestep32(p, i, gr);
    const unsigned long long b = (unsigned long long)__double_as_longlong(dt * tbase_inv(p, k));
    const unsigned long long frac = b & ((1ull << 52) - 1ull);  // distance of the mantissa from 1 and from 2
    const unsigned long long near = 1ull << 35;                 // 2^-17 ~ 7.6e-6
    if (is_finite64(dt) && (frac < near || frac > (1ull << 52) - near)) {
        W(p, F_MSV, i, msv);
        return particle_timestep(p, i);
    }
    return dt;
}

__device__ __forceinline__ void gradients32_cell(const KP& p, int i) {
    unsigned long long my_dti = MAX_NR_TIMESTEPS;
    int my_tb = 127;
    unsigned int err = 0;
    int k = i >= 0 ? inst_of(p, i) : -1;
    if (k >= 0 && p.tl[k].done) k = -1;
    if (k >= 0) {
        int tb = p.timebin[i];
        if (p.active[i]) {
            mark_dirty(p, i);
          V3<float> gr[5];
#pragma unroll
          for (int q = 0; q < 5; q++) gr[q] = v3(0.f, 0.f, 0.f);
          if (!p.godunov) {  // GodunovHydroRunner::step has no gradient stage (godunov.rs:14-58)
            St<float> prim = G5(p, G_PRIM, i);
            float a00 = 0.f, a01 = 0.f, a02 = 0.f, a11 = 0.f, a12 = 0.f, a22 = 0.f;
            if (p.dim == 1) { a11 = 1.f; a22 = 1.f; }
            else if (p.dim == 2) { a22 = 1.f; }
            // LimiterData (gradients.rs:58-103) on differences to this cell's
            // state: the neighbours' differences are gathered here, the
            // extrapolations (which need the gradient) in a second pass
            float dmn[5], dmx[5];
#pragma unroll
            for (int q = 0; q < 5; q++) {
                dmn[q] = 0.f;
                dmx[q] = 0.f;
            }
            int k0 = p.csr_off[i], k1 = p.csr_off[i + 1];
            for (int k = k0; k < k1; k++) {
                int f = p.csr_face[k];
                St<float> op;
                V3<float> ds, d;
                other_side32(p, i, f, prim, op, ds, d);
                float w = p.geo[GE_W * (size_t)p.nf + f];
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    const float dq = op.q[q] - prim.q[q];
                    gr[q] = gr[q] + (w * dq) * ds;
                    dmn[q] = fminf(dmn[q], dq);
                    dmx[q] = fmaxf(dmx[q], dq);
                }
                a00 += w * ds.x * ds.x;
                a01 += w * ds.x * ds.y;
                a02 += w * ds.x * ds.z;
                a11 += w * ds.y * ds.y;
                a12 += w * ds.y * ds.z;
                a22 += w * ds.z * ds.z;
            }
            V3<float> m0 = v3(a00, a01, a02), m1 = v3(a01, a11, a12), m2 = v3(a02, a12, a22);
            V3<float> t0 = cross(m1, m2), t1 = cross(m2, m0), t2 = cross(m0, m1);
            float inv_det = 1.f / dot(m2, t2);
            V3<float> r0 = inv_det * t0, r1 = inv_det * t1, r2 = inv_det * t2;
            bool finite = true;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                V3<float> x = gr[q];
                gr[q] = v3(dot(r0, x), dot(r1, x), dot(r2, x));  // symmetric inverse: rows = columns
                finite = finite && isfinite(gr[q].x) && isfinite(gr[q].y) && isfinite(gr[q].z);
            }
            if (!finite) {
#pragma unroll
                for (int q = 0; q < 5; q++) gr[q] = v3(0.f, 0.f, 0.f);
            }
            float emn[5], emx[5];
#pragma unroll
            for (int q = 0; q < 5; q++) {
                emn[q] = INFINITY;
                emx[q] = -INFINITY;
            }
            for (int k = k0; k < k1; k++) {
                const int f = p.csr_face[k];
                // the limiter's extrapolation vector seen from cell i (as other_side32)
                const V3<float> d = p.left[f] == i ? GE3(p, GE_DL, f) : GE3(p, GE_DR, f);
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    float ex = dot(gr[q], d);
                    emn[q] = fminf(emn[q], ex);
                    emx[q] = fmaxf(emx[q], ex);
                }
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
                float alpha = (emx[q] == 0.f || emn[q] == 0.f) ? 1.f : fminf(1.f, fminf(dmx[q] / emx[q], dmn[q] / emn[q]));
                gr[q] = alpha * gr[q];
                W3(p, F_GRAD + 3 * q, i, f64v(gr[q]));
            }
            V3<double> cen = C3(p, F_CEN, i);
            W3(p, F_GC, i, cen);
            if (p.cf_fresh) {
                // the FP32 copies next predict would make from these rows; on a
                // fixed mesh the timestep sets the mesh velocity to zero
                const size_t n = (size_t)p.n;
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    p.cf[(G_GRAD + 3 * q + 0) * n + i] = gr[q].x;
                    p.cf[(G_GRAD + 3 * q + 1) * n + i] = gr[q].y;
                    p.cf[(G_GRAD + 3 * q + 2) * n + i] = gr[q].z;
                }
                const V3<double> dgc = cen - C3(p, F_LOC, i);
                p.cf[(G_DGC + 0) * n + i] = f32(dgc.x);
                p.cf[(G_DGC + 1) * n + i] = f32(dgc.y);
                p.cf[(G_DGC + 2) * n + i] = f32(dgc.z);
#pragma unroll
                for (int a = 0; a < 3; a++) p.cf[(G_V + a) * n + i] = 0.f;
                p.cf_fresh[i] = 1;
            }
          } else {
            // no gradient stage: the stored gradients (velocity rows) feed the timestep
#pragma unroll
            for (int q = 1; q < 4; q++) gr[q] = f32v(C3(p, F_GRAD + 3 * q, i));
          }
            double dt_new = limit_by_gravity(p, i, cell_timestep32(p, i, k, gr));
            unsigned long long tc = p.tl[k].ti_current;
            unsigned long long dti = make_integer_timestep(dt_new, tb, NUM_TIME_BINS, tc, tbase_inv(p, k));
            if (dti == 0) err |= 1u << 6;
            W(p, F_DT, i, (double)dti * tbase(p, k));
            tb = get_time_bin(dti);
            my_dti = dti;
        }
        p.tb_tmp[i] = (int8_t)tb;
        my_tb = tb;
    }
    if (err) set_err(p, k, err);
    inst_min_dti_tb(p, k, my_dti, my_tb);
}
// Hierarchical steps: a warp per listed cell (lanes over the faces, the WLS
// sums folded in CSR order from the lanes' registers, the limiter's minima and
// maxima reduced across the warp), as gradients_cell_warp in the plain form.
__device__ __forceinline__ void gradients32_cell_warp(const KP& p, int i, int lane) {
    unsigned long long my_dti = MAX_NR_TIMESTEPS;
    int my_tb = 127;
    unsigned int err = 0;
    int k = inst_of(p, i);
    if (p.tl[k].done) k = -1;
    if (k >= 0) {
        int tb = p.timebin[i];
        if (p.active[i]) {
            mark_dirty(p, i);
          V3<float> gr[5];
#pragma unroll
          for (int q = 0; q < 5; q++) gr[q] = v3(0.f, 0.f, 0.f);
          if (!p.godunov) {
            St<float> prim = G5(p, G_PRIM, i);
            float a00 = 0.f, a01 = 0.f, a02 = 0.f, a11 = 0.f, a12 = 0.f, a22 = 0.f;
            if (p.dim == 1) { a11 = 1.f; a22 = 1.f; }
            else if (p.dim == 2) { a22 = 1.f; }
            const int k0 = p.csr_off[i], deg = p.csr_off[i + 1] - k0;
            for (int j0 = 0; j0 < deg; j0 += 32) {  // warp-uniform
                float w = 0.f, dq[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
                V3<float> ds = v3(0.f, 0.f, 0.f);
                if (j0 + lane < deg) {
                    int f = p.csr_face[k0 + j0 + lane];
                    St<float> op;
                    V3<float> d;
                    other_side32(p, i, f, prim, op, ds, d);
                    w = p.geo[GE_W * (size_t)p.nf + f];
#pragma unroll
                    for (int q = 0; q < 5; q++) dq[q] = op.q[q] - prim.q[q];
                }
                const int n = min(32, deg - j0);
                for (int t = 0; t < n; t++) {
                    const float wt = __shfl_sync(0xffffffffu, w, t);
                    const V3<float> dst = v3(__shfl_sync(0xffffffffu, ds.x, t), __shfl_sync(0xffffffffu, ds.y, t),
                                             __shfl_sync(0xffffffffu, ds.z, t));
#pragma unroll
                    for (int q = 0; q < 5; q++) gr[q] = gr[q] + (wt * __shfl_sync(0xffffffffu, dq[q], t)) * dst;
                    a00 += wt * dst.x * dst.x;
                    a01 += wt * dst.x * dst.y;
                    a02 += wt * dst.x * dst.z;
                    a11 += wt * dst.y * dst.y;
                    a12 += wt * dst.y * dst.z;
                    a22 += wt * dst.z * dst.z;
                }
            }
            V3<float> m0 = v3(a00, a01, a02), m1 = v3(a01, a11, a12), m2 = v3(a02, a12, a22);
            V3<float> t0 = cross(m1, m2), t1 = cross(m2, m0), t2 = cross(m0, m1);
            float inv_det = 1.f / dot(m2, t2);
            V3<float> r0 = inv_det * t0, r1 = inv_det * t1, r2 = inv_det * t2;
            bool finite = true;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                V3<float> x = gr[q];
                gr[q] = v3(dot(r0, x), dot(r1, x), dot(r2, x));
                finite = finite && isfinite(gr[q].x) && isfinite(gr[q].y) && isfinite(gr[q].z);
            }
            if (!finite) {
#pragma unroll
                for (int q = 0; q < 5; q++) gr[q] = v3(0.f, 0.f, 0.f);
            }
            float dmn[5], dmx[5], emn[5], emx[5];
#pragma unroll
            for (int q = 0; q < 5; q++) {
                dmn[q] = 0.f;
                dmx[q] = 0.f;
                emn[q] = INFINITY;
                emx[q] = -INFINITY;
            }
            for (int j = lane; j < deg; j += 32) {
                int f = p.csr_face[k0 + j];
                St<float> op;
                V3<float> ds, d;
                other_side32(p, i, f, prim, op, ds, d);
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    float ex = dot(gr[q], d);
                    float dq = op.q[q] - prim.q[q];
                    dmn[q] = fminf(dmn[q], dq);
                    dmx[q] = fmaxf(dmx[q], dq);
                    emn[q] = fminf(emn[q], ex);
                    emx[q] = fmaxf(emx[q], ex);
                }
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    dmn[q] = fminf(dmn[q], __shfl_xor_sync(0xffffffffu, dmn[q], o));
                    dmx[q] = fmaxf(dmx[q], __shfl_xor_sync(0xffffffffu, dmx[q], o));
                    emn[q] = fminf(emn[q], __shfl_xor_sync(0xffffffffu, emn[q], o));
                    emx[q] = fmaxf(emx[q], __shfl_xor_sync(0xffffffffu, emx[q], o));
                }
                float alpha = (emx[q] == 0.f || emn[q] == 0.f) ? 1.f : fminf(1.f, fminf(dmx[q] / emx[q], dmn[q] / emn[q]));
                gr[q] = alpha * gr[q];
                if (lane == 0) W3(p, F_GRAD + 3 * q, i, f64v(gr[q]));
            }
            if (lane == 0) W3(p, F_GC, i, C3(p, F_CEN, i));
          } else {
#pragma unroll
            for (int q = 1; q < 4; q++) gr[q] = f32v(C3(p, F_GRAD + 3 * q, i));
          }
            if (lane == 0) {
                double dt_new = limit_by_gravity(p, i, cell_timestep32(p, i, k, gr));
                unsigned long long tc = p.tl[k].ti_current;
                unsigned long long dti = make_integer_timestep(dt_new, tb, NUM_TIME_BINS, tc, tbase_inv(p, k));
                if (dti == 0) err |= 1u << 6;
                W(p, F_DT, i, (double)dti * tbase(p, k));
                tb = get_time_bin(dti);
                my_dti = dti;
            }
        }
        if (lane == 0) {
            p.tb_tmp[i] = (int8_t)tb;
            my_tb = tb;
        }
    }
    if (err) set_err(p, k, err);
    inst_min_dti_tb(p, lane == 0 ? k : -1, my_dti, my_tb);
}

// LIST: hierarchical step, a warp per listed cell.  The two forms are separate
// instantiations so that the all-cells kernel keeps its own register budget.
template <bool LIST>
__global__ void __launch_bounds__(kMaxBlock) k_gradients32(KP p) {
    const int n_items = cell_items(p);
    if (LIST) {
        const int lane = threadIdx.x & 31, n_warps = (gridDim.x * blockDim.x) >> 5;
        for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n_items; w += n_warps)
            gradients32_cell_warp(p, p.cell_list[w], lane);
        return;
    }
    // warp-uniform trip count: the per-instance reductions need every lane
    for (int base = blockIdx.x * blockDim.x; base < n_items; base += gridDim.x * blockDim.x) {
        int idx = base + threadIdx.x;
        gradients32_cell(p, idx < n_items ? cell_at(p, idx) : -1);
    }
}

template <int SOLVER, bool SAMPLE>
__global__ void k_riemann32(double gamma, int64_t n, const double* l, const double* r, const double* vf,
                            const double* nrm, double* out, unsigned int* errp, RSx x) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Gas<float> g = make_gas<float>(gamma, 0, 0.);
    Gas<double> g64 = make_gas<double>(gamma, 0, 0.);
    St<float> L, R;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        L.q[q] = (float)l[q * n + i];
        R.q[q] = (float)r[q * n + i];
    }
    V3<float> nn = v3((float)nrm[i], (float)nrm[n + i], (float)nrm[2 * n + i]);
    unsigned int err = 0;
    St<float> o;
    if (SAMPLE) {
        o = star_half_state<float, SOLVER>(L, R, nn, g, g64, 1000, &err, &x);
    } else {
        V3<float> iv = v3((float)vf[i], (float)vf[n + i], (float)vf[2 * n + i]);
        o = solve_for_flux<float, SOLVER>(L, R, iv, nn, g, g64, 1000, &err, &x);
    }
#pragma unroll
    for (int q = 0; q < 5; q++) out[q * n + i] = (double)o.q[q];
    err &= ~kInfoFallback;
    if (err) atomicOr(errp, err);
}

inline int grid(int n, int b = kBlock) { return (n + b - 1) / b; }

}  // namespace

void launch_predict32(const KP& p, cudaStream_t s) {
    if (p.n > 0) k_predict32<<<dim3(grid(p.n, p.blk_cell), 2), p.blk_cell, 0, s>>>(p);
}

void launch_prep32(const KP& p, cudaStream_t s) {
    if (p.n > 0) k_prep32<<<cell_grid(p), p.blk_cell, 0, s>>>(p);
}

void launch_geom32(const KP& p, bool check, cudaStream_t s) {
    KP q = p;
    q.geo_check = check ? 1 : 0;
    if (q.n > 0) k_geom_check<<<grid(q.n, kBlock), kBlock, 0, s>>>(q, check ? 0 : 1);
    if (q.nf > 0) k_geom32<<<grid(q.nf, kBlock), kBlock, 0, s>>>(q);
}

void launch_gradients32(const KP& p, cudaStream_t s) {
    if (p.n <= 0) return;
    if (p.use_list) k_gradients32<true><<<cell_grid(p), p.blk_cell, 0, s>>>(p);
    else k_gradients32<false><<<cell_grid(p), p.blk_cell, 0, s>>>(p);
}

void launch_face_flux_fp32(const KP& p, int solver, cudaStream_t s) {
    if (p.nf <= 0) return;
    int g = grid(p.nf, p.blk_face), cap = p.n_sms * 512 / p.blk_face;
    if (p.use_list && g > cap) g = cap;
    if (solver == SOLVER_HLLC) k_face_flux32<SOLVER_HLLC><<<g, p.blk_face, 0, s>>>(p);
    else if (solver == SOLVER_EXACT) k_face_flux32<SOLVER_EXACT><<<g, p.blk_face, 0, s>>>(p);
    else if (solver == SOLVER_PVRS) k_face_flux32<SOLVER_PVRS><<<g, p.blk_face, 0, s>>>(p);
    else k_face_flux32<SOLVER_EXTRA><<<g, p.blk_face, 0, s>>>(p);
}

void launch_riemann_fp32(int kind, int sample, double gamma, int64_t n, const double* l, const double* r,
                         const double* vf, const double* nrm, double* out, unsigned int* err, const RSx& x,
                         cudaStream_t s) {
    if (n <= 0) return;
    int g = (int)((n + kBlock - 1) / kBlock);
    if (sample) {
        if (kind == SOLVER_PVRS) k_riemann32<SOLVER_PVRS, true><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else if (kind >= SOLVER_AIRS && kind <= SOLVER_TRRS)
            k_riemann32<SOLVER_EXTRA, true><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else k_riemann32<SOLVER_EXACT, true><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
    } else {
        if (kind == SOLVER_HLLC) k_riemann32<SOLVER_HLLC, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else if (kind == SOLVER_EXACT) k_riemann32<SOLVER_EXACT, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else if (kind == SOLVER_PVRS) k_riemann32<SOLVER_PVRS, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
        else k_riemann32<SOLVER_EXTRA, false><<<g, kBlock, 0, s>>>(gamma, n, l, r, vf, nrm, out, err, x);
    }
}

}  // namespace mvmm
