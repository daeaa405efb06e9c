// Cell-state accessors and per-cell helpers shared by the kernels of both
// arithmetic forms (each translation unit gets its own copy: the plain form is
// compiled without FMA contraction, the FP32-face form with it).
#pragma once

#include "mvmm_device.cuh"
#include "mvmm_gpu.h"
#include "mvmm_internal.h"

namespace mvmm {
namespace {

constexpr int kBlock = 128;     // default block of the step kernels
constexpr int kMaxBlock = 256;  // largest block the autotuner may choose

__device__ __forceinline__ double C(const KP& p, int f, int i) { return p.cd[(size_t)f * p.n + i]; }
__device__ __forceinline__ void W(const KP& p, int f, int i, double v) { p.cd[(size_t)f * p.n + i] = v; }
__device__ __forceinline__ V3<double> C3(const KP& p, int f, int i) {
    return {C(p, f, i), C(p, f + 1, i), C(p, f + 2, i)};
}
__device__ __forceinline__ void W3(const KP& p, int f, int i, V3<double> v) {
    W(p, f, i, v.x);
    W(p, f + 1, i, v.y);
    W(p, f + 2, i, v.z);
}
__device__ __forceinline__ St<double> C5(const KP& p, int f, int i) {
    St<double> s;
#pragma unroll
    for (int q = 0; q < 5; q++) s.q[q] = C(p, f + q, i);
    return s;
}
__device__ __forceinline__ void W5(const KP& p, int f, int i, const St<double>& s) {
#pragma unroll
    for (int q = 0; q < 5; q++) W(p, f + q, i, s.q[q]);
}
__device__ __forceinline__ V3<double> F3(const double* a, int nf, int f) { return {a[f], a[nf + f], a[2 * nf + f]}; }
// The gas law in type T from the host-evaluated constants; equal to
// make_gas<T>(p.gamma, p.eos, p.iso_u) member by member.
template <typename T>
__device__ __forceinline__ Gas<T> gas_t(const KP& p) {
    Gas<T> g;
    g.gamma = T(p.gk.gamma);
    g.gamma_inv = T(p.gk.gamma_inv);
    g.odgm1_ = T(p.gk.odgm1);
    g.odgp1_ = T(p.gk.odgp1);
    g.iso_u = T(p.gk.iso_u);
    g.eos = p.gk.eos;
    g.rm = p.gk.rm;
    g.inv_m = p.gk.inv_m;
    return g;
}
__device__ __forceinline__ Gas<double> gas(const KP& p) { return gas_t<double>(p); }
__device__ __forceinline__ int inst_of(const KP& p, int cell) { return p.inst ? p.inst[cell] : 0; }
// A kernel rewrote rows of cell i that the host holds (mvmm_step_cells_changed
// copies back only such cells): its extrapolations only (kDirtyExtrap), or any
// of its rows (kDirtyAll).  One thread, or the lanes of one warp with the same
// bits, marks a cell in a kernel.
__device__ __forceinline__ void mark_dirty(const KP& p, int i, uint8_t bits = kDirtyAll) {
    if (p.dirty) p.dirty[i] |= bits;
}
__device__ __forceinline__ double tbase(const KP& p, int k) { return p.inst_tb ? p.inst_tb[k] : p.time_base; }
__device__ __forceinline__ double tbase_inv(const KP& p, int k) { return p.inst_tbi ? p.inst_tbi[k] : p.time_base_inv; }
__device__ __forceinline__ void set_err(const KP& p, int k, unsigned int bits) {
    if (bits) atomicOr(&p.tl[k].err, bits);
}
// The cells a cell kernel visits: all cells, or in a hierarchical step the
// compacted list of active cells and the cells next to an active face (the
// other cells are left unchanged by every stage after predict).
__device__ __forceinline__ int cell_items(const KP& p) { return p.use_list ? (int)p.tl[0].n_clist : p.n; }
__device__ __forceinline__ int cell_at(const KP& p, int idx) { return p.use_list ? p.cell_list[idx] : idx; }
// Puts cell i on this step's cell list once (want: the lane has a candidate);
// aggregated over the warp.  Every lane of the warp calls it.  The active
// cells (predict) come first and are also counted in n_alist.
// Returns true on the lane that put the cell on the list.
__device__ __forceinline__ bool list_cell_warp(const KP& p, bool want, int i, bool active_cells = false) {
    want = want && atomicExch(&p.touch[i], 1u) == 0u;
    unsigned int b = __ballot_sync(0xffffffffu, want);
    if (!b) return false;
    int lane = threadIdx.x & 31, leader = __ffs(b) - 1;
    unsigned int start = 0;
    if (lane == leader) {
        start = atomicAdd(&p.tl[0].n_clist, (unsigned int)__popc(b));
        if (active_cells) atomicAdd(&p.tl[0].n_alist, (unsigned int)__popc(b));
    }
    start = __shfl_sync(0xffffffffu, start, leader);
    if (want) p.cell_list[start + __popc(b & ((1u << lane) - 1u))] = i;
    return want;
}
// The stamp of faces active in this step (hierarchical steps, one simulation).
__device__ __forceinline__ unsigned int face_stamp_now(const KP& p) { return (unsigned int)p.tl[0].steps + 1u; }

// Counter add per instance, aggregated over the lanes of a warp that share an
// instance (k < 0: the lane contributes nothing).  Every lane of the warp calls it.
enum { CNT_FACES = 0, CNT_CELLS = 1, CNT_FALLBACK = 2 };
__device__ __forceinline__ void inst_count(const KP& p, int k, bool flag, int which) {
    unsigned int grp = __match_any_sync(0xffffffffu, k);
    unsigned int cnt = __popc(__ballot_sync(0xffffffffu, flag) & grp);
    if (k >= 0 && cnt && (int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        DevTimeline* T = p.tl + k;
        unsigned long long* c = which == CNT_FACES ? &T->active_faces
                                : which == CNT_CELLS ? &T->active_cells : &T->fallback_faces;
        atomicAdd(c, (unsigned long long)cnt);
    }
}
// Per-instance minima of the integer timestep and the new time bin
// (timesteps_apply / timestep_sync reductions).  dti is 0 or a power of two
// (make_integer_timestep), so its bit index is an order-preserving 32-bit key.
__device__ __forceinline__ void inst_min_dti_tb(const KP& p, int k, unsigned long long dti, int tb) {
    unsigned int grp = __match_any_sync(0xffffffffu, k);
    unsigned int key = dti == 0 ? 0u : (unsigned int)(64 - __clzll((long long)dti));
    unsigned int kmin = __reduce_min_sync(grp, key);
    int tbmin = __reduce_min_sync(grp, tb);
    if (k >= 0 && (int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        atomicMin(&p.tl[k].min_dti, kmin == 0 ? 0ull : (1ull << (kmin - 1)));
        atomicMin(&p.tl[k].min_timebin, tbmin);
    }
}

// Gradients::dot row q with dx (physical_quantities.rs:122-133)
__device__ __forceinline__ double gdot(const KP& p, int i, int q, V3<double> dx) {
    return C(p, F_GRAD + 3 * q, i) * dx.x + C(p, F_GRAD + 3 * q + 1, i) * dx.y + C(p, F_GRAD + 3 * q + 2, i) * dx.z;
}

// The other side of face f as seen from cell i: Space::get_boundary_part for
// walls (space.rs:213-229), else the neighbour (runner/hydrodynamics.rs:59-65).
__device__ __forceinline__ void other_side(const KP& p, int i, int f, const St<double>& prim, V3<double> cen,
                                           St<double>& oprim, V3<double>& ocen, V3<double>& sh) {
    int l = p.left[f], r = p.right[f];
    V3<double> s = F3(p.shift, p.nf, f);
    sh = (i == l) ? s : neg(s);
    if (i == l && r < 0) {
        V3<double> fc = F3(p.fcen, p.nf, f);
        V3<double> n = F3(p.normal, p.nf, f);
        ocen = cen + (2. * dot(fc - cen, n)) * n;
        if (p.boundary == 1) oprim = reflect(prim, n);
        else if (p.boundary == 2) oprim = prim;
        else oprim = st_zero<double>();
    } else {
        int o = (i == l) ? r : l;
        ocen = C3(p, F_CEN, o);
        oprim = C5(p, F_PRIM, o);
    }
}

// Particle::radius (part.rs:439-447)
__device__ __forceinline__ double radius(double volume, int dim) {
    if (dim == 1) return 0.5 * volume;
    if (dim == 2) return sqrt(0.31830988618379067154 * volume);
    double x = 0.25 * 3. * 0.31830988618379067154 * volume, y, r;
    if (rat_root(x, 3, 1. / 3., y, r)) return r;  // x^(1/3) (cube root by Newton, see rat_root)
    return pow(x, 1. / 3.);
}

// ---- gravity (gravity.rs) ----
// ExternalPotentialGravity::compute_accelerations at a generator position:
// Potential::Constant, or KeplerianPotential::acceleration (gravity.rs:125-136).
__device__ __forceinline__ V3<double> grav_acceleration(const KP& p, V3<double> pos) {
    if (p.grav == MVMM_GRAVITY_CONSTANT) return v3(p.grav_avec[0], p.grav_avec[1], p.grav_avec[2]);
    const V3<double> dx = pos - v3(p.grav_pos[0], p.grav_pos[1], p.grav_pos[2]);
    double r2 = len2(dx);
    const double r = sqrt(r2);
    if (r < p.grav_soft) r2 = r2 + p.grav_soft * p.grav_soft;
    const double d = r * r2;
    return v3(-dx.x / d, -dx.y / d, -dx.z / d);
}
// Cell i's a_grav where the accelerations are computed: self-gravity's from
// the last SelfGravity::compute_accelerations (k_self_gravity), an external
// potential's at the generator position.
__device__ __forceinline__ V3<double> cell_acceleration(const KP& p, int i) {
    if (p.grav == MVMM_GRAVITY_SELF) return v3(p.agrav[i], p.agrav[p.n + i], p.agrav[2 * p.n + i]);
    return grav_acceleration(p, C3(p, F_LOC, i));
}
// GravitySolver::compute_timesteps of cell i (gravity.rs:45-53, 71-73, 90-95,
// 119-123).  Self-gravity: sqrt(softening / |a_grav|), INFINITY where a_grav
// is zero (always, unless its accelerations are computed); the Keplerian
// potential: eta * r_2D / v_circ; the constant potential: INFINITY.
__device__ __forceinline__ double grav_timestep(const KP& p, int i) {
    if (p.grav == MVMM_GRAVITY_SELF) {
        if (!p.agrav) return INFINITY;
        const double a2 = len2(v3(p.agrav[i], p.agrav[p.n + i], p.agrav[2 * p.n + i]));
        if (a2 == 0.) return INFINITY;
        return sqrt(p.grav_soft / sqrt(a2));
    }
    if (p.grav != MVMM_GRAVITY_KEPLERIAN) return INFINITY;
    // eta * radius (in 2D whatever the dimensionality) / circular_velocity
    const V3<double> dx = C3(p, F_LOC, i) - v3(p.grav_pos[0], p.grav_pos[1], p.grav_pos[2]);
    const double r = sqrt(len2(dx));
    const double r_softened = r < p.grav_soft ? r + p.grav_soft : r;
    return 0.5 * sqrt(0.31830988618379067154 * C(p, F_VOL, i)) / sqrt(1. / r_softened);
}
// The runners take the gravity solver's timestep where it is smaller
// (runner/hydrodynamics/optimal_order.rs:47-50, godunov.rs:41-44).
__device__ __forceinline__ double limit_by_gravity(const KP& p, int i, double dt) {
    return p.grav ? m_min(dt, grav_timestep(p, i)) : dt;
}

// Particle::set_particle_velocity (part.rs:328-372): the velocity the
// generator drifts with over its next timestep.
__device__ __forceinline__ V3<double> particle_velocity(const KP& p, int i, V3<double> fluid_v, double sound_speed,
                                                        double vol) {
    if (p.motion == 0) return v3(0., 0., 0.);  // Fixed
    if (p.motion == 3) return fluid_v;         // Fluid
    V3<double> d = C3(p, F_CEN, i) - C3(p, F_LOC, i);
    if (p.motion == 1) {  // Steer
        double abs_d = len(d);
        double eta = 0.25;
        double eta_r = eta * radius(vol, p.dim);
        double xi = 0.99;
        if (abs_d > 0.9 * eta_r) {
            double fac = xi * sound_speed / abs_d;
            if (abs_d < 1.1 * eta_r) fac *= 5. * (abs_d - 0.9 * eta_r) / eta_r;
            return fluid_v + fac * d;
        }
        return fluid_v;
    }
    // SteerPakmor
    double alpha = 2. / (double)p.dim * C(p, F_MAOR, i);
    double beta = 2.25;
    double eta = m_max(0., m_min(0.5, 2. / beta * (alpha - 0.75 * beta)));
    V3<double> dn = (1.0 / len(d)) * d;  // DVec3::normalize: d * length_recip
    // curl of the velocity gradient (physical_quantities.rs:149-155), grad row 3q+k
    V3<double> curl = v3(C(p, F_GRAD + 10, i) - C(p, F_GRAD + 8, i), C(p, F_GRAD + 5, i) - C(p, F_GRAD + 9, i),
                         C(p, F_GRAD + 6, i) - C(p, F_GRAD + 4, i));
    double v_reg = radius(vol, p.dim) * len(curl);
    V3<double> vr = (eta * m_max(sound_speed, v_reg)) * dn;
    return fluid_v + vr;
}

// Particle::timestep (part.rs:42-84, 328-372); returns the dt.
__device__ __forceinline__ double particle_timestep(const KP& p, int i) {
    St<double> cons = C5(p, F_CONS, i);
    if (is_zero64(cons.q[0])) {
        W3(p, F_V, i, v3(0., 0., 0.));
        return INFINITY;
    }
    const Gas<double> g = gas(p);
    double m_inv = 1. / cons.q[0];
    V3<double> dxg = C3(p, F_LOC, i) - C3(p, F_GC, i);
    V3<double> d_v = v3(gdot(p, i, 1, dxg), gdot(p, i, 2, dxg), gdot(p, i, 3, dxg));
    V3<double> fluid_v = m_inv * vel(cons) + d_v;
    St<double> prim = C5(p, F_PRIM, i);
    double u = (cons.q[4] - 0.5 * dot(vel(cons), vel(prim))) / cons.q[0];  // Particle::internal_energy
    double vol = C(p, F_VOL, i);
    double c = g.sound_speed(g.pressure_from_internal_energy(u, prim.q[0]), vol * m_inv);
    V3<double> v = particle_velocity(p, i, fluid_v, c, vol);
    if (!is_finite64(v.x) || !is_finite64(v.y) || !is_finite64(v.z)) set_err(p, inst_of(p, i), 1u << 4);  // part.rs:366
    V3<double> v_rel = fluid_v - v;
    W3(p, F_V, i, v);
    W3(p, F_VREL, i, v_rel);
    W(p, F_MAOR, i, 0.);
    double v_max = m_max(C(p, F_MSV, i), len(v_rel) + c);
    W(p, F_MSV, i, 0.);
    if (v_max > 0.) return p.cfl * radius(vol, p.dim) / v_max;
    return INFINITY;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ int warp_min_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace
}  // namespace mvmm
