// Plain-FP64 face and cell-update physics shared by the context kernels
// (step_fp64.cu) and the allocation-free entry point (noalloc.cu).  Both
// translation units are compiled with -fmad=false, so every expression rounds
// as the Rust reference evaluates it.
//
// The face functions read the cell state through an accessor A, which hides
// where the state lives (the context's 60-row block, or the caller's
// mvmm_cells arrays).  An accessor provides, for cell i and face f:
//   St<double> prim(i); V3<double> gc(i), cen(i), loc(i), v(i);
//   double dt(i), cs(i)          (sound speed for v_max, 0 where rho <= 0);
//   double gdot(i, q, dx)        (Gradients::dot row q);
//   double extrap(i, q);
//   St<double> src(i, prim)      (time_extrapolations source, part.rs:134-149;
//                                 read only where prim.rho > 0);
//   V3<double> fcen(f), shift(f), normal(f); double area(f);
//   int boundary()               (MVMM_BOUNDARY_*).
#pragma once

#include "mvmm_device.cuh"
#include "mvmm_gpu.h"

namespace mvmm {
namespace {

struct FaceOut {
    St<double> fl;
    V3<double> mflux;
    double v_max, a_over_r;
};
// A face up to its Riemann solve: the two states handed to the solver (in the
// face frame), the face velocity and normal, and what the result needs.
struct FacePre {
    St<double> l, r;
    V3<double> iv, n, dx;
    double dt, area, v_max;
};
// ... and from the solver's flux on (flux_exchange, flux.rs:85-99)
__device__ __forceinline__ FaceOut face_finish(const FacePre& q, const St<double>& F) {
    St<double> fluxes = q.area * F;
    FaceOut o;
    o.fl = q.dt * fluxes;
    o.mflux = fluxes.q[0] * q.dx;
    o.v_max = q.v_max;
    o.a_over_r = q.area / len(q.dx);
    return o;
}
__device__ __forceinline__ FaceOut face_zero() {
    FaceOut o;
    o.fl = st_zero<double>();
    o.mflux = v3(0., 0., 0.);
    o.v_max = 0.;
    o.a_over_r = 0.;
    return o;
}

// reconstructed state: ((prim + grad.dx) + extrap) + time_extrapolations(-0.5 dt)
// (flux.rs:52-60, part.rs:134-149)
template <class A>
__device__ __forceinline__ St<double> reconstruct(const A& a, int i, const St<double>& prim, V3<double> dx, double td) {
    St<double> r;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        double v = prim.q[q] + a.gdot(i, q, dx);
        v = v + a.extrap(i, q);
        r.q[q] = v;
    }
    if (prim.q[0] > 0.) {
        const St<double> s = a.src(i, prim);
#pragma unroll
        for (int q = 0; q < 5; q++) r.q[q] = r.q[q] + td * s.q[q];
    } else {
#pragma unroll
        for (int q = 0; q < 5; q++) r.q[q] = r.q[q] + 0.;
    }
    return r;
}

// flux_exchange (flux.rs:23-100) up to the Riemann solve
template <class A>
__device__ __forceinline__ FacePre face_interior_pre(const A& a, int f, int l, int r, double dt) {
    V3<double> fc = a.fcen(f);
    V3<double> sh = a.shift(f);
    V3<double> dx_left = fc - a.gc(l);
    V3<double> dx_right = (fc - a.gc(r)) - sh;
    double dx_gradients = len(dx_left - dx_right);
    V3<double> dx_centroid = (a.cen(r) + sh) - a.cen(l);
    V3<double> locl = a.loc(l), locr = a.loc(r);
    V3<double> dx = (locr + sh) - locl;
    St<double> pl = a.prim(l), pr = a.prim(r);
    double v_max = 0. + a.cs(l);
    v_max = v_max + a.cs(r);
    v_max -= m_min(dot(vel(pr) - vel(pl), dx_centroid), 0.);
    double td = -(-0.5 * dt);  // -dt_extrapolate in time_extrapolations
    St<double> ldash = reconstruct(a, l, pl, dx_left, td);
    St<double> rdash = reconstruct(a, r, pr, dx_right, td);
    St<double> prim_left = pairwise_limiter(pl, pr, ldash, len(dx_left) / dx_gradients);
    St<double> prim_right = pairwise_limiter(pr, pl, rdash, len(dx_right) / dx_gradients);
    V3<double> vl = a.v(l), vr = a.v(r);
    V3<double> midpoint = 0.5 * ((locl + locr) + sh);
    double fac = dot(vr - vl, fc - midpoint) / len2(dx);
    V3<double> v_face = 0.5 * (vl + vr) - fac * dx;
    V3<double> mvf = neg(v_face);
    FacePre q;
    q.l = boost(prim_left, mvf);
    q.r = boost(prim_right, mvf);
    q.iv = v_face;
    q.n = a.normal(f);
    q.dx = dx;
    q.dt = dt;
    q.area = a.area(f);
    q.v_max = v_max;
    return q;
}

// flux_exchange_boundary (flux.rs:102-195) with Space::get_boundary_part
// semantics (space.rs:213-229) up to the Riemann solve
template <class A>
__device__ __forceinline__ FacePre face_boundary_pre(const A& a, int f, int i) {
    V3<double> fc = a.fcen(f);
    V3<double> n = a.normal(f);
    V3<double> loc = a.loc(i), cen = a.cen(i), gc = a.gc(i);
    // Particle::reflect (part.rs:374-383)
    V3<double> rloc = loc + (2. * dot(fc - loc, n)) * n;
    V3<double> rcen = cen + (2. * dot(fc - cen, n)) * n;
    V3<double> rgc = gc + (2. * dot(fc - gc, n)) * n;
    V3<double> dx_face = fc - gc;
    double dx_gradients = len(rgc - gc);
    V3<double> dx_centroid = rcen - cen;
    V3<double> dx = rloc - loc;
    St<double> prim = a.prim(i);
    double v_max = 0. + a.cs(i);
    double dt = a.dt(i);
    double td = -(-0.5 * dt);
    St<double> dash = reconstruct(a, i, prim, dx_face, td);
    double dx_fac = len(dx_face) / dx_gradients;
    St<double> bnd;
    const int boundary = a.boundary();
    if (boundary == MVMM_BOUNDARY_REFLECTIVE) {
        St<double> rprim = reflect(prim, n);
        dash = pairwise_limiter(prim, rprim, dash, dx_fac);
        v_max -= m_min(dot(vel(rprim) - vel(prim), dx_centroid), 0.);
        bnd = reflect(dash, n);
    } else if (boundary == MVMM_BOUNDARY_OPEN) {
        dash = pairwise_limiter(prim, prim, dash, dx_fac);
        bnd = dash;
    } else {  // vacuum
        St<double> vac = st_zero<double>();
        dash = pairwise_limiter(prim, vac, dash, dx_fac);
        v_max += m_min(dot(vel(prim), dx_centroid), 0.);
        bnd = vac;
    }
    FacePre q;
    q.l = dash;
    q.r = bnd;
    q.iv = v3(0., 0., 0.);
    q.n = n;
    q.dx = dx;
    q.dt = dt;
    q.area = a.area(f);
    q.v_max = v_max;
    return q;
}

// Particle::apply_flux (part.rs:178-193) of an active cell: the conserved
// state after adding the summed fluxes.
__device__ __forceinline__ St<double> apply_flux64(const St<double>& cons_in, const St<double>& facc,
                                                   unsigned int* err) {
    St<double> cons = cons_in + facc;
    if (!is_finite64(cons.q[0]) || !is_finite64(cons.q[1]) || !is_finite64(cons.q[2]) || !is_finite64(cons.q[3]) ||
        !is_finite64(cons.q[4]))
        *err |= MVMM_ERR_NONFINITE;
    if (lt0_64(cons.q[0])) cons = st_zero<double>();
    if (lt0_64(cons.q[4])) cons = st_zero<double>();
    return cons;
}
// kick2 / kick1 as the reference's runners run them: Particle::grav_kick with
// the zero acceleration they leave in a_grav adds +0 to the momentum
// (part.rs:303-312); the mass and energy additions leave those rows' bits as
// they are.
__device__ __forceinline__ St<double> zero_kick64(St<double> cons) {
    cons.q[1] = cons.q[1] + 0.;
    cons.q[2] = cons.q[2] + 0.;
    cons.q[3] = cons.q[3] + 0.;
    return cons;
}
// Particle::grav_kick (part.rs:303-312) with acceleration a over half of dt.
// gravity_mflux is zero whenever a kick runs (apply_flux resets it before
// kick2, and nothing accumulates into an active cell's after that), so the
// energy gains (dt/2) a . momentum.
__device__ __forceinline__ St<double> grav_kick64(const St<double>& cons, double dt, V3<double> a) {
    const V3<double> k = (0.5 * dt) * a;
    const double mass = cons.q[0];
    const V3<double> mom = vel(cons);
    const V3<double> mflux0 = v3(0., 0., 0.);
    St<double> out;
    out.q[0] = cons.q[0] + 0.;
    out.q[1] = cons.q[1] + k.x * mass;
    out.q[2] = cons.q[2] + k.y * mass;
    out.q[3] = cons.q[3] + k.z * mass;
    out.q[4] = cons.q[4] + dot(k, mom - mflux0);
    return out;
}

// Particle::convert_conserved_to_primitive (part.rs:219-261) with
// State<Primitive>::from_conserved (physical_quantities.rs:213-226).
__device__ __forceinline__ St<double> c2p64(const St<double>& cons, double volume, const Gas<double>& g,
                                            unsigned int* err) {
    if (!ge0_64(cons.q[0])) *err |= MVMM_ERR_NEG_MASS;
    if (!ge0_64(cons.q[4])) *err |= MVMM_ERR_NEG_ENERGY;
    St<double> prim;
    if (is_zero64(cons.q[0])) {
        if (!is_zero64(cons.q[4])) *err |= MVMM_ERR_NEG_ENERGY;
        prim = st_zero<double>();
    } else if (gt0_64(cons.q[0])) {
        double m_inv = 1. / cons.q[0];
        double density = cons.q[0] / volume;
        V3<double> velocity = m_inv * vel(cons);
        double thermal = cons.q[4] - 0.5 * len2(vel(cons)) * m_inv;
        double u = thermal * m_inv;
        double pressure = g.pressure_from_internal_energy(u, density);
        prim = st(density, velocity, pressure);
    } else {
        prim = st_zero<double>();
    }
    if (!ge0_64(prim.q[0]) || !ge0_64(prim.q[4])) *err |= MVMM_ERR_NEG_PRIM;
    if (!is_finite64(prim.q[0]) || !is_finite64(prim.q[1]) || !is_finite64(prim.q[2]) || !is_finite64(prim.q[3]) ||
        !is_finite64(prim.q[4]))
        *err |= MVMM_ERR_NONFINITE;
    return prim;
}

}  // namespace
}  // namespace mvmm
