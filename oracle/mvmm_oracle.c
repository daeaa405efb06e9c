/*
 * CPU oracle: plain-C restatement of mvmm_hydro's OptimalOrderRunner::step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Nothing in the GPU product links or
 * calls this file.  Compile with -ffp-contract=off so that every expression is
 * evaluated in the same order and rounding as the Rust source (Rust never
 * contracts a*b+c into an FMA).  Rust semantics reproduced:
 *   - f64::min / f64::max  -> fmin / fmax (return the non-NaN operand);
 *   - `x as u64`           -> saturating conversion (NaN -> 0);
 *   - powf                 -> pow; glam dot products are x*x' + y*y' + z*z'
 *     evaluated left to right; glam DMat3::inverse is the cross-product
 *     adjugate divided by det = z_axis . (x_axis x y_axis).
 * All citations are paths inside the mvmm_hydro source tree.
 */
#include "mvmm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* glam-like value types                                               */
/* ------------------------------------------------------------------ */
typedef struct { double x, y, z; } vec3;
/* State<T>(f64, DVec3, f64): index 0 density/mass, 1..3 velocity/momentum,
 * 4 pressure/energy (physical_quantities.rs:16, 86-112). */
typedef struct { double q[5]; } state;
/* Gradients<T>(DVec3, [DVec3;3], DVec3) (physical_quantities.rs:115). */
typedef struct { vec3 g[5]; } grads;
/* DMat3: three columns. */
typedef struct { vec3 c0, c1, c2; } mat3;

static inline vec3 v3(double x, double y, double z) { vec3 r = {x, y, z}; return r; }
static inline vec3 vadd(vec3 a, vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3 vsub(vec3 a, vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 vscale(double s, vec3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline double vdot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vlen2(vec3 a) { return vdot(a, a); }
static inline double vlen(vec3 a) { return sqrt(vdot(a, a)); }
static inline vec3 vcross(vec3 a, vec3 b) {
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline int visfinite(vec3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
static inline double vcomp(vec3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

static inline state st(double a, vec3 b, double c) { state s = {{a, b.x, b.y, b.z, c}}; return s; }
static inline state st_vacuum(void) { state s = {{0., 0., 0., 0., 0.}}; return s; }
static inline state st_add(state a, state b) {
    state r; for (int i = 0; i < 5; i++) r.q[i] = a.q[i] + b.q[i]; return r;
}
static inline state st_sub(state a, state b) {
    state r; for (int i = 0; i < 5; i++) r.q[i] = a.q[i] - b.q[i]; return r;
}
static inline state st_scale(double s, state a) {
    state r; for (int i = 0; i < 5; i++) r.q[i] = s * a.q[i]; return r;
}
static inline vec3 st_vel(state s) { return v3(s.q[1], s.q[2], s.q[3]); }

/* Gradients::dot (physical_quantities.rs:122-133) */
static inline state gr_dot(const grads *g, vec3 dx) {
    state r;
    for (int i = 0; i < 5; i++) r.q[i] = vdot(g->g[i], dx);
    return r;
}
/* Gradients::div_v (physical_quantities.rs:145-147) */
static inline double gr_div_v(const grads *g) { return g->g[1].x + g->g[2].y + g->g[3].z; }
static inline int gr_isfinite(const grads *g) {
    for (int i = 0; i < 5; i++) if (!visfinite(g->g[i])) return 0;
    return 1;
}

/* ------------------------------------------------------------------ */
/* Gas law (gas_law.rs)                                                 */
/* ------------------------------------------------------------------ */
typedef struct { double gamma, gamma_inv, odgm1, odgp1; } adiabatic;
typedef struct { adiabatic g; int eos; double iso_u; } gaslaw;

static adiabatic adiabatic_from(double value) { /* gas_law.rs:9-18 */
    adiabatic a = {value, 1. / value, 1. / (value - 1.), 1. / (value + 1.)};
    return a;
}
static inline double gp1dg(const adiabatic *a) { return (a->gamma + 1.) * a->gamma_inv; }       /* :31-33 */
static inline double gm1d2g(const adiabatic *a) { return 0.5 * (a->gamma - 1.) * a->gamma_inv; } /* :35-37 */
static inline double gm1dgp1(const adiabatic *a) { return (a->gamma - 1.) * a->odgp1; }          /* :39-41 */
static inline double odgm1(const adiabatic *a) { return a->odgm1; }
static inline double tdgm1(const adiabatic *a) { return 2. * a->odgm1; }                          /* :47-49 */
static inline double tdgp1(const adiabatic *a) { return 2. * a->odgp1; }                          /* :51-53 */

/* gas_law.rs:81-88 */
static inline double gas_internal_energy_from_pressure(const gaslaw *e, double p, double rho_inv) {
    if (e->eos == ORC_EOS_IDEAL) return p * rho_inv * e->g.odgm1;
    return e->iso_u;
}
/* gas_law.rs:90-97 */
static inline double gas_pressure_from_internal_energy(const gaslaw *e, double u, double rho) {
    if (e->eos == ORC_EOS_IDEAL) return (e->g.gamma - 1.) * u * rho;
    return (e->g.gamma - 1.) * e->iso_u * rho;
}
/* gas_law.rs:99-106 */
static inline double sound_speed(const gaslaw *e, double p, double rho_inv) {
    if (e->eos == ORC_EOS_IDEAL) return sqrt(e->g.gamma * p * rho_inv);
    return sqrt(e->iso_u * e->g.gamma * (e->g.gamma - 1.));
}

/* ------------------------------------------------------------------ */
/* State helpers (physical_quantities.rs)                              */
/* ------------------------------------------------------------------ */
/* State<Primitive>::boost (:228-236) */
static inline state prim_boost(state s, vec3 vel) {
    if (s.q[0] > 0.) return st(s.q[0], vadd(st_vel(s), vel), s.q[4]);
    return s;
}
/* State<Primitive>::reflect (:239-242) */
static inline state prim_reflect(state s, vec3 n) {
    vec3 vel = st_vel(s);
    vec3 v = vsub(vel, vscale(2. * vdot(vel, n), n));
    return st(s.q[0], v, s.q[4]);
}
/* State<Primitive>::check_physical (:245-254); the eprintln is dropped. */
static inline void check_physical(state *s) {
    if (s->q[0] < 0.) *s = st_vacuum();
    if (s->q[4] < 0.) *s = st_vacuum();
}
/* State<Conserved>::internal_energy (:288-292) */
static inline double cons_internal_energy(state c) {
    double m_inv = 1. / c.q[0];
    double thermal = c.q[4] - 0.5 * vlen2(st_vel(c)) * m_inv;
    return thermal * m_inv;
}
/* State<Primitive>::from_conserved (:213-226) */
static state prim_from_conserved(state c, double volume, const gaslaw *e, uint32_t *err) {
    if (c.q[0] > 0.) {
        double m_inv = 1. / c.q[0];
        double density = c.q[0] / volume;
        vec3 velocity = vscale(m_inv, st_vel(c));
        double u = cons_internal_energy(c);
        double pressure = gas_pressure_from_internal_energy(e, u, density);
        if (!(density >= 0.) || !(pressure >= 0.)) *err |= ORC_ERR_NEG_PRIM;
        /* DVec3 * f64 multiplies each component: velocity.k * m_inv. */
        velocity = v3(c.q[1] * m_inv, c.q[2] * m_inv, c.q[3] * m_inv);
        return st(density, velocity, pressure);
    }
    return st_vacuum();
}
/* State<Conserved>::from_primitives (:294-304) */
static state cons_from_primitives(state p, double volume, const gaslaw *e) {
    double mass = p.q[0] * volume;
    vec3 mom = vscale(mass, st_vel(p));
    double energy = 0.5 * vdot(mom, st_vel(p)) + mass * gas_internal_energy_from_pressure(e, p.q[4], 1. / p.q[0]);
    return st(mass, mom, energy);
}

/* ------------------------------------------------------------------ */
/* Riemann solvers                                                      */
/* ------------------------------------------------------------------ */
/* riemann_solver.rs:46-76 */
static state flux_from_half_state(state half, vec3 iv, vec3 n, const adiabatic *g) {
    vec3 hv = st_vel(half);
    double rho = half.q[0], p = half.q[4];
    vec3 v_tot = vadd(iv, hv);
    vec3 f0 = vscale(rho, hv);
    vec3 f1 = vscale(rho * v_tot.x, hv); f1.x += p;
    vec3 f2 = vscale(rho * v_tot.y, hv); f2.y += p;
    vec3 f3 = vscale(rho * v_tot.z, hv); f3.z += p;
    double roe = p * odgm1(g) + 0.5 * rho * vlen2(v_tot);
    vec3 f4 = vadd(vscale(roe, hv), vscale(p, v_tot));
    return st(vdot(f0, n), v3(vdot(f1, n), vdot(f2, n), vdot(f3, n)), vdot(f4, n));
}

/* RiemannStarSolver default methods (riemann_solver.rs:108-221) */
static inline double shock_speed(double v, double a, double pdps, const adiabatic *g) {
    return v - a * sqrt(0.5 * gp1dg(g) * pdps + gm1d2g(g));
}
static inline double rarefaction_head_speed(double v, double a) { return v - a; }
static inline double rarefaction_tail_speed(double u, double a, double pdps, const adiabatic *g) {
    return u - a * pow(pdps, gm1d2g(g));
}
static state sample_rarefaction_fan(state s, double a, double v, vec3 n, const adiabatic *g) {
    double v_half = tdgp1(g) * (a + 0.5 * (g->gamma - 1.) * v);
    double base = tdgp1(g) + gm1dgp1(g) / a * v;
    return st(s.q[0] * pow(base, tdgm1(g)), vadd(st_vel(s), vscale(v_half - v, n)),
              s.q[4] * pow(base, g->gamma * tdgm1(g)));
}
static inline state sample_middle_state(double rho, double u, double p, state s, double v, vec3 n) {
    return st(rho, vadd(st_vel(s), vscale(u - v, n)), p);
}
static state sample_left_rarefaction_wave(double rho, double u, double p, state l, double v, double a,
                                          vec3 n, const adiabatic *g) {
    if (rarefaction_head_speed(v, a) < 0.) {
        if (rarefaction_tail_speed(u, a, p / l.q[4], g) > 0.) return sample_rarefaction_fan(l, a, v, n, g);
        return sample_middle_state(rho, u, p, l, v, n);
    }
    return l;
}
static state sample_right_rarefaction_wave(double rho, double u, double p, state r, double v, double a,
                                           vec3 n, const adiabatic *g) {
    if (rarefaction_head_speed(v, -a) > 0.) {
        if (rarefaction_tail_speed(u, -a, p / r.q[4], g) < 0.) return sample_rarefaction_fan(r, -a, v, n, g);
        return sample_middle_state(rho, u, p, r, v, n);
    }
    return r;
}
static state sample_left_shock_wave(double rho, double u, double p, state l, double v, double a, vec3 n,
                                    const adiabatic *g) {
    if (shock_speed(v, a, p / l.q[4], g) < 0.) return sample_middle_state(rho, u, p, l, v, n);
    return l;
}
static state sample_right_shock_wave(double rho, double u, double p, state r, double v, double a, vec3 n,
                                     const adiabatic *g) {
    if (shock_speed(v, -a, p / r.q[4], g) > 0.) return sample_middle_state(rho, u, p, r, v, n);
    return r;
}

typedef struct { double rho_l, rho_r, u, p; } star_values; /* riemann_solver.rs:89-95 */

/* --- Exact solver (riemann_solver/exact.rs) --- */
static inline double ex_fb(double p, state s, double a, const adiabatic *g) { /* :12-20 */
    if (p > s.q[4]) {
        double cap_a = tdgp1(g) / s.q[0];
        double cap_b = gm1dgp1(g) * s.q[4];
        return (p - s.q[4]) * sqrt(cap_a / (p + cap_b));
    }
    return tdgm1(g) * a * (pow(p / s.q[4], gm1d2g(g)) - 1.);
}
static inline double ex_f(double p, state l, state r, double vl, double vr, double al, double ar,
                          const adiabatic *g) { /* :23-34 */
    return ex_fb(p, l, al, g) + ex_fb(p, r, ar, g) + (vr - vl);
}
static inline double ex_fprimeb(double p, state s, double a, const adiabatic *g) { /* :37-45 */
    if (p > s.q[4]) {
        double cap_a = tdgp1(g) / s.q[0];
        double cap_b = gm1dgp1(g) * s.q[4];
        return (1. - 0.5 * (p - s.q[4]) / (cap_b + p)) * sqrt(cap_a / (p + cap_b));
    }
    return 1. / s.q[0] / a * pow(p / s.q[4], -gm1d2g(g));
}
static inline double ex_fprime(double p, state l, state r, double al, double ar, const adiabatic *g) {
    return ex_fprimeb(p, l, al, g) + ex_fprimeb(p, r, ar, g); /* :48-57 */
}
static inline double ex_gb(double p, state s, const adiabatic *g) { /* :60-64 */
    double cap_a = tdgp1(g) / s.q[0];
    double cap_b = gm1dgp1(g) * s.q[4];
    return sqrt(cap_a / (p + cap_b));
}
static double ex_guess_p(state l, state r, double vl, double vr, double al, double ar, const adiabatic *g) {
    /* :70-103 */
    double p_min = fmin(l.q[4], r.q[4]);
    double p_max = fmax(l.q[4], r.q[4]);
    double q_max = p_max / p_min;
    double ppv = 0.5 * (l.q[4] + r.q[4]) - 0.125 * (vr - vl) * (l.q[0] + r.q[0]) * (al + ar);
    ppv = fmax(ppv, 1e-8);
    double p_guess;
    if (q_max <= 2. && p_min <= ppv && ppv <= p_max) {
        p_guess = ppv;
    } else if (ppv < p_min) {
        double base = (al + ar - 0.5 * (g->gamma - 1.) * (vr - vl)) /
                      (al / pow(l.q[4], gm1d2g(g)) + ar / pow(r.q[4], gm1d2g(g)));
        p_guess = pow(base, g->gamma * tdgm1(g));
    } else {
        p_guess = (ex_gb(ppv, l, g) * l.q[4] + ex_gb(ppv, r, g) * r.q[4] - vr + vl) /
                  (ex_gb(ppv, l, g) + ex_gb(ppv, r, g));
    }
    return fmax(p_guess, 1e-8);
}
static double ex_solve_brent(double lower, double upper, double low_f, double up_f, double tol, state l,
                             state r, double vl, double vr, double al, double ar, const adiabatic *g,
                             uint32_t *err) { /* :106-191 */
    double a = lower, b = upper, c, d = INFINITY;
    double fa = low_f, fb = up_f, fc;
    double s, fs, t;
    if (fa * fb > 0.) { *err |= ORC_ERR_BRENT_BRACKET; return b; }
    if (fabs(fa) < fabs(fb)) { t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    c = a; fc = fa;
    int mflag = 1;
    while (fb != 0. && fabs(a - b) > tol * 0.5 * (a + b)) {
        if (fa != fc && fb != fc)
            s = a * fb * fc / (fa - fb) / (fa - fc) + b * fa * fc / (fb - fa) / (fb - fc) +
                c * fa * fb / (fc - fa) / (fc - fb);
        else
            s = b - fb * (b - a) / (fb - fa);
        double tmp = 0.25 * (3. * a + b);
        if (!((s > tmp && s < b) || (s < tmp && s > b)) || (mflag && fabs(s - b) >= (0.5 * fabs(b - c))) ||
            (!mflag && fabs(s - b) >= (0.5 * fabs(c - d))) || (mflag && fabs(b - c) < 0.5 * tol * (b + c)) ||
            (!mflag && fabs(c - d) < 0.5 * tol * (c + d))) {
            s = 0.5 * (a + b);
            mflag = 1;
        } else {
            mflag = 0;
        }
        fs = ex_f(s, l, r, vl, vr, al, ar, g);
        d = c; c = b; fc = fb;
        if (fa * fs < 0.) { b = s; fb = fs; } else { a = s; fa = fs; }
        if (fabs(fa) < fabs(fb)) { t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    }
    return b;
}
static inline double ex_middle_density(double p, state s, const adiabatic *g) { /* :193-212 */
    double pdps = p / s.q[4];
    if (pdps > 1.) return s.q[0] * (pdps + gm1dgp1(g)) / (gm1dgp1(g) * pdps + 1.);
    return s.q[0] * pow(pdps, 1. / g->gamma);
}
/* ExactRiemannSolver::star_state_from_pstar (exact.rs:214-238) */
static star_values ex_star_from_pstar(double p, state l, state r, double vl, double vr, double al, double ar,
                                      const adiabatic *g) {
    star_values sv;
    sv.u = 0.5 * (vl + vr) + 0.5 * (ex_fb(p, r, ar, g) - ex_fb(p, l, al, g));
    sv.rho_l = ex_middle_density(p, l, g);
    sv.rho_r = ex_middle_density(p, r, g);
    sv.p = p;
    return sv;
}
static star_values ex_star_state(state l, state r, double vl, double vr, double al, double ar,
                                 const adiabatic *g, int max_iter, uint32_t *err) { /* :241-291 */
    double p = 0.;
    double p_guess = ex_guess_p(l, r, vl, vr, al, ar, g);
    double fp = ex_f(p, l, r, vl, vr, al, ar, g);
    double fp_guess = ex_f(p_guess, l, r, vl, vr, al, ar, g);
    if (fp * fp_guess >= 0.) {
        int counter = 0;
        while (fabs(p - p_guess) > 1e-6 * 0.5 * (p + p_guess) && fp_guess < 0.0) {
            p = p_guess;
            p_guess = p_guess - fp_guess / ex_fprime(p_guess, l, r, al, ar, g);
            fp_guess = ex_f(p_guess, l, r, vl, vr, al, ar, g);
            counter += 1;
            if (counter > max_iter) { *err |= ORC_ERR_NEWTON_CAP; break; }
        }
    }
    if (fabs(p - p_guess) > 1e-6 * 0.5 * (p + p_guess) && fp_guess > 0.) {
        p = 0.;
        fp = ex_f(p, l, r, vl, vr, al, ar, g);
        p = ex_solve_brent(p, p_guess, fp, fp_guess, 1e-6, l, r, vl, vr, al, ar, g, err);
    } else {
        p = p_guess;
    }
    return ex_star_from_pstar(p, l, r, vl, vr, al, ar, g);
}

/* --- PVRS (riemann_solver/pvrs.rs:26-46) --- */
static star_values pv_star_state(state l, state r, double vl, double vr, double al, double ar) {
    double rho_bar = 0.5 * (l.q[0] + r.q[0]);
    double p_bar = 0.5 * (l.q[4] + r.q[4]);
    double a_bar = 0.5 * (al + ar);
    star_values sv;
    sv.p = p_bar + 0.5 * (vl - vr) * rho_bar * a_bar;
    sv.u = 0.5 * ((vl + vr) + (l.q[4] - r.q[4]) / (rho_bar * a_bar));
    sv.rho_l = l.q[0] + (vl - sv.u) * rho_bar / a_bar;
    sv.rho_r = r.q[0] + (sv.u - vr) * rho_bar / a_bar;
    return sv;
}

/* --- TSRS (riemann_solver/tsrs.rs:18-51) --- */
static star_values ts_star_state(state l, state r, double vl, double vr, double al, double ar, const adiabatic *g) {
    /* PVRiemannSolver::p_star(rho_bar, p_bar, a_bar, v_l, v_r) (pvrs.rs:8-22) */
    double rho_bar = 0.5 * (l.q[0] + r.q[0]);
    double p_bar = 0.5 * (l.q[4] + r.q[4]);
    double a_bar = 0.5 * (al + ar);
    double p_guess = p_bar + 0.5 * (vl - vr) * rho_bar * a_bar;
    /* TSRiemannSolver::g (tsrs.rs:18-22) */
    double g_l = sqrt((tdgp1(g) / l.q[0]) / (p_guess + gm1dgp1(g) * l.q[4]));
    double g_r = sqrt((tdgp1(g) / r.q[0]) / (p_guess + gm1dgp1(g) * r.q[4]));
    double pstar = (g_l * l.q[4] + g_r * r.q[4] - (vr - vl)) / (g_l + g_r);
    return ex_star_from_pstar(pstar, l, r, vl, vr, al, ar, g);
}

/* --- TRRS (riemann_solver/trrs.rs:14-32) --- */
static star_values tr_star_state(state l, state r, double vl, double vr, double al, double ar, const adiabatic *g) {
    double beta = gm1d2g(g);
    double gm1d2 = 0.5 * (g->gamma - 1.);
    double num = al + ar - gm1d2 * (vr - vl);
    double denom = al * pow(l.q[4], -beta) + ar * pow(r.q[4], -beta);
    double pstar = pow(num / denom, 1. / beta);
    return ex_star_from_pstar(pstar, l, r, vl, vr, al, ar, g);
}

/* The flux solver of a run: riemann_solver.rs:28-44 and bin/main.rs:625-642
 * (kind, AIRS threshold, LinearAdvection velocity). */
typedef struct { int kind; double airs_threshold; vec3 adv; } rsolver;

static star_values star_state(const rsolver *rs, state l, state r, double vl, double vr, double al, double ar,
                              const adiabatic *g, int max_iter, uint32_t *err) {
    switch (rs->kind) {
    case ORC_EXACT: return ex_star_state(l, r, vl, vr, al, ar, g, max_iter, err);
    case ORC_TSRS: return ts_star_state(l, r, vl, vr, al, ar, g);
    case ORC_TRRS: return tr_star_state(l, r, vl, vr, al, ar, g);
    case ORC_AIRS: { /* AIRiemannSolver (airs.rs:18-38) */
        star_values s = pv_star_state(l, r, vl, vr, al, ar);
        double p_max = fmax(l.q[4], r.q[4]);
        double p_min = fmin(l.q[4], r.q[4]);
        if (p_max / p_min < rs->airs_threshold) return s;
        return ex_star_state(l, r, vl, vr, al, ar, g, max_iter, err);
    }
    default: return pv_star_state(l, r, vl, vr, al, ar);
    }
}

/* RiemannStarSolver::sample (riemann_solver.rs:224-255) */
static state star_sample(const rsolver *rs, state l, state r, double vl, double vr, double al, double ar, vec3 n,
                         const adiabatic *g, int max_iter, uint32_t *err) {
    star_values s = star_state(rs, l, r, vl, vr, al, ar, g, max_iter, err);
    if (s.u < 0.) {
        if (s.p > r.q[4]) return sample_right_shock_wave(s.rho_r, s.u, s.p, r, vr, ar, n, g);
        return sample_right_rarefaction_wave(s.rho_r, s.u, s.p, r, vr, ar, n, g);
    } else if (s.p > l.q[4]) {
        return sample_left_shock_wave(s.rho_l, s.u, s.p, l, vl, al, n, g);
    }
    return sample_left_rarefaction_wave(s.rho_l, s.u, s.p, l, vl, al, n, g);
}

/* --- Vacuum (riemann_solver/vacuum.rs) --- */
static inline int is_vacuum(state l, state r, double al, double ar, double vrml, const adiabatic *g) {
    if (l.q[0] == 0. || r.q[0] == 0.) return 1; /* :23-25 */
    if (tdgm1(g) * (al + ar) <= vrml) return 1; /* :27-29 */
    return 0;
}
static state sample_right_vacuum(state l, double vl, double al, double sl, vec3 n, const adiabatic *g) {
    if (0. <= vl - al) return l; /* :48-56 */
    if (0. < sl) return sample_rarefaction_fan(l, al, vl, n, g);
    return st_vacuum();
}
static state sample_left_vacuum(state r, double vr, double ar, double sr, vec3 n, const adiabatic *g) {
    if (0. <= sr) return st_vacuum(); /* :67-75 */
    if (0. < vr + ar) return sample_rarefaction_fan(r, -ar, vr, n, g);
    return r;
}
static state vacuum_sample(state l, state r, double vl, double vr, double al, double ar, vec3 n,
                           const adiabatic *g) { /* :116-138 */
    if (r.q[0] == 0.) {
        double sl = vl + tdgm1(g) * al;
        return sample_right_vacuum(l, vl, al, sl, n, g);
    } else if (l.q[0] == 0.) {
        double sr = vr - tdgm1(g) * ar;
        return sample_left_vacuum(r, vr, ar, sr, n, g);
    }
    /* sample_vacuum_creation (:78-99) */
    double sl = vl + tdgm1(g) * al;
    double sr = vr - tdgm1(g) * ar;
    if (0. <= sl) return sample_right_vacuum(l, vl, al, sl, n, g);
    if (0. < sr) return st_vacuum();
    return sample_left_vacuum(r, vr, ar, sr, n, g);
}

/* HLLC (riemann_solver/hllc.rs:12-123) */
static state hllc_flux(state s, double v, double e, vec3 n) { /* :97-104 */
    double rho_v = s.q[0] * v;
    return st(rho_v, vadd(vscale(rho_v, st_vel(s)), vscale(s.q[4], n)), ((s.q[0] * e) + s.q[4]) * v);
}
static state hllc_flux_star(state s, double v, double e, double S, double s_star, vec3 n) { /* :107-123 */
    double s_m_v = S - v;
    double rho = s.q[0];
    double starfac = rho * s_m_v / (S - s_star);
    vec3 v_star = vadd(vscale(s_star - v, n), st_vel(s));
    double e_star = e + (s_star - v) * (s_star + s.q[4] / (rho * s_m_v));
    state u_star = st_scale(starfac, st(1., v_star, e_star));
    state u_l = st(rho, vscale(rho, st_vel(s)), rho * e);
    return st_scale(S, st_sub(u_star, u_l));
}
static state hllc_solve(state l, state r, vec3 iv, vec3 n, const gaslaw *eos) {
    const adiabatic *g = &eos->g;
    double rho_l_inv = 1. / l.q[0];
    double rho_r_inv = 1. / r.q[0];
    double vl = vdot(st_vel(l), n);
    double vr = vdot(st_vel(r), n);
    double al = sound_speed(eos, l.q[4], rho_l_inv);
    double ar = sound_speed(eos, r.q[4], rho_r_inv);
    double vrml = vr - vl;
    if (is_vacuum(l, r, al, ar, vrml, g)) {
        state w = vacuum_sample(l, r, vl, vr, al, ar, n, g);
        return flux_from_half_state(w, iv, n, g);
    }
    double ppvrs = 0.5 * (l.q[4] + r.q[4]) - 0.125 * vrml * (l.q[0] + r.q[0]) * (al + ar);
    double p_star = fmax(ppvrs, 0.);
    double q_l = 1.;
    if (p_star > l.q[4] && l.q[4] > 0.) q_l = sqrt(1. + 0.5 * gp1dg(g) * (p_star / l.q[4] - 1.));
    double q_r = 1.;
    if (p_star > r.q[4] && r.q[4] > 0.) q_r = sqrt(1. + 0.5 * gp1dg(g) * (p_star / r.q[4] - 1.));
    double s_l_m_v_l = -al * q_l;
    double s_r_m_v_r = ar * q_r;
    double s_star = (r.q[4] - l.q[4] + l.q[0] * vl * s_l_m_v_l - r.q[0] * vr * s_r_m_v_r) /
                    (l.q[0] * s_l_m_v_l - r.q[0] * s_r_m_v_r);
    state flux;
    if (s_star >= 0.) {
        double v_l2 = vlen2(st_vel(l));
        double e_l = gas_internal_energy_from_pressure(eos, l.q[4], rho_l_inv) + 0.5 * v_l2;
        flux = hllc_flux(l, vl, e_l, n);
        double s_l = s_l_m_v_l + vl;
        if (s_l < 0.) flux = st_add(flux, hllc_flux_star(l, vl, e_l, s_l, s_star, n));
    } else {
        double v_r2 = vlen2(st_vel(r));
        double e_r = gas_internal_energy_from_pressure(eos, r.q[4], rho_r_inv) + 0.5 * v_r2;
        flux = hllc_flux(r, vr, e_r, n);
        double s_r = s_r_m_v_r + vr;
        if (s_r > 0.) flux = st_add(flux, hllc_flux_star(r, vr, e_r, s_r, s_star, n));
    }
    /* de-boost (:85-90): the added State is built from the pre-update flux */
    state add = st(0., vscale(flux.q[0], iv), vdot(iv, st_vel(flux)) + 0.5 * vlen2(iv) * flux.q[0]);
    /* `interface_velocity * flux.mass()` is DVec3 * f64: component * mass */
    add.q[1] = iv.x * flux.q[0];
    add.q[2] = iv.y * flux.q[0];
    add.q[3] = iv.z * flux.q[0];
    return st_add(flux, add);
}

/* Blanket RiemannFluxSolver impl for star solvers (riemann_solver.rs:258-287) */
static state star_half_state(const rsolver *rs, state l, state r, vec3 n, const gaslaw *eos, int max_iter,
                             uint32_t *err) {
    const adiabatic *g = &eos->g;
    double vl = vdot(st_vel(l), n);
    double vr = vdot(st_vel(r), n);
    double al = sound_speed(eos, l.q[4], 1. / l.q[0]);
    double ar = sound_speed(eos, r.q[4], 1. / r.q[0]);
    double vrml = vr - vl;
    if (is_vacuum(l, r, al, ar, vrml, g)) return vacuum_sample(l, r, vl, vr, al, ar, n, g);
    return star_sample(rs, l, r, vl, vr, al, ar, n, g, max_iter, err);
}

/* LinearAdvectionRiemannSover::solve_for_flux (riemann_solver/linear_advection.rs:17-34) */
static state linear_advection_flux(const rsolver *rs, state l, state r, vec3 iv, vec3 n) {
    double v = vdot(vsub(rs->adv, iv), n);
    state s = v > 0. ? l : r;
    return st_scale(v, s);
}

static state riemann_solve_for_flux(const rsolver *rs, state l, state r, vec3 iv, vec3 n, const gaslaw *eos,
                                    int max_iter, uint32_t *err) {
    if (rs->kind == ORC_HLLC) return hllc_solve(l, r, iv, n, eos);
    if (rs->kind == ORC_LINEAR_ADVECTION) return linear_advection_flux(rs, l, r, iv, n);
    state w = star_half_state(rs, l, r, n, eos, max_iter, err);
    return flux_from_half_state(w, iv, n, &eos->g);
}

/* ------------------------------------------------------------------ */
/* Timeline (timeline.rs)                                              */
/* ------------------------------------------------------------------ */
#define NUM_TIME_BINS 56
#define TIME_BIN_NEIGHBOUR_MAX_DELTA_BIN 2
static inline uint64_t get_integer_timestep(int bin) { /* :18-24 */
    if (bin <= 0) return 0;
    return (uint64_t)1 << (bin + 1);
}
#define MAX_NR_TIMESTEPS (get_integer_timestep(NUM_TIME_BINS))
static inline int get_time_bin(uint64_t dti) { /* :31-33; u32 wrap then `as i8` */
    uint32_t lz = dti == 0 ? 64u : (uint32_t)__builtin_clzll(dti);
    uint32_t v = 64u - lz - 2u;
    return (int)(int8_t)(uint8_t)(v & 0xffu);
}
static inline uint64_t get_integer_time_end(uint64_t ti, int bin) { /* :53-67 */
    uint64_t dti = get_integer_timestep(bin);
    if (dti == 0) return 0;
    uint64_t mod = ti % dti;
    if (mod == 0) return ti;
    return ti - mod + dti;
}
static inline int get_max_active_bin(uint64_t ti) { /* :72-83 */
    if (ti == 0) return NUM_TIME_BINS;
    int bin = 1;
    while ((((uint64_t)1 << ((bin + 1) & 63)) & ti) == 0) bin += 1;
    return bin;
}
/* Rust `f64 as u64` (saturating, NaN -> 0). */
static inline uint64_t sat_u64(double x) {
    if (!(x > 0.)) return 0;
    if (x >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)x;
}
static uint64_t make_integer_timestep(double dt, int old_bin, int min_ngb_bin, uint64_t ti_current,
                                      double time_base_inv, uint32_t *err) { /* :103-139 */
    uint64_t new_dti = sat_u64(dt * time_base_inv);
    int nb = get_time_bin(new_dti);
    int lim = min_ngb_bin + TIME_BIN_NEIGHBOUR_MAX_DELTA_BIN;
    int new_bin = nb < lim ? nb : lim;
    new_dti = get_integer_timestep(new_bin);
    uint64_t current_dti = get_integer_timestep(old_bin);
    if (old_bin > 0) new_dti = new_dti < 2 * current_dti ? new_dti : 2 * current_dti;
    uint64_t timeline_dti = MAX_NR_TIMESTEPS;
    while (new_dti < timeline_dti) timeline_dti /= 2;
    new_dti = timeline_dti;
    if (new_dti > current_dti) {
        uint64_t ti_end = get_integer_time_end(ti_current, old_bin);
        if ((MAX_NR_TIMESTEPS - ti_end) % new_dti != 0) new_dti = current_dti;
    }
    if (new_dti == 0) *err |= ORC_ERR_ZERO_DTI;
    return new_dti;
}

/* ------------------------------------------------------------------ */
/* Particle (part.rs) and faces                                         */
/* ------------------------------------------------------------------ */
typedef struct particle {
    state prim;
    grads grad;
    vec3 gc;
    state extrap;
    state cons;
    state fluxes;
    vec3 gravity_mflux;
    double volume;
    vec3 loc, centroid, v, v_rel;
    double max_a_over_r, max_signal_velocity;
    int timebin;
    double dt;
    double dvdt;
    vec3 a_grav;
} particle;

typedef struct face {
    int64_t left, right; /* right < 0: None */
    double area;
    vec3 normal, centroid, shift;
} face;

typedef struct { state fluxes; vec3 mflux; double v_max, a_over_r; } flux_info; /* flux.rs:10-21 */

struct orc_ctx {
    orc_params p;
    gaslaw eos;
    rsolver rs;
    /* moving meshes: geometry of the rebuilt cells, applied after the next predict */
    double *pend_vol, *pend_cen;
    int pending_geometry;
    int64_t n, nf;
    particle *parts;
    face *faces;
    int32_t *csr_off, *csr_face;
    double time_base, time_base_inv;
    uint32_t err;
    /* scratch */
    flux_info *fi;
    uint8_t *active;
    grads *gtmp;
    uint8_t *has_g;
    double *dts;
    int *wake;
};

static inline vec3 m_vec(const double *a, int64_t n, int64_t i) { return v3(a[i], a[n + i], a[2 * n + i]); }

/* Particle::time_extrapolations (part.rs:134-149) */
static state time_extrapolations(const particle *pt, double dt, const gaslaw *eos) {
    double rho = pt->prim.q[0];
    if (rho > 0.) {
        double rho_inv = 1. / rho;
        double p = pt->prim.q[4];
        double div_v = gr_div_v(&pt->grad);
        vec3 g4 = pt->grad.g[4];
        state s = st(rho * div_v + vdot(pt->v_rel, pt->grad.g[0]),
                     vadd(vscale(div_v, pt->v_rel), vscale(rho_inv, g4)),
                     eos->g.gamma * p * div_v + vdot(pt->v_rel, g4));
        /* v_rel * div_v: DVec3 * f64 -> component * div_v */
        s.q[1] = pt->v_rel.x * div_v + rho_inv * g4.x;
        s.q[2] = pt->v_rel.y * div_v + rho_inv * g4.y;
        s.q[3] = pt->v_rel.z * div_v + rho_inv * g4.z;
        return st_scale(-dt, s);
    }
    return st_vacuum();
}

/* Particle::extrapolate_state (part.rs:123-132) */
static void extrapolate_state(particle *pt, double dt, const gaslaw *eos) {
    pt->extrap = st_add(pt->extrap, time_extrapolations(pt, dt, eos));
    check_physical(&pt->prim);
    double volume = pt->volume + pt->dvdt * dt;
    double lo = 0.5 * pt->volume, hi = 2. * pt->volume;
    pt->volume = volume < lo ? lo : (volume > hi ? hi : volume);
}

/* Particle::reflect (part.rs:374-383) */
static particle reflect_part(const particle *pt, vec3 around, vec3 n) {
    particle r = *pt;
    r.loc = vadd(r.loc, vscale(2. * vdot(vsub(around, pt->loc), n), n));
    r.centroid = vadd(r.centroid, vscale(2. * vdot(vsub(around, pt->centroid), n), n));
    r.gc = vadd(r.gc, vscale(2. * vdot(vsub(around, pt->gc), n), n));
    r.v = vsub(r.v, vscale(2. * vdot(r.v, n), n));
    return r;
}

/* Space::get_boundary_part (space.rs:213-229) */
static particle boundary_part(const orc_ctx *c, const particle *pt, const face *f) {
    particle r = reflect_part(pt, f->centroid, f->normal);
    if (c->p.boundary == ORC_REFLECTIVE) r.prim = prim_reflect(r.prim, f->normal);
    else if (c->p.boundary == ORC_VACUUM) r.prim = st_vacuum();
    return r;
}

/* gradients.rs:105-132 */
static double pairwise_limiter_single_quantity(double q_l, double q_r, double q_dash, double dx_fac) {
    if (q_l == q_r) return q_l;
    double q_bar = q_l + dx_fac * (q_r - q_l);
    double q_diff = fabs(q_l - q_r);
    double delta1 = 0.5 * q_diff;
    double delta2 = 0.25 * q_diff;
    if (q_l < q_r) {
        double q_min = fmin(q_l, q_r);
        double qmin = (q_min - delta1) * q_min > 0. ? q_min - delta1 : q_min * fabs(q_min) / (fabs(q_min) + delta1);
        return fmax(qmin, fmin(q_bar + delta2, q_dash));
    }
    double q_max = fmax(q_l, q_r);
    double qplu = (q_max + delta1) * q_max > 0. ? q_max + delta1 : q_max * fabs(q_max) / (fabs(q_max) + delta1);
    return fmin(qplu, fmax(q_bar - delta2, q_dash));
}
/* gradients.rs:134-152 */
static state pairwise_limiter(state l, state r, state dash, double dx_fac) {
    state lim;
    for (int i = 0; i < 5; i++) lim.q[i] = pairwise_limiter_single_quantity(l.q[i], r.q[i], dash.q[i], dx_fac);
    check_physical(&lim);
    return lim;
}

/* flux.rs:23-100 */
static flux_info flux_exchange(const orc_ctx *c, const particle *L, const particle *R, double dt,
                               const face *f, double tef, uint32_t *err) {
    const gaslaw *eos = &c->eos;
    vec3 dx_left = vsub(f->centroid, L->gc);
    vec3 shift = f->shift;
    vec3 dx_right = vsub(vsub(f->centroid, R->gc), shift);
    double dx_gradients = vlen(vsub(dx_left, dx_right));
    vec3 dx_centroid = vsub(vadd(R->centroid, shift), L->centroid);
    vec3 dx = vsub(vadd(R->loc, shift), L->loc);

    double v_max = 0.;
    if (L->prim.q[0] > 0.) v_max += sound_speed(eos, L->prim.q[4], 1. / L->prim.q[0]);
    if (R->prim.q[0] > 0.) v_max += sound_speed(eos, R->prim.q[4], 1. / R->prim.q[0]);
    v_max -= fmin(vdot(vsub(st_vel(R->prim), st_vel(L->prim)), dx_centroid), 0.);

    double dt_extrapolate = -tef * dt;
    state left_dash = st_add(st_add(st_add(L->prim, gr_dot(&L->grad, dx_left)), L->extrap),
                             time_extrapolations(L, dt_extrapolate, eos));
    state right_dash = st_add(st_add(st_add(R->prim, gr_dot(&R->grad, dx_right)), R->extrap),
                              time_extrapolations(R, dt_extrapolate, eos));
    state prim_left = pairwise_limiter(L->prim, R->prim, left_dash, vlen(dx_left) / dx_gradients);
    state prim_right = pairwise_limiter(R->prim, L->prim, right_dash, vlen(dx_right) / dx_gradients);

    vec3 midpoint = vscale(0.5, vadd(vadd(L->loc, R->loc), shift));
    double fac = vdot(vsub(R->v, L->v), vsub(f->centroid, midpoint)) / vlen2(dx);
    vec3 v_face = vsub(vscale(0.5, vadd(L->v, R->v)), vscale(fac, dx));
    vec3 mvf = v3(-v_face.x, -v_face.y, -v_face.z);

    state F = riemann_solve_for_flux(&c->rs, prim_boost(prim_left, mvf), prim_boost(prim_right, mvf),
                                     v_face, f->normal, eos, c->p.max_newton_iter, err);
    state fluxes = st_scale(f->area, F);
    flux_info fi;
    fi.fluxes = st_scale(dt, fluxes);
    fi.mflux = v3(dx.x * fluxes.q[0], dx.y * fluxes.q[0], dx.z * fluxes.q[0]);
    fi.v_max = v_max;
    fi.a_over_r = f->area / vlen(dx);
    return fi;
}

/* flux.rs:102-195 */
static flux_info flux_exchange_boundary(const orc_ctx *c, const particle *P, const face *f, double tef,
                                        uint32_t *err) {
    const gaslaw *eos = &c->eos;
    vec3 n = f->normal;
    particle refl = reflect_part(P, f->centroid, n);
    vec3 dx_face = vsub(f->centroid, P->gc);
    double dx_gradients = vlen(vsub(refl.gc, P->gc));
    vec3 dx_centroid = vsub(refl.centroid, P->centroid);
    vec3 dx = vsub(refl.loc, P->loc);

    double v_max = 0.;
    if (P->prim.q[0] > 0.) v_max += sound_speed(eos, P->prim.q[4], 1. / P->prim.q[0]);

    double dt_extrapolate = -tef * P->dt;
    state dash = st_add(st_add(st_add(P->prim, gr_dot(&P->grad, dx_face)), P->extrap),
                        time_extrapolations(P, dt_extrapolate, eos));
    state bnd;
    double dx_fac = vlen(dx_face) / dx_gradients;
    if (c->p.boundary == ORC_REFLECTIVE) {
        refl.prim = prim_reflect(refl.prim, n);
        dash = pairwise_limiter(P->prim, refl.prim, dash, dx_fac);
        v_max -= fmin(vdot(vsub(st_vel(refl.prim), st_vel(P->prim)), dx_centroid), 0.);
        bnd = prim_reflect(dash, n);
    } else if (c->p.boundary == ORC_OPEN) {
        dash = pairwise_limiter(P->prim, P->prim, dash, dx_fac);
        bnd = dash;
    } else { /* vacuum */
        state vac = st_vacuum();
        dash = pairwise_limiter(P->prim, vac, dash, dx_fac);
        v_max += fmin(vdot(st_vel(P->prim), dx_centroid), 0.);
        bnd = vac;
    }
    state F = riemann_solve_for_flux(&c->rs, dash, bnd, v3(0., 0., 0.), n, eos, c->p.max_newton_iter, err);
    state fluxes = st_scale(f->area, F);
    flux_info fi;
    fi.fluxes = st_scale(P->dt, fluxes);
    fi.mflux = v3(dx.x * fluxes.q[0], dx.y * fluxes.q[0], dx.z * fluxes.q[0]);
    fi.v_max = v_max;
    fi.a_over_r = f->area / vlen(dx);
    return fi;
}

static flux_info flux_info_zero(void) {
    flux_info fi;
    fi.fluxes = st_vacuum();
    fi.mflux = v3(0., 0., 0.);
    fi.v_max = 0.;
    fi.a_over_r = 0.;
    return fi;
}

/* EulerEqnsFvs::compute_fluxes (finite_volume_solver/euler_eqns_fvs.rs:26-48) */
static int64_t compute_fluxes(orc_ctx *c, const uint8_t *active, flux_info *out) {
    int64_t count = 0;
    uint32_t err = 0;
#pragma omp parallel for schedule(static) reduction(+ : count) reduction(| : err)
    for (int64_t fi = 0; fi < c->nf; fi++) {
        const face *f = &c->faces[fi];
        const particle *L = &c->parts[f->left];
        int la = active[f->left];
        if (f->right >= 0) {
            const particle *R = &c->parts[f->right];
            int ra = active[f->right];
            if ((!la && !ra) || (R->dt < L->dt && !ra) || (L->dt < R->dt && !la)) {
                out[fi] = flux_info_zero();
                continue;
            }
            double dt = fmin(L->dt, R->dt);
            out[fi] = flux_exchange(c, L, R, dt, f, 0.5, &err);
            count++;
        } else if (la) {
            out[fi] = flux_exchange_boundary(c, L, f, 0.5, &err);
            count++;
        } else {
            out[fi] = flux_info_zero();
        }
    }
    c->err |= err;
    return count;
}

/* Particle::apply_flux (part.rs:178-193) */
static void apply_flux(particle *pt, uint32_t *err) {
    pt->cons = st_add(pt->cons, pt->fluxes);
    if (!isfinite(pt->cons.q[0]) || !visfinite(st_vel(pt->cons)) || !isfinite(pt->cons.q[4]))
        *err |= ORC_ERR_NONFINITE;
    if (pt->cons.q[0] < 0.) pt->cons = st_vacuum();
    if (pt->cons.q[4] < 0.) pt->cons = st_vacuum();
    pt->fluxes = st_vacuum();
    pt->gravity_mflux = v3(0., 0., 0.);
}

/* Particle::hydro_kick1 (part.rs:87-104) */
static void hydro_kick1(particle *pt, int motion, int dim) {
    if (motion == ORC_MOTION_FIXED) return;
    double rho = pt->prim.q[0];
    if (rho > 0.) {
        double kick_fac = 0.5 * pt->dt / rho;
        if (dim > 0) pt->v.x -= kick_fac * pt->grad.g[4].x;
        if (dim > 1) pt->v.y -= kick_fac * pt->grad.g[4].y;
        if (dim > 2) pt->v.z -= kick_fac * pt->grad.g[4].z;
    }
}

/* Particle::grav_kick (part.rs:303-312) */
static void grav_kick(particle *pt) {
    double mass = pt->cons.q[0];
    vec3 mom = st_vel(pt->cons);
    vec3 k = vscale(0.5 * pt->dt, pt->a_grav);
    state add = st(0., vscale(mass, k), vdot(k, vsub(mom, pt->gravity_mflux)));
    add.q[1] = k.x * mass;
    add.q[2] = k.y * mass;
    add.q[3] = k.z * mass;
    pt->cons = st_add(pt->cons, add);
}

/* runner/hydrodynamics.rs:13-39 (+ kick2 :51-57) */
static void apply_fluxes(orc_ctx *c, const flux_info *fl, const uint8_t *active) {
    uint32_t err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int64_t i = 0; i < c->n; i++) {
        particle *pt = &c->parts[i];
        int act = active[i];
        for (int32_t k = c->csr_off[i]; k < c->csr_off[i + 1]; k++) {
            int32_t idx = c->csr_face[k];
            const face *f = &c->faces[idx];
            const flux_info *fi = &fl[idx];
            if (f->left == i) { /* update_fluxes_left (part.rs:160-167) */
                pt->fluxes = st_sub(pt->fluxes, fi->fluxes);
                pt->gravity_mflux = vsub(pt->gravity_mflux, fi->mflux);
            } else { /* update_fluxes_right (part.rs:169-176) */
                pt->fluxes = st_add(pt->fluxes, fi->fluxes);
                pt->gravity_mflux = vsub(pt->gravity_mflux, fi->mflux);
            }
            if (act) {
                pt->max_signal_velocity = fmax(fi->v_max, pt->max_signal_velocity);
                pt->max_a_over_r = fmax(pt->max_a_over_r, fi->a_over_r);
            }
        }
        if (act) apply_flux(pt, &err);
    }
    c->err |= err;
}

static void kick2(orc_ctx *c, const uint8_t *active) { /* runner/hydrodynamics.rs:51-57 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++)
        if (active[i]) grav_kick(&c->parts[i]);
}

/* Particle::convert_conserved_to_primitive (part.rs:219-261) */
static void convert_c2p(orc_ctx *c, const uint8_t *active) {
    uint32_t err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int64_t i = 0; i < c->n; i++) {
        if (!active[i]) continue;
        particle *pt = &c->parts[i];
        if (!(pt->cons.q[0] >= 0.)) err |= ORC_ERR_NEG_MASS;
        if (!(pt->cons.q[4] >= 0.)) err |= ORC_ERR_NEG_ENERGY;
        if (pt->cons.q[0] == 0.) {
            if (pt->cons.q[4] != 0.) err |= ORC_ERR_NEG_ENERGY;
            pt->prim = st_vacuum();
        } else {
            pt->prim = prim_from_conserved(pt->cons, pt->volume, &c->eos, &err);
        }
        if (!(pt->prim.q[0] >= 0.) || !(pt->prim.q[4] >= 0.)) err |= ORC_ERR_NEG_PRIM;
        if (!isfinite(pt->prim.q[0]) || !visfinite(st_vel(pt->prim)) || !isfinite(pt->prim.q[4]))
            err |= ORC_ERR_NONFINITE;
    }
    c->err |= err;
}

/* GradientData::init (gradients.rs:14-33) */
static mat3 wls_init(int dim) {
    mat3 m;
    memset(&m, 0, sizeof(m));
    if (dim == 1) { m.c0.x = 0.; m.c1.y = 1.; m.c2.z = 1.; }
    else if (dim == 2) { m.c2.z = 1.; }
    return m;
}
/* GradientData::collect (gradients.rs:35-41) */
static inline void wls_collect(grads *g, mat3 *m, state sl, state sr, double w, vec3 ds) {
    for (int i = 0; i < 5; i++) g->g[i] = vadd(g->g[i], vscale(w * (sr.q[i] - sl.q[i]), ds));
    m->c0 = vadd(m->c0, vscale(w, vscale(ds.x, ds)));
    m->c1 = vadd(m->c1, vscale(w, vscale(ds.y, ds)));
    m->c2 = vadd(m->c2, vscale(w, vscale(ds.z, ds)));
}
/* glam DMat3::inverse + GradientData::finalize (gradients.rs:43-55) */
static grads wls_finalize(grads g, mat3 m) {
    vec3 t0 = vcross(m.c1, m.c2);
    vec3 t1 = vcross(m.c2, m.c0);
    vec3 t2 = vcross(m.c0, m.c1);
    double det = vdot(m.c2, t2);
    double inv_det = 1.0 / det;
    /* inverse = transpose(from_cols(t0*inv, t1*inv, t2*inv)) -> rows t0, t1, t2 */
    vec3 r0 = vscale(inv_det, t0), r1 = vscale(inv_det, t1), r2 = vscale(inv_det, t2);
    /* columns of the inverse */
    vec3 c0 = v3(r0.x, r1.x, r2.x), c1 = v3(r0.y, r1.y, r2.y), c2 = v3(r0.z, r1.z, r2.z);
    for (int i = 0; i < 5; i++) {
        vec3 x = g.g[i];
        /* mul_vec3: x_axis * x.x + y_axis * x.y + z_axis * x.z */
        vec3 res = vscale(x.x, c0);
        res = v3(c0.x * x.x, c0.y * x.x, c0.z * x.x);
        res = vadd(res, v3(c1.x * x.y, c1.y * x.y, c1.z * x.y));
        res = vadd(res, v3(c2.x * x.z, c2.y * x.z, c2.z * x.z));
        g.g[i] = res;
    }
    if (!gr_isfinite(&g)) memset(&g, 0, sizeof(g));
    return g;
}

/* runner/hydrodynamics.rs:67-143 (estimate, limit, apply) */
static void gradients(orc_ctx *c, const uint8_t *active) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) {
        c->has_g[i] = 0;
        if (!active[i]) continue;
        const particle *pt = &c->parts[i];
        vec3 centroid = pt->centroid;
        grads g;
        memset(&g, 0, sizeof(g));
        mat3 m = wls_init(c->p.dimensionality);
        for (int32_t k = c->csr_off[i]; k < c->csr_off[i + 1]; k++) {
            const face *f = &c->faces[c->csr_face[k]];
            vec3 shift = (i == f->left) ? f->shift : v3(-f->shift.x, -f->shift.y, -f->shift.z);
            if (f->left == i && f->right < 0) {
                particle o = boundary_part(c, pt, f);
                vec3 ds = vsub(vadd(o.centroid, shift), centroid);
                wls_collect(&g, &m, pt->prim, o.prim, f->area / vlen2(ds), ds);
            } else {
                int64_t oi = (i == f->left) ? f->right : f->left;
                const particle *o = &c->parts[oi];
                vec3 ds = vsub(vadd(o->centroid, shift), centroid);
                wls_collect(&g, &m, pt->prim, o->prim, f->area / vlen2(ds), ds);
            }
        }
        c->gtmp[i] = wls_finalize(g, m);
        c->has_g[i] = 1;
    }
    /* gradient_limit (runner/hydrodynamics.rs:104-134; LimiterData gradients.rs:58-103) */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) {
        if (!c->has_g[i]) continue;
        const particle *pt = &c->parts[i];
        vec3 centroid = pt->centroid;
        grads *g = &c->gtmp[i];
        state mn = pt->prim, mx = pt->prim;
        state emn, emx;
        for (int q = 0; q < 5; q++) { emn.q[q] = INFINITY; emx.q[q] = -INFINITY; }
        for (int32_t k = c->csr_off[i]; k < c->csr_off[i + 1]; k++) {
            const face *f = &c->faces[c->csr_face[k]];
            vec3 shift = (i == f->left) ? f->shift : v3(-f->shift.x, -f->shift.y, -f->shift.z);
            /* the reference's offset: face centroid - centroid - shift (runner/hydrodynamics.rs:119); with
               limiter_frame set, the frame flux_exchange uses (flux.rs:33-35): the face centroid is in the
               left cell's frame, so the right cell's offset is face centroid - shift - centroid */
            vec3 off = vsub(f->centroid, centroid);
            if (!c->p.limiter_frame) off = vsub(off, shift);
            else if (i != f->left) off = vadd(off, shift);
            state ex = gr_dot(g, off);
            state op;
            if (f->left == i && f->right < 0) {
                particle o = boundary_part(c, pt, f);
                op = o.prim;
            } else {
                int64_t oi = (i == f->left) ? f->right : f->left;
                op = c->parts[oi].prim;
            }
            for (int q = 0; q < 5; q++) {
                mn.q[q] = fmin(mn.q[q], op.q[q]);
                mx.q[q] = fmax(mx.q[q], op.q[q]);
                emn.q[q] = fmin(emn.q[q], ex.q[q]);
                emx.q[q] = fmax(emx.q[q], ex.q[q]);
            }
        }
        for (int q = 0; q < 5; q++) {
            double d_max = mx.q[q] - pt->prim.q[q];
            double d_min = mn.q[q] - pt->prim.q[q];
            double alpha;
            if (emx.q[q] == 0. || emn.q[q] == 0.) alpha = 1.;
            else alpha = fmin(1.0, fmin(d_max / emx.q[q], d_min / emn.q[q]));
            g->g[q] = vscale(alpha, g->g[q]);
            g->g[q] = v3(g->g[q].x, g->g[q].y, g->g[q].z);
        }
    }
    /* gradient_apply (runner/hydrodynamics.rs:136-143) */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) {
        if (!c->has_g[i]) continue;
        c->parts[i].grad = c->gtmp[i];
        c->parts[i].gc = c->parts[i].centroid;
    }
}

/* Particle::radius (part.rs:439-447) */
static inline double radius(const particle *pt, int dim) {
    if (dim == 1) return 0.5 * pt->volume;
    if (dim == 2) return sqrt(0.31830988618379067154 * pt->volume);
    return pow(0.25 * 3. * 0.31830988618379067154 * pt->volume, 1. / 3.);
}

/* Particle::set_particle_velocity (part.rs:328-372) */
static vec3 particle_velocity(const particle *pt, vec3 fluid_v, double sound_speed, int motion, int dim) {
    if (motion == ORC_MOTION_FIXED) return v3(0., 0., 0.);
    if (motion == ORC_MOTION_FLUID) return fluid_v;
    vec3 d = vsub(pt->centroid, pt->loc);
    if (motion == ORC_MOTION_STEER) {
        double abs_d = vlen(d);
        double eta = 0.25;
        double eta_r = eta * radius(pt, dim);
        double xi = 0.99;
        if (abs_d > 0.9 * eta_r) {
            double fac = xi * sound_speed / abs_d;
            if (abs_d < 1.1 * eta_r) fac *= 5. * (abs_d - 0.9 * eta_r) / eta_r;
            return vadd(fluid_v, vscale(fac, d));
        }
        return fluid_v;
    }
    /* SteerPakmor */
    double alpha = 2. / (double)dim * pt->max_a_over_r;
    double beta = 2.25;
    double eta = fmax(0., fmin(0.5, 2. / beta * (alpha - 0.75 * beta)));
    vec3 dn = vscale(1.0 / vlen(d), d); /* DVec3::normalize */
    /* Gradients::curl_v (physical_quantities.rs:149-155) */
    vec3 curl = v3(pt->grad.g[3].y - pt->grad.g[2].z, pt->grad.g[1].z - pt->grad.g[3].x,
                   pt->grad.g[2].x - pt->grad.g[1].y);
    double v_reg = radius(pt, dim) * vlen(curl);
    return vadd(fluid_v, vscale(eta * fmax(sound_speed, v_reg), dn));
}

/* Particle::timestep (part.rs:42-84) */
static double particle_timestep(particle *pt, double cfl, const gaslaw *eos, int dim, int motion, uint32_t *err) {
    if (pt->cons.q[0] == 0.) {
        pt->v = v3(0., 0., 0.);
        return INFINITY;
    }
    double m_inv = 1. / pt->cons.q[0];
    vec3 d_v = st_vel(gr_dot(&pt->grad, vsub(pt->loc, pt->gc)));
    vec3 mom = st_vel(pt->cons);
    vec3 fluid_v = vadd(v3(mom.x * m_inv, mom.y * m_inv, mom.z * m_inv), d_v);
    /* Particle::internal_energy (part.rs:314-317) */
    double u = (pt->cons.q[4] - 0.5 * vdot(mom, st_vel(pt->prim))) / pt->cons.q[0];
    double c = sound_speed(eos, gas_pressure_from_internal_energy(eos, u, pt->prim.q[0]), pt->volume * m_inv);
    pt->v = particle_velocity(pt, fluid_v, c, motion, dim);
    if (!isfinite(pt->v.x) || !isfinite(pt->v.y) || !isfinite(pt->v.z)) *err |= ORC_ERR_NONFINITE; /* :366 */
    pt->v_rel = vsub(fluid_v, pt->v);
    pt->max_a_over_r = 0.;
    double v_max = fmax(pt->max_signal_velocity, vlen(pt->v_rel) + c);
    pt->max_signal_velocity = 0.;
    if (v_max > 0.) return cfl * radius(pt, dim) / v_max;
    return INFINITY;
}

/* --- gravity (gravity.rs) --- */
/* KeplerianPotential::acceleration (gravity.rs:125-136) */
static vec3 kepler_acceleration(const orc_params *p, vec3 pos) {
    vec3 dx = vsub(pos, v3(p->gravity_position[0], p->gravity_position[1], p->gravity_position[2]));
    double r2 = vdot(dx, dx);
    double r = sqrt(r2);
    if (r < p->gravity_softening) r2 = r2 + p->gravity_softening * p->gravity_softening;
    double d = r * r2;
    return v3(-dx.x / d, -dx.y / d, -dx.z / d);
}
/* KeplerianPotential::circular_velocity (gravity.rs:138-147) */
static double kepler_circular_velocity(const orc_params *p, vec3 pos) {
    vec3 dx = vsub(pos, v3(p->gravity_position[0], p->gravity_position[1], p->gravity_position[2]));
    double r = sqrt(vdot(dx, dx));
    double r_softened = r < p->gravity_softening ? r + p->gravity_softening : r;
    return sqrt(1. / r_softened);
}
/* GravitySolver::compute_timesteps (gravity.rs:45-53, 71-73, 90-95, 119-123) */
static double gravity_timestep(const orc_ctx *c, const particle *pt) {
    switch (c->p.gravity) {
        case ORC_GRAVITY_SELF: {
            double a2 = vdot(pt->a_grav, pt->a_grav);
            if (a2 == 0.) return INFINITY;
            return sqrt(c->p.gravity_softening / sqrt(a2));
        }
        case ORC_GRAVITY_KEPLERIAN: /* eta = 0.5, radius in 2D whatever the dimensionality */
            return 0.5 * radius(pt, 2) / kepler_circular_velocity(&c->p, pt->loc);
        default:
            return INFINITY;
    }
}
/* SelfGravity::compute_accelerations (gravity.rs:22-43): particle i sums the
   pull of the particles after it only (j > i), in index order, with the
   softening added to the distance; every particle's a_grav is replaced. */
static void self_gravity_accelerations(orc_ctx *c) {
    const double eps = c->p.gravity_softening;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < c->n; i++) {
        const vec3 li = c->parts[i].loc;
        vec3 a = v3(0., 0., 0.);
        for (int64_t j = i + 1; j < c->n; j++) {
            const particle *pj = &c->parts[j];
            double r = vlen(vsub(pj->loc, li)) + eps;
            vec3 dir = vsub(pj->loc, li);
            vec3 m = vscale(pj->cons.q[0], dir); /* mass * dir */
            double r3 = r * r * r;
            a = vadd(a, v3(m.x / r3, m.y / r3, m.z / r3));
        }
        c->parts[i].a_grav = a;
    }
}

/* GravitySolver::compute_accelerations: SelfGravity, or
   ExternalPotentialGravity (gravity.rs:67-70, 81-86) */
static void gravity_accelerations(orc_ctx *c) {
    if (c->p.gravity == ORC_GRAVITY_SELF) {
        self_gravity_accelerations(c);
        return;
    }
    if (c->p.gravity != ORC_GRAVITY_CONSTANT && c->p.gravity != ORC_GRAVITY_KEPLERIAN) return;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) {
        particle *pt = &c->parts[i];
        if (c->p.gravity == ORC_GRAVITY_CONSTANT)
            pt->a_grav = v3(c->p.gravity_acceleration[0], c->p.gravity_acceleration[1], c->p.gravity_acceleration[2]);
        else
            pt->a_grav = kepler_acceleration(&c->p, pt->loc);
    }
}

static void compute_timesteps(orc_ctx *c, const uint8_t *active, double *out) {
    uint32_t e = 0;
#pragma omp parallel for schedule(static) reduction(| : e)
    for (int64_t i = 0; i < c->n; i++) {
        if (!active[i]) { out[i] = INFINITY; continue; }
        out[i] = particle_timestep(&c->parts[i], c->p.cfl, &c->eos, c->p.dimensionality, c->p.particle_motion, &e);
    }
    c->err |= e;
}
/* The runners take the gravity solver's timestep per cell where it is smaller
   (runner/hydrodynamics/optimal_order.rs:47-50, godunov.rs:41-44). */
static void gravity_timestep_limit(orc_ctx *c, double *dts) {
    if (c->p.gravity == ORC_GRAVITY_NONE) return;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) dts[i] = fmin(dts[i], gravity_timestep(c, &c->parts[i]));
}

void orc_gravity_timesteps(orc_ctx *c, double *dt_out) {
    for (int64_t i = 0; i < c->n; i++) dt_out[i] = gravity_timestep(c, &c->parts[i]);
}
void orc_gravity_accelerations(orc_ctx *c, double *a_out) {
    gravity_accelerations(c);
    for (int64_t i = 0; i < c->n; i++) {
        a_out[i] = c->parts[i].a_grav.x;
        a_out[c->n + i] = c->parts[i].a_grav.y;
        a_out[2 * c->n + i] = c->parts[i].a_grav.z;
    }
}

/* TimestepInfo helpers (engine.rs:55-80) */
static inline double dt_from_dti(const orc_ctx *c, uint64_t dti) { return (double)dti * c->time_base; }

/* Particle::timestep_limit (part.rs:263-297) */
static void timestep_limit(const orc_ctx *c, particle *pt, int wakeup, uint64_t ti_current) {
    if (wakeup >= pt->timebin) return;
    if (pt->timebin <= get_max_active_bin(ti_current)) { /* bin_is_starting */
        pt->timebin = wakeup;
        pt->dt = dt_from_dti(c, get_integer_timestep(pt->timebin));
    } else {
        uint64_t ti_end_old = get_integer_time_end(ti_current, pt->timebin);
        pt->dt -= dt_from_dti(c, ti_end_old - ti_current);
        pt->timebin = wakeup;
        uint64_t dti_new = get_integer_timestep(pt->timebin);
        uint64_t ti_end = get_integer_time_end(ti_current, pt->timebin);
        pt->dt += (ti_end == ti_current) ? dt_from_dti(c, dti_new) : dt_from_dti(c, ti_end - ti_current);
    }
}

/* timesteps_apply (runner/hydrodynamics.rs:145-158) */
static uint64_t timesteps_apply(orc_ctx *c, const double *dts, const uint8_t *active, uint64_t ti_current) {
    uint64_t mn = UINT64_MAX;
    uint32_t err = 0;
#pragma omp parallel for schedule(static) reduction(min : mn) reduction(| : err)
    for (int64_t i = 0; i < c->n; i++) {
        uint64_t dti;
        if (!active[i]) {
            dti = MAX_NR_TIMESTEPS;
        } else {
            particle *pt = &c->parts[i];
            dti = make_integer_timestep(dts[i], pt->timebin, NUM_TIME_BINS, ti_current, c->time_base_inv, &err);
            pt->dt = dt_from_dti(c, dti); /* set_timestep (part.rs:319-322) */
            pt->timebin = get_time_bin(dti);
        }
        if (dti < mn) mn = dti;
    }
    c->err |= err;
    return mn;
}

/* timestep_limiter (runner/hydrodynamics.rs:160-184) */
static void timestep_limiter(orc_ctx *c, const uint8_t *active, uint64_t ti_current) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) {
        int wakeup = c->parts[i].timebin;
        for (int32_t k = c->csr_off[i]; k < c->csr_off[i + 1]; k++) {
            const face *f = &c->faces[c->csr_face[k]];
            int64_t oi;
            if (i == f->left) {
                if (f->right < 0) continue;
                oi = f->right;
            } else {
                oi = f->left;
            }
            if (!active[oi]) continue;
            int cand = c->parts[oi].timebin + TIME_BIN_NEIGHBOUR_MAX_DELTA_BIN;
            if (cand < wakeup) wakeup = cand;
        }
        c->wake[i] = wakeup;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) timestep_limit(c, &c->parts[i], c->wake[i], ti_current);
}

/* timestep_sync (runner/hydrodynamics.rs:186-191) */
static void timestep_sync(orc_ctx *c, uint64_t ti_current) {
    int mn = 127;
    for (int64_t i = 0; i < c->n; i++)
        if (c->parts[i].timebin < mn) mn = c->parts[i].timebin;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) timestep_limit(c, &c->parts[i], mn, ti_current);
}

/* ------------------------------------------------------------------ */
/* Host API                                                             */
/* ------------------------------------------------------------------ */
orc_ctx *orc_create(const orc_params *p, const orc_mesh *m) {
    orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    c->p = *p;
    if (c->p.max_newton_iter <= 0) c->p.max_newton_iter = 1000;
    c->eos.g = adiabatic_from(p->gamma);
    c->eos.eos = p->eos;
    c->eos.iso_u = p->isothermal_internal_energy;
    c->rs.kind = p->riemann;
    c->rs.airs_threshold = p->airs_threshold;
    c->rs.adv = v3(p->advection_velocity[0], p->advection_velocity[1], p->advection_velocity[2]);
    c->n = m->n_cells;
    c->nf = m->n_faces;
    c->parts = (particle *)calloc((size_t)c->n, sizeof(particle));
    c->faces = (face *)calloc((size_t)(c->nf > 0 ? c->nf : 1), sizeof(face));
    for (int64_t f = 0; f < c->nf; f++) {
        face *fc = &c->faces[f];
        fc->left = m->left[f];
        fc->right = m->right[f] < 0 ? -1 : m->right[f];
        fc->area = m->area[f];
        fc->normal = m_vec(m->normal, c->nf, f);
        fc->centroid = m_vec(m->centroid, c->nf, f);
        fc->shift = m_vec(m->shift, c->nf, f);
    }
    c->csr_off = (int32_t *)malloc(sizeof(int32_t) * (size_t)(c->n + 1));
    memcpy(c->csr_off, m->csr_off, sizeof(int32_t) * (size_t)(c->n + 1));
    int64_t nc = m->csr_off[c->n];
    c->csr_face = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nc > 0 ? nc : 1));
    memcpy(c->csr_face, m->csr_face, sizeof(int32_t) * (size_t)nc);
    /* Engine::new: time_base = t_end / MAX_NR_TIMESTEPS (engine.rs:118-119) */
    c->time_base = p->t_end / (double)MAX_NR_TIMESTEPS;
    c->time_base_inv = 1. / c->time_base;
    c->fi = (flux_info *)malloc(sizeof(flux_info) * (size_t)(c->nf > 0 ? c->nf : 1));
    c->active = (uint8_t *)malloc((size_t)c->n + 1);
    c->gtmp = (grads *)malloc(sizeof(grads) * (size_t)c->n);
    c->has_g = (uint8_t *)malloc((size_t)c->n + 1);
    c->dts = (double *)malloc(sizeof(double) * (size_t)c->n);
    c->wake = (int *)malloc(sizeof(int) * (size_t)c->n);
#ifdef _OPENMP
    if (p->n_threads > 0) omp_set_num_threads(p->n_threads);
#endif
    return c;
}

/* Space::drift (space.rs:833-854), Particle::drift (part.rs:107-119), box_wrap (part.rs:449-455) */
/* Particle::reflect_gradients (part.rs:390-428), the reference's steps as
   they are: the pressure gradient is reflected with the density gradient's
   already reflected normal component, and the velocity gradients first take
   the velocity's sign change, then are reflected themselves. */
static grads grads_reflect(grads g, vec3 n) {
    g.g[0] = vsub(g.g[0], vscale(2. * vdot(g.g[0], n), n));
    g.g[4] = vsub(g.g[4], vscale(2. * vdot(g.g[0], n), n));
    const vec3 dv_dx = v3(g.g[1].x, g.g[2].x, g.g[3].x);
    const vec3 dv_dy = v3(g.g[1].y, g.g[2].y, g.g[3].y);
    const vec3 dv_dz = v3(g.g[1].z, g.g[2].z, g.g[3].z);
    const vec3 twice = vscale(2., v3(vdot(dv_dx, n), vdot(dv_dy, n), vdot(dv_dz, n)));
    g.g[1] = vsub(g.g[1], vscale(n.x, twice));
    g.g[2] = vsub(g.g[2], vscale(n.y, twice));
    g.g[3] = vsub(g.g[3], vscale(n.z, twice));
    for (int q = 1; q <= 3; q++) g.g[q] = vsub(g.g[q], vscale(2. * vdot(g.g[q], n), n));
    return g;
}

/* utils.rs contains (:15-21) */
static int box_contains(const orc_ctx *c, vec3 pos) {
    const double *p3[3] = {&pos.x, &pos.y, &pos.z};
    int in = 1;
    for (int a = 0; a < c->p.dimensionality; a++) in = in && *p3[a] >= 0. && *p3[a] < c->p.box_size[a];
    return in;
}

/* Particle::box_reflect (part.rs:457-469) with utils.rs box_reflect
   (:34-43): the generator is mirrored into the box; where it moved, its
   primitive velocity and its gradients are reflected about the direction of
   the move.  Only loc moves (centroid and gradients_centroid stay).  A
   generator still outside (exactly on the upper face, or more than a box
   length out) fails the reference's assert. */
static void part_box_reflect(orc_ctx *c, particle *pt) {
    const vec3 old = pt->loc;
    double *loc[3] = {&pt->loc.x, &pt->loc.y, &pt->loc.z};
    for (int a = 0; a < c->p.dimensionality; a++) {
        if (*loc[a] < 0.) *loc[a] -= 2. * *loc[a];
        if (*loc[a] > c->p.box_size[a]) *loc[a] -= 2. * (*loc[a] - c->p.box_size[a]);
    }
    if (!box_contains(c, pt->loc)) c->err |= ORC_ERR_NONFINITE;
    const vec3 shift = vsub(pt->loc, old);
    if (vlen2(shift) > 0.) {
        const vec3 n = vscale(1. / vlen(shift), shift); /* shift * shift.length_recip() */
        pt->prim = prim_reflect(pt->prim, n);
        pt->grad = grads_reflect(pt->grad, n);
    }
}

/* Space::drift (space.rs:833-854) of every particle.  Outside the box a
   generator is wrapped (periodic) or reflected (reflective); in an open or
   vacuum box it stays where it drifted and the host removes it (orc_outside
   lists them). */
void orc_drift(orc_ctx *c, double dt) {
    int dim = c->p.dimensionality;
    for (int64_t i = 0; i < c->n; i++) {
        particle *pt = &c->parts[i];
        double *loc[3] = {&pt->loc.x, &pt->loc.y, &pt->loc.z};
        double *cen[3] = {&pt->centroid.x, &pt->centroid.y, &pt->centroid.z};
        double *gc[3] = {&pt->gc.x, &pt->gc.y, &pt->gc.z};
        const double v[3] = {pt->v.x, pt->v.y, pt->v.z};
        for (int a = 0; a < dim; a++) {
            *loc[a] += v[a] * dt;
            *cen[a] += v[a] * dt;
            *gc[a] += v[a] * dt;
        }
        if (!isfinite(pt->loc.x) || !isfinite(pt->loc.y) || !isfinite(pt->loc.z)) {
            c->err |= ORC_ERR_NONFINITE;
            continue;
        }
        if (box_contains(c, pt->loc)) continue;
        if (c->p.boundary == ORC_REFLECTIVE) {
            part_box_reflect(c, pt);
            continue;
        }
        if (c->p.boundary != ORC_PERIODIC) continue; /* removed by the host */
        vec3 old = pt->loc;
        for (int a = 0; a < dim; a++) {
            while (*loc[a] < 0.) *loc[a] += c->p.box_size[a];
            while (*loc[a] >= c->p.box_size[a]) *loc[a] -= c->p.box_size[a];
        }
        vec3 shift = vsub(pt->loc, old);
        pt->gc = vadd(pt->gc, shift);
        pt->centroid = vadd(pt->centroid, shift);
    }
}

void orc_set_mesh(orc_ctx *c, const orc_mesh *m, const double *volume, const double *centroid) {
    free(c->faces);
    free(c->fi);
    free(c->csr_face);
    c->nf = m->n_faces;
    c->faces = (face *)calloc((size_t)(c->nf > 0 ? c->nf : 1), sizeof(face));
    for (int64_t f = 0; f < c->nf; f++) {
        face *fc = &c->faces[f];
        fc->left = m->left[f];
        fc->right = m->right[f] < 0 ? -1 : m->right[f];
        fc->area = m->area[f];
        fc->normal = m_vec(m->normal, c->nf, f);
        fc->centroid = m_vec(m->centroid, c->nf, f);
        fc->shift = m_vec(m->shift, c->nf, f);
    }
    memcpy(c->csr_off, m->csr_off, sizeof(int32_t) * (size_t)(c->n + 1));
    int64_t nc = m->csr_off[c->n];
    c->csr_face = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nc > 0 ? nc : 1));
    memcpy(c->csr_face, m->csr_face, sizeof(int32_t) * (size_t)nc);
    c->fi = (flux_info *)malloc(sizeof(flux_info) * (size_t)(c->nf > 0 ? c->nf : 1));
    if (!c->pend_vol) {
        c->pend_vol = (double *)malloc(sizeof(double) * (size_t)c->n);
        c->pend_cen = (double *)malloc(sizeof(double) * 3 * (size_t)c->n);
    }
    memcpy(c->pend_vol, volume, sizeof(double) * (size_t)c->n);
    memcpy(c->pend_cen, centroid, sizeof(double) * 3 * (size_t)c->n);
    c->pending_geometry = 1;
}

void orc_destroy(orc_ctx *c) {
    if (!c) return;
    free(c->pend_vol);
    free(c->pend_cen);
    free(c->parts); free(c->faces); free(c->csr_off); free(c->csr_face);
    free(c->fi); free(c->active); free(c->gtmp); free(c->has_g); free(c->dts); free(c->wake);
    free(c);
}

uint32_t orc_error(const orc_ctx *c) { return c->err; }

void orc_set_cells(orc_ctx *c, const orc_cells *in) {
    int64_t n = c->n;
    for (int64_t i = 0; i < n; i++) {
        particle *pt = &c->parts[i];
        memset(pt, 0, sizeof(*pt));
        for (int q = 0; q < 5; q++) {
            pt->cons.q[q] = in->cons[q * n + i];
            pt->prim.q[q] = in->prim[q * n + i];
            pt->extrap.q[q] = in->extrap[q * n + i];
            pt->fluxes.q[q] = in->facc[q * n + i];
            pt->grad.g[q] = v3(in->grad[(3 * q) * n + i], in->grad[(3 * q + 1) * n + i], in->grad[(3 * q + 2) * n + i]);
        }
        pt->gc = m_vec(in->gc, n, i);
        pt->volume = in->volume[i];
        pt->loc = m_vec(in->loc, n, i);
        pt->centroid = m_vec(in->centroid, n, i);
        pt->v = m_vec(in->v, n, i);
        pt->v_rel = m_vec(in->v_rel, n, i);
        pt->max_a_over_r = in->max_a_over_r[i];
        pt->max_signal_velocity = in->max_signal_velocity[i];
        pt->dt = in->dt[i];
        pt->timebin = in->timebin[i];
    }
}

static inline void put3(double *a, int64_t n, int64_t i, vec3 v) { a[i] = v.x; a[n + i] = v.y; a[2 * n + i] = v.z; }

void orc_get_cells(const orc_ctx *c, orc_cells *out) {
    int64_t n = c->n;
    for (int64_t i = 0; i < n; i++) {
        const particle *pt = &c->parts[i];
        for (int q = 0; q < 5; q++) {
            out->cons[q * n + i] = pt->cons.q[q];
            out->prim[q * n + i] = pt->prim.q[q];
            out->extrap[q * n + i] = pt->extrap.q[q];
            out->facc[q * n + i] = pt->fluxes.q[q];
            out->grad[(3 * q) * n + i] = pt->grad.g[q].x;
            out->grad[(3 * q + 1) * n + i] = pt->grad.g[q].y;
            out->grad[(3 * q + 2) * n + i] = pt->grad.g[q].z;
        }
        put3(out->gc, n, i, pt->gc);
        out->volume[i] = pt->volume;
        put3(out->loc, n, i, pt->loc);
        put3(out->centroid, n, i, pt->centroid);
        put3(out->v, n, i, pt->v);
        put3(out->v_rel, n, i, pt->v_rel);
        out->max_a_over_r[i] = pt->max_a_over_r;
        out->max_signal_velocity[i] = pt->max_signal_velocity;
        out->dt[i] = pt->dt;
        out->timebin[i] = (int8_t)pt->timebin;
    }
}

/* OptimalOrderRunner::step (runner/hydrodynamics/optimal_order.rs:15-64), or
 * GodunovHydroRunner::step (runner/hydrodynamics/godunov.rs:14-58): the same
 * sequence without gradient_estimate / gradient_limit / gradient_apply. */
uint64_t orc_step(orc_ctx *c, uint64_t ti_current, uint64_t ti_old, int64_t *n_active_faces) {
    int max_bin = get_max_active_bin(ti_current);
    for (int64_t i = 0; i < c->n; i++) c->active[i] = c->parts[i].timebin <= max_bin; /* bin_is_ending */
    double dt = dt_from_dti(c, ti_current - ti_old);
    orc_predict(c, dt);
    if (c->pending_geometry) { /* Space::volume_calculation -> Particle::update_geometry (part.rs:151-158) */
        for (int64_t i = 0; i < c->n; i++) {
            if (!c->active[i]) continue;
            particle *pt = &c->parts[i];
            pt->volume = c->pend_vol[i];
            pt->centroid = v3(c->pend_cen[i], c->pend_cen[c->n + i], c->pend_cen[2 * c->n + i]);
            if (!(pt->volume >= 0.)) c->err |= ORC_ERR_NONFINITE;
        }
        c->pending_geometry = 0;
    }
    int64_t nf = compute_fluxes(c, c->active, c->fi);
    if (n_active_faces) *n_active_faces = nf;
    apply_fluxes(c, c->fi, c->active);
    /* "TODO: gravity" (runner/hydrodynamics/optimal_order.rs:33): the
       reference computes no accelerations here, so a_grav stays zero; with
       gravity_accelerations set the external potential's accelerations are
       computed at this point */
    if (c->p.gravity_accelerations) gravity_accelerations(c);
    kick2(c, c->active);
    convert_c2p(c, c->active);
    if (c->p.runner != ORC_RUNNER_GODUNOV) gradients(c, c->active);
    compute_timesteps(c, c->active, c->dts);
    gravity_timestep_limit(c, c->dts);
    uint64_t ti_next = ti_current + timesteps_apply(c, c->dts, c->active, ti_current);
    if (c->p.sync_all) timestep_sync(c, ti_current);
    else timestep_limiter(c, c->active, ti_current);
    /* reset_extrapolations (runner/hydrodynamics.rs:193-195) and kick1 (:41-49) */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) {
        if (!c->active[i]) continue;
        c->parts[i].extrap = st_vacuum();
        hydro_kick1(&c->parts[i], c->p.particle_motion, c->p.dimensionality);
        grav_kick(&c->parts[i]);
    }
    return ti_next;
}

/* Engine::run with Step sync points only (engine.rs:152-199).  Dump sync
 * points do not change the state for a fixed mesh and are not modelled. */
int64_t orc_run(orc_ctx *c, int64_t max_steps, uint64_t *ti_current, uint64_t *ti_old, int64_t *n_active_faces) {
    int64_t steps = 0, faces = 0;
    uint64_t tc = *ti_current, to = *ti_old;
    while (max_steps <= 0 || steps < max_steps) {
        int64_t nf = 0;
        uint64_t tn = orc_step(c, tc, to, &nf);
        faces += nf;
        steps++;
        if (tc >= MAX_NR_TIMESTEPS || c->err) { to = tc; tc = tn; break; }
        to = tc;
        tc = tn;
    }
    *ti_current = tc;
    *ti_old = to;
    if (n_active_faces) *n_active_faces = faces;
    return steps;
}

void orc_predict(orc_ctx *c, double dt) { /* euler_eqns_fvs.rs:20-24 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->n; i++) extrapolate_state(&c->parts[i], dt, &c->eos);
}

int64_t orc_compute_fluxes(orc_ctx *c, const uint8_t *active, double *out) {
    int64_t n = compute_fluxes(c, active, c->fi);
    int64_t nf = c->nf;
    for (int64_t f = 0; f < nf; f++) {
        const flux_info *fi = &c->fi[f];
        for (int q = 0; q < 5; q++) out[q * nf + f] = fi->fluxes.q[q];
        out[5 * nf + f] = fi->mflux.x;
        out[6 * nf + f] = fi->mflux.y;
        out[7 * nf + f] = fi->mflux.z;
        out[8 * nf + f] = fi->v_max;
        out[9 * nf + f] = fi->a_over_r;
    }
    return n;
}

void orc_apply_fluxes(orc_ctx *c, const double *in, const uint8_t *active) {
    int64_t nf = c->nf;
    for (int64_t f = 0; f < nf; f++) {
        flux_info *fi = &c->fi[f];
        for (int q = 0; q < 5; q++) fi->fluxes.q[q] = in[q * nf + f];
        fi->mflux = v3(in[5 * nf + f], in[6 * nf + f], in[7 * nf + f]);
        fi->v_max = in[8 * nf + f];
        fi->a_over_r = in[9 * nf + f];
    }
    apply_fluxes(c, c->fi, active);
    if (c->p.gravity_accelerations) gravity_accelerations(c);
    kick2(c, active);
}

void orc_convert_conserved_to_primitive(orc_ctx *c, const uint8_t *active) { convert_c2p(c, active); }
void orc_gradients(orc_ctx *c, const uint8_t *active) { gradients(c, active); }
void orc_compute_timesteps(orc_ctx *c, const uint8_t *active, double *dt_out) { compute_timesteps(c, active, dt_out); }

static inline state soa_state(const double *a, int64_t n, int64_t i) {
    state s;
    for (int q = 0; q < 5; q++) s.q[q] = a[q * n + i];
    return s;
}

void orc_riemann_flux_ex(int kind, double gamma, double airs_threshold, const double *adv, int64_t n,
                         const double *left, const double *right, const double *v_face, const double *normal,
                         double *out, uint32_t *err) {
    gaslaw eos;
    eos.g = adiabatic_from(gamma);
    eos.eos = ORC_EOS_IDEAL;
    eos.iso_u = 0.;
    rsolver rs = {kind, airs_threshold, adv ? v3(adv[0], adv[1], adv[2]) : v3(0., 0., 0.)};
    uint32_t e = 0;
    for (int64_t i = 0; i < n; i++) {
        state f = riemann_solve_for_flux(&rs, soa_state(left, n, i), soa_state(right, n, i), m_vec(v_face, n, i),
                                         m_vec(normal, n, i), &eos, 1000, &e);
        for (int q = 0; q < 5; q++) out[q * n + i] = f.q[q];
    }
    if (err) *err = e;
}

void orc_riemann_flux(int kind, double gamma, int64_t n, const double *left, const double *right,
                      const double *v_face, const double *normal, double *out, uint32_t *err) {
    orc_riemann_flux_ex(kind, gamma, 2., NULL, n, left, right, v_face, normal, out, err);
}

void orc_riemann_sample_ex(int kind, double gamma, double airs_threshold, int64_t n, const double *left,
                           const double *right, const double *normal, double *out, uint32_t *err) {
    gaslaw eos;
    eos.g = adiabatic_from(gamma);
    eos.eos = ORC_EOS_IDEAL;
    eos.iso_u = 0.;
    /* HLLC and LinearAdvection are not star solvers: sample the exact solution */
    int k = (kind == ORC_HLLC || kind == ORC_LINEAR_ADVECTION) ? ORC_EXACT : kind;
    rsolver rs = {k, airs_threshold, v3(0., 0., 0.)};
    uint32_t e = 0;
    for (int64_t i = 0; i < n; i++) {
        state w = star_half_state(&rs, soa_state(left, n, i), soa_state(right, n, i), m_vec(normal, n, i), &eos,
                                  1000, &e);
        for (int q = 0; q < 5; q++) out[q * n + i] = w.q[q];
    }
    if (err) *err = e;
}

void orc_riemann_sample(int kind, double gamma, int64_t n, const double *left, const double *right,
                        const double *normal, double *out, uint32_t *err) {
    orc_riemann_sample_ex(kind, gamma, 2., n, left, right, normal, out, err);
}

uint64_t orc_get_integer_timestep(int bin) { return get_integer_timestep(bin); }
int orc_get_time_bin(uint64_t dti) { return get_time_bin(dti); }
int orc_get_max_active_bin(uint64_t ti) { return get_max_active_bin(ti); }
uint64_t orc_make_integer_timestep(double dt, int old_bin, int min_ngb_bin, uint64_t ti_current,
                                   double time_base_inv, uint32_t *err) {
    uint32_t e = 0;
    uint64_t r = make_integer_timestep(dt, old_bin, min_ngb_bin, ti_current, time_base_inv, &e);
    if (err) *err = e;
    return r;
}

/* ExactRiemannSolver::solve_for_star_state with explicit wave inputs
 * (exact.rs:241-291), as called by the reference's regression test
 * exact.rs:440-460.  out = (rho_l, rho_r, u, p). */
void orc_exact_star(double gamma, double rho_l, double p_l, double a_l, double rho_r, double p_r, double a_r,
                    double v_l, double v_r, double *out, uint32_t *err) {
    adiabatic g = adiabatic_from(gamma);
    state l = st(rho_l, v3(0., 0., 0.), p_l), r = st(rho_r, v3(0., 0., 0.), p_r);
    uint32_t e = 0;
    star_values s = ex_star_state(l, r, v_l, v_r, a_l, a_r, &g, 1000, &e);
    out[0] = s.rho_l;
    out[1] = s.rho_r;
    out[2] = s.u;
    out[3] = s.p;
    if (err) *err = e;
}

/* keep cons_from_primitives referenced (used by the conversion round trip test) */
void orc_cons_from_primitives(double gamma, const double *prim5, double volume, double *cons5) {
    gaslaw eos;
    eos.g = adiabatic_from(gamma);
    eos.eos = ORC_EOS_IDEAL;
    eos.iso_u = 0.;
    state p;
    for (int q = 0; q < 5; q++) p.q[q] = prim5[q];
    state c = cons_from_primitives(p, volume, &eos);
    for (int q = 0; q < 5; q++) cons5[q] = c.q[q];
}
void orc_prim_from_conserved(double gamma, const double *cons5, double volume, double *prim5) {
    gaslaw eos;
    eos.g = adiabatic_from(gamma);
    eos.eos = ORC_EOS_IDEAL;
    eos.iso_u = 0.;
    uint32_t e = 0;
    state c;
    for (int q = 0; q < 5; q++) c.q[q] = cons5[q];
    state p = prim_from_conserved(c, volume, &eos, &e);
    for (int q = 0; q < 5; q++) prim5[q] = p.q[q];
}
