// Device-side physics of the per-face finite-volume update.
//
// Templated over the arithmetic type T of the face stage (double for the plain
// form, float for the FP32-face form).  Expressions keep the reference's
// evaluation order term by term; the plain form is compiled with -fmad=false so
// that nothing is contracted into an FMA (Rust never contracts), which makes
// the FP64 path reproduce the reference's arithmetic except inside pow().
// References are paths inside the mvmm_hydro source tree.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "bitconv.cuh"
#include "mvmm_internal.h"

namespace mvmm {

// ------------------------------------------------------------------ math --
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float m_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
// Rust f64::min / f64::max: IEEE minNum / maxNum (the non-NaN operand wins).
__device__ __forceinline__ double m_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float m_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double m_max(double a, double b) { return fmax(a, b); }

// Comparisons of a double with zero, and isfinite, evaluated on its bit
// pattern with integer instructions: the same truth values as the
// floating-point forms (NaN compares false, -0.0 == 0.0), without occupying
// the FP64 pipe, which on this GPU runs at 1/64 of the FP32 rate.
__device__ __forceinline__ unsigned long long mag64(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
constexpr unsigned long long kInf64 = 0x7ff0000000000000ull;
__device__ __forceinline__ bool is_nan64(double x) { return mag64(x) > kInf64; }
__device__ __forceinline__ bool is_finite64(double x) { return mag64(x) < kInf64; }
__device__ __forceinline__ bool is_zero64(double x) { return mag64(x) == 0; }  // x == 0.
__device__ __forceinline__ bool lt0_64(double x) {                              // x < 0.
    return __double_as_longlong(x) < 0 && mag64(x) != 0 && mag64(x) <= kInf64;
}
__device__ __forceinline__ bool gt0_64(double x) {  // x > 0.
    return __double_as_longlong(x) > 0 && mag64(x) <= kInf64;
}
__device__ __forceinline__ bool ge0_64(double x) { return !is_nan64(x) && (__double_as_longlong(x) >= 0 || mag64(x) == 0); }
__device__ __forceinline__ float m_max(float a, float b) { return fmaxf(a, b); }

// The active-face rule of compute_fluxes (euler_eqns_fvs.rs:35-45) for an
// interior face: false where the face is skipped.
__device__ __forceinline__ bool interior_face_active(bool la, bool ra, double dtl, double dtr) {
    return !((!la && !ra) || (dtr < dtl && !ra) || (dtl < dtr && !la));
}

template <typename T>
struct V3 {
    T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3<T> v3(T x, T y, T z) { return {x, y, z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T>
__device__ __forceinline__ V3<T> neg(V3<T> a) { return {-a.x, -a.y, -a.z}; }
// glam DVec3::dot: x*x' + y*y' + z*z' left to right.
template <typename T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T>
__device__ __forceinline__ T len2(V3<T> a) { return dot(a, a); }
template <typename T>
__device__ __forceinline__ T len(V3<T> a) { return m_sqrt(dot(a, a)); }
template <typename T>
__device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {  // glam DVec3::cross
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <typename T, typename U>
__device__ __forceinline__ V3<T> cvt(V3<U> a) { return {T(a.x), T(a.y), T(a.z)}; }
// FP64 <-> FP32 conversions of the cell kernels, on the integer pipe
// (bitconv.cuh): the same values as the conversion instructions, which share
// the slow FP64 pipe.
__device__ __forceinline__ float f32(double x) { return bitconv::to_f32_rn(x); }
__device__ __forceinline__ double f64(float x) { return bitconv::to_f64(x); }
__device__ __forceinline__ V3<float> f32v(V3<double> a) { return {f32(a.x), f32(a.y), f32(a.z)}; }
__device__ __forceinline__ V3<double> f64v(V3<float> a) { return {f64(a.x), f64(a.y), f64(a.z)}; }

// State<T>(f64, DVec3, f64): 0 density/mass, 1..3 velocity/momentum, 4 pressure/energy.
template <typename T>
struct St {
    T q[5];
};
template <typename T>
__device__ __forceinline__ St<T> st(T a, V3<T> b, T c) { return {{a, b.x, b.y, b.z, c}}; }
template <typename T>
__device__ __forceinline__ St<T> st_zero() { return {{T(0), T(0), T(0), T(0), T(0)}}; }
template <typename T>
__device__ __forceinline__ V3<T> vel(const St<T>& s) { return {s.q[1], s.q[2], s.q[3]}; }
template <typename T>
__device__ __forceinline__ St<T> operator+(const St<T>& a, const St<T>& b) {
    St<T> r;
#pragma unroll
    for (int i = 0; i < 5; i++) r.q[i] = a.q[i] + b.q[i];
    return r;
}
template <typename T>
__device__ __forceinline__ St<T> operator-(const St<T>& a, const St<T>& b) {
    St<T> r;
#pragma unroll
    for (int i = 0; i < 5; i++) r.q[i] = a.q[i] - b.q[i];
    return r;
}
template <typename T>
__device__ __forceinline__ St<T> operator*(T s, const St<T>& a) {
    St<T> r;
#pragma unroll
    for (int i = 0; i < 5; i++) r.q[i] = s * a.q[i];
    return r;
}

// ------------------------------------------------- rational powers --
// For gamma = m/(m-2) (m integer: 5/3 -> 5, 7/5 -> 7) every exponent the
// Riemann solvers raise to is k/m for an integer k: gm1d2g = 1/m,
// tdgm1 = m-2, gamma*tdgm1 = m, 1/gamma = (m-2)/m.  GB300 runs FP64 at a small
// fraction of its FP32 rate, so instead of a general double pow() these powers
// are built from y = x^(-1/m), computed by range reduction (x = 2^(q m + r) f),
// an FP32 seed and two division-free Newton steps y <- y + y (1 - x y^m) / m
// (quadratic convergence: ~1e-7 -> ~1e-14 -> rounding), plus integer powers by
// repeated squaring.  Accuracy is a few ulp, the same class as pow() itself.

// x^k for a small integer k >= 0 by repeated squaring
template <typename T>
__device__ __forceinline__ T ipow(T x, int k) {
    T r = T(1);
    T b = x;
    while (k) {
        if (k & 1) r = r * b;
        k >>= 1;
        if (k) b = b * b;
    }
    return r;
}

// y = x^(-1/m), r = x^(1/m) for finite normal x > 0; false otherwise.
template <int ITERS = 2>
__device__ __forceinline__ bool rat_root(double x, int m, double inv_m, double& y, double& r) {
    long long bits = __double_as_longlong(x);
    int ex = (int)((bits >> 52) & 0x7ff);
    if (!(x > 0.0) || ex == 0 || ex == 0x7ff) return false;
    int e = ex - 1023;
    int q = e >= 0 ? e / m : -((-e + m - 1) / m);  // floor(e / m)
    int rr = e - q * m;                             // 0 <= rr < m
    double xr = __longlong_as_double((bits & 0x000fffffffffffffLL) | ((long long)(rr + 1023) << 52));
    double yy = (double)exp2f(-log2f((float)xr) * (float)inv_m);
#pragma unroll
    for (int it = 0; it < ITERS; it++) {
        double t = fma(-xr, ipow(yy, m), 1.0);
        yy = fma(yy * inv_m, t, yy);
    }
    double rs = xr * ipow(yy, m - 1);  // xr^(1/m) = 1/yy; one reciprocal Newton step
    rs = fma(rs, fma(-rs, yy, 1.0), rs);  // removes the rounding of the power chain
    y = yy * __longlong_as_double((long long)(1023 - q) << 52);
    r = rs * __longlong_as_double((long long)(1023 + q) << 52);
    return true;
}
__device__ __forceinline__ float rat_root_f(float x, int m) { return powf(x, 1.0f / (float)m); }

// ------------------------------------------------------------- gas law --
// AdiabaticIndex + GasLaw (gas_law.rs:1-106).
template <typename T>
struct Gas {
    T gamma, gamma_inv, odgm1_, odgp1_, iso_u;
    int eos;  // 0 ideal, 1 isothermal
    int rm;   // m when gamma == m/(m-2) for an integer m in [3, 15], else 0
    double inv_m;
    __device__ __forceinline__ T gp1dg() const { return (gamma + T(1)) * gamma_inv; }
    __device__ __forceinline__ T gm1d2g() const { return T(0.5) * (gamma - T(1)) * gamma_inv; }
    __device__ __forceinline__ T gm1dgp1() const { return (gamma - T(1)) * odgp1_; }
    __device__ __forceinline__ T odgm1() const { return odgm1_; }
    __device__ __forceinline__ T tdgm1() const { return T(2) * odgm1_; }
    __device__ __forceinline__ T tdgp1() const { return T(2) * odgp1_; }
    __device__ __forceinline__ T internal_energy_from_pressure(T p, T rho_inv) const {
        return eos == 0 ? p * rho_inv * odgm1_ : iso_u;
    }
    __device__ __forceinline__ T pressure_from_internal_energy(T u, T rho) const {
        return eos == 0 ? (gamma - T(1)) * u * rho : (gamma - T(1)) * iso_u * rho;
    }
    __device__ __forceinline__ T sound_speed(T p, T rho_inv) const {
        return eos == 0 ? m_sqrt(gamma * p * rho_inv) : m_sqrt(iso_u * gamma * (gamma - T(1)));
    }
    // x^gm1d2g, x^-gm1d2g, x^tdgm1, x^(gamma*tdgm1), x^(1/gamma)
    __device__ __forceinline__ T pow_e1(T x) const;
    __device__ __forceinline__ T pow_me1(T x) const;
    __device__ __forceinline__ T pow_tdgm1(T x) const {
        if (rm && x > T(0)) return ipow(x, rm - 2);
        return m_pow(x, tdgm1());
    }
    __device__ __forceinline__ T pow_gtdgm1(T x) const {
        if (rm && x > T(0)) return ipow(x, rm);
        return m_pow(x, gamma * tdgm1());
    }
    __device__ __forceinline__ T pow_ginv(T x) const;
    // x^(1 / gm1d2g) with the exponent rounded as `1. / beta` is (trrs.rs:28-29):
    // an integer power when that exponent is the integer m
    __device__ __forceinline__ T pow_igm1d2g(T x) const {
        T e = T(1) / gm1d2g();
        if (rm && e == T(rm)) return ipow(x, rm);
        return m_pow(x, e);
    }
};
// pow(+-0, y) is +0 for y > 0 and +inf for y < 0 (IEEE 754 / C99 F.9.4.4):
// answered directly, as the exact solver evaluates f(0) on every face.
template <>
__device__ __forceinline__ double Gas<double>::pow_e1(double x) const {
    double y, r;
    if (x == 0.0) return 0.0;
    if (rm && rat_root(x, rm, inv_m, y, r)) return r;
    return pow(x, gm1d2g());
}
template <>
__device__ __forceinline__ double Gas<double>::pow_me1(double x) const {
    double y, r;
    if (x == 0.0) return INFINITY;
    if (rm && rat_root(x, rm, inv_m, y, r)) return y;
    return pow(x, -gm1d2g());
}
template <>
__device__ __forceinline__ double Gas<double>::pow_ginv(double x) const {
    double y, r;
    if (x == 0.0) return 0.0;
    if (rm && rat_root(x, rm, inv_m, y, r)) return ipow(r, rm - 2);
    return pow(x, 1. / gamma);
}
template <>
__device__ __forceinline__ float Gas<float>::pow_e1(float x) const { return powf(x, gm1d2g()); }
template <>
__device__ __forceinline__ float Gas<float>::pow_me1(float x) const { return powf(x, -gm1d2g()); }
template <>
__device__ __forceinline__ float Gas<float>::pow_ginv(float x) const { return powf(x, 1.0f / gamma); }

// m with gamma == m/(m-2) to within 4 ulp (3 <= m <= 15), else 0
__host__ __device__ inline int rational_gamma(double gamma) {
    if (!(gamma > 1.0) || !(gamma < 4.0)) return 0;
    double mm = 2.0 * gamma / (gamma - 1.0);
    int m = (int)(mm + 0.5);
    if (m < 3 || m > 15) return 0;
    double g = (double)m / (double)(m - 2);
    double d = g > gamma ? g - gamma : gamma - g;
    return d <= 4.0 * 2.220446049250313e-16 * gamma ? m : 0;
}
template <typename T>
__host__ __device__ inline Gas<T> make_gas(double gamma, int eos, double iso_u) {
    // AdiabaticIndex::from (gas_law.rs:9-18), constants evaluated in double
    Gas<T> g;
    g.gamma = T(gamma);
    g.gamma_inv = T(1. / gamma);
    g.odgm1_ = T(1. / (gamma - 1.));
    g.odgp1_ = T(1. / (gamma + 1.));
    g.iso_u = T(iso_u);
    g.eos = eos;
    g.rm = rational_gamma(gamma);
    g.inv_m = g.rm ? 1.0 / g.rm : 0.0;
    return g;
}

// -------------------------------------------------------- state helpers --
template <typename T>
__device__ __forceinline__ St<T> boost(const St<T>& s, V3<T> v) {  // physical_quantities.rs:228-236
    if (s.q[0] > T(0)) return st(s.q[0], vel(s) + v, s.q[4]);
    return s;
}
template <typename T>
__device__ __forceinline__ St<T> reflect(const St<T>& s, V3<T> n) {  // physical_quantities.rs:239-242
    V3<T> v = vel(s);
    return st(s.q[0], v - (T(2) * dot(v, n)) * n, s.q[4]);
}
template <typename T>
__device__ __forceinline__ void check_physical(St<T>& s) {  // physical_quantities.rs:245-254
    if (s.q[0] < T(0)) s = st_zero<T>();
    if (s.q[4] < T(0)) s = st_zero<T>();
}

// ------------------------------------------------------------- Riemann --
// flux_from_half_state (riemann_solver.rs:46-76)
template <typename T>
__device__ __forceinline__ St<T> flux_from_half_state(const St<T>& h, V3<T> iv, V3<T> n, const Gas<T>& g) {
    V3<T> hv = vel(h);
    T rho = h.q[0], p = h.q[4];
    V3<T> vt = iv + hv;
    V3<T> f0 = rho * hv;
    V3<T> f1 = (rho * vt.x) * hv;
    f1.x += p;
    V3<T> f2 = (rho * vt.y) * hv;
    f2.y += p;
    V3<T> f3 = (rho * vt.z) * hv;
    f3.z += p;
    T roe = p * g.odgm1() + T(0.5) * rho * len2(vt);
    V3<T> f4 = roe * hv + p * vt;
    return st(dot(f0, n), v3(dot(f1, n), dot(f2, n), dot(f3, n)), dot(f4, n));
}

// RiemannStarSolver samplers (riemann_solver.rs:108-221)
template <typename T>
__device__ __forceinline__ T shock_speed(T v, T a, T pdps, const Gas<T>& g) {
    return v - a * m_sqrt(T(0.5) * g.gp1dg() * pdps + g.gm1d2g());
}
template <typename T>
__device__ __forceinline__ T rarefaction_tail_speed(T u, T a, T pdps, const Gas<T>& g) {
    return u - a * g.pow_e1(pdps);
}
template <typename T>
__device__ __noinline__ St<T> sample_rarefaction_fan(St<T> s, T a, T v, V3<T> n, Gas<T> g) {
    T v_half = g.tdgp1() * (a + T(0.5) * (g.gamma - T(1)) * v);
    T base = g.tdgp1() + g.gm1dgp1() / a * v;
    return st(s.q[0] * g.pow_tdgm1(base), vel(s) + (v_half - v) * n, s.q[4] * g.pow_gtdgm1(base));
}
template <typename T>
__device__ __forceinline__ St<T> sample_middle(T rho, T u, T p, const St<T>& s, T v, V3<T> n) {
    return st(rho, vel(s) + (u - v) * n, p);
}

template <typename T>
struct Star {
    T rho_l, rho_r, u, p;
};

// Toro sampling at x/t = 0 given the star state (riemann_solver.rs:224-255)
template <typename T>
// The reference's two sides (u < 0: the right side, with -a_R; else the left)
// are written once for the side x/t = 0 falls on: that side's state, velocity,
// middle density and signed sound speed are selected, and its comparisons carry
// the side's sign (right: shock speed > 0, head speed v - a > 0, tail speed < 0
// as sg * x < 0 or > 0 with sg = -1), so the lanes of a warp run one code path
// whichever side each samples.  Each comparison and value is the one the
// reference forms on that side.
__device__ St<T> sample_star(const Star<T>& s, const St<T>& l, const St<T>& r, T vl, T vr, T al, T ar, V3<T> n,
                             const Gas<T>& g) {
    const bool right = s.u < T(0);
    const St<T> w = right ? r : l;
    const T v = right ? vr : vl;
    const T a = right ? -ar : al;
    const T rho = right ? s.rho_r : s.rho_l;
    const T sg = right ? T(-1) : T(1);
    if (s.p > w.q[4]) {  // shock
        if (sg * shock_speed(v, a, s.p / w.q[4], g) < T(0)) return sample_middle(rho, s.u, s.p, w, v, n);
        return w;
    }
    // rarefaction
    if (sg * (v - a) < T(0)) {
        if (sg * rarefaction_tail_speed(s.u, a, s.p / w.q[4], g) > T(0)) return sample_rarefaction_fan(w, a, v, n, g);
        return sample_middle(rho, s.u, s.p, w, v, n);
    }
    return w;
}

// VacuumRiemannSolver (riemann_solver/vacuum.rs:14-138)
template <typename T>
__device__ __forceinline__ bool is_vacuum(const St<T>& l, const St<T>& r, T al, T ar, T vrml, const Gas<T>& g) {
    if (l.q[0] == T(0) || r.q[0] == T(0)) return true;
    if (g.tdgm1() * (al + ar) <= vrml) return true;
    return false;
}
template <typename T>
__device__ __noinline__ St<T> vacuum_sample(St<T> l, St<T> r, T vl, T vr, T al, T ar, V3<T> n, Gas<T> g) {
    bool right_vac, left_vac;
    T sl = T(0), sr = T(0);
    if (r.q[0] == T(0)) {
        sl = vl + g.tdgm1() * al;
        right_vac = true;
        left_vac = false;
    } else if (l.q[0] == T(0)) {
        sr = vr - g.tdgm1() * ar;
        right_vac = false;
        left_vac = true;
    } else {  // vacuum creation (:78-99)
        sl = vl + g.tdgm1() * al;
        sr = vr - g.tdgm1() * ar;
        if (T(0) <= sl) {
            right_vac = true;
            left_vac = false;
        } else if (T(0) < sr) {
            return st_zero<T>();
        } else {
            right_vac = false;
            left_vac = true;
        }
    }
    if (right_vac) {  // sample_right_vacuum (:40-57)
        if (T(0) <= vl - al) return l;
        if (T(0) < sl) return sample_rarefaction_fan(l, al, vl, n, g);
        return st_zero<T>();
    }
    (void)left_vac;  // sample_left_vacuum (:59-76)
    if (T(0) <= sr) return st_zero<T>();
    if (T(0) < vr + ar) return sample_rarefaction_fan(r, -ar, vr, n, g);
    return r;
}

// ---- exact solver (riemann_solver/exact.rs), always evaluated in FP64 ----
// One side of the exact solver's Riemann problem: density, pressure, sound
// speed, and the shock terms A = 2/((gamma+1) rho), B = (gamma-1)/(gamma+1) p
// (exact.rs:14-15, 39-40, 61-62), formed once per face instead of at every
// evaluation of fb, fb' and gb (the same operations on the same inputs).
struct ExSide {
    double rho, p, a, A, B;
};
__device__ __forceinline__ ExSide ex_side(double rho, double p, double a, const Gas<double>& g) {
    return ExSide{rho, p, a, g.tdgp1() / rho, g.gm1dgp1() * p};
}
__device__ __forceinline__ double ex_fb(double p, const ExSide& s, const Gas<double>& g) {  // :12-20
    if (p > s.p) return (p - s.p) * sqrt(s.A / (p + s.B));
    return g.tdgm1() * s.a * (g.pow_e1(p / s.p) - 1.);
}
// The two sides' terms are evaluated lower-pressure side first: for a pressure
// between the two side pressures (the usual case) that side takes the shock
// branch of fb and the other the rarefaction branch, so the lanes of a warp
// take the same branches; the terms are then added in the reference's order
// (left, right), so the value is the same.
__device__ __forceinline__ double ex_f(double p, const ExSide& l, const ExSide& r, double vl, double vr,
                                       const Gas<double>& g) {  // :23-34
    const bool lo_left = l.p <= r.p;
    const double t_lo = ex_fb(p, lo_left ? l : r, g);
    const double t_hi = ex_fb(p, lo_left ? r : l, g);
    return (lo_left ? t_lo : t_hi) + (lo_left ? t_hi : t_lo) + (vr - vl);
}
// ex_f at p = 0, where a side with p_s > 0 takes the rarefaction branch with
// (0 / p_s)^e = 0: its term is (2/(gamma-1)) a (0 - 1), the same bits without
// the division and the power.
__device__ __forceinline__ double ex_fb0(const ExSide& s, const Gas<double>& g) {
    return gt0_64(s.p) ? g.tdgm1() * s.a * (0. - 1.) : ex_fb(0., s, g);
}
__device__ __forceinline__ double ex_f0(const ExSide& l, const ExSide& r, double vl, double vr, const Gas<double>& g) {
    return ex_fb0(l, g) + ex_fb0(r, g) + (vr - vl);
}
__device__ __forceinline__ double ex_fprimeb(double p, const ExSide& s, const Gas<double>& g) {  // :37-45
    if (p > s.p) return (1. - 0.5 * (p - s.p) / (s.B + p)) * sqrt(s.A / (p + s.B));
    return 1. / s.rho / s.a * g.pow_me1(p / s.p);
}
__device__ __forceinline__ double ex_gb(double p, const ExSide& s, const Gas<double>& g) {  // :60-64
    return sqrt(s.A / (p + s.B));
}
static __device__ __noinline__ double ex_guess_p(ExSide l, ExSide r, double vl, double vr, Gas<double> g) {  // :70-103
    double p_min = fmin(l.p, r.p);
    double p_max = fmax(l.p, r.p);
    double q_max = p_max / p_min;
    double ppv = 0.5 * (l.p + r.p) - 0.125 * (vr - vl) * (l.rho + r.rho) * (l.a + r.a);
    ppv = fmax(ppv, 1e-8);
    double p_guess;
    if (q_max <= 2. && p_min <= ppv && ppv <= p_max) {
        p_guess = ppv;
    } else if (ppv < p_min) {
        double base = (l.a + r.a - 0.5 * (g.gamma - 1.) * (vr - vl)) /
                      (l.a / g.pow_e1(l.p) + r.a / g.pow_e1(r.p));
        p_guess = g.pow_gtdgm1(base);
    } else {
        p_guess = (ex_gb(ppv, l, g) * l.p + ex_gb(ppv, r, g) * r.p - vr + vl) / (ex_gb(ppv, l, g) + ex_gb(ppv, r, g));
    }
    return fmax(p_guess, 1e-8);
}
// Brent's method (exact.rs:106-191); the iteration count is bounded by
// max_iter (the reference has no bound; it converges for a bracketed root).
static __device__ __noinline__ double ex_brent(double lower, double upper, double low_f, double up_f, double tol, ExSide l,
                                        ExSide r, double vl, double vr, Gas<double> g, int max_iter,
                                        unsigned int* err) {
    double a = lower, b = upper, c, d = INFINITY;
    double fa = low_f, fb = up_f, fc, s, fs, t;
    if (fa * fb > 0.) {
        *err |= 2u;
        return b;
    }
    if (fabs(fa) < fabs(fb)) { t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    c = a;
    fc = fa;
    bool mflag = true;
    int it = 0;
    while (fb != 0. && fabs(a - b) > tol * 0.5 * (a + b)) {
        if (++it > 100 * max_iter) {
            *err |= 1u;
            break;
        }
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
            mflag = true;
        } else {
            mflag = false;
        }
        const bool bisected = mflag;
        fs = ex_f(s, l, r, vl, vr, g);
        d = c;
        c = b;
        fc = fb;
        const bool b_kept = !(fa * fs < 0.);
        if (fa * fs < 0.) { b = s; fb = fs; } else { a = s; fa = fs; }
        const bool swapped = fabs(fa) < fabs(fb);
        if (swapped) { t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
        // A bisection that left b in place (and so set c = b) starts a run in
        // which every later iteration bisects too: with mflag set and c == b,
        // the test |b - c| < tol (b + c) / 2 chooses the midpoint whatever the
        // interpolant.  While each midpoint keeps fa's sign and does not
        // undercut |fb|, b stays the answer and only a moves until the bracket
        // is within the tolerance, and the loop returns b.  f is increasing in
        // p, so that holds for every midpoint if it holds at one point closer
        // to b on a's side than all of them: every midpoint is 0.5 (a_j + b)
        // with |a_j - b| > tol (a_j + b) / 2 and a_j, b in [0, p_guess], so it
        // lies more than tol b / 4 from b, and the point tol b / 8 from b
        // towards a is closer.  f is evaluated there once; where the check
        // fails the loop resumes as if the run had not been looked at.  Same
        // iterates, same result, and the ~20 evaluations of the run (the usual
        // case for nearly uniform states, whose guess lands above the root)
        // become one.
        if (bisected && b_kept && !swapped && fb != 0. && fabs(a - b) > tol * 0.5 * (a + b) &&
            it + 64 <= 100 * max_iter) {
            const double s_chk = b + copysign(0.125 * tol * fabs(b), a - b);
            const double fl = ex_f(s_chk, l, r, vl, vr, g);
            if (fl != 0. && !(fa * fl < 0.) && !(fabs(fl) < fabs(fb))) return b;
        }
    }
    return b;
}
// ex_brent's loop one evaluation of f at a time, so that a kernel can hand a
// lane whose search has ended the next search while the other lanes of its
// warp go on.  start() and step() leave either done set (the root in b, the
// error bits in err) or the next point to evaluate in x; the points, and so
// the iterates and the result, are ex_brent's: x is its s, or the point of its
// forced-bisection check (phase 1).
struct BrentMachine {
    double a, b, c, d, fa, fb, fc, x, tol;
    int it, max_it;
    bool mflag, bisected, done;
    int phase;  // 0: x is the iteration's s; 1: x is the check point
    unsigned int err;

    __device__ __forceinline__ void start(double lower, double upper, double low_f, double up_f, double tol_,
                                          int max_iter) {
        a = lower;
        b = upper;
        d = INFINITY;
        fa = low_f;
        fb = up_f;
        tol = tol_;
        max_it = 100 * max_iter;
        err = 0;
        done = false;
        phase = 0;
        if (fa * fb > 0.) {
            err |= 2u;
            done = true;
            return;
        }
        if (fabs(fa) < fabs(fb)) swap_ab();
        c = a;
        fc = fa;
        mflag = true;
        it = 0;
        next_s();
    }
    __device__ __forceinline__ void swap_ab() {
        double t = a;
        a = b;
        b = t;
        t = fa;
        fa = fb;
        fb = t;
    }
    // the loop test, then the iteration's s (or done)
    __device__ __forceinline__ void next_s() {
        if (!(fb != 0. && fabs(a - b) > tol * 0.5 * (a + b))) {
            done = true;
            return;
        }
        if (++it > max_it) {
            err |= 1u;
            done = true;
            return;
        }
        double s;
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
            mflag = true;
        } else {
            mflag = false;
        }
        bisected = mflag;
        x = s;
        phase = 0;
    }
    // f(x) given
    __device__ __forceinline__ void step(double fx) {
        if (phase == 1) {
            if (fx != 0. && !(fa * fx < 0.) && !(fabs(fx) < fabs(fb))) done = true;
            else next_s();
            return;
        }
        const double s = x, fs = fx;
        d = c;
        c = b;
        fc = fb;
        const bool b_kept = !(fa * fs < 0.);
        if (fa * fs < 0.) {
            b = s;
            fb = fs;
        } else {
            a = s;
            fa = fs;
        }
        const bool swapped = fabs(fa) < fabs(fb);
        if (swapped) swap_ab();
        if (bisected && b_kept && !swapped && fb != 0. && fabs(a - b) > tol * 0.5 * (a + b) && it + 64 <= max_it) {
            x = b + copysign(0.125 * tol * fabs(b), a - b);
            phase = 1;
        } else {
            next_s();
        }
    }
};

// The Newton loop of ex_star_pre (exact.rs:255-275) from p = 0, the guess and
// f(guess), one evaluation of f at a time (as BrentMachine for ex_brent):
// start() and step() leave either done set (the pressure in pg, brent set where
// Brent's method must follow on [0, pg] with f(pg) = fpg, the error bits in
// err) or the next point to evaluate in x.
struct NewtonMachine {
    double p, pg, fpg, x;
    int counter, max_iter;
    bool done, brent;
    unsigned int err;

    __device__ __forceinline__ void start(double p_guess, double fp_guess, int max_iter_, const ExSide& l,
                                          const ExSide& r, const Gas<double>& g) {
        p = 0.;
        pg = p_guess;
        fpg = fp_guess;
        counter = 0;
        max_iter = max_iter_;
        err = 0;
        done = false;
        brent = false;
        next_x(l, r, g);
    }
    __device__ __forceinline__ void end() {
        brent = fabs(p - pg) > 1e-6 * 0.5 * (p + pg) && fpg > 0.;
        done = true;
    }
    // the loop test, then the next iterate (or done)
    __device__ __forceinline__ void next_x(const ExSide& l, const ExSide& r, const Gas<double>& g) {
        if (!(fabs(p - pg) > 1e-6 * 0.5 * (p + pg) && fpg < 0.0)) {
            end();
            return;
        }
        p = pg;
        const bool lo_left = l.p <= r.p;
        const double d_lo = ex_fprimeb(pg, lo_left ? l : r, g);
        const double d_hi = ex_fprimeb(pg, lo_left ? r : l, g);
        pg = pg - fpg / ((lo_left ? d_lo : d_hi) + (lo_left ? d_hi : d_lo));
        x = pg;
    }
    // f(x) given
    __device__ __forceinline__ void step(double fx, const ExSide& l, const ExSide& r, const Gas<double>& g) {
        fpg = fx;
        counter += 1;
        if (counter > max_iter) {  // the reference panics here
            err |= 1u;
            end();
            return;
        }
        next_x(l, r, g);
    }
};

__device__ __forceinline__ double ex_middle_density(double p, const ExSide& s, const Gas<double>& g) {  // :193-212
    double pdps = p / s.p;
    if (pdps > 1.) return s.rho * (pdps + g.gm1dgp1()) / (g.gm1dgp1() * pdps + 1.);
    return s.rho * g.pow_ginv(pdps);
}
// ExactRiemannSolver::solve_for_star_state (exact.rs:241-291), in two parts
// around its Brent fallback so that a face kernel can hand the Brent searches
// to a second kernel (ex_star composes them).  ex_star_pre: guess_p and the
// Newton iteration; returns true where Brent's method must run on
// [0, *p_guess] (with f(*p_guess) = *fp_guess), else *p is the pressure.
static __device__ __noinline__ bool ex_star_pre(ExSide l, ExSide r, double vl, double vr, Gas<double> g, int max_iter,
                                                unsigned int* err, double* p_out, double* p_guess_out,
                                                double* fp_guess_out) {
    double p = 0.;
    double p_guess = ex_guess_p(l, r, vl, vr, g);
    double fp = ex_f0(l, r, vl, vr, g);  // p = 0
    double fp_guess = ex_f(p_guess, l, r, vl, vr, g);
    if (fp * fp_guess >= 0.) {
        int counter = 0;
        while (fabs(p - p_guess) > 1e-6 * 0.5 * (p + p_guess) && fp_guess < 0.0) {
            p = p_guess;
            // f' = f'_l + f'_r, the terms evaluated in ex_f's branch-coherent order
            const bool lo_left = l.p <= r.p;
            const double d_lo = ex_fprimeb(p_guess, lo_left ? l : r, g);
            const double d_hi = ex_fprimeb(p_guess, lo_left ? r : l, g);
            p_guess = p_guess - fp_guess / ((lo_left ? d_lo : d_hi) + (lo_left ? d_hi : d_lo));
            fp_guess = ex_f(p_guess, l, r, vl, vr, g);
            counter += 1;
            if (counter > max_iter) {  // the reference panics here
                *err |= 1u;
                break;
            }
        }
    }
    *p_guess_out = p_guess;
    *fp_guess_out = fp_guess;
    *p_out = p_guess;
    return fabs(p - p_guess) > 1e-6 * 0.5 * (p + p_guess) && fp_guess > 0.;
}
// The same in two parts, so that a face kernel can queue the Newton searches
// as well as the Brent searches and each runs with full warps.  ex_star_start:
// guess_p and the function values at 0 and at the guess (exact.rs:244-254);
// returns which stage follows: EX_DONE (the pressure is the guess), EX_NEWTON
// (the Newton loop from p = 0, exact.rs:255-275) or EX_BRENT (Brent's method
// on [0, p_guess], exact.rs:278-283).  The tests are ex_star_pre's with p = 0.
enum { EX_DONE = 0, EX_NEWTON = 1, EX_BRENT = 2 };
static __device__ __noinline__ int ex_star_start(ExSide l, ExSide r, double vl, double vr, Gas<double> g,
                                                 double* p_guess_out, double* fp_guess_out, double* fp0_out) {
    const double p = 0.;
    const double p_guess = ex_guess_p(l, r, vl, vr, g);
    const double fp = ex_f0(l, r, vl, vr, g);  // p = 0
    const double fp_guess = ex_f(p_guess, l, r, vl, vr, g);
    *p_guess_out = p_guess;
    *fp_guess_out = fp_guess;
    *fp0_out = fp;
    const bool apart = fabs(p - p_guess) > 1e-6 * 0.5 * (p + p_guess);
    if (fp * fp_guess >= 0. && apart && fp_guess < 0.0) return EX_NEWTON;
    return apart && fp_guess > 0. ? EX_BRENT : EX_DONE;
}
// Brent's method on [0, p_guess] as the reference calls it
__device__ __forceinline__ double ex_star_brent(double p_guess, double fp_guess, const ExSide& l, const ExSide& r,
                                                double vl, double vr, const Gas<double>& g, int max_iter,
                                                unsigned int* err) {
    double p = 0.;
    double fp = ex_f0(l, r, vl, vr, g);  // p = 0
    return ex_brent(p, p_guess, fp, fp_guess, 1e-6, l, r, vl, vr, g, max_iter, err);
}
// star_state_from_pstar (:214-238)
__device__ __forceinline__ Star<double> ex_star_post(double p, const ExSide& l, const ExSide& r, double vl, double vr,
                                                     const Gas<double>& g) {
    Star<double> s;
    s.u = 0.5 * (vl + vr) + 0.5 * (ex_fb(p, r, g) - ex_fb(p, l, g));
    s.rho_l = ex_middle_density(p, l, g);
    s.rho_r = ex_middle_density(p, r, g);
    s.p = p;
    return s;
}
static __device__ __noinline__ Star<double> ex_star(ExSide l, ExSide r, double vl, double vr, Gas<double> g, int max_iter,
                                            unsigned int* err) {
    double p, p_guess, fp_guess;
    if (ex_star_pre(l, r, vl, vr, g, max_iter, err, &p, &p_guess, &fp_guess))
        p = ex_star_brent(p_guess, fp_guess, l, r, vl, vr, g, max_iter, err);
    return ex_star_post(p, l, r, vl, vr, g);
}

// Exact star state for the FP32-face form: the same iteration as ex_star
// (guess_p, Newton while f < 0, else Brent, relative tolerance 1e-6, FP64;
// roots to ~1e-13 with one Newton step, as the result is rounded to FP32),
// evaluated with algebraically equal but cheaper expressions: per-side
// constants hoisted out of the loop, one m-th root per pressure (shared by
// both sides: (p/p_s)^(1/m) = p^(1/m) p_s^(-1/m)), rsqrt for the shock branch
// and a single division in Brent's inverse quadratic interpolation.  Used
// only when gamma = m/(m-2) (Gas::rm != 0).
struct ExFast {
    double rho, p, a, sqA, B, c_rar, ps_rm, ps_r, k_fp;
};
__device__ __forceinline__ ExFast ex_fast_side(const ExSide& s, const Gas<double>& g) {
    ExFast e;
    e.rho = s.rho;
    e.p = s.p;
    e.a = s.a;
    // multiplicative per-side constants from the FP32 face-stage inputs (no
    // cancellation downstream); the p_s roots below stay FP64, they meet
    // p^(1/m) in (p/p_s)^(1/m) - 1
    e.sqA = (double)sqrtf((float)g.tdgp1() / (float)s.rho);
    e.B = g.gm1dgp1() * s.p;
    e.c_rar = g.tdgm1() * s.a;
    double y, r;
    if (!rat_root<1>(s.p, g.rm, g.inv_m, y, r)) {
        y = pow(s.p, -g.inv_m);
        r = pow(s.p, g.inv_m);
    }
    e.ps_rm = y;
    e.ps_r = r;
    e.k_fp = (double)(1.0f / ((float)s.rho * (float)s.a));
    return e;
}
struct PRoot {
    double y, r;  // p^(-1/m), p^(1/m)
};
__device__ __forceinline__ PRoot proot(double p, const Gas<double>& g) {
    PRoot q;
    if (p == 0.0) {
        q.y = INFINITY;
        q.r = 0.0;
    } else if (!rat_root<1>(p, g.rm, g.inv_m, q.y, q.r)) {
        q.y = pow(p, -g.inv_m);
        q.r = pow(p, g.inv_m);
    }
    return q;
}
__device__ __forceinline__ double exf_fb(double p, const ExFast& s, const PRoot& q) {
    if (p > s.p) return (p - s.p) * s.sqA * rsqrt(p + s.B);
    return s.c_rar * (q.r * s.ps_rm - 1.);
}
__device__ __forceinline__ double exf_fpb(double p, const ExFast& s, const PRoot& q) {
    if (p > s.p) {
        double w = rsqrt(p + s.B);
        return s.sqA * w * (1. - 0.5 * (p - s.p) * (w * w));
    }
    return s.k_fp * s.ps_r * q.y;
}
__device__ __forceinline__ double exf_f(double p, const ExFast& l, const ExFast& r, double dv, const Gas<double>& g) {
    PRoot q{0., 0.};
    if (p <= l.p || p <= r.p) q = proot(p, g);
    return exf_fb(p, l, q) + exf_fb(p, r, q) + dv;
}
static __device__ __noinline__ Star<double> ex_star_fast(ExSide L, ExSide R, double vl, double vr, Gas<double> g,
                                                        int max_iter, unsigned int* err) {
    ExFast l = ex_fast_side(L, g), r = ex_fast_side(R, g);
    double dv = vr - vl;
    // guess_p (exact.rs:70-103)
    double p_min = fmin(l.p, r.p), p_max = fmax(l.p, r.p);
    double ppv = 0.5 * (l.p + r.p) - 0.125 * dv * (l.rho + r.rho) * (l.a + r.a);
    ppv = fmax(ppv, 1e-8);
    double p_guess;
    if (p_max <= 2. * p_min && p_min <= ppv && ppv <= p_max) {
        p_guess = ppv;
    } else if (ppv < p_min) {
        double base = (l.a + r.a - 0.5 * (g.gamma - 1.) * dv) / (l.a * l.ps_rm + r.a * r.ps_rm);
        p_guess = base > 0. ? ipow(base, g.rm) : pow(base, g.gamma * g.tdgm1());
    } else {
        double gl = l.sqA * rsqrt(ppv + l.B), gr = r.sqA * rsqrt(ppv + r.B);
        p_guess = (gl * l.p + gr * r.p - dv) / (gl + gr);
    }
    p_guess = fmax(p_guess, 1e-8);
    double p = 0.;
    double fp = exf_f(p, l, r, dv, g);
    double fpg = exf_f(p_guess, l, r, dv, g);
    if (fp * fpg >= 0.) {
        int counter = 0;
        while (fabs(p - p_guess) > 5e-7 * (p + p_guess) && fpg < 0.0) {
            p = p_guess;
            PRoot q{0., 0.};
            if (p_guess <= l.p || p_guess <= r.p) q = proot(p_guess, g);
            double fpr = exf_fpb(p_guess, l, q) + exf_fpb(p_guess, r, q);
            p_guess = p_guess - fpg / fpr;
            fpg = exf_f(p_guess, l, r, dv, g);
            if (++counter > max_iter) {
                *err |= 1u;
                break;
            }
        }
    }
    if (fabs(p - p_guess) > 5e-7 * (p + p_guess) && fpg > 0.) {
        // Brent's method on [0, p_guess] (exact.rs:106-191)
        double a = 0., b = p_guess, c, d = INFINITY, fa = exf_f(0., l, r, dv, g), fb = fpg, fc, s, fs, t;
        const double tol = 1e-6;
        if (fa * fb > 0.) {
            *err |= 2u;
        } else {
            if (fabs(fa) < fabs(fb)) { t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
            c = a;
            fc = fa;
            bool mflag = true;
            int it = 0;
            while (fb != 0. && fabs(a - b) > tol * 0.5 * (a + b)) {
                if (++it > 100 * max_iter) {
                    *err |= 1u;
                    break;
                }
                if (fa != fc && fb != fc) {
                    double dab = fa - fb, dac = fa - fc, dbc = fb - fc;
                    s = (a * fb * fc * dbc - b * fa * fc * dac + c * fa * fb * dab) / (dab * dac * dbc);
                } else {
                    s = b - fb * (b - a) / (fb - fa);
                }
                double tmp = 0.25 * (3. * a + b);
                if (!((s > tmp && s < b) || (s < tmp && s > b)) || (mflag && fabs(s - b) >= (0.5 * fabs(b - c))) ||
                    (!mflag && fabs(s - b) >= (0.5 * fabs(c - d))) || (mflag && fabs(b - c) < 0.5 * tol * (b + c)) ||
                    (!mflag && fabs(c - d) < 0.5 * tol * (c + d))) {
                    s = 0.5 * (a + b);
                    mflag = true;
                } else {
                    mflag = false;
                }
                fs = exf_f(s, l, r, dv, g);
                d = c;
                c = b;
                fc = fb;
                if (fa * fs < 0.) { b = s; fb = fs; } else { a = s; fa = fs; }
                if (fabs(fa) < fabs(fb)) { t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
            }
        }
        p = b;
    } else {
        p = p_guess;
    }
    // star_state_from_pstar (exact.rs:214-238)
    PRoot q{0., 0.};
    if (p <= l.p || p <= r.p) q = proot(p, g);
    Star<double> st_;
    st_.u = 0.5 * (vl + vr) + 0.5 * (exf_fb(p, r, q) - exf_fb(p, l, q));
    double gg = g.gm1dgp1();
    double pl = p / l.p, pr = p / r.p;
    st_.rho_l = pl > 1. ? l.rho * (pl + gg) / (gg * pl + 1.) : l.rho * ipow(q.r * l.ps_rm, g.rm - 2);
    st_.rho_r = pr > 1. ? r.rho * (pr + gg) / (gg * pr + 1.) : r.rho * ipow(q.r * r.ps_rm, g.rm - 2);
    st_.p = p;
    return st_;
}

// Exact star state for the FP32-face form.  GB300 runs FP64 at a small
// fraction of its FP32 rate, so the reference's search (guess_p, then Newton
// on f(p) = f_L + f_R + (v_R - v_L), exact.rs:23-34, 70-103) runs in FP32:
// Newton on x = p^(1/m) to 1e-6, then one Newton step whose f is the sum of
// the accurate FP32 terms formed without rounding (a TwoSum pair), which is
// where the near-root cancellation of f_L + f_R + dv happens; f' from FP32
// (an approximate derivative keeps Newton's convergence, at a rate set by its
// 1e-7 error).  A correction above 1e-4 of the pressure (a search that did
// not converge), a non-finite or non-positive result (near vacuum, extreme
// ratios) sends the face to the full FP64 reference iteration (ex_star_fast).
// Requires gamma = m/(m-2).
__device__ __forceinline__ double rsqrt64(double x) {  // FP32 seed + one Newton step (~1e-14)
    double w = (double)rsqrtf((float)x);
    return w * (1.5 - 0.5 * x * (w * w));
}
struct F32Side {
    float rho, p, a, sqA, B, c_rar, k_fp, ps_rm, k_fp_rm;  // ps_rm = p^(-1/m), k_fp_rm = k_fp / ps_rm
};
__device__ __forceinline__ F32Side f32_side(float rho, float p, float a, const Gas<float>& g) {
    F32Side s;
    s.rho = rho;
    s.p = p;
    s.a = a;
    s.sqA = sqrtf(g.tdgp1() / rho);
    s.B = g.gm1dgp1() * p;
    s.c_rar = g.tdgm1() * a;
    s.k_fp = 1.f / (rho * a);
    s.ps_rm = __powf(p, -g.gm1d2g());
    s.k_fp_rm = s.k_fp / s.ps_rm;
    return s;
}
// Error-free FP32 sum (Knuth's TwoSum): hi + lo carries the sum of the FP32
// addends to ~1e-14 relative.  The rounded-addition intrinsics keep a product
// passed in as x from being fused into the first addition.
struct Sum2 {
    float hi, lo;
};
__device__ __forceinline__ void sum2_add(Sum2& a, float x) {
    const float s = __fadd_rn(a.hi, x);
    const float bp = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, e);
}

// One side's f term and its derivative (exact.rs:12-20, 37-45) in FP32 at
// pp = x^m with x known: the rarefaction's (pp/p_s)^(1/m) is x p_s^(-1/m) and
// its derivative term k_fp / t is k_fp_rm / x (inv_x = 1/x), so the iteration
// takes no power.
__device__ __forceinline__ void f32_eval_x(float pp, float x, float inv_x, const F32Side& s, float& fb, float& fpb) {
    if (pp > s.p) {
        float w = rsqrtf(pp + s.B);
        float sw = s.sqA * w;
        fb = (pp - s.p) * sw;
        fpb = sw * (1.f - 0.5f * (pp - s.p) * (w * w));
    } else {
        fb = s.c_rar * fmaf(x, s.ps_rm, -1.f);
        fpb = s.k_fp_rm * inv_x;
    }
}
// One side's term of f (exact.rs:12-20) in FP32 to a few ulp of the term
// itself: (p - p_s) sqrt(A / (p + B)) for a shock, and for a rarefaction
// c ((p/p_s)^(1/m) - 1) = c expm1(log1p((p - p_s) / p_s) / m), which does not
// lose the digits of t - 1 when p is close to p_s.
__device__ __forceinline__ float side_acc(float p, const F32Side& s, float inv_m) {
    if (p > s.p) return (p - s.p) * s.sqA * rsqrtf(p + s.B);
    return s.c_rar * expm1f(log1pf((p - s.p) / s.p) * inv_m);
}
// M: the gamma's m when known at compile time (5 for 5/3, 7 for 7/5), else 0
template <int M>
static __device__ __noinline__ Star<float> ex_star_split(float rl, float pl, float al, float rr, float pr, float ar,
                                                         float vl, float vr, Gas<float> g, Gas<double> g64,
                                                         int max_iter, unsigned int* err) {
    const float z = g.gm1d2g();
    F32Side L = f32_side(rl, pl, al, g), R = f32_side(rr, pr, ar, g);
    float dv = vr - vl;
    // starting pressure: guess_p (exact.rs:70-103) in FP32
    float p_min = fminf(pl, pr), p_max = fmaxf(pl, pr);
    float ppv = fmaxf(0.5f * (pl + pr) - 0.125f * dv * (rl + rr) * (al + ar), 1e-8f);
    float p;
    if (p_max <= 2.f * p_min && p_min <= ppv && ppv <= p_max) {
        p = ppv;
    } else if (ppv < p_min) {
        float base = (al + ar - 0.5f * (g.gamma - 1.f) * dv) / (al * L.ps_rm + ar * R.ps_rm);
        p = base > 0.f ? ipow(base, M > 0 ? M : g64.rm) : 1e-8f;
    } else {
        float gl = L.sqA * rsqrtf(ppv + L.B), gr = R.sqA * rsqrtf(ppv + R.B);
        p = (gl * pl + gr * pr - dv) / (gl + gr);
    }
    p = fmaxf(p, 1e-8f);
    // Newton in FP32 on x = p^(1/m): the rarefaction terms of f are linear in
    // x (two rarefactions converge in one step) and the shock terms convex, so
    // after at most one overshoot the iterates approach the root monotonically;
    // Newton in p crawls where a step lands at small p and (p/p_s)^(1/m) is steep.
    const int m = M > 0 ? M : g64.rm;
    const float inv_m = 1.f / (float)m;
    float x = __powf(p, inv_m);
    for (int it = 0; it < 16; it++) {
        float xm1 = ipow(x, m - 1);
        float pp = xm1 * x;
        const float inv_x = 1.f / x;
        float fbl, fpl, fbr, fpr;
        f32_eval_x(pp, x, inv_x, L, fbl, fpl);
        f32_eval_x(pp, x, inv_x, R, fbr, fpr);
        float dx = (fbl + fbr + dv) / ((fpl + fpr) * (float)m * xm1);
        float xn = x - dx;
        if (!(xn > 0.f)) xn = 0.5f * x;
        bool done = fabsf(dx) <= 1e-6f * x;
        x = xn;
        if (done) break;
    }
    p = ipow(x, m);
    // one Newton step with the cancelling sum f = (v_r - v_l) + f_l + f_r of
    // accurate FP32 terms formed without rounding (a TwoSum pair, rounded once
    // at the end); f' in FP32
    float fbl, fpl, fbr, fpr;
    const float inv_x = 1.f / x;
    f32_eval_x(p, x, inv_x, L, fbl, fpl);
    f32_eval_x(p, x, inv_x, R, fbr, fpr);
    Sum2 f{vr, 0.f};
    sum2_add(f, -vl);
    sum2_add(f, side_acc(p, L, inv_m));
    sum2_add(f, side_acc(p, R, inv_m));
    const float dP = (f.hi + f.lo) / (fpl + fpr);
    const float P = p - dP;
    Star<float> s;
    // a search that ended more than 1e-4 from the root (after the step the
    // error is of order dP^2) is redone by the full FP64 iteration
    if (!(P > 0.f) || !isfinite(P) || !(fabsf(dP) <= 1e-4f * P)) {
        *err |= 1u << 16;  // counted by the face kernel as a fallback face
        Star<double> sd = ex_star_fast(ex_side((double)rl, (double)pl, (double)al, g64),
                                       ex_side((double)rr, (double)pr, (double)ar, g64), (double)vl, (double)vr, g64,
                                       max_iter, err);
        s.rho_l = (float)sd.rho_l;
        s.rho_r = (float)sd.rho_r;
        s.u = (float)sd.u;
        s.p = (float)sd.p;
        return s;
    }
    // star_state_from_pstar (exact.rs:214-238) in FP32 at the polished pressure
    const float ps = P;
    s.u = 0.5f * (vl + vr) + 0.5f * (side_acc(ps, R, inv_m) - side_acc(ps, L, inv_m));
    float gg = g.gm1dgp1();
    float qlr = ps / pl, qrr = ps / pr;
    s.rho_l = qlr > 1.f ? rl * (qlr + gg) / (gg * qlr + 1.f) : rl * ipow(__powf(qlr, z), m - 2);
    s.rho_r = qrr > 1.f ? rr * (qrr + gg) / (gg * qrr + 1.f) : rr * ipow(__powf(qrr, z), m - 2);
    s.p = ps;
    return s;
}

// PVRiemannSolver::solve_for_star_state (riemann_solver/pvrs.rs:26-46)
template <typename T>
__device__ __forceinline__ Star<T> pv_star(const St<T>& l, const St<T>& r, T vl, T vr, T al, T ar) {
    T rho_bar = T(0.5) * (l.q[0] + r.q[0]);
    T p_bar = T(0.5) * (l.q[4] + r.q[4]);
    T a_bar = T(0.5) * (al + ar);
    Star<T> s;
    s.p = p_bar + T(0.5) * (vl - vr) * rho_bar * a_bar;
    s.u = T(0.5) * ((vl + vr) + (l.q[4] - r.q[4]) / (rho_bar * a_bar));
    s.rho_l = l.q[0] + (vl - s.u) * rho_bar / a_bar;
    s.rho_r = r.q[0] + (s.u - vr) * rho_bar / a_bar;
    return s;
}

// ExactRiemannSolver::fb, middle_density and star_state_from_pstar
// (exact.rs:12-20, 193-238) in the face type T, for the star solvers that
// estimate p* in closed form and take the rest from the exact relations.
template <typename T>
__device__ __forceinline__ T xs_fb(T p, T rho, T ps, T a, const Gas<T>& g) {
    if (p > ps) {
        T cap_a = g.tdgp1() / rho;
        T cap_b = g.gm1dgp1() * ps;
        return (p - ps) * m_sqrt(cap_a / (p + cap_b));
    }
    return g.tdgm1() * a * (g.pow_e1(p / ps) - T(1));
}
template <typename T>
__device__ __forceinline__ T xs_middle_density(T p, T rho, T ps, const Gas<T>& g) {
    T pdps = p / ps;
    if (pdps > T(1)) return rho * (pdps + g.gm1dgp1()) / (g.gm1dgp1() * pdps + T(1));
    return rho * g.pow_ginv(pdps);
}
template <typename T>
__device__ __forceinline__ Star<T> star_from_pstar(T ps, const St<T>& l, const St<T>& r, T vl, T vr, T al, T ar,
                                                   const Gas<T>& g) {
    Star<T> s;
    s.u = T(0.5) * (vl + vr) + T(0.5) * (xs_fb(ps, r.q[0], r.q[4], ar, g) - xs_fb(ps, l.q[0], l.q[4], al, g));
    s.rho_l = xs_middle_density(ps, l.q[0], l.q[4], g);
    s.rho_r = xs_middle_density(ps, r.q[0], r.q[4], g);
    s.p = ps;
    return s;
}
// TSRiemannSolver (riemann_solver/tsrs.rs:18-51): two-shock p* from the PVRS guess
template <typename T>
__device__ __forceinline__ Star<T> ts_star(const St<T>& l, const St<T>& r, T vl, T vr, T al, T ar,
                                           const Gas<T>& g) {
    T rho_bar = T(0.5) * (l.q[0] + r.q[0]);
    T p_bar = T(0.5) * (l.q[4] + r.q[4]);
    T a_bar = T(0.5) * (al + ar);
    T p_guess = p_bar + T(0.5) * (vl - vr) * rho_bar * a_bar;  // PVRiemannSolver::p_star (pvrs.rs:20-22)
    T g_l = m_sqrt((g.tdgp1() / l.q[0]) / (p_guess + g.gm1dgp1() * l.q[4]));
    T g_r = m_sqrt((g.tdgp1() / r.q[0]) / (p_guess + g.gm1dgp1() * r.q[4]));
    T ps = (g_l * l.q[4] + g_r * r.q[4] - (vr - vl)) / (g_l + g_r);
    return star_from_pstar(ps, l, r, vl, vr, al, ar, g);
}
// TRRiemannSolver (riemann_solver/trrs.rs:14-32): two-rarefaction p*
template <typename T>
__device__ __forceinline__ Star<T> tr_star(const St<T>& l, const St<T>& r, T vl, T vr, T al, T ar,
                                           const Gas<T>& g) {
    T gm1d2 = T(0.5) * (g.gamma - T(1));
    T num = al + ar - gm1d2 * (vr - vl);
    T denom = al * g.pow_me1(l.q[4]) + ar * g.pow_me1(r.q[4]);  // p^-beta
    T ps = g.pow_igm1d2g(num / denom);
    return star_from_pstar(ps, l, r, vl, vr, al, ar, g);
}

// Solver kinds (riemann_solver.rs:28-44, bin/main.rs:625-642).  The face
// kernels are instantiated for HLLC, EXACT and PVRS; the other kinds share one
// instantiation (SOLVER_EXTRA) that switches on RSx::kind at run time.
enum {
    SOLVER_HLLC = 0,
    SOLVER_EXACT = 1,
    SOLVER_PVRS = 2,
    SOLVER_AIRS = 3,
    SOLVER_TSRS = 4,
    SOLVER_TRRS = 5,
    SOLVER_LINADV = 6,
    SOLVER_EXTRA = 7
};

// The FP32 gas law of a face stage (already FP32 in the FP32-face form).
__device__ __forceinline__ const Gas<float>& gas32(const Gas<float>& g) { return g; }
__device__ __forceinline__ Gas<float> gas32(const Gas<double>& g) { return make_gas<float>(g.gamma, g.eos, g.iso_u); }

// Exact star state in the face type: the FP32 search above for the
// FP32-face form with a rational gamma, else the FP64 reference iteration.
template <typename T>
__device__ __forceinline__ Star<T> exact_star(const St<T>& l, const St<T>& r, T vl, T vr, T al, T ar,
                                              const Gas<T>& g, const Gas<double>& g64, int max_iter,
                                              unsigned int* err) {
    Star<T> s;
    if (sizeof(T) == 4 && g64.rm) {
        const float a0 = float(l.q[0]), a1 = float(l.q[4]), a2 = float(al), b0 = float(r.q[0]), b1 = float(r.q[4]),
                    b2 = float(ar), u0 = float(vl), u1 = float(vr);
        Star<float> sf = g64.rm == 5   ? ex_star_split<5>(a0, a1, a2, b0, b1, b2, u0, u1, gas32(g), g64, max_iter, err)
                         : g64.rm == 7 ? ex_star_split<7>(a0, a1, a2, b0, b1, b2, u0, u1, gas32(g), g64, max_iter, err)
                                       : ex_star_split<0>(a0, a1, a2, b0, b1, b2, u0, u1, gas32(g), g64, max_iter, err);
        s.rho_l = T(sf.rho_l);
        s.rho_r = T(sf.rho_r);
        s.u = T(sf.u);
        s.p = T(sf.p);
    } else {
        ExSide L = ex_side(double(l.q[0]), double(l.q[4]), double(al), g64);
        ExSide R = ex_side(double(r.q[0]), double(r.q[4]), double(ar), g64);
        Star<double> sd = ex_star(L, R, double(vl), double(vr), g64, max_iter, err);
        s.rho_l = T(sd.rho_l);
        s.rho_r = T(sd.rho_r);
        s.u = T(sd.u);
        s.p = T(sd.p);
    }
    return s;
}

// Blanket RiemannFluxSolver impl for star solvers: half state (riemann_solver.rs:258-284).
template <typename T, int SOLVER>
__device__ __forceinline__ St<T> star_half_state(const St<T>& l, const St<T>& r, V3<T> n, const Gas<T>& g,
                                                 const Gas<double>& g64, int max_iter, unsigned int* err,
                                                 const RSx* x = nullptr) {
    T vl = dot(vel(l), n);
    T vr = dot(vel(r), n);
    T al = g.sound_speed(l.q[4], T(1) / l.q[0]);
    T ar = g.sound_speed(r.q[4], T(1) / r.q[0]);
    T vrml = vr - vl;
    if (is_vacuum(l, r, al, ar, vrml, g)) return vacuum_sample(l, r, vl, vr, al, ar, n, g);
    const int kind = SOLVER == SOLVER_EXTRA ? x->kind : SOLVER;
    Star<T> s;
    if (kind == SOLVER_EXACT) {
        s = exact_star(l, r, vl, vr, al, ar, g, g64, max_iter, err);
    } else if (kind == SOLVER_TSRS) {
        s = ts_star(l, r, vl, vr, al, ar, g);
    } else if (kind == SOLVER_TRRS) {
        s = tr_star(l, r, vl, vr, al, ar, g);
    } else {
        s = pv_star(l, r, vl, vr, al, ar);
        if (kind == SOLVER_AIRS) {  // AIRiemannSolver (airs.rs:18-38)
            T p_max = m_max(l.q[4], r.q[4]);
            T p_min = m_min(l.q[4], r.q[4]);
            if (!(p_max / p_min < T(x->airs_threshold))) s = exact_star(l, r, vl, vr, al, ar, g, g64, max_iter, err);
        }
    }
    return sample_star(s, l, r, vl, vr, al, ar, n, g);
}

// HLLCRiemannSolver (riemann_solver/hllc.rs:12-123)
template <typename T>
__device__ __forceinline__ St<T> hllc_flux_single(const St<T>& s, T v, T e, V3<T> n) {  // :97-104
    T rho_v = s.q[0] * v;
    return st(rho_v, rho_v * vel(s) + s.q[4] * n, ((s.q[0] * e) + s.q[4]) * v);
}
template <typename T>
__device__ __forceinline__ St<T> hllc_flux_star(const St<T>& s, T v, T e, T S, T s_star, V3<T> n) {  // :107-123
    T s_m_v = S - v;
    T rho = s.q[0];
    T starfac = rho * s_m_v / (S - s_star);
    V3<T> v_star = (s_star - v) * n + vel(s);
    T e_star = e + (s_star - v) * (s_star + s.q[4] / (rho * s_m_v));
    St<T> u_star = starfac * st(T(1), v_star, e_star);
    St<T> u_l = st(rho, rho * vel(s), rho * e);
    return S * (u_star - u_l);
}
template <typename T>
__device__ St<T> hllc_solve(const St<T>& l, const St<T>& r, V3<T> iv, V3<T> n, const Gas<T>& g) {
    T rho_l_inv = T(1) / l.q[0];
    T rho_r_inv = T(1) / r.q[0];
    T vl = dot(vel(l), n);
    T vr = dot(vel(r), n);
    T al = g.sound_speed(l.q[4], rho_l_inv);
    T ar = g.sound_speed(r.q[4], rho_r_inv);
    T vrml = vr - vl;
    if (is_vacuum(l, r, al, ar, vrml, g)) {
        St<T> w = vacuum_sample(l, r, vl, vr, al, ar, n, g);
        return flux_from_half_state(w, iv, n, g);
    }
    T ppvrs = T(0.5) * (l.q[4] + r.q[4]) - T(0.125) * vrml * (l.q[0] + r.q[0]) * (al + ar);
    T p_star = m_max(ppvrs, T(0));
    T q_l = T(1);
    if (p_star > l.q[4] && l.q[4] > T(0)) q_l = m_sqrt(T(1) + T(0.5) * g.gp1dg() * (p_star / l.q[4] - T(1)));
    T q_r = T(1);
    if (p_star > r.q[4] && r.q[4] > T(0)) q_r = m_sqrt(T(1) + T(0.5) * g.gp1dg() * (p_star / r.q[4] - T(1)));
    T s_l_m_v_l = -al * q_l;
    T s_r_m_v_r = ar * q_r;
    T s_star = (r.q[4] - l.q[4] + l.q[0] * vl * s_l_m_v_l - r.q[0] * vr * s_r_m_v_r) /
               (l.q[0] * s_l_m_v_l - r.q[0] * s_r_m_v_r);
    St<T> flux;
    if (s_star >= T(0)) {
        T v_l2 = len2(vel(l));
        T e_l = g.internal_energy_from_pressure(l.q[4], rho_l_inv) + T(0.5) * v_l2;
        flux = hllc_flux_single(l, vl, e_l, n);
        T s_l = s_l_m_v_l + vl;
        if (s_l < T(0)) flux = flux + hllc_flux_star(l, vl, e_l, s_l, s_star, n);
    } else {
        T v_r2 = len2(vel(r));
        T e_r = g.internal_energy_from_pressure(r.q[4], rho_r_inv) + T(0.5) * v_r2;
        flux = hllc_flux_single(r, vr, e_r, n);
        T s_r = s_r_m_v_r + vr;
        if (s_r > T(0)) flux = flux + hllc_flux_star(r, vr, e_r, s_r, s_star, n);
    }
    // de-boost to the lab frame (:85-90)
    St<T> add = st(T(0), flux.q[0] * iv, dot(iv, vel(flux)) + T(0.5) * len2(iv) * flux.q[0]);
    return flux + add;
}

// LinearAdvectionRiemannSover::solve_for_flux (riemann_solver/linear_advection.rs:17-34):
// the upwind (density, velocity, pressure) vector times the advection speed
template <typename T>
__device__ __forceinline__ St<T> linear_advection_flux(const St<T>& l, const St<T>& r, V3<T> iv, V3<T> n,
                                                       const RSx& x) {
    V3<T> va = {T(x.adv[0]), T(x.adv[1]), T(x.adv[2])};
    T v = dot(va - iv, n);
    if (v > T(0)) return v * l;
    return v * r;
}

template <typename T, int SOLVER>
__device__ __forceinline__ St<T> solve_for_flux(const St<T>& l, const St<T>& r, V3<T> iv, V3<T> n, const Gas<T>& g,
                                                const Gas<double>& g64, int max_iter, unsigned int* err,
                                                const RSx* x = nullptr) {
    if (SOLVER == SOLVER_HLLC) return hllc_solve(l, r, iv, n, g);
    if (SOLVER == SOLVER_EXTRA && x->kind == SOLVER_LINADV) return linear_advection_flux(l, r, iv, n, *x);
    St<T> w = star_half_state<T, SOLVER>(l, r, n, g, g64, max_iter, err, x);
    return flux_from_half_state(w, iv, n, g);
}

// ------------------------------------------------------------ limiters --
// pairwise_limiter_single_quantity (gradients.rs:105-132)
template <typename T>
__device__ __forceinline__ T pairwise_limiter_q(T q_l, T q_r, T q_dash, T dx_fac) {
    if (q_l == q_r) return q_l;
    T q_bar = q_l + dx_fac * (q_r - q_l);
    T q_diff = m_abs(q_l - q_r);
    T delta1 = T(0.5) * q_diff;
    T delta2 = T(0.25) * q_diff;
    if (q_l < q_r) {
        T q_min = m_min(q_l, q_r);
        T qmin = (q_min - delta1) * q_min > T(0) ? q_min - delta1 : q_min * m_abs(q_min) / (m_abs(q_min) + delta1);
        return m_max(qmin, m_min(q_bar + delta2, q_dash));
    }
    T q_max = m_max(q_l, q_r);
    T qplu = (q_max + delta1) * q_max > T(0) ? q_max + delta1 : q_max * m_abs(q_max) / (m_abs(q_max) + delta1);
    return m_min(qplu, m_max(q_bar - delta2, q_dash));
}
// pairwise_limiter (gradients.rs:134-152)
template <typename T>
__device__ __forceinline__ St<T> pairwise_limiter(const St<T>& l, const St<T>& r, const St<T>& dash, T dx_fac) {
    St<T> o;
#pragma unroll
    for (int i = 0; i < 5; i++) o.q[i] = pairwise_limiter_q(l.q[i], r.q[i], dash.q[i], dx_fac);
    check_physical(o);
    return o;
}

// ------------------------------------------------------------ timeline --
// timeline.rs constants and helpers
constexpr int NUM_TIME_BINS = 56;
constexpr int TIME_BIN_NEIGHBOUR_MAX_DELTA_BIN = 2;
__host__ __device__ __forceinline__ uint64_t get_integer_timestep(int bin) {  // :18-24
    return bin <= 0 ? 0ull : (1ull << (bin + 1));
}
constexpr uint64_t MAX_NR_TIMESTEPS = 1ull << 57;
__device__ __forceinline__ int get_time_bin(uint64_t dti) {  // :31-33 (u32 wrap, then `as i8`)
    uint32_t lz = (uint32_t)__clzll((long long)dti);
    uint32_t v = 64u - lz - 2u;
    return (int)(int8_t)(uint8_t)(v & 0xffu);
}
__device__ __forceinline__ uint64_t get_integer_time_end(uint64_t ti, int bin) {  // :53-67
    uint64_t dti = get_integer_timestep(bin);
    if (dti == 0) return 0;
    uint64_t mod = ti % dti;
    return mod == 0 ? ti : ti - mod + dti;
}
__host__ __device__ __forceinline__ int get_max_active_bin(uint64_t ti) {  // :72-83
    if (ti == 0) return NUM_TIME_BINS;
    int bin = 1;
    while (((1ull << ((bin + 1) & 63)) & ti) == 0) bin += 1;
    return bin;
}
// get_max_active_bin without the bit loop: the lowest set bit p >= 2 gives
// bin p - 1; with only bits 0/1 set the loop's shift wraps at bin 63.
__device__ __forceinline__ int max_active_bin_bits(uint64_t ti) {
    if (ti == 0) return NUM_TIME_BINS;
    uint64_t hi = ti & ~3ull;
    if (hi) return __ffsll((long long)hi) - 2;
    return (ti & 1ull) ? 63 : 64;
}
__device__ __forceinline__ uint64_t sat_u64(double x) {  // Rust `f64 as u64`
    if (!(x > 0.)) return 0;
    if (x >= 18446744073709551616.0) return ~0ull;
    return (uint64_t)x;
}
// make_integer_timestep (timeline.rs:103-139)
__device__ __forceinline__ uint64_t make_integer_timestep(double dt, int old_bin, int min_ngb_bin, uint64_t ti_current,
                                                          double time_base_inv) {
    uint64_t new_dti = sat_u64(dt * time_base_inv);
    int nb = get_time_bin(new_dti);
    int lim = min_ngb_bin + TIME_BIN_NEIGHBOUR_MAX_DELTA_BIN;
    new_dti = get_integer_timestep(nb < lim ? nb : lim);
    uint64_t current_dti = get_integer_timestep(old_bin);
    if (old_bin > 0) new_dti = new_dti < 2 * current_dti ? new_dti : 2 * current_dti;
    uint64_t timeline_dti = MAX_NR_TIMESTEPS;
    // the halving loop of the reference, as a bit operation: largest power of
    // two <= new_dti, capped at MAX (0 stays 0)
    if (new_dti < timeline_dti) timeline_dti = new_dti == 0 ? 0ull : (1ull << (63 - __clzll((long long)new_dti)));
    new_dti = timeline_dti;
    if (new_dti > current_dti) {
        uint64_t ti_end = get_integer_time_end(ti_current, old_bin);
        if ((MAX_NR_TIMESTEPS - ti_end) % new_dti != 0) new_dti = current_dti;
    }
    return new_dti;
}

}  // namespace mvmm
