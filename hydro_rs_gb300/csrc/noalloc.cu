// Allocation-free flux exchange + scatter on caller-owned device arrays.
//
// Some callers cannot call cudaMalloc: a host application that owns the whole
// device memory budget and hands this library slices of it (a serving process
// that partitions HBM up front), code that runs while its own CUDA graph is
// being captured, or code that must not risk the implicit device
// synchronisation cudaMalloc/cudaFree can cause.  mvmm_flux_update_noalloc
// serves them: the caller passes the mesh, the cell state and the active mask
// as device arrays and receives the updated state in place; the only
// intermediate, the per-face flux results, lives in the file-scope array
// g_face_scratch below, sized for MVMM_NOALLOC_MAX_FACES faces.
//
// Arithmetic is the plain FP64 form (this file is compiled with -fmad=false),
// so the result equals mvmm_compute_fluxes + mvmm_apply_fluxes +
// mvmm_convert_conserved_to_primitive on a context.
#include <mutex>

#include "../../include/mvmm_gpu.h"
#include "mvmm_device.cuh"

namespace mvmm {
namespace {

constexpr int kRows = 7;  // 5 fluxes, v_max, a_over_r
// Shared by every call on this device; kept until the process exits.
static __device__ __align__(256) double g_face_scratch[kRows * MVMM_NOALLOC_MAX_FACES];

constexpr int kBlock = 128;
constexpr int kMaxDevices = 64;

struct NA {
    int n, nf;
    mvmm_mesh m;      // device pointers
    mvmm_cells c;     // device pointers
    const uint8_t* active;
    uint32_t* err;
    double* scratch;  // device address of g_face_scratch
    double gamma, iso_u;
    int eos, boundary, max_iter;
};

__device__ __forceinline__ V3<double> R3(const double* a, int n, int i) { return {a[i], a[n + i], a[2 * n + i]}; }
__device__ __forceinline__ St<double> R5(const double* a, int n, int i) {
    St<double> s;
#pragma unroll
    for (int q = 0; q < 5; q++) s.q[q] = a[q * n + i];
    return s;
}
__device__ __forceinline__ Gas<double> gas(const NA& p) { return make_gas<double>(p.gamma, p.eos, p.iso_u); }
__device__ __forceinline__ double gdot(const NA& p, int i, int q, V3<double> dx) {
    const double* g = p.c.grad;
    int n = p.n;
    return g[(3 * q) * n + i] * dx.x + g[(3 * q + 1) * n + i] * dx.y + g[(3 * q + 2) * n + i] * dx.z;
}
// time_extrapolations source (part.rs:134-149) and v_max sound speed, from the cell state
__device__ __forceinline__ St<double> source(const NA& p, int i, const St<double>& prim) {
    int n = p.n;
    const double* g = p.c.grad;
    V3<double> vr = R3(p.c.v_rel, n, i);
    V3<double> g0 = v3(g[0 * n + i], g[1 * n + i], g[2 * n + i]);
    V3<double> g4 = v3(g[12 * n + i], g[13 * n + i], g[14 * n + i]);
    double div_v = g[3 * n + i] + g[7 * n + i] + g[11 * n + i];
    double rho_inv = 1. / prim.q[0];
    St<double> s;
    s.q[0] = prim.q[0] * div_v + dot(vr, g0);
    s.q[1] = vr.x * div_v + rho_inv * g4.x;
    s.q[2] = vr.y * div_v + rho_inv * g4.y;
    s.q[3] = vr.z * div_v + rho_inv * g4.z;
    s.q[4] = p.gamma * prim.q[4] * div_v + dot(vr, g4);
    return s;
}
__device__ __forceinline__ double vmax_c(const NA& p, const St<double>& prim) {
    return prim.q[0] > 0. ? gas(p).sound_speed(prim.q[4], 1. / prim.q[0]) : 0.;
}
__device__ __forceinline__ St<double> reconstruct(const NA& p, int i, const St<double>& prim, V3<double> dx, double td) {
    St<double> r;
#pragma unroll
    for (int q = 0; q < 5; q++) r.q[q] = (prim.q[q] + gdot(p, i, q, dx)) + p.c.extrap[q * p.n + i];
    if (prim.q[0] > 0.) {
        St<double> s = source(p, i, prim);
#pragma unroll
        for (int q = 0; q < 5; q++) r.q[q] = r.q[q] + td * s.q[q];
    } else {
#pragma unroll
        for (int q = 0; q < 5; q++) r.q[q] = r.q[q] + 0.;
    }
    return r;
}

// flux_exchange (flux.rs:23-100)
template <int SOLVER>
__device__ void face_interior(const NA& p, int f, int l, int r, double dt, double out[kRows], unsigned int* err) {
    const Gas<double> g = gas(p);
    int n = p.n, nf = p.nf;
    V3<double> fc = R3(p.m.centroid, nf, f);
    V3<double> sh = R3(p.m.shift, nf, f);
    V3<double> dx_left = fc - R3(p.c.gc, n, l);
    V3<double> dx_right = (fc - R3(p.c.gc, n, r)) - sh;
    double dx_gradients = len(dx_left - dx_right);
    V3<double> dx_centroid = (R3(p.c.centroid, n, r) + sh) - R3(p.c.centroid, n, l);
    V3<double> locl = R3(p.c.loc, n, l), locr = R3(p.c.loc, n, r);
    V3<double> dx = (locr + sh) - locl;
    St<double> pl = R5(p.c.prim, n, l), pr = R5(p.c.prim, n, r);
    double v_max = 0. + vmax_c(p, pl);
    v_max = v_max + vmax_c(p, pr);
    v_max -= m_min(dot(vel(pr) - vel(pl), dx_centroid), 0.);
    double td = -(-0.5 * dt);
    St<double> ldash = reconstruct(p, l, pl, dx_left, td);
    St<double> rdash = reconstruct(p, r, pr, dx_right, td);
    St<double> prim_left = pairwise_limiter(pl, pr, ldash, len(dx_left) / dx_gradients);
    St<double> prim_right = pairwise_limiter(pr, pl, rdash, len(dx_right) / dx_gradients);
    V3<double> vl = R3(p.c.v, n, l), vr = R3(p.c.v, n, r);
    V3<double> midpoint = 0.5 * ((locl + locr) + sh);
    double fac = dot(vr - vl, fc - midpoint) / len2(dx);
    V3<double> v_face = 0.5 * (vl + vr) - fac * dx;
    V3<double> mvf = neg(v_face);
    St<double> F = solve_for_flux<double, SOLVER>(boost(prim_left, mvf), boost(prim_right, mvf), v_face,
                                                  R3(p.m.normal, nf, f), g, g, p.max_iter, err);
    double area = p.m.area[f];
    St<double> fluxes = area * F;
#pragma unroll
    for (int q = 0; q < 5; q++) out[q] = dt * fluxes.q[q];
    out[5] = v_max;
    out[6] = area / len(dx);
}

// flux_exchange_boundary (flux.rs:102-195)
template <int SOLVER>
__device__ void face_boundary(const NA& p, int f, int i, double out[kRows], unsigned int* err) {
    const Gas<double> g = gas(p);
    int n = p.n, nf = p.nf;
    V3<double> fc = R3(p.m.centroid, nf, f);
    V3<double> nn = R3(p.m.normal, nf, f);
    V3<double> loc = R3(p.c.loc, n, i), cen = R3(p.c.centroid, n, i), gc = R3(p.c.gc, n, i);
    V3<double> rloc = loc + (2. * dot(fc - loc, nn)) * nn;
    V3<double> rcen = cen + (2. * dot(fc - cen, nn)) * nn;
    V3<double> rgc = gc + (2. * dot(fc - gc, nn)) * nn;
    V3<double> dx_face = fc - gc;
    double dx_gradients = len(rgc - gc);
    V3<double> dx_centroid = rcen - cen;
    V3<double> dx = rloc - loc;
    St<double> prim = R5(p.c.prim, n, i);
    double v_max = 0. + vmax_c(p, prim);
    double dt = p.c.dt[i];
    St<double> dash = reconstruct(p, i, prim, dx_face, -(-0.5 * dt));
    double dx_fac = len(dx_face) / dx_gradients;
    St<double> bnd;
    if (p.boundary == MVMM_BOUNDARY_REFLECTIVE) {
        St<double> rprim = reflect(prim, nn);
        dash = pairwise_limiter(prim, rprim, dash, dx_fac);
        v_max -= m_min(dot(vel(rprim) - vel(prim), dx_centroid), 0.);
        bnd = reflect(dash, nn);
    } else if (p.boundary == MVMM_BOUNDARY_OPEN) {
        dash = pairwise_limiter(prim, prim, dash, dx_fac);
        bnd = dash;
    } else {
        St<double> vac = st_zero<double>();
        dash = pairwise_limiter(prim, vac, dash, dx_fac);
        v_max += m_min(dot(vel(prim), dx_centroid), 0.);
        bnd = vac;
    }
    St<double> F = solve_for_flux<double, SOLVER>(dash, bnd, v3(0., 0., 0.), nn, g, g, p.max_iter, err);
    double area = p.m.area[f];
    St<double> fluxes = area * F;
#pragma unroll
    for (int q = 0; q < 5; q++) out[q] = dt * fluxes.q[q];
    out[5] = v_max;
    out[6] = area / len(dx);
}

// compute_fluxes (euler_eqns_fvs.rs:26-48) into the static scratch rows
template <int SOLVER>
__global__ void __launch_bounds__(kBlock) k_na_face(NA p) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= p.nf) return;
    int l = p.m.left[f], r = p.m.right[f];
    bool la = p.active[l] != 0;
    double out[kRows] = {0., 0., 0., 0., 0., 0., 0.};
    unsigned int err = 0;
    if (r >= 0) {
        bool ra = p.active[r] != 0;
        double dtl = p.c.dt[l], dtr = p.c.dt[r];
        if (!((!la && !ra) || (dtr < dtl && !ra) || (dtl < dtr && !la)))
            face_interior<SOLVER>(p, f, l, r, m_min(dtl, dtr), out, &err);
    } else if (la) {
        face_boundary<SOLVER>(p, f, l, out, &err);
    }
#pragma unroll
    for (int q = 0; q < kRows; q++) p.scratch[(size_t)q * p.nf + f] = out[q];
    if (err && p.err) atomicOr(p.err, err);
}

// apply_fluxes + kick2 + convert_conserved_to_primitive (runner/hydrodynamics.rs:13-57,
// part.rs:160-261) as a CSR gather from the scratch rows
__global__ void __launch_bounds__(kBlock) k_na_update(NA p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    int n = p.n;
    size_t nf = (size_t)p.nf;
    bool act = p.active[i] != 0;
    St<double> facc = R5(p.c.facc, n, i);
    double msv = p.c.max_signal_velocity[i], maor = p.c.max_a_over_r[i];
    for (int k = p.m.csr_off[i]; k < p.m.csr_off[i + 1]; k++) {
        int f = p.m.csr_face[k];
        St<double> x;
#pragma unroll
        for (int q = 0; q < 5; q++) x.q[q] = p.scratch[q * nf + f];
        if (p.m.left[f] == i) facc = facc - x;
        else facc = facc + x;
        if (act) {
            msv = m_max(p.scratch[5 * nf + f], msv);
            maor = m_max(maor, p.scratch[6 * nf + f]);
        }
    }
    unsigned int err = 0;
    if (act) {
        St<double> cons = R5(p.c.cons, n, i) + facc;
        for (int q = 0; q < 5; q++)
            if (!isfinite(cons.q[q])) err |= MVMM_ERR_NONFINITE;
        if (cons.q[0] < 0.) cons = st_zero<double>();
        if (cons.q[4] < 0.) cons = st_zero<double>();
        facc = st_zero<double>();
        cons.q[1] = cons.q[1] + 0.;  // kick2 with zero acceleration
        cons.q[2] = cons.q[2] + 0.;
        cons.q[3] = cons.q[3] + 0.;
#pragma unroll
        for (int q = 0; q < 5; q++) p.c.cons[q * n + i] = cons.q[q];
        p.c.max_signal_velocity[i] = msv;
        p.c.max_a_over_r[i] = maor;
        // convert_conserved_to_primitive (part.rs:219-261)
        if (!(cons.q[0] >= 0.)) err |= MVMM_ERR_NEG_MASS;
        if (!(cons.q[4] >= 0.)) err |= MVMM_ERR_NEG_ENERGY;
        St<double> prim;
        if (cons.q[0] == 0.) {
            if (cons.q[4] != 0.) err |= MVMM_ERR_NEG_ENERGY;
            prim = st_zero<double>();
        } else if (cons.q[0] > 0.) {
            double m_inv = 1. / cons.q[0];
            double density = cons.q[0] / p.c.volume[i];
            V3<double> velocity = m_inv * vel(cons);
            double thermal = cons.q[4] - 0.5 * len2(vel(cons)) * m_inv;
            double u = thermal * m_inv;
            prim = st(density, velocity, gas(p).pressure_from_internal_energy(u, density));
        } else {
            prim = st_zero<double>();
        }
        if (!(prim.q[0] >= 0.) || !(prim.q[4] >= 0.)) err |= MVMM_ERR_NEG_PRIM;
#pragma unroll
        for (int q = 0; q < 5; q++) p.c.prim[q * n + i] = prim.q[q];
    }
#pragma unroll
    for (int q = 0; q < 5; q++) p.c.facc[q * n + i] = facc.q[q];
    if (err && p.err) atomicOr(p.err, err);
}

// Device address of g_face_scratch, looked up once per device.
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

}  // namespace
}  // namespace mvmm

using namespace mvmm;

extern "C" int mvmm_flux_update_noalloc(const mvmm_params* prm, const mvmm_mesh* dm, mvmm_cells* dc,
                                        const uint8_t* d_active, uint32_t* d_err, void* stream) {
    if (!prm || !dm || !dc || !d_active) return MVMM_E_INVALID;
    if (prm->precision != MVMM_PRECISION_FP64 || prm->riemann < 0 || prm->riemann > 2 || !(prm->gamma > 1.) ||
        prm->boundary < 0 || prm->boundary > 3 || prm->eos < 0 || prm->eos > 1)
        return MVMM_E_INVALID;
    if (dm->n_cells <= 0 || dm->n_faces < 0 || dc->n != dm->n_cells) return MVMM_E_INVALID;
    if (dm->n_faces > MVMM_NOALLOC_MAX_FACES) return MVMM_E_INVALID;  // scratch holds at most this many faces
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MVMM_E_CUDA;
    double* scratch;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_face_scratch);
            if (e != cudaSuccess || !ptr) return MVMM_E_CUDA;
            g_scratch_addr[dev] = static_cast<double*>(ptr);
        }
        scratch = g_scratch_addr[dev];
    }
    NA p{};
    p.n = (int)dm->n_cells;
    p.nf = (int)dm->n_faces;
    p.m = *dm;
    p.c = *dc;
    p.active = d_active;
    p.err = d_err;
    p.scratch = scratch;
    p.gamma = prm->gamma;
    p.iso_u = prm->isothermal_internal_energy;
    p.eos = prm->eos;
    p.boundary = prm->boundary;
    p.max_iter = prm->max_newton_iter > 0 ? prm->max_newton_iter : 1000;
    cudaStream_t s = (cudaStream_t)stream;
    if (p.nf > 0) {
        int g = (p.nf + kBlock - 1) / kBlock;
        if (prm->riemann == MVMM_RIEMANN_HLLC) k_na_face<SOLVER_HLLC><<<g, kBlock, 0, s>>>(p);
        else if (prm->riemann == MVMM_RIEMANN_EXACT) k_na_face<SOLVER_EXACT><<<g, kBlock, 0, s>>>(p);
        else k_na_face<SOLVER_PVRS><<<g, kBlock, 0, s>>>(p);
    }
    k_na_update<<<(p.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(p);
    return cudaGetLastError() == cudaSuccess ? MVMM_OK : MVMM_E_CUDA;
}
