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
// The physics is the plain FP64 form the context kernels use (face64.cuh; this
// file is compiled with -fmad=false), so the result equals
// mvmm_compute_fluxes + mvmm_apply_fluxes + mvmm_convert_conserved_to_primitive
// on a context.  Unlike a context, which validates the mesh on upload, the
// caller's device arrays are checked by the kernels as they read them: an index
// outside its array is skipped and reported as MVMM_ERR_BOUNDS.
#include <mutex>
#include <string>

#include "../../include/mvmm_gpu.h"
#include "face64.cuh"

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

// The face physics' view of the caller's arrays.  The derived face-stage
// values a context keeps in rows written by predict (the time-extrapolation
// source and the v_max sound speed) are formed here from the state, with the
// same expressions.
struct AccNA {
    const NA& p;
    __device__ __forceinline__ St<double> prim(int i) const { return R5(p.c.prim, p.n, i); }
    __device__ __forceinline__ V3<double> gc(int i) const { return R3(p.c.gc, p.n, i); }
    __device__ __forceinline__ V3<double> cen(int i) const { return R3(p.c.centroid, p.n, i); }
    __device__ __forceinline__ V3<double> loc(int i) const { return R3(p.c.loc, p.n, i); }
    __device__ __forceinline__ V3<double> v(int i) const { return R3(p.c.v, p.n, i); }
    __device__ __forceinline__ double dt(int i) const { return p.c.dt[i]; }
    __device__ __forceinline__ double cs(int i) const {
        const double rho = p.c.prim[i];
        return gt0_64(rho) ? gas(p).sound_speed(p.c.prim[4 * p.n + i], 1. / rho) : 0.;
    }
    __device__ __forceinline__ double gdot(int i, int q, V3<double> dx) const {
        const double* g = p.c.grad;
        const int n = p.n;
        return g[(3 * q) * n + i] * dx.x + g[(3 * q + 1) * n + i] * dx.y + g[(3 * q + 2) * n + i] * dx.z;
    }
    __device__ __forceinline__ double extrap(int i, int q) const { return p.c.extrap[q * p.n + i]; }
    // Particle::time_extrapolations body before the -dt factor (part.rs:134-149)
    __device__ __forceinline__ St<double> src(int i, const St<double>& prim) const {
        const int n = p.n;
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
    __device__ __forceinline__ V3<double> fcen(int f) const { return R3(p.m.centroid, p.nf, f); }
    __device__ __forceinline__ V3<double> shift(int f) const { return R3(p.m.shift, p.nf, f); }
    __device__ __forceinline__ V3<double> normal(int f) const { return R3(p.m.normal, p.nf, f); }
    __device__ __forceinline__ double area(int f) const { return p.m.area[f]; }
    __device__ __forceinline__ int boundary() const { return p.boundary; }
};

// compute_fluxes (euler_eqns_fvs.rs:26-48) into the static scratch rows
template <int SOLVER>
__global__ void __launch_bounds__(kBlock) k_na_face(NA p) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= p.nf) return;
    const int l = p.m.left[f], r = p.m.right[f];
    FaceOut o = face_zero();
    unsigned int err = 0;
    if (l < 0 || l >= p.n || r >= p.n || r < -1 || (r < 0 && p.boundary == MVMM_BOUNDARY_PERIODIC)) {
        err |= MVMM_ERR_BOUNDS;  // the face is skipped
    } else {
        const AccNA a{p};
        const Gas<double> g = gas(p);
        const bool la = p.active[l] != 0;
        if (r >= 0) {
            const bool ra = p.active[r] != 0;
            const double dtl = p.c.dt[l], dtr = p.c.dt[r];
            if (interior_face_active(la, ra, dtl, dtr)) {
                const FacePre q = face_interior_pre(a, f, l, r, m_min(dtl, dtr));
                o = face_finish(q, solve_for_flux<double, SOLVER>(q.l, q.r, q.iv, q.n, g, g, p.max_iter, &err));
            }
        } else if (la) {
            const FacePre q = face_boundary_pre(a, f, l);
            o = face_finish(q, solve_for_flux<double, SOLVER>(q.l, q.r, q.iv, q.n, g, g, p.max_iter, &err));
        }
    }
    const size_t nf = (size_t)p.nf;
#pragma unroll
    for (int q = 0; q < 5; q++) p.scratch[q * nf + f] = o.fl.q[q];
    p.scratch[5 * nf + f] = o.v_max;
    p.scratch[6 * nf + f] = o.a_over_r;
    if (err && p.err) atomicOr(p.err, err);
}

// apply_fluxes + kick2 + convert_conserved_to_primitive (runner/hydrodynamics.rs:13-57,
// part.rs:160-261) as a CSR gather from the scratch rows
__global__ void __launch_bounds__(kBlock) k_na_update(NA p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const int n = p.n;
    const size_t nf = (size_t)p.nf;
    const bool act = p.active[i] != 0;
    unsigned int err = 0;
    St<double> facc = R5(p.c.facc, n, i);
    double msv = p.c.max_signal_velocity[i], maor = p.c.max_a_over_r[i];
    // the cell's CSR range must lie inside the caller's csr_face[csr_off[n]]
    const int k0 = p.m.csr_off[i], k1 = p.m.csr_off[i + 1], kend = p.m.csr_off[n];
    if (k0 < 0 || k1 < k0 || k1 > kend) {
        err |= MVMM_ERR_BOUNDS;
    } else {
        for (int k = k0; k < k1; k++) {
            const int f = p.m.csr_face[k];
            if (f < 0 || f >= p.nf) {
                err |= MVMM_ERR_BOUNDS;
                continue;
            }
            St<double> x;
#pragma unroll
            for (int q = 0; q < 5; q++) x.q[q] = p.scratch[q * nf + f];
            if (p.m.left[f] == i) facc = facc - x;  // update_fluxes_left (part.rs:160-167)
            else facc = facc + x;                   // update_fluxes_right (part.rs:169-176)
            if (act) {
                msv = m_max(p.scratch[5 * nf + f], msv);
                maor = m_max(maor, p.scratch[6 * nf + f]);
            }
        }
    }
    if (act) {
        const St<double> cons = zero_kick64(apply_flux64(R5(p.c.cons, n, i), facc, &err));  // + kick2
        facc = st_zero<double>();
#pragma unroll
        for (int q = 0; q < 5; q++) p.c.cons[q * n + i] = cons.q[q];
        p.c.max_signal_velocity[i] = msv;
        p.c.max_a_over_r[i] = maor;
        const St<double> prim = c2p64(cons, p.c.volume[i], gas(p), &err);
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

int cuda_fail(const char* what, cudaError_t e) {
    return report_error(MVMM_E_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
}

}  // namespace
}  // namespace mvmm

using namespace mvmm;

extern "C" int mvmm_flux_update_noalloc(const mvmm_params* prm, const mvmm_mesh* dm, mvmm_cells* dc,
                                        const uint8_t* d_active, uint32_t* d_err, void* stream) {
    if (!prm || !dm || !dc || !d_active) return report_error(MVMM_E_INVALID, "noalloc: null argument");
    if (prm->riemann >= MVMM_RIEMANN_AIRS && prm->riemann <= MVMM_RIEMANN_LINEAR_ADVECTION)
        return report_error(MVMM_E_UNSUPPORTED, "noalloc: only the HLLC, exact and PVRS solvers are supported");
    if (prm->riemann < 0 || prm->riemann > MVMM_RIEMANN_LINEAR_ADVECTION)
        return report_error(MVMM_E_INVALID, "noalloc: unknown Riemann solver");
    if (prm->precision != MVMM_PRECISION_FP64)
        return report_error(MVMM_E_UNSUPPORTED, "noalloc: only the plain FP64 form is supported");
    if (!(prm->gamma > 1.)) return report_error(MVMM_E_INVALID, "noalloc: gamma must be > 1");
    if (prm->boundary < 0 || prm->boundary > 3) return report_error(MVMM_E_INVALID, "noalloc: unknown boundary");
    if (prm->eos < 0 || prm->eos > 1) return report_error(MVMM_E_INVALID, "noalloc: unknown equation of state");
    if (dm->n_cells <= 0 || dm->n_faces < 0 || dc->n != dm->n_cells)
        return report_error(MVMM_E_INVALID, "noalloc: empty mesh or cell count differs from the mesh's");
    if (dm->n_cells > (1ll << 30)) return report_error(MVMM_E_INVALID, "noalloc: too many cells");
    if (dm->n_faces > MVMM_NOALLOC_MAX_FACES)  // the scratch array holds at most this many faces
        return report_error(MVMM_E_INVALID, "noalloc: more faces than MVMM_NOALLOC_MAX_FACES");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail("noalloc: cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return report_error(MVMM_E_CUDA, "noalloc: device ordinal above 63");
    double* scratch;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_face_scratch);
            if (e != cudaSuccess) return cuda_fail("noalloc: cudaGetSymbolAddress", e);
            if (!ptr) return report_error(MVMM_E_CUDA, "noalloc: cudaGetSymbolAddress returned null");
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
    void* args[] = {&p};
    // cudaLaunchKernel reports this launch's own status (not an earlier error of the thread)
    if (p.nf > 0) {
        const void* fn = prm->riemann == MVMM_RIEMANN_HLLC    ? (const void*)k_na_face<SOLVER_HLLC>
                         : prm->riemann == MVMM_RIEMANN_EXACT ? (const void*)k_na_face<SOLVER_EXACT>
                                                              : (const void*)k_na_face<SOLVER_PVRS>;
        e = cudaLaunchKernel(fn, dim3((p.nf + kBlock - 1) / kBlock), dim3(kBlock), args, 0, s);
        if (e != cudaSuccess) return cuda_fail("noalloc: face kernel launch", e);
    }
    e = cudaLaunchKernel((const void*)k_na_update, dim3((p.n + kBlock - 1) / kBlock), dim3(kBlock), args, 0, s);
    if (e != cudaSuccess) return cuda_fail("noalloc: update kernel launch", e);
    return MVMM_OK;
}
