"""ctypes bindings of ``libmvmm_gpu.so`` (the C ABI in ``include/mvmm_gpu.h``).

There is no CPU fallback: if the CUDA library is missing, or no GPU is present,
every entry point raises.  ``GpuSim`` drives one simulation through the
reference-shaped API (Engine / Runner / FiniteVolumeSolver); the module-level
functions expose the RiemannFluxSolver over arrays.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .layout import Cells

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmvmm_gpu.so")
MAX_NR_TIMESTEPS = 1 << 57
KERNEL_NAMES = ("predict", "face_flux", "update", "gradient_timestep", "limiter", "end")

EXPORTED = (
    "mvmm_ctx_create", "mvmm_ctx_destroy", "mvmm_ctx_set_stream", "mvmm_upload_cells", "mvmm_download_cells",
    "mvmm_error_bits", "mvmm_last_error", "mvmm_predict", "mvmm_compute_fluxes",
    "mvmm_convert_conserved_to_primitive", "mvmm_compute_timesteps", "mvmm_apply_fluxes", "mvmm_gradients",
    "mvmm_step", "mvmm_run", "mvmm_enqueue_steps", "mvmm_set_time", "mvmm_get_time", "mvmm_profile_enable",
    "mvmm_profile_read", "mvmm_riemann_flux", "mvmm_riemann_sample", "mvmm_get_stats",
    "mvmm_ctx_create_batched", "mvmm_batch_state", "mvmm_autotune", "mvmm_riemann_flux_p", "mvmm_riemann_sample_p",
    "mvmm_step_cells", "mvmm_drift", "mvmm_get_positions", "mvmm_set_mesh", "mvmm_flush_deferred",
    "mvmm_gravity_timesteps", "mvmm_gravity_accelerations", "mvmm_step_cells_changed", "mvmm_host_alloc",
    "mvmm_host_free",
)


class MvmmError(RuntimeError):
    def __init__(self, code: int, msg: str, bits: int = 0):
        super().__init__(f"mvmm error {code}: {msg}" + (f" (bits 0x{bits:x})" if bits else ""))
        self.code = code
        self.bits = bits


class _Params(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("eos", ctypes.c_int), ("isothermal_internal_energy", ctypes.c_double),
                ("cfl", ctypes.c_double), ("riemann", ctypes.c_int), ("boundary", ctypes.c_int),
                ("dimensionality", ctypes.c_int), ("sync_all", ctypes.c_int), ("t_end", ctypes.c_double),
                ("max_newton_iter", ctypes.c_int), ("precision", ctypes.c_int), ("particle_motion", ctypes.c_int),
                ("runner", ctypes.c_int), ("airs_threshold", ctypes.c_double),
                ("advection_velocity", ctypes.c_double * 3), ("box_size", ctypes.c_double * 3),
                ("gravity", ctypes.c_int), ("gravity_softening", ctypes.c_double),
                ("gravity_acceleration", ctypes.c_double * 3), ("gravity_position", ctypes.c_double * 3),
                ("gravity_accelerations", ctypes.c_int), ("limiter_frame", ctypes.c_int)]


def make_params(p, precision=None, box=(1.0, 1.0, 1.0)) -> _Params:
    """mvmm_params from an ics.Params (precision overrides p.precision; box: the mesh's box)."""
    thr, adv = p.solver_extras()
    prec = p.precision if precision is None else precision
    return _Params(p.gamma, p.eos, p.isothermal_internal_energy, p.cfl, p.riemann, p.boundary, p.dimensionality,
                   int(p.sync_all), p.t_end,
                   p.max_newton_iter, prec, p.particle_motion, p.runner, thr, (ctypes.c_double * 3)(*adv),
                   (ctypes.c_double * 3)(*[float(b) for b in box]), *p.gravity_fields())


_LIB = None


def load_library(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    vp, i64, u64, dbl, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
    pu64, pi64, pi32 = ctypes.POINTER(u64), ctypes.POINTER(i64), ctypes.POINTER(i32)
    sig = {
        "mvmm_ctx_create": (i32, [vp, vp, ctypes.POINTER(vp)]),
        "mvmm_ctx_destroy": (i32, [vp]),
        "mvmm_ctx_set_stream": (i32, [vp, vp]),
        "mvmm_upload_cells": (i32, [vp, vp]),
        "mvmm_download_cells": (i32, [vp, vp]),
        "mvmm_error_bits": (ctypes.c_uint32, [vp]),
        "mvmm_last_error": (ctypes.c_char_p, []),
        "mvmm_predict": (i32, [vp, dbl]),
        "mvmm_compute_fluxes": (i32, [vp, vp, vp, pi64]),
        "mvmm_convert_conserved_to_primitive": (i32, [vp, vp]),
        "mvmm_compute_timesteps": (i32, [vp, vp, vp]),
        "mvmm_gravity_timesteps": (i32, [vp, vp]),
        "mvmm_gravity_accelerations": (i32, [vp, vp]),
        "mvmm_apply_fluxes": (i32, [vp, vp, vp]),
        "mvmm_gradients": (i32, [vp, vp]),
        "mvmm_step": (i32, [vp, u64, u64, pu64, pi64]),
        "mvmm_run": (i32, [vp, i64, pu64, pu64, pi64, pi64, pi32]),
        "mvmm_enqueue_steps": (i32, [vp, i64]),
        "mvmm_set_time": (i32, [vp, u64, u64]),
        "mvmm_get_time": (i32, [vp, pu64, pu64, pi64, pi64, pi32]),
        "mvmm_profile_enable": (i32, [vp, i32]),
        "mvmm_profile_read": (i32, [vp, vp, vp]),
        "mvmm_riemann_flux": (i32, [i32, i32, dbl, i64, vp, vp, vp, vp, vp]),
        "mvmm_riemann_sample": (i32, [i32, i32, dbl, i64, vp, vp, vp, vp]),
        "mvmm_riemann_flux_p": (i32, [vp, i64, vp, vp, vp, vp, vp]),
        "mvmm_step_cells": (i32, [vp, vp, vp, u64, u64, pu64, pi64]),
        "mvmm_step_cells_changed": (i32, [vp, vp, vp, i64, u64, u64, pu64, pi64, pi64]),
        "mvmm_drift": (i32, [vp, dbl]),
        "mvmm_flush_deferred": (i32, [vp]),
        "mvmm_get_positions": (i32, [vp, vp]),
        "mvmm_set_mesh": (i32, [vp, vp, vp, vp]),
        "mvmm_host_alloc": (i32, [ctypes.c_size_t, ctypes.POINTER(vp)]),
        "mvmm_host_free": (i32, [vp]),
        "mvmm_riemann_sample_p": (i32, [vp, i64, vp, vp, vp, vp]),
        "mvmm_get_stats": (i32, [vp, vp]),
        "mvmm_ctx_create_batched": (i32, [vp, vp, i64, vp, vp, ctypes.POINTER(vp)]),
        "mvmm_batch_state": (i32, [vp, vp, vp, vp, vp, vp, vp]),
        "mvmm_autotune": (i32, [vp, i32, pi32, pi32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _check(rc: int, ctx=None):
    if rc != 0:
        L = load_library()
        bits = int(L.mvmm_error_bits(ctx)) if ctx else 0
        raise MvmmError(rc, L.mvmm_last_error().decode(), bits)


def _soa(a, k):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(k, -1))


def _solver_params(kind, gamma, precision, airs_threshold, velocity):
    from .ics import Params
    return make_params(Params(gamma=gamma, riemann=kind, precision=precision, airs_threshold=airs_threshold,
                              advection_velocity=velocity))


def riemann_flux(kind: int, gamma: float, left, right, v_face, normal, precision: int = 0,
                 airs_threshold=None, velocity=None):
    """RiemannFluxSolver::solve_for_flux over arrays on the GPU."""
    L = load_library()
    left, right, v_face, normal = _soa(left, 5), _soa(right, 5), _soa(v_face, 3), _soa(normal, 3)
    n = left.shape[1]
    out = np.zeros((5, n))
    if airs_threshold is None and velocity is None:
        _check(L.mvmm_riemann_flux(kind, precision, gamma, n, left.ctypes.data, right.ctypes.data,
                                   v_face.ctypes.data, normal.ctypes.data, out.ctypes.data))
    else:
        prm = _solver_params(kind, gamma, precision, airs_threshold, velocity)
        _check(L.mvmm_riemann_flux_p(ctypes.byref(prm), n, left.ctypes.data, right.ctypes.data, v_face.ctypes.data,
                                     normal.ctypes.data, out.ctypes.data))
    return out


def riemann_sample(kind: int, gamma: float, left, right, normal, precision: int = 0, airs_threshold=None):
    """Half state at x/t = 0 (RiemannStarSolver::sample after the vacuum test) on the GPU."""
    L = load_library()
    left, right, normal = _soa(left, 5), _soa(right, 5), _soa(normal, 3)
    n = left.shape[1]
    out = np.zeros((5, n))
    if airs_threshold is None:
        _check(L.mvmm_riemann_sample(kind, precision, gamma, n, left.ctypes.data, right.ctypes.data,
                                     normal.ctypes.data, out.ctypes.data))
    else:
        prm = _solver_params(kind, gamma, precision, airs_threshold, None)
        _check(L.mvmm_riemann_sample_p(ctypes.byref(prm), n, left.ctypes.data, right.ctypes.data, normal.ctypes.data,
                                       out.ctypes.data))
    return out


class _HostBlock:
    """A page-locked host block (mvmm_host_alloc), freed when the last array
    viewing it goes (the arrays hold it as their base)."""

    def __init__(self, nbytes: int):
        p = ctypes.c_void_p(0)
        _check(load_library().mvmm_host_alloc(nbytes, ctypes.byref(p)))
        self.ptr, self.nbytes = p.value, nbytes
        self.__array_interface__ = {"data": (self.ptr, False), "shape": (nbytes,), "typestr": "|u1", "version": 3}

    def __del__(self):
        ptr = getattr(self, "ptr", None)
        if ptr:
            self.ptr = None
            try:
                load_library().mvmm_host_free(ctypes.c_void_p(ptr))
            except Exception:
                pass


class PinnedArrays:
    """``arrays(specs)`` for :func:`mesh.mesh_voronoi`: the arrays of one call
    carved from one page-locked block, which is kept and reused by the next
    call (grown when too small), so a caller alternates two of these to keep
    the previous result intact while it builds the next."""

    def __init__(self):
        self.block = None

    def __call__(self, specs):
        sizes = [int(np.prod(shape)) * np.dtype(dt).itemsize for shape, dt in specs]
        offs, total = [], 0
        for b in sizes:
            offs.append(total)
            total += (b + 63) // 64 * 64
        if self.block is None or self.block.nbytes < total:
            self.block = _HostBlock(max(total + total // 4, 64))
        raw = np.asarray(self.block)
        return [raw[o:o + b].view(dt).reshape(shape) for (shape, dt), o, b in zip(specs, offs, sizes)]


class GpuSim:
    """One simulation resident on the GPU (Engine + OptimalOrderRunner + EulerEqnsFvs).

    With ``cell_offsets`` / ``t_end`` (from :func:`hydro_rs_gb300.ics.pack`) the
    context is a batch of independent simulations stepped together."""

    def __init__(self, problem, precision: int | None = None, stream=None, cell_offsets=None, t_end=None):
        L = load_library()
        p = problem.params
        self.problem = problem
        self.mesh = problem.mesh
        prec = p.precision if precision is None else precision
        self.precision, self.stream = prec, stream
        self._p = make_params(p, prec, problem.mesh.box)
        self._mv = self.mesh.cview()
        h = ctypes.c_void_p(0)
        self.n_instances = 1
        if cell_offsets is not None:
            self._off = np.ascontiguousarray(cell_offsets, dtype=np.int64)
            self._tend = np.ascontiguousarray(t_end, dtype=np.float64)
            self.n_instances = len(self._off) - 1
            _check(L.mvmm_ctx_create_batched(ctypes.byref(self._p), ctypes.byref(self._mv), self.n_instances,
                                             self._off.ctypes.data, self._tend.ctypes.data, ctypes.byref(h)))
        else:
            _check(L.mvmm_ctx_create(ctypes.byref(self._p), ctypes.byref(self._mv), ctypes.byref(h)))
        self.h = h
        if stream is not None:
            _check(L.mvmm_ctx_set_stream(self.h, ctypes.c_void_p(stream)), self.h)
        self.cells = problem.cells.copy()
        self.upload(self.cells)
        self.ti_current = 0
        self.ti_old = 0
        self.steps = 0
        self.active_faces = 0
        self.finished = False

    def close(self):
        if getattr(self, "h", None):
            load_library().mvmm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state ----
    def upload(self, cells: Cells):
        cv = cells.cview()
        _check(load_library().mvmm_upload_cells(self.h, ctypes.byref(cv)), self.h)

    def state(self, out: Cells | None = None) -> Cells:
        out = self.cells.copy() if out is None else out
        cv = out.cview()
        _check(load_library().mvmm_download_cells(self.h, ctypes.byref(cv)), self.h)
        return out

    def error_bits(self) -> int:
        return int(load_library().mvmm_error_bits(self.h))

    # ---- Runner::step / Engine::run ----
    def step(self) -> bool:
        tn = ctypes.c_uint64(0)
        nf = ctypes.c_int64(0)
        _check(load_library().mvmm_step(self.h, self.ti_current, self.ti_old, ctypes.byref(tn), ctypes.byref(nf)),
               self.h)
        self.steps += 1
        self.active_faces += nf.value
        done = self.ti_current >= MAX_NR_TIMESTEPS
        self.ti_old, self.ti_current = self.ti_current, tn.value
        self.finished = done
        return done

    # ---- moving meshes (host-driven: drift, rebuild the Voronoi mesh, step)
    def drift(self, dt: float):
        """Space::drift of every generator by v*dt: wrapped in a periodic box,
        mirrored back into a reflective one; in an open or vacuum box a
        generator that left stays outside for the host to remove."""
        _check(load_library().mvmm_drift(self.h, float(dt)), self.h)

    def rebuilt(self, keep, mesh) -> "GpuSim":
        """A context over the cells ``keep`` (indices into this one, in order)
        with this one's parameters, form, stream and timeline, created with
        ``mesh`` over them: the removal of generators that left an open or
        vacuum box (a context's cell count is fixed)."""
        from .ics import Problem

        st = self.state()
        cells = Cells(n=len(keep), arrays={k: np.ascontiguousarray(v[..., keep]) for k, v in st.arrays.items()})
        new = GpuSim(Problem(self.problem.name, self.problem.params, mesh, cells), precision=self.precision,
                     stream=self.stream)
        new.ti_current, new.ti_old, new.steps = self.ti_current, self.ti_old, self.steps
        new.active_faces, new.finished = self.active_faces, self.finished
        return new

    def host_arrays(self) -> PinnedArrays:
        """Page-locked output arrays for the host mesh builder: mvmm_set_mesh
        then copies the mesh at the link's speed."""
        return PinnedArrays()

    def positions(self) -> np.ndarray:
        loc = np.zeros((3, self.mesh.n_cells))
        _check(load_library().mvmm_get_positions(self.h, loc.ctypes.data), self.h)
        return loc

    def set_mesh(self, mesh):
        """Space::volume_calculation's result: new faces now, new volumes and
        centroids for the next step's active cells."""
        self._mv = mesh.cview()
        self._new_mesh = mesh  # keep the arrays alive while the context copies them
        vol = np.ascontiguousarray(mesh.volume, dtype=np.float64)
        cen = np.ascontiguousarray(mesh.cell_centroid, dtype=np.float64)
        _check(load_library().mvmm_set_mesh(self.h, ctypes.byref(self._mv), vol.ctypes.data, cen.ctypes.data), self.h)
        self.mesh = mesh

    def step_cells(self, cells_in: Cells, cells_out: Cells | None = None) -> bool:
        """One step on host-resident state (mvmm_step_cells): upload, step and
        download in one call; cells_out defaults to cells_in."""
        ci = cells_in.cview()
        co = ci if cells_out is None or cells_out is cells_in else cells_out.cview()
        tn = ctypes.c_uint64(0)
        nf = ctypes.c_int64(0)
        _check(load_library().mvmm_step_cells(self.h, ctypes.byref(ci), ctypes.byref(co), self.ti_current,
                                              self.ti_old, ctypes.byref(tn), ctypes.byref(nf)), self.h)
        self.steps += 1
        self.active_faces += nf.value
        done = self.ti_current >= MAX_NR_TIMESTEPS
        self.ti_old, self.ti_current = self.ti_current, tn.value
        self.finished = done
        return done

    def step_cells_changed(self, cells: Cells, changed=None) -> int:
        """One step on host-resident state that moves only what changed
        (mvmm_step_cells_changed): ``cells`` holds what the previous call left,
        but for the cells listed in ``changed`` (None: upload every cell); the
        cells the step rewrote are written back into ``cells``.  Returns the
        bytes written back."""
        cv = cells.cview()
        if changed is None:
            ptr, m = None, 0
        else:
            idx = np.ascontiguousarray(changed, dtype=np.int32)
            ptr, m = idx.ctypes.data, idx.size
        tn = ctypes.c_uint64(0)
        nf = ctypes.c_int64(0)
        stored = ctypes.c_int64(0)
        _check(load_library().mvmm_step_cells_changed(self.h, ctypes.byref(cv), ptr, m, self.ti_current,
                                                      self.ti_old, ctypes.byref(tn), ctypes.byref(nf),
                                                      ctypes.byref(stored)), self.h)
        self.steps += 1
        self.active_faces += nf.value
        done = self.ti_current >= MAX_NR_TIMESTEPS
        self.ti_old, self.ti_current = self.ti_current, tn.value
        self.finished = done
        return stored.value

    def run(self, max_steps: int = 0) -> int:
        tc = ctypes.c_uint64(self.ti_current)
        to = ctypes.c_uint64(self.ti_old)
        s = ctypes.c_int64(0)
        nf = ctypes.c_int64(0)
        fin = ctypes.c_int(0)
        _check(load_library().mvmm_run(self.h, max_steps, ctypes.byref(tc), ctypes.byref(to), ctypes.byref(s),
                                       ctypes.byref(nf), ctypes.byref(fin)), self.h)
        self.ti_current, self.ti_old = tc.value, to.value
        self.steps += s.value
        self.active_faces += nf.value
        self.finished = bool(fin.value)
        return s.value

    # ---- asynchronous stepping for timing ----
    def set_time(self):
        """Writes the host's sync point to the device timeline (a batch keeps
        each simulation's own device timeline, so this is a no-op for it)."""
        if self.n_instances > 1:
            return
        _check(load_library().mvmm_set_time(self.h, self.ti_current, self.ti_old), self.h)

    def enqueue_steps(self, n: int):
        _check(load_library().mvmm_enqueue_steps(self.h, n), self.h)

    def sync_time(self):
        tc, to, st, af, fin = (ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int())
        _check(load_library().mvmm_get_time(self.h, ctypes.byref(tc), ctypes.byref(to), ctypes.byref(st),
                                            ctypes.byref(af), ctypes.byref(fin)), self.h)
        self.ti_current, self.ti_old, self.finished = tc.value, to.value, bool(fin.value)
        return st.value, af.value

    def batch_state(self) -> dict:
        k = self.n_instances
        tc, to = np.zeros(k, np.uint64), np.zeros(k, np.uint64)
        st, af = np.zeros(k, np.int64), np.zeros(k, np.int64)
        err, fin = np.zeros(k, np.uint32), np.zeros(k, np.int32)
        _check(load_library().mvmm_batch_state(self.h, tc.ctypes.data, to.ctypes.data, st.ctypes.data, af.ctypes.data,
                                               err.ctypes.data, fin.ctypes.data), self.h)
        return {"ti_current": tc, "ti_old": to, "steps": st, "active_faces": af, "err": err, "finished": fin}

    def flush_deferred(self):
        """Enqueues the deferred extrapolations of hierarchical steps (no sync)."""
        _check(load_library().mvmm_flush_deferred(self.h), self.h)

    def autotune(self, steps: int = 3):
        """Picks the thread-block sizes by timing this workload (state is restored)."""
        bf, bc = ctypes.c_int(0), ctypes.c_int(0)
        _check(load_library().mvmm_autotune(self.h, steps, ctypes.byref(bf), ctypes.byref(bc)), self.h)
        return bf.value, bc.value

    def stats(self) -> dict:
        a = np.zeros(6, dtype=np.int64)
        _check(load_library().mvmm_get_stats(self.h, a.ctypes.data), self.h)
        return dict(zip(("steps", "active_faces", "active_cells", "fp64_fallback_faces", "host_bytes_in",
                         "host_bytes_out"), a.tolist()))

    def profile(self, enable: bool):
        _check(load_library().mvmm_profile_enable(self.h, int(enable)), self.h)

    def profile_read(self):
        ms = np.zeros(len(KERNEL_NAMES))
        n = np.zeros(len(KERNEL_NAMES), dtype=np.int64)
        _check(load_library().mvmm_profile_read(self.h, ms.ctypes.data, n.ctypes.data), self.h)
        return dict(zip(KERNEL_NAMES, zip(ms.tolist(), n.tolist())))

    # ---- FiniteVolumeSolver trait, per stage ----
    def predict(self, dt: float):
        _check(load_library().mvmm_predict(self.h, dt), self.h)

    def compute_fluxes(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        out = np.zeros((10, self.mesh.n_faces))
        nf = ctypes.c_int64(0)
        _check(load_library().mvmm_compute_fluxes(self.h, active.ctypes.data, out.ctypes.data, ctypes.byref(nf)),
               self.h)
        return out, nf.value

    def apply_fluxes(self, fluxes, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        fluxes = np.ascontiguousarray(fluxes, dtype=np.float64)
        _check(load_library().mvmm_apply_fluxes(self.h, fluxes.ctypes.data, active.ctypes.data), self.h)

    def convert(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        _check(load_library().mvmm_convert_conserved_to_primitive(self.h, active.ctypes.data), self.h)

    def gradients(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        _check(load_library().mvmm_gradients(self.h, active.ctypes.data), self.h)

    def compute_timesteps(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        out = np.zeros(self.mesh.n_cells)
        _check(load_library().mvmm_compute_timesteps(self.h, active.ctypes.data, out.ctypes.data), self.h)
        return out

    # ---- GravitySolver trait ----
    def gravity_timesteps(self):
        out = np.zeros(self.mesh.n_cells)
        _check(load_library().mvmm_gravity_timesteps(self.h, out.ctypes.data), self.h)
        return out

    def gravity_accelerations(self):
        out = np.zeros((3, self.mesh.n_cells))
        _check(load_library().mvmm_gravity_accelerations(self.h, out.ctypes.data), self.h)
        return out
