"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker for the GPU library: only ``tests/``, the smoke
check in ``__graft_entry__`` and the CPU-baseline leg of ``bench.py`` may use
it.  The product (``hydro_rs_gb300``) never imports this module.

``OracleSim`` mirrors the reference's ``Engine``/``OptimalOrderRunner`` over
one problem; the free functions expose the Riemann solvers and the timeline
helpers for the golden-vector tests.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmvmm_oracle.so")
_LIB = None


class _Params(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("eos", ctypes.c_int), ("isothermal_internal_energy", ctypes.c_double),
                ("cfl", ctypes.c_double), ("riemann", ctypes.c_int), ("boundary", ctypes.c_int),
                ("dimensionality", ctypes.c_int), ("sync_all", ctypes.c_int), ("t_end", ctypes.c_double),
                ("max_newton_iter", ctypes.c_int), ("n_threads", ctypes.c_int), ("runner", ctypes.c_int),
                ("airs_threshold", ctypes.c_double), ("advection_velocity", ctypes.c_double * 3),
                ("particle_motion", ctypes.c_int), ("box_size", ctypes.c_double * 3),
                ("gravity", ctypes.c_int), ("gravity_softening", ctypes.c_double),
                ("gravity_acceleration", ctypes.c_double * 3), ("gravity_position", ctypes.c_double * 3),
                ("gravity_accelerations", ctypes.c_int), ("limiter_frame", ctypes.c_int)]


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, u64, dbl, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(_Params), vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_cells.argtypes = [vp, vp]
        L.orc_get_cells.argtypes = [vp, vp]
        L.orc_error.restype = ctypes.c_uint32
        L.orc_error.argtypes = [vp]
        L.orc_step.restype = u64
        L.orc_step.argtypes = [vp, u64, u64, ctypes.POINTER(i64)]
        L.orc_run.restype = i64
        L.orc_run.argtypes = [vp, i64, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(i64)]
        L.orc_predict.argtypes = [vp, dbl]
        L.orc_compute_fluxes.restype = i64
        L.orc_compute_fluxes.argtypes = [vp, vp, vp]
        L.orc_apply_fluxes.argtypes = [vp, vp, vp]
        L.orc_convert_conserved_to_primitive.argtypes = [vp, vp]
        L.orc_gradients.argtypes = [vp, vp]
        L.orc_compute_timesteps.argtypes = [vp, vp, vp]
        L.orc_riemann_flux.argtypes = [i32, dbl, i64, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_riemann_sample.argtypes = [i32, dbl, i64, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_drift.argtypes = [vp, dbl]
        L.orc_set_mesh.argtypes = [vp, vp, vp, vp]
        L.orc_riemann_flux_ex.argtypes = [i32, dbl, dbl, vp, i64, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_riemann_sample_ex.argtypes = [i32, dbl, dbl, i64, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_get_integer_timestep.restype = u64
        L.orc_get_integer_timestep.argtypes = [i32]
        L.orc_get_time_bin.restype = i32
        L.orc_get_time_bin.argtypes = [u64]
        L.orc_get_max_active_bin.restype = i32
        L.orc_get_max_active_bin.argtypes = [u64]
        L.orc_make_integer_timestep.restype = u64
        L.orc_make_integer_timestep.argtypes = [dbl, i32, i32, u64, dbl, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_cons_from_primitives.argtypes = [dbl, vp, dbl, vp]
        L.orc_prim_from_conserved.argtypes = [dbl, vp, dbl, vp]
        L.orc_exact_star.argtypes = [dbl] + [dbl] * 8 + [vp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_gravity_timesteps.argtypes = [vp, vp]
        L.orc_gravity_accelerations.argtypes = [vp, vp]
        _LIB = L
    return _LIB


MAX_NR_TIMESTEPS = 1 << 57


class OracleSim:
    """Engine + OptimalOrderRunner over one problem (mesh + cells + params)."""

    def __init__(self, problem, n_threads: int = 0):
        p = problem.params
        self.problem = problem
        self.n_threads = n_threads
        self.mesh = problem.mesh
        self.cells = problem.cells.copy()
        thr, adv = p.solver_extras()
        self._p = _Params(p.gamma, p.eos, p.isothermal_internal_energy, p.cfl, p.riemann, p.boundary,
                          p.dimensionality, int(p.sync_all),
                          p.t_end, p.max_newton_iter, n_threads, p.runner, thr, (ctypes.c_double * 3)(*adv),
                          p.particle_motion, (ctypes.c_double * 3)(*[float(b) for b in problem.mesh.box]),
                          *p.gravity_fields())
        self._mv = self.mesh.cview()
        self.h = lib().orc_create(ctypes.byref(self._p), ctypes.byref(self._mv))
        self._cv = self.cells.cview()
        lib().orc_set_cells(self.h, ctypes.byref(self._cv))
        self.ti_current = 0
        self.ti_old = 0
        self.steps = 0
        self.active_faces = 0

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_destroy(h)
            self.h = None

    def error(self) -> int:
        return int(lib().orc_error(self.h))

    def step(self) -> int:
        nf = ctypes.c_int64(0)
        tn = lib().orc_step(self.h, self.ti_current, self.ti_old, ctypes.byref(nf))
        self.steps += 1
        self.active_faces += nf.value
        done = self.ti_current >= MAX_NR_TIMESTEPS
        self.ti_old, self.ti_current = self.ti_current, tn
        return done

    def run(self, max_steps: int = 0) -> int:
        tc = ctypes.c_uint64(self.ti_current)
        to = ctypes.c_uint64(self.ti_old)
        nf = ctypes.c_int64(0)
        s = lib().orc_run(self.h, max_steps, ctypes.byref(tc), ctypes.byref(to), ctypes.byref(nf))
        self.ti_current, self.ti_old = tc.value, to.value
        self.steps += s
        self.active_faces += nf.value
        return s

    @property
    def finished(self) -> bool:
        return self.ti_old >= MAX_NR_TIMESTEPS

    def state(self):
        out = self.cells.copy()
        cv = out.cview()
        lib().orc_get_cells(self.h, ctypes.byref(cv))
        return out

    # ---- moving meshes ----
    def drift(self, dt: float):
        lib().orc_drift(self.h, float(dt))

    def positions(self) -> np.ndarray:
        return self.state().loc.copy()

    def rebuilt(self, keep, mesh) -> "OracleSim":
        """An oracle over the particles ``keep`` with this one's parameters and
        timeline, on ``mesh`` (the removal of generators that left an open or
        vacuum box)."""
        from hydro_rs_gb300.ics import Problem
        from hydro_rs_gb300.layout import Cells

        st = self.state()
        cells = Cells(n=len(keep), arrays={k: np.ascontiguousarray(v[..., keep]) for k, v in st.arrays.items()})
        new = OracleSim(Problem(self.problem.name, self.problem.params, mesh, cells), n_threads=self.n_threads)
        new.ti_current, new.ti_old, new.steps, new.active_faces = (self.ti_current, self.ti_old, self.steps,
                                                                   self.active_faces)
        return new

    def set_mesh(self, mesh):
        self._mv = mesh.cview()
        self._new_mesh = mesh
        vol = np.ascontiguousarray(mesh.volume, dtype=np.float64)
        cen = np.ascontiguousarray(mesh.cell_centroid, dtype=np.float64)
        lib().orc_set_mesh(self.h, ctypes.byref(self._mv), vol.ctypes.data, cen.ctypes.data)
        self.mesh = mesh

    # ---- per-stage (FiniteVolumeSolver trait / runner free functions) ----
    def predict(self, dt: float):
        lib().orc_predict(self.h, dt)

    def compute_fluxes(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        out = np.zeros((10, self.mesh.n_faces))
        n = lib().orc_compute_fluxes(self.h, active.ctypes.data, out.ctypes.data)
        return out, n

    def apply_fluxes(self, fluxes, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        fluxes = np.ascontiguousarray(fluxes, dtype=np.float64)
        lib().orc_apply_fluxes(self.h, fluxes.ctypes.data, active.ctypes.data)

    def convert(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        lib().orc_convert_conserved_to_primitive(self.h, active.ctypes.data)

    def gradients(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        lib().orc_gradients(self.h, active.ctypes.data)

    def compute_timesteps(self, active):
        active = np.ascontiguousarray(active, dtype=np.uint8)
        out = np.zeros(self.mesh.n_cells)
        lib().orc_compute_timesteps(self.h, active.ctypes.data, out.ctypes.data)
        return out

    def gravity_timesteps(self):
        out = np.zeros(self.mesh.n_cells)
        lib().orc_gravity_timesteps(self.h, out.ctypes.data)
        return out

    def gravity_accelerations(self):
        out = np.zeros((3, self.mesh.n_cells))
        lib().orc_gravity_accelerations(self.h, out.ctypes.data)
        return out


def _soa(a, k):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(k, -1))
    return a


def riemann_flux(kind, gamma, left, right, v_face, normal, airs_threshold=2.0, velocity=None):
    """RiemannFluxSolver::solve_for_flux over arrays ([5][n], [5][n], [3][n], [3][n])."""
    left, right, v_face, normal = _soa(left, 5), _soa(right, 5), _soa(v_face, 3), _soa(normal, 3)
    n = left.shape[1]
    out = np.zeros((5, n))
    err = ctypes.c_uint32(0)
    adv = np.zeros(3) if velocity is None else np.ascontiguousarray(velocity, dtype=np.float64)
    lib().orc_riemann_flux_ex(kind, gamma, airs_threshold, adv.ctypes.data, n, left.ctypes.data, right.ctypes.data,
                              v_face.ctypes.data, normal.ctypes.data, out.ctypes.data, ctypes.byref(err))
    return out, err.value


def riemann_sample(kind, gamma, left, right, normal, airs_threshold=2.0):
    """Half state at x/t=0 (vacuum-aware), [5][n]."""
    left, right, normal = _soa(left, 5), _soa(right, 5), _soa(normal, 3)
    n = left.shape[1]
    out = np.zeros((5, n))
    err = ctypes.c_uint32(0)
    lib().orc_riemann_sample_ex(kind, gamma, airs_threshold, n, left.ctypes.data, right.ctypes.data,
                                normal.ctypes.data, out.ctypes.data, ctypes.byref(err))
    return out, err.value


def cons_from_primitives(gamma, prim5, volume):
    p = np.ascontiguousarray(prim5, dtype=np.float64)
    out = np.zeros(5)
    lib().orc_cons_from_primitives(gamma, p.ctypes.data, volume, out.ctypes.data)
    return out


def prim_from_conserved(gamma, cons5, volume):
    c = np.ascontiguousarray(cons5, dtype=np.float64)
    out = np.zeros(5)
    lib().orc_prim_from_conserved(gamma, c.ctypes.data, volume, out.ctypes.data)
    return out


def exact_star(gamma, rho_l, p_l, a_l, rho_r, p_r, a_r, v_l, v_r):
    """(rho_l*, rho_r*, u*, p*) and the error bits of the exact star solver."""
    out = np.zeros(4)
    err = ctypes.c_uint32(0)
    lib().orc_exact_star(gamma, rho_l, p_l, a_l, rho_r, p_r, a_r, v_l, v_r, out.ctypes.data, ctypes.byref(err))
    return out, err.value


def get_integer_timestep(b):
    return int(lib().orc_get_integer_timestep(b))


def get_time_bin(dti):
    return int(lib().orc_get_time_bin(dti))


def get_max_active_bin(ti):
    return int(lib().orc_get_max_active_bin(ti))


def make_integer_timestep(dt, old_bin, min_ngb_bin, ti_current, time_base_inv):
    err = ctypes.c_uint32(0)
    r = lib().orc_make_integer_timestep(dt, old_bin, min_ngb_bin, ti_current, time_base_inv, ctypes.byref(err))
    return int(r), err.value
