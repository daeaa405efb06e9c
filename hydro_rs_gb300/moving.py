"""Moving-mesh stepping: the host half of Engine::run for particle motion other
than ``fixed``.

The reference drifts every generator to the next sync point
(``Engine::run``, ``src/engine.rs:164-176``; ``Space::drift``,
``src/space.rs:833-854``) and, inside the runner's step, rebuilds the Voronoi
mesh from the drifted generators (``Space::volume_calculation``,
``src/space.rs:236-263``).  Here the drift and the step run on the device; the
generator positions come back, the host builds the new mesh (the same C++
builder as for the initial conditions) and hands it to the context, whose next
step applies the new faces, volumes and centroids.  Each part is timed, so the
host mesh build and the upload appear as their own lines.

``sim`` is a ``gpu.GpuSim`` (or the oracle's ``OracleSim``, which has the same
methods), created with ``params.particle_motion`` set.

Walls: a generator that drifts out of a reflective box is mirrored back by
the drift itself (``Particle::box_reflect``).  In an open or vacuum box the
reference removes the generators that left (``src/space.rs:840-853``): it
collects their indices in ascending order and removes them one by one from its
particle vector, so after the first removal each later index names the
particle that followed the intended one (an index past the end panics).
``removal_keep`` restates that, and the stepper replaces the simulation by one
over the particles kept (the context's cell count is fixed).
"""
from __future__ import annotations

import time

import numpy as np

from .mesh import mesh_voronoi

MAX_NR_TIMESTEPS = 1 << 57
BOUNDARY_OPEN, BOUNDARY_VACUUM = 2, 3


class RemovalError(RuntimeError):
    """The reference's removal would panic (an index past the end), or kept a
    generator outside the box (its mesh has no cell there)."""


def outside_box(loc, box, dim: int) -> np.ndarray:
    """Particles utils.rs ``contains`` (:15-21) puts outside the box."""
    inside = np.ones(loc.shape[1], dtype=bool)
    for a in range(dim):
        inside &= (loc[a] >= 0.0) & (loc[a] < box[a])
    return ~inside


def removal_keep(n: int, to_remove) -> np.ndarray:
    """Original indices left after ``for idx in to_remove { parts.remove(idx) }``
    (space.rs:851-853) over a vector of n particles."""
    keep = list(range(n))
    for idx in to_remove:
        if idx >= len(keep):
            raise RemovalError(f"removal index {idx} past the end of {len(keep)} particles")
        del keep[idx]
    return np.asarray(keep, dtype=np.int64)


class MovingMeshStepper:
    def __init__(self, sim, mesh, n_threads: int = 0):
        self.sim = sim
        self.dim = mesh.dimensionality
        self.box = mesh.box
        self.periodic = mesh.periodic
        self.time_base = sim.problem.params.t_end / MAX_NR_TIMESTEPS
        self.n_threads = n_threads
        self.seconds = {"drift": 0.0, "positions": 0.0, "mesh_build": 0.0, "mesh_upload": 0.0, "step": 0.0}
        self.removed = 0  # generators that left an open or vacuum box
        # the GPU context's meshes are built into two alternating page-locked
        # blocks (the one the context holds stays intact while the next is built)
        self._arrays = [sim.host_arrays(), sim.host_arrays()] if hasattr(sim, "host_arrays") else None
        self._turn = 0

    def step(self) -> bool:
        sim, s = self.sim, self.seconds
        t0 = time.perf_counter()
        if sim.ti_current > sim.ti_old:  # drift to this sync point
            sim.drift((sim.ti_current - sim.ti_old) * self.time_base)
        t1 = time.perf_counter()
        loc = sim.positions()
        keep = None
        if sim.problem.params.boundary in (BOUNDARY_OPEN, BOUNDARY_VACUUM):
            out = outside_box(loc, self.box, self.dim)
            if out.any():
                keep = removal_keep(loc.shape[1], np.flatnonzero(out).tolist())
                if out[keep].any():
                    raise RemovalError("the reference's removal kept a generator outside the box")
                self.removed += loc.shape[1] - keep.size
                loc = np.ascontiguousarray(loc[:, keep])
        t2 = time.perf_counter()
        arrays = None
        if self._arrays is not None:
            arrays = self._arrays[self._turn]
            self._turn ^= 1
        mesh = mesh_voronoi(loc, self.dim, self.box, self.periodic, self.n_threads, arrays=arrays)
        t3 = time.perf_counter()
        if keep is not None:  # a simulation over the particles kept
            sim = self.sim = sim.rebuilt(keep, mesh)
        sim.set_mesh(mesh)
        t4 = time.perf_counter()
        done = sim.step()
        t5 = time.perf_counter()
        s["drift"] += t1 - t0
        s["positions"] += t2 - t1
        s["mesh_build"] += t3 - t2
        s["mesh_upload"] += t4 - t3
        s["step"] += t5 - t4
        return done
