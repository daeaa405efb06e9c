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
"""
from __future__ import annotations

import time

from .mesh import mesh_voronoi

MAX_NR_TIMESTEPS = 1 << 57


class MovingMeshStepper:
    def __init__(self, sim, mesh, n_threads: int = 0):
        self.sim = sim
        self.dim = mesh.dimensionality
        self.box = mesh.box
        self.periodic = mesh.periodic
        self.time_base = sim.problem.params.t_end / MAX_NR_TIMESTEPS
        self.n_threads = n_threads
        self.seconds = {"drift": 0.0, "positions": 0.0, "mesh_build": 0.0, "mesh_upload": 0.0, "step": 0.0}

    def step(self) -> bool:
        sim, s = self.sim, self.seconds
        t0 = time.perf_counter()
        if sim.ti_current > sim.ti_old:  # drift to this sync point
            sim.drift((sim.ti_current - sim.ti_old) * self.time_base)
        t1 = time.perf_counter()
        loc = sim.positions()
        t2 = time.perf_counter()
        mesh = mesh_voronoi(loc, self.dim, self.box, self.periodic, self.n_threads)
        t3 = time.perf_counter()
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
