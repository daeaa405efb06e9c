"""Serving: a continuous-batching request loop over resident GPU simulations.

No counterpart in the reference (one simulation per process).  Each request is
a simulation to run to its t_end (here an isentropic vortex at a given
resolution).  The server keeps a pool of *slots*: a slot is a GPU context
(mesh + state, ``libmvmm_gpu`` C ABI) with its own CUDA stream, built once
per resolution and reused by later requests of that resolution.  The loop:

* admits waiting requests in arrival order while the slots' device memory stays
  within a fixed HBM budget (a new slot is created only if it fits; a free slot
  of the right resolution is reused first);
* enqueues a chunk of steps (CUDA-graph launches) for every running
  simulation on its own stream, so simulations overlap on the device;
* polls a CUDA event after each chunk (no blocking), reads the device timeline
  of simulations whose chunk completed and retires the finished ones, which
  frees their slot for the next request.

Results do not depend on the mix: a simulation's kernels only touch its own
context, and the kernels are deterministic.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import ics
from .layout import Cells


@dataclass
class Request:
    rid: int
    arrival: float       # seconds after the start of the run
    nx: int              # resolution nx^2
    beta: float
    v_adv: tuple
    t_end: float = 1.0


@dataclass
class Result:
    rid: int
    nx: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    active_faces: int
    state: Cells | None = None
    err: int = 0

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def poisson_requests(n: int, rate: float, seed: int = 5, resolutions=(32, 64, 128, 256, 512), t_end: float = 1.0):
    """n requests with exponential inter-arrival times (mean 1/rate); resolution,
    vortex strength beta ~ U[3,7] and advection velocity ~ U[-1,1]^2 drawn per request."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    out = []
    for k in range(n):
        out.append(Request(k, float(t[k]), int(rng.choice(resolutions)), float(rng.uniform(3, 7)),
                           (float(rng.uniform(-1, 1)), float(rng.uniform(-1, 1))), t_end))
    return out


def context_bytes(n_cells: int, n_faces: int, precision: int) -> int:
    """Device memory of one context (mvmm_ctx_create's allocations)."""
    n, f = n_cells, max(n_faces, 1)
    cells = n * (60 * 8 + 3 + 8 + 4) + (n * 40 * 4 if precision == 1 else 0)
    faces = f * (4 + 4 + 8 + 72 + 80 + 1 + 4) + (f * 7 * 4 if precision == 1 else 0)
    csr = (n + 1) * 4 + 2 * f * 4
    return int(cells + faces + csr + 4096)


class _Slot:
    def __init__(self, gpu, torch, template, precision):
        self.stream = torch.cuda.Stream()
        self.sim = gpu.GpuSim(template, precision=precision, stream=self.stream.cuda_stream)
        # a context's time base is t_end / 2^57, so a slot serves one (resolution, t_end)
        self.key = (template.extra["nx"], template.params.t_end)
        self.bytes = context_bytes(template.mesh.n_cells, template.mesh.n_faces, precision)
        self.req = None
        self.event = None
        self.admitted = 0.0


class Server:
    """Runs requests to completion with continuous batching under an HBM budget."""

    def __init__(self, budget_bytes: int = 32 << 30, chunk: int = 16, precision: int = 1, riemann: int = ics.HLLC,
                 jitter_seed: int = 5, keep_states: bool = False, gpu_module=None, torch_module=None):
        if torch_module is None:
            import torch as torch_module
        if gpu_module is None:
            from . import gpu as gpu_module
        self.torch = torch_module
        self.gpu = gpu_module
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.precision = precision
        self.riemann = riemann
        self.jitter_seed = jitter_seed
        self.keep_states = keep_states
        self.templates = {}
        self.slots = []
        self.used = 0
        self.peak_running = 0

    # one jittered mesh per resolution, built on the host once and reused
    def template(self, nx: int):
        if nx not in self.templates:
            self.templates[nx] = ics.yee_vortex_2d(nx, 5.0, (0.0, 0.0), seed=self.jitter_seed, riemann=self.riemann)
            self.templates[nx].extra["nx"] = nx
        return self.templates[nx]

    def problem_for(self, r: Request):
        p = self.template(r.nx)
        cells = ics.yee_cells(p.mesh, p.cells.loc, r.beta, r.v_adv, p.params.gamma, box_len=10.0)
        q = ics.Problem("yee_vortex_2d", ics.Params(**vars(p.params)), p.mesh, cells, extra={"nx": r.nx})
        q.params.t_end = r.t_end
        return q

    def _free_slot(self, key):
        for s in self.slots:
            if s.req is None and s.key == key:
                return s
        return None

    def _admit(self, r: Request, now: float):
        q = self.problem_for(r)
        s = self._free_slot((r.nx, r.t_end))
        if s is None:
            need = context_bytes(q.mesh.n_cells, q.mesh.n_faces, self.precision)
            if self.used + need > self.budget:
                # evict an idle slot of another resolution if that makes room
                for idle in [x for x in self.slots if x.req is None]:
                    if self.used + need - idle.bytes <= self.budget:
                        idle.sim.close()
                        self.slots.remove(idle)
                        self.used -= idle.bytes
                        break
                else:
                    return False
            s = _Slot(self.gpu, self.torch, q, self.precision)
            self.slots.append(s)
            self.used += s.bytes
        s.sim.upload(q.cells)
        s.sim.ti_current = s.sim.ti_old = 0
        s.sim.finished = False
        s.sim.set_time()
        s.base = s.sim.stats()
        s.req = r
        s.admitted = now
        self._enqueue(s)
        return True

    def _enqueue(self, s):
        s.sim.enqueue_steps(self.chunk)
        s.event = self.torch.cuda.Event()
        s.event.record(s.stream)

    def run(self, requests, realtime: bool = True):
        """Serves the requests; returns (results, wall seconds)."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        results = []
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: math.inf)
        while pending or any(s.req is not None for s in self.slots):
            now = clock()
            while pending and pending[0].arrival <= now:
                if not self._admit(pending[0], time.perf_counter() - t0):
                    break  # the head waits for memory (arrival order is kept)
                pending.popleft()
            progressed = False
            self.peak_running = max(self.peak_running, sum(1 for s in self.slots if s.req is not None))
            for s in self.slots:
                if s.req is None or not s.event.query():
                    continue
                progressed = True
                st, af = s.sim.sync_time()
                if s.sim.finished:
                    stats = s.sim.stats()
                    r = s.req
                    results.append(Result(r.rid, r.nx, r.arrival, s.admitted, time.perf_counter() - t0,
                                          stats["steps"] - s.base["steps"],
                                          stats["active_faces"] - s.base["active_faces"],
                                          s.sim.state() if self.keep_states else None, s.sim.error_bits()))
                    s.req = None
                else:
                    self._enqueue(s)
            if not progressed:
                if pending and not any(s.req is not None for s in self.slots) and realtime:
                    time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.01)))
                else:
                    time.sleep(20e-6)
        wall = time.perf_counter() - t0
        return sorted(results, key=lambda r: r.rid), wall

    def close(self):
        for s in self.slots:
            s.sim.close()
        self.slots = []
        self.used = 0


def latency_summary(results, wall: float) -> dict:
    lat = np.array([r.latency for r in results])
    return {"requests": len(results), "solves_per_s": len(results) / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "active_faces": int(sum(r.active_faces for r in results)), "wall_s": wall}
