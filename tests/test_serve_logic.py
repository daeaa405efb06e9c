"""Host logic of the serving loop, with fake GPU contexts (no GPU needed).

Checks arrival-order admission, the HBM budget (never exceeded), slot reuse
per resolution, eviction of idle slots, and that every request completes.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import ics, serve


class _FakeEvent:
    def record(self, stream):
        pass

    def query(self):
        return True


class _FakeStream:
    cuda_stream = 0


class _FakeCuda:
    Event = _FakeEvent
    Stream = _FakeStream


class _FakeTorch:
    cuda = _FakeCuda


class _FakeSim:
    live = 0
    created = 0

    def __init__(self, problem, precision=1, stream=None):
        self.problem = problem
        self.ti_current = self.ti_old = 0
        self.finished = False
        self._left = 0
        self._steps = 0
        _FakeSim.live += 1
        _FakeSim.created += 1

    def upload(self, cells):
        # a resolution-dependent number of chunks to finish
        self._left = int(np.sqrt(cells.n)) // 8

    def set_time(self):
        pass

    def stats(self):
        return {"steps": self._steps, "active_faces": 3 * self._steps, "active_cells": 0, "fp64_fallback_faces": 0}

    def enqueue_steps(self, n):
        self._steps += n
        self._left -= 1

    def sync_time(self):
        self.finished = self._left < 0
        return self._steps, 3 * self._steps

    def state(self):
        return None

    def error_bits(self):
        return 0

    def close(self):
        _FakeSim.live -= 1


class _FakeGpu:
    GpuSim = _FakeSim


def test_admission_budget_and_reuse():
    reqs = serve.poisson_requests(40, rate=1000.0, seed=1, resolutions=(8, 16, 32))
    big = serve.context_bytes(32 * 32, 3 * 32 * 32, 1)
    srv = serve.Server(budget_bytes=int(2.5 * big), chunk=4, gpu_module=_FakeGpu, torch_module=_FakeTorch)
    peak = [0]
    orig = srv._admit

    def admit(r, now):
        ok = orig(r, now)
        peak[0] = max(peak[0], srv.used)
        assert srv.used <= srv.budget
        return ok

    srv._admit = admit
    res, wall = srv.run(reqs, realtime=False)
    assert [r.rid for r in res] == list(range(40))
    assert peak[0] <= srv.budget
    # slots are reused: far fewer contexts than requests
    assert _FakeSim.created < 20
    summ = serve.latency_summary(res, wall)
    assert summ["requests"] == 40 and summ["p99_latency_s"] >= summ["p50_latency_s"]
    srv.close()
    assert _FakeSim.live == 0


def test_context_bytes_grows_with_mesh():
    assert serve.context_bytes(1000, 3000, 1) < serve.context_bytes(4000, 12000, 1)
    assert serve.context_bytes(1000, 3000, 0) < serve.context_bytes(1000, 3000, 1)
