"""Serving on the GPU: requests run concurrently on separate streams, and each
result is identical to the same simulation run alone."""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import serve

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix(gpu_lib):
    reqs = serve.poisson_requests(8, rate=1e6, seed=9, resolutions=(8, 16, 24), t_end=0.3)
    srv = serve.Server(chunk=4, keep_states=True)
    res, wall = srv.run(reqs, realtime=False)
    assert srv.peak_running > 1  # requests really overlapped on the device
    assert [r.rid for r in res] == list(range(8))
    for r in res:
        assert r.err == 0
        q = srv.problem_for(reqs[r.rid])
        alone = G.GpuSim(q, precision=1)
        alone.run()
        assert alone.finished
        a = alone.state()
        for f in ("cons", "prim", "grad", "dt"):
            assert np.array_equal(r.state.arrays[f], a.arrays[f]), (r.rid, f)
    summ = serve.latency_summary(res, wall)
    assert summ["solves_per_s"] > 0
    srv.close()


def test_budget_limits_concurrency(gpu_lib):
    reqs = serve.poisson_requests(6, rate=1e6, seed=10, resolutions=(16,), t_end=0.2)
    one = serve.context_bytes(256, 3 * 256, 1)
    srv = serve.Server(budget_bytes=int(1.5 * one), chunk=4)
    res, wall = srv.run(reqs, realtime=False)
    assert len(res) == 6 and srv.peak_running == 1 and len(srv.slots) == 1
    srv.close()
