"""Hierarchical time bins on the GPU against the oracle (sync_timesteps = false).

Inactive cells keep accumulating fluxes, the active-face rule uses the
strictly-smaller-dt side, and the neighbour limiter wakes cells up
(euler_eqns_fvs.rs:35, runner/hydrodynamics.rs:160-184, part.rs:263-297).
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import compare_cells, totals

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("riemann", [ics.HLLC, ics.EXACT])
def test_point_blast_3d_bins(gpu_lib, riemann):
    p = ics.point_blast_3d(8, riemann=riemann, sync_all=False, t_end=0.05)
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p)
    bins_seen = set()
    for _ in range(40):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
        bins_seen.update(np.unique(orc.state().timebin).tolist())
    assert gpu.active_faces == orc.active_faces
    assert len(bins_seen) >= 2, bins_seen  # the run really is hierarchical
    a, b = gpu.state(), orc.state()
    errs = compare_cells(a, b, fields=("cons", "prim", "facc", "dt", "grad", "gc", "extrap"))
    assert max(errs.values()) <= 1e-10, errs
    assert np.array_equal(a.timebin, b.timebin)
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-13 and abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])


def test_point_blast_3d_bins_fp32(gpu_lib):
    """FP32-face form with hierarchical bins: the compacted face and cell lists
    (only active cells and their neighbours are visited after predict) give the
    oracle's timeline, time bins and active faces, and the density within 1e-5 L1."""
    p = ics.point_blast_3d(8, riemann=ics.HLLC, sync_all=False, t_end=0.05)
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p, precision=1)
    for _ in range(40):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
    a, b = gpu.state(), orc.state()
    assert gpu.active_faces == orc.active_faces
    assert np.array_equal(a.timebin, b.timebin)
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-13 and abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])


def test_kh_unsynchronised_bins(gpu_lib):
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.HLLC)
    p.params.sync_all = False
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p)
    for _ in range(30):
        orc.step()
        gpu.step()
    assert gpu.ti_current == orc.ti_current and gpu.active_faces == orc.active_faces
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim"))
    assert max(errs.values()) <= 1e-11, errs


def test_deferred_extrapolation(gpu_lib):
    """Hierarchical steps defer the extrapolation of inactive cells until a
    step reads them (mvmm_flush_deferred completes the rest).  A run that
    completes them after every step and one that leaves them deferred end on
    the same bits, over more steps than the log of step sizes holds (4,096);
    a download in the middle changes nothing; the oracle agrees at t_end."""
    p = ics.sod_1d(1500, riemann=ics.HLLC, t_end=0.2)  # 8,193 steps
    p.params.sync_all = False
    lazy, eager = G.GpuSim(p), G.GpuSim(p)
    lazy.run(max_steps=1000)
    mid = lazy.state()
    lazy.run()
    while not eager.finished:
        eager.step()
        eager.flush_deferred()
        if eager.steps == 1000:
            assert all(np.array_equal(x.view(np.uint8), y.view(np.uint8))
                       for x, y in zip(mid.arrays.values(), eager.state().arrays.values()))
    assert lazy.steps == eager.steps > 4096
    a, b = lazy.state(), eager.state()
    for k, x in a.arrays.items():
        assert np.array_equal(x.view(np.uint8), b.arrays[k].view(np.uint8)), k
    orc = O.OracleSim(p)
    orc.run()
    assert orc.steps == lazy.steps
    errs = compare_cells(a, orc.state(), fields=("cons", "prim", "extrap"))
    assert max(errs.values()) <= 1e-9, errs
