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
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim", "facc", "dt"))
    assert max(errs.values()) <= 1e-10, errs
    t0, t1 = totals(p.cells), totals(gpu.state())
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
