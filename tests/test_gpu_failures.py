"""Failure detection on the GPU without a GPU fault.

Failures are made on the host (a one-iteration Newton cap, a negative energy
written into the uploaded state); the kernels record them in a device error
word, the host reads it after the step and returns MVMM_E_NUMERIC with the
bits, and the context stays usable.  No trap, assert or bad address is used.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_newton_cap_reported_and_context_survives(gpu_lib):
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.EXACT)
    p.params.max_newton_iter = 1
    sim = G.GpuSim(p)
    with pytest.raises(G.MvmmError) as ei:
        sim.run(max_steps=4)
    assert ei.value.code == -3 and ei.value.bits & 1
    # the oracle flags the same condition
    o = O.OracleSim(p)
    o.run(max_steps=4)
    assert o.error() & 1
    # the context is still usable after the reported failure
    st = sim.state()
    assert np.all(np.isfinite(st.cons))
    sim.upload(p.cells)
    sim.ti_current = sim.ti_old = 0
    sim.step()


def test_negative_energy_reported(gpu_lib):
    p = ics.sod_1d(64)
    sim = G.GpuSim(p)
    c = p.cells.copy()
    c.cons[4][10] = -1.0
    sim.upload(c)
    with pytest.raises(G.MvmmError) as ei:
        sim.convert(np.ones(64, np.uint8))
    assert ei.value.bits & (1 << 3)
    sim.upload(p.cells)
    sim.compute_timesteps(np.ones(64, np.uint8))
