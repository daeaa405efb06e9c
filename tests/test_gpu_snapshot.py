"""Space::dump from resident device state: a GPU run written as an HDF5 snapshot
(hydro_rs_gb300/snapshot.py) holds the state the oracle reaches, at the run's
simulated time."""
import os

import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from hydro_rs_gb300 import snapshot as S
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_snapshot_of_device_state(gpu_lib, tmp_path, precision):
    p = ics.sod_1d(400, riemann=ics.EXACT)
    sim = G.GpuSim(p, precision=precision)
    sim.run(max_steps=60)
    fn = os.path.join(tmp_path, "snap.hdf5")
    S.snapshot_of(sim, fn)
    t = S.read(fn)["children"]
    st = sim.state()
    d = t["PartType0"]["children"]
    assert np.array_equal(d["Masses"], st.cons[0]) and np.array_equal(d["Densities"], st.prim[0])
    assert np.array_equal(d["Momenta"], st.cons[1:4].T) and np.array_equal(d["Timestep"], st.dt)
    assert t["Header"]["attrs"]["Time"][0] == sim.ti_current * (p.params.t_end / 2.0 ** 57)
    o = O.OracleSim(p)
    o.run(max_steps=60)
    tol = 1e-12 if precision == 0 else 1e-5
    assert rel_err(d["Densities"], o.state().prim[0]) <= tol
