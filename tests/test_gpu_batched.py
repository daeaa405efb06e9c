"""Batched simulations: many independent problems packed into one context.

Each simulation keeps its own integer timeline and finishes after its own
number of steps; every stage is one launch over all of them.  The result of
each simulation must be the same alone and in the batch (bit for bit: the
kernels have no cross-simulation data flow and no floating-point atomics).
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _batch(problems, precision=0):
    packed, off, te = ics.pack(problems)
    sim = G.GpuSim(packed, precision=precision, cell_offsets=off, t_end=te)
    return sim, packed, off


def _run(sim):
    """Runs to the end; a simulation that fails (PVRS has no pressure floor,
    pvrs.rs:40, so strong rarefactions can give a negative pressure) stops and
    is reported per simulation, the call then returns MVMM_E_NUMERIC."""
    try:
        sim.run()
    except G.MvmmError as e:
        assert e.code == -3


@pytest.mark.parametrize("riemann,precision", [(ics.EXACT, 0), (ics.PVRS, 0), (ics.EXACT, 1)])
def test_batch_equals_alone(gpu_lib, riemann, precision):
    probs = ics.riemann_batch_1d(8, seed=41, n_min=40, n_max=240, riemann=riemann, t_end=0.02)
    sim, packed, off = _batch(probs, precision)
    _run(sim)
    st = sim.batch_state()
    assert st["finished"].all() or (st["err"] != 0).any()
    parts = ics.unpack_cells(sim.state(), off)
    for k, p in enumerate(probs):
        if st["err"][k]:
            continue
        alone = G.GpuSim(p, precision=precision)
        _run(alone)
        assert alone.finished and alone.steps == st["steps"][k]
        a = alone.state()
        for f in ("cons", "prim", "grad", "dt"):
            assert np.array_equal(parts[k].arrays[f], a.arrays[f]), (k, f)
        assert np.array_equal(parts[k].timebin, a.timebin)
    assert len(set(st["steps"].tolist())) > 1  # the simulations took different numbers of steps


def test_batch_matches_oracle(gpu_lib):
    probs = ics.riemann_batch_1d(4, seed=42, n_min=60, n_max=160, riemann=ics.EXACT, t_end=0.02)
    sim, packed, off = _batch(probs)
    _run(sim)
    parts = ics.unpack_cells(sim.state(), off)
    st = sim.batch_state()
    for k, p in enumerate(probs):
        if st["err"][k]:
            continue
        o = O.OracleSim(p)
        o.run()
        assert o.steps == st["steps"][k]
        ref = o.state()
        for q in range(5):
            assert rel_err(parts[k].cons[q], ref.cons[q]) <= 1e-9, (k, q)


def test_failed_simulation_stops_alone(gpu_lib):
    """A host-made failure in one simulation stops it; the others finish unchanged.

    The failure: a cell whose kinetic energy exceeds its total energy, so
    cons->prim yields a negative pressure, which the reference asserts against
    (physical_quantities.rs:220-221).  (A negative total energy would not do:
    the reference resets such a cell to vacuum, part.rs:184-191.)"""
    probs = ics.riemann_batch_1d(5, seed=43, n_min=40, n_max=120, riemann=ics.HLLC, t_end=0.02)
    packed, off, te = ics.pack(probs)
    bad = 2
    i = int(off[bad]) + 3
    c = packed.cells.cons
    c[1][i] = 4.0 * np.sqrt(2.0 * c[0][i] * c[4][i])
    sim = G.GpuSim(packed, cell_offsets=off, t_end=te)
    with pytest.raises(G.MvmmError):
        sim.run()
    st = sim.batch_state()
    assert st["err"][bad] != 0 and st["finished"].all()
    parts = ics.unpack_cells(sim.state(), off)
    for k, p in enumerate(probs):
        if k == bad:
            continue
        assert st["err"][k] == 0
        alone = G.GpuSim(p)
        alone.run()
        assert np.array_equal(parts[k].cons, alone.state().cons), k


def test_autotune_keeps_state_and_results(gpu_lib):
    """The autotuner restores the state it timed from; block sizes do not change results."""
    p = ics.kelvin_helmholtz_2d(32, riemann=ics.EXACT)
    a = G.GpuSim(p, precision=1)
    b = G.GpuSim(p, precision=1)
    a.run(max_steps=3)
    b.run(max_steps=3)
    before = a.state()
    bf, bc = a.autotune(2)
    assert bf in (64, 128, 256) and bc in (64, 128, 256)
    after = a.state()
    for f in ("cons", "prim", "grad", "dt"):
        assert np.array_equal(before.arrays[f], after.arrays[f]), f
    a.run(max_steps=5)
    b.run(max_steps=5)
    assert a.ti_current == b.ti_current
    for f in ("cons", "prim", "grad"):
        assert np.array_equal(a.state().arrays[f], b.state().arrays[f]), f
