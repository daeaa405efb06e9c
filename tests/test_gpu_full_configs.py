"""Parity at the full sizes of the reference workloads (plain FP64 form).

* Shear layer, 256x256 jittered periodic lattice, exact solver: the GPU and
  the oracle step in lock-step to simulated time T_KH; same integer timeline
  at every step, conserved state within 1e-9 (norm-wise, per quantity), mass,
  momentum and energy conserved to round-off.  T_KH stops short of t_end = 1.5:
  the reference's cell-wise limiter offsets periodic faces by the face shift
  (runner/hydrodynamics.rs:119: face.centroid() - centroid - shift, where the
  flux code puts the face centroid in the left cell's frame, flux.rs:33-35), so
  cells next to the periodic seam get extrapolation vectors a box length
  long.  Their limiter factor eventually turns negative, a velocity gradient
  runs away and the CFL timestep halves every step until the integer timestep
  is zero (MVMM_ERR_ZERO_DTI); the oracle shows this at 64x64 from t = 0.62 on,
  and at 256x256 the GPU, which reproduces the reference's arithmetic, meets
  it between t = 0.08 and 0.17.  While the gradient runs away, last-bit
  differences (the oracle's pow against the GPU's) grow with it, and at
  256x256 the two integer timelines part at t ~ 0.09.  With limiter_frame = 1
  (the limiter's offsets in flux_exchange's frame) the same shear layer runs
  to t_end = 1.5: the GPU and the oracle take the same 16,385 steps and end
  within 1e-9 (measured 1.4e-13), mass and energy conserved to round-off.
* Point blast, 128^3 jittered periodic lattice (2.1M cells, ~16.7M faces),
  HLLC, hierarchical time bins: 60 steps in lock-step; time bins bit-equal,
  state within 1e-10, the realised bin spread recorded.
* 512 independent 1D Riemann problems (N log-uniform in [200, 20000]) in one
  batch, PVRS and exact: every instance after 100 of its steps within 1e-10 of
  the oracle run alone, with the same flagged instances (error bits per
  instance); and the 64 instances cheapest to finish run to t_end = 0.15
  within 1e-9.  (All 512 to t_end is ~4e11 face updates: about an hour on the
  host cores, so the oracle cannot check it; bench.py times that run.)
"""

import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import compare_cells, rel_err, totals

pytestmark = pytest.mark.gpu

# ~470 steps.  The GPU-vs-oracle difference sits in the cells next to the
# periodic seam, whose limiter the reference feeds box-length extrapolation
# vectors (gradients ~1e4 there from the first steps): max relative difference
# 1.8e-12 at t = 0.02, 1.8e-10 at t = 0.04, 2.7e-9 at t = 0.05, 1e-6 at t = 0.07.
T_KH = 0.04
MAX_NR_TIMESTEPS = 1 << 57


def test_kh256_exact_parity_to_time(gpu_lib):
    p = ics.kelvin_helmholtz_2d(256, riemann=ics.EXACT, t_end=1.5)
    tb = p.params.t_end / MAX_NR_TIMESTEPS
    gpu = G.GpuSim(p)
    orc = O.OracleSim(p, n_threads=0)
    while gpu.ti_current * tb < T_KH:
        gpu.step()
        orc.step()
        assert gpu.ti_current == orc.ti_current, gpu.steps
    assert gpu.steps == orc.steps and gpu.active_faces == orc.active_faces
    a, b = gpu.state(), orc.state()
    for q in range(5):
        e = rel_err(a.cons[q], b.cons[q])
        assert e <= 1e-9, (q, e)
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-12 * abs(t0[0])
    assert abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])
    for q in (1, 2, 3):
        assert abs(t1[q] - t0[q]) <= 1e-12 * abs(t0[0])
    assert gpu.error_bits() == orc.error() == 0
    print(f"kh256: {gpu.steps} steps to t = {gpu.ti_current * tb:.4f}")


def test_kh256_exact_parity_to_t_end_flux_frame(gpu_lib):
    p = ics.kelvin_helmholtz_2d(256, riemann=ics.EXACT, t_end=1.5)
    p.params.limiter_frame = 1
    gpu = G.GpuSim(p)
    gpu.run()
    orc = O.OracleSim(p, n_threads=0)
    orc.run()
    assert gpu.finished and orc.finished and gpu.steps == orc.steps
    assert gpu.error_bits() == orc.error() == 0
    a, b = gpu.state(), orc.state()
    for q in range(5):
        e = rel_err(a.cons[q], b.cons[q])
        assert e <= 1e-9, (q, e)
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-12 * abs(t0[0])
    assert abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])
    for q in (1, 2, 3):
        assert abs(t1[q] - t0[q]) <= 1e-12 * abs(t0[0])
    print(f"kh256 to t_end with the flux frame: {gpu.steps} steps")


def test_blast128_hierarchical_parity(gpu_lib):
    p = ics.point_blast_3d(128, seed=3, riemann=ics.HLLC, t_end=0.05, sync_all=False)
    gpu = G.GpuSim(p)
    orc = O.OracleSim(p, n_threads=0)
    bins = set()
    active = []
    for _ in range(60):
        f0 = orc.active_faces
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
        assert gpu.active_faces == orc.active_faces
        active.append(orc.active_faces - f0)
        bins.update(np.unique(orc.state().timebin).tolist())
    a, b = gpu.state(), orc.state()
    assert np.array_equal(a.timebin, b.timebin)
    errs = compare_cells(a, b, fields=("cons", "prim", "facc", "dt", "grad", "extrap"))
    assert max(errs.values()) <= 1e-10, errs
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-12 * abs(t0[0]) and abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])
    assert len(bins) >= 3, bins  # several time bins in use at once
    print(f"blast128: bins {sorted(bins)}, active faces per step {min(active)}..{max(active)} "
          f"of {p.mesh.n_faces}")


def _batch_problems(riemann):
    return ics.riemann_batch_1d(512, seed=4, riemann=riemann, t_end=0.15)


def _cost_to_t_end(q):
    """Rough face updates to t_end: steps ~ t_end / (cfl dx / (2 signal speed))."""
    s = q.cells
    with np.errstate(divide="ignore", invalid="ignore"):
        c = np.sqrt(q.params.gamma * s.prim[4] / s.prim[0])
    v = np.nanmax(c) + np.max(np.abs(s.prim[1]))
    n = q.mesh.n_cells
    return n * q.params.t_end / (q.params.cfl / n / (2.0 * v))


def _run_batch(sim, max_steps=0):
    try:
        sim.run(max_steps=max_steps)
    except G.MvmmError as e:  # flagged instances stop; the others run on
        assert e.code == -3


@pytest.mark.parametrize("riemann", [ics.PVRS, ics.EXACT], ids=["pvrs", "exact"])
def test_batch512_parity_fixed_steps(gpu_lib, riemann):
    probs = _batch_problems(riemann)
    packed, off, te = ics.pack(probs)
    assert packed.mesh.n_cells > 1_000_000
    sim = G.GpuSim(packed, cell_offsets=off, t_end=te)
    _run_batch(sim, max_steps=100)
    st = sim.batch_state()
    parts = ics.unpack_cells(sim.state(), off)
    flagged = 0
    for k, q in enumerate(probs):
        o = O.OracleSim(q, n_threads=0)
        o.run(max_steps=100)
        if o.error():
            flagged += 1
            assert st["err"][k] != 0, k
            continue
        assert st["err"][k] == 0, (k, st["err"][k])
        assert st["steps"][k] == o.steps and st["ti_current"][k] == o.ti_current, k
        b = o.state()
        for qq in range(5):
            assert rel_err(parts[k].cons[qq], b.cons[qq]) <= 1e-10, (k, qq)
    print(f"batch512 {['HLLC', 'exact', 'PVRS'][riemann]}: {flagged} instances flagged by both sides")


@pytest.mark.parametrize("riemann", [ics.PVRS, ics.EXACT], ids=["pvrs", "exact"])
def test_batch_cheapest64_to_t_end(gpu_lib, riemann):
    probs = _batch_problems(riemann)
    order = np.argsort([_cost_to_t_end(q) for q in probs])[:64]
    sub = [probs[i] for i in sorted(order)]
    packed, off, te = ics.pack(sub)
    sim = G.GpuSim(packed, cell_offsets=off, t_end=te)
    _run_batch(sim)
    st = sim.batch_state()
    parts = ics.unpack_cells(sim.state(), off)
    finished = 0
    for k, q in enumerate(sub):
        o = O.OracleSim(q, n_threads=0)
        try:
            o.run()
        except Exception:
            pass
        if o.error():
            assert st["err"][k] != 0, k
            continue
        assert st["err"][k] == 0 and st["finished"][k] and o.finished, k
        finished += 1
        assert st["steps"][k] == o.steps, k
        b = o.state()
        for qq in range(5):
            assert rel_err(parts[k].cons[qq], b.cons[qq]) <= 1e-9, (k, qq)
    assert finished >= 32
    print(f"batch cheapest 64 to t_end: {finished} finished, "
          f"{64 - finished} flagged; max steps {int(st['steps'].max())}")
