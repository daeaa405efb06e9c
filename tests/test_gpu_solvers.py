"""GPU parity for the AIRS, TSRS, TRRS and LinearAdvection solvers and the
Godunov runner, through the C ABI, against the CPU oracle.

Same bar as the HLLC / exact / PVRS paths: single Riemann problems within
1e-11 (pow() is the only operation that is not correctly rounded on either
side), whole runs within 1e-9 at t_end and 1e-10 after a dozen steps on a
Voronoi mesh; the FP32-face form by its L1 density error.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import compare_cells, rel_err, totals
from tests.test_gpu_parity import _random_states

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0
ADV = np.array([0.7, -0.4, 0.2])
EXTRA = [ics.AIRS, ics.TSRS, ics.TRRS, ics.LINEAR_ADVECTION]


def _settings(kind):
    return {"airs_threshold": 2.0, "velocity": ADV if kind == ics.LINEAR_ADVECTION else None}


@pytest.mark.parametrize("kind", EXTRA)
def test_riemann_flux_fp64_matches_oracle(gpu_lib, kind):
    rng = np.random.default_rng(40 + kind)
    L, R, vf, nrm = _random_states(rng, 4096)
    kw = _settings(kind)
    ref, _ = O.riemann_flux(kind, GAMMA, L, R, vf, nrm, **kw)
    got = G.riemann_flux(kind, GAMMA, L, R, vf, nrm, **kw)
    ok = np.isfinite(ref).all(axis=0)
    assert ok.sum() > 3000
    assert np.array_equal(np.isfinite(got).all(axis=0), ok)
    for q in range(5):
        d = np.abs(got[q, ok] - ref[q, ok])
        s = np.abs(ref[q, ok]) + 1e-300
        assert np.max(d / np.maximum(s, np.max(s) * 1e-12)) < 1e-11, (kind, q)


@pytest.mark.parametrize("kind", [ics.AIRS, ics.TSRS, ics.TRRS])
def test_riemann_sample_fp64_matches_oracle(gpu_lib, kind):
    rng = np.random.default_rng(50 + kind)
    L, R, _, nrm = _random_states(rng, 2048)
    ref, _ = O.riemann_sample(kind, GAMMA, L, R, nrm, airs_threshold=2.0)
    got = G.riemann_sample(kind, GAMMA, L, R, nrm, airs_threshold=2.0)
    ok = np.isfinite(ref).all(axis=0)
    assert np.array_equal(np.isfinite(got).all(axis=0), ok)
    for q in range(5):
        d = np.abs(got[q, ok] - ref[q, ok])
        s = np.abs(ref[q, ok])
        assert np.max(d / np.maximum(s, np.max(s) * 1e-12)) < 1e-11, (kind, q)


@pytest.mark.parametrize("kind", EXTRA)
def test_riemann_flux_fp32_close_to_oracle(gpu_lib, kind):
    rng = np.random.default_rng(60 + kind)
    L, R, vf, nrm = _random_states(rng, 4096)
    L, R, vf, nrm = L[:, 32:], R[:, 32:], vf[:, 32:], nrm[:, 32:]
    kw = _settings(kind)
    ref, _ = O.riemann_flux(kind, GAMMA, L, R, vf, nrm, **kw)
    got = G.riemann_flux(kind, GAMMA, L, R, vf, nrm, precision=1, **kw)
    ok = np.isfinite(ref).all(axis=0) & np.isfinite(got).all(axis=0)
    assert ok.sum() > 3000
    for q in range(5):
        scale = np.abs(ref[q, ok]).max()
        assert np.median(np.abs(got[q, ok] - ref[q, ok])) / scale < 1e-5, (kind, q)


def test_missing_settings_rejected(gpu_lib):
    L = np.ones((5, 1))
    N = np.array([[1.0], [0.0], [0.0]])
    for kind in (ics.AIRS, ics.LINEAR_ADVECTION):
        with pytest.raises(G.MvmmError):
            G.riemann_flux(kind, GAMMA, L, L, np.zeros((3, 1)), N)
    p = ics.sod_1d(50, riemann=ics.AIRS)
    with pytest.raises(G.MvmmError):
        G.GpuSim(p)  # AIRS without a threshold (MissingAIRSThreshold)
    p = ics.sod_1d(50)
    p.params.runner = 7
    with pytest.raises(G.MvmmError):
        G.GpuSim(p)


@pytest.mark.parametrize("kind,runner", [(ics.AIRS, ics.OPTIMAL_ORDER), (ics.TSRS, ics.OPTIMAL_ORDER),
                                         (ics.TRRS, ics.OPTIMAL_ORDER), (ics.HLLC, ics.GODUNOV),
                                         (ics.AIRS, ics.GODUNOV)])
def test_sod_t_end_parity(gpu_lib, kind, runner):
    """Sod (N=1000) to t_end = 0.2 with each solver / runner: conserved state within 1e-9."""
    p = ics.sod_1d(1000, riemann=kind)
    p.params.runner = runner
    p.params.airs_threshold = 2.0
    orc = O.OracleSim(p)
    orc.run()
    gpu = G.GpuSim(p)
    gpu.run()
    assert gpu.finished and orc.finished
    assert gpu.steps == orc.steps and gpu.active_faces == orc.active_faces
    a, b = gpu.state(), orc.state()
    for q in range(5):
        assert rel_err(a.cons[q], b.cons[q]) <= 1e-9, q
    if runner == ics.GODUNOV:
        assert np.all(a.grad == 0.0)
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-13 * abs(t0[0])
    assert abs(t1[4] - t0[4]) <= 1e-13 * abs(t0[4])


def _advection_problem(nx):
    """Periodic 2D Voronoi mesh, uniform pressure and velocity, a dense square (run/config.yml pairs
    LinearAdvection with the Godunov runner)."""
    p = ics.kelvin_helmholtz_2d(nx, riemann=ics.LINEAR_ADVECTION, t_end=0.5)
    p.params.runner = ics.GODUNOV
    p.params.advection_velocity = tuple(ADV)
    loc = p.cells.loc
    rho = np.where((np.abs(loc[0] - 0.5) < 0.25) & (np.abs(loc[1] - 0.5) < 0.25), 2.0, 1.0)
    vel = np.zeros((3, loc.shape[1]))
    vel[:2] = ADV[:2, None]
    u = ics.gas_internal_energy_from_pressure(p.params.gamma, 2.5, 1.0 / rho)
    p.cells = ics.cells_from_ic(p.mesh, loc, rho * p.cells.volume, vel, u, p.params.gamma)
    return p


def test_linear_advection_godunov_parity(gpu_lib):
    p = _advection_problem(32)
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p)
    for _ in range(12):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim"))
    assert max(errs.values()) <= 1e-10, errs
    assert gpu.error_bits() == 0 and orc.error() == 0
    assert np.all(gpu.state().grad == 0.0)


@pytest.mark.parametrize("kind", [ics.AIRS, ics.TSRS, ics.TRRS])
def test_kh_small_parity(gpu_lib, kind):
    p = ics.kelvin_helmholtz_2d(32, riemann=kind, t_end=1.5)
    p.params.airs_threshold = 2.0
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p)
    for _ in range(12):
        orc.step()
        gpu.step()
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim", "grad"))
    assert max(errs.values()) <= 1e-10, errs


@pytest.mark.parametrize("kind", [ics.AIRS, ics.TSRS, ics.TRRS])
def test_fp32_face_l1(gpu_lib, kind):
    """20 steps on the same integer timeline as the oracle.  (With PVRS star
    states, which AIRS picks here since the pressure is near uniform, this
    32x32 shear layer collapses its timestep after about 25 steps in the FP64
    oracle too; past that point any perturbation is amplified.)"""
    p = ics.kelvin_helmholtz_2d(32, riemann=kind)
    p.params.airs_threshold = 2.0
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p, precision=1)
    for _ in range(20):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1
