"""The gravity solver (gravity.rs) on the GPU against the oracle.

The reference's runners take the gravity solver's timestep per cell where it
is smaller (runner/hydrodynamics/optimal_order.rs:47-50) but never compute
accelerations ("TODO: gravity", :33), so a_grav stays zero and the kicks add
nothing: with the Keplerian potential the timestep limit is the whole effect.
With gravity_accelerations set, the external potential's accelerations
(Potential::Constant, KeplerianPotential::acceleration) are computed at that
point and kick2 / kick1 apply them (Particle::grav_kick, part.rs:303-312).
Plain FP64 form within 1e-12 of the oracle; the GravitySolver entry points
within 1e-14.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import compare_cells, rel_err

pytestmark = pytest.mark.gpu


def _gas_2d(nx=32, riemann=ics.HLLC, **grav):
    """The periodic shear layer at 32^2 with the given gravity settings."""
    p = ics.kelvin_helmholtz_2d(nx, riemann=riemann, t_end=0.5)
    for k, v in grav.items():
        setattr(p.params, k, v)
    return p


def _generator(i=528):
    """A generator position of the 32^2 lattice (a potential centred on it
    gives its cell the softened circular velocity)."""
    return tuple(float(x) for x in ics.kelvin_helmholtz_2d(32).cells.loc[:, i])


CASES = {
    # centred on a generator with a small softening: its cell's limit is below the CFL step
    "keplerian_timestep": dict(gravity=ics.GRAVITY_KEPLERIAN, gravity_softening=1e-4, gravity_position=_generator()),
    "self_timestep": dict(gravity=ics.GRAVITY_SELF, gravity_softening=0.01),
    "constant_kicks": dict(gravity=ics.GRAVITY_CONSTANT, gravity_acceleration=(0.0, -1.0, 0.0),
                           gravity_accelerations=True),
    # a point mass below the box: accelerations of order one
    "keplerian_kicks": dict(gravity=ics.GRAVITY_KEPLERIAN, gravity_softening=0.05, gravity_position=(0.5, -1.0, 0.5),
                            gravity_accelerations=True),
}


@pytest.mark.parametrize("case", list(CASES))
def test_gravity_step_parity(gpu_lib, case):
    p = _gas_2d(**CASES[case])
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    for _ in range(12):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim", "grad", "dt"))
    assert max(errs.values()) <= 1e-12, errs
    assert gpu.error_bits() == orc.error() == 0


def test_keplerian_timestep_limits_the_step(gpu_lib):
    """The Keplerian limit is what sets the step: the same run without gravity
    steps further in the same number of steps, and self-gravity (zero
    accelerations) changes nothing, bit for bit."""
    plain = G.GpuSim(_gas_2d())
    kep = G.GpuSim(_gas_2d(**CASES["keplerian_timestep"]))
    slf = G.GpuSim(_gas_2d(**CASES["self_timestep"]))
    for s in (plain, kep, slf):
        s.run(max_steps=6)
    assert kep.ti_current < plain.ti_current
    a, b = plain.state(), slf.state()
    for k, v in a.arrays.items():
        assert np.array_equal(np.ascontiguousarray(v).view(np.uint8), np.ascontiguousarray(b.arrays[k]).view(np.uint8))


@pytest.mark.parametrize("case", ["keplerian_timestep", "constant_kicks", "keplerian_kicks"])
def test_gravity_solver_entry_points(gpu_lib, case):
    p = _gas_2d(**CASES[case])
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    tg, to = gpu.gravity_timesteps(), orc.gravity_timesteps()
    fin = np.isfinite(to)
    assert np.array_equal(np.isfinite(tg), fin)
    if fin.any():
        assert rel_err(tg[fin], to[fin]) <= 1e-14
    ag, ao = gpu.gravity_accelerations(), orc.gravity_accelerations()
    # a generator at the Keplerian centre gets -0 / 0 (gravity.rs:133-135), NaN on both sides
    ok = np.isfinite(ao)
    assert np.array_equal(np.isfinite(ag), ok)
    for a in range(3):
        assert rel_err(ag[a][ok[a]], ao[a][ok[a]]) <= 1e-14, a


def test_gravity_rejections(gpu_lib):
    p = _gas_2d(gravity=ics.GRAVITY_SELF, gravity_softening=0.01, gravity_accelerations=True)
    with pytest.raises(G.MvmmError) as e:
        G.GpuSim(p)
    assert e.value.code == -5  # MVMM_E_UNSUPPORTED
    p = _gas_2d(**CASES["self_timestep"])
    with pytest.raises(G.MvmmError) as e:
        G.GpuSim(p).gravity_accelerations()
    assert e.value.code == -5
    p = _gas_2d(**CASES["constant_kicks"])
    sim = G.GpuSim(p)
    with pytest.raises(G.MvmmError) as e:
        sim.step_cells(p.cells.copy())
    assert e.value.code == -5
