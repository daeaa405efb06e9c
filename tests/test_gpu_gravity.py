"""The gravity solver (gravity.rs) on the GPU against the oracle.

The reference's runners take the gravity solver's timestep per cell where it
is smaller (runner/hydrodynamics/optimal_order.rs:47-50) but never compute
accelerations ("TODO: gravity", :33), so a_grav stays zero and the kicks add
nothing: with the Keplerian potential the timestep limit is the whole effect.
With gravity_accelerations set, the accelerations (Potential::Constant,
KeplerianPotential::acceleration, or SelfGravity's direct sum over j > i) are
computed at that point and kick2 / kick1 apply them (Particle::grav_kick,
part.rs:303-312).  Plain FP64 form within 1e-12 of the oracle; the
GravitySolver entry points within 1e-14, self-gravity's bit for bit.
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
    # the direct sum over the cells after each one: its accelerations kick and limit the timestep
    "self_kicks": dict(gravity=ics.GRAVITY_SELF, gravity_softening=0.02, gravity_accelerations=True),
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


@pytest.mark.parametrize("case", ["keplerian_timestep", "constant_kicks", "keplerian_kicks", "self_kicks"])
def test_gravity_solver_entry_points(gpu_lib, case):
    p = _gas_2d(**CASES[case])
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    if case == "self_kicks":  # a stepped state: updated masses, and a_grav set by the last step
        for _ in range(3):
            orc.step()
            gpu.step()
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
    if case == "self_kicks":
        # the same sums in the same order with IEEE division and square root
        assert np.array_equal(ag, ao)
        assert np.array_equal(gpu.gravity_timesteps(), orc.gravity_timesteps())


def test_self_gravity_hierarchical(gpu_lib):
    """The shear layer 16^2 on hierarchical time bins with self-gravity kicks:
    the self-gravity timestep sqrt(softening / |a|) spreads the cells over
    about ten bins; every cell's acceleration is summed each step (as
    compute_accelerations sets every a_grav), the active ones kick."""
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.HLLC)
    p.params.sync_all = False
    p.params.gravity, p.params.gravity_softening, p.params.gravity_accelerations = ics.GRAVITY_SELF, 0.01, True
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    bins = set()
    for _ in range(30):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
        bins.update(np.unique(orc.state().timebin).tolist())
    assert len(bins) >= 5, bins
    assert gpu.active_faces == orc.active_faces
    a, b = gpu.state(), orc.state()
    assert np.array_equal(a.timebin, b.timebin)
    errs = compare_cells(a, b, fields=("cons", "prim", "facc", "dt", "grad"))
    assert max(errs.values()) <= 1e-10, errs
    assert gpu.error_bits() == orc.error() == 0


def test_self_gravity_flags_as_the_oracle(gpu_lib):
    """grav_kick is not positivity preserving: it takes (dt/2)^2 |a|^2 m / 2 of
    internal energy, and the cold background of the point blast goes negative.
    Both sides flag the negative pressure (MVMM_ERR_NEG_PRIM) at the same step."""
    p = ics.point_blast_3d(6, riemann=ics.HLLC, sync_all=False, t_end=0.05)
    p.params.gravity, p.params.gravity_softening, p.params.gravity_accelerations = ics.GRAVITY_SELF, 0.05, True
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    for k in range(25):
        orc.step()
        try:
            gpu.step()
        except G.MvmmError as e:
            assert e.code == -3 and e.bits == orc.error() == 0x20, (k, e.bits, orc.error())
            return
        assert orc.error() == 0, k
    raise AssertionError("no step flagged")


def test_self_gravity_batch(gpu_lib):
    """Batched 1D problems with self-gravity kicks: each simulation sums over its
    own cells only, so it is the same alone and in the batch, bit for bit, and
    matches the oracle."""
    probs = ics.riemann_batch_1d(3, seed=5, n_min=50, n_max=120, riemann=ics.HLLC, t_end=0.01)
    for q in probs:  # the softening keeps the kicks within what the cold states take (no flags)
        q.params.gravity, q.params.gravity_softening, q.params.gravity_accelerations = ics.GRAVITY_SELF, 0.1, True
    packed, off, te = ics.pack(probs)
    sim = G.GpuSim(packed, cell_offsets=off, t_end=te)
    sim.run(max_steps=40)
    parts = ics.unpack_cells(sim.state(), off)
    st = sim.batch_state()
    for k, q in enumerate(probs):
        alone, orc = G.GpuSim(q), O.OracleSim(q)
        for _ in range(int(st["steps"][k])):
            alone.step()
            orc.step()
        a = alone.state()
        for f in ("cons", "prim", "grad", "dt"):
            assert np.array_equal(parts[k].arrays[f], a.arrays[f]), (k, f)
        errs = compare_cells(a, orc.state(), fields=("cons", "prim", "dt"))
        assert max(errs.values()) <= 1e-12, (k, errs)


def test_self_gravity_fp32_face_form(gpu_lib):
    """The FP32-face form with self-gravity kicks (kick2 and the FP32 copies of
    the primitives after the FP64 accumulation) stays close to the FP64
    oracle."""
    p = _gas_2d(**CASES["self_kicks"])
    orc, gpu = O.OracleSim(p), G.GpuSim(p, precision=1)
    for _ in range(10):
        orc.step()
        gpu.step()
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1


def test_self_gravity_stage_apply_fluxes(gpu_lib):
    """FiniteVolumeSolver::apply_fluxes per stage with self-gravity kicks:
    accelerations from the updated masses, then kick2 of the active cells."""
    p = _gas_2d(**CASES["self_kicks"])
    orc = O.OracleSim(p)
    for _ in range(2):
        orc.step()
    p2 = ics.Problem(p.name, p.params, p.mesh, orc.state())
    gpu, o2 = G.GpuSim(p2), O.OracleSim(p2)
    active = (np.random.default_rng(3).random(p.mesh.n_cells) < 0.6).astype(np.uint8)
    fo, _ = o2.compute_fluxes(active)
    gpu.apply_fluxes(fo, active)
    o2.apply_fluxes(fo, active)
    assert max(compare_cells(gpu.state(), o2.state(), fields=("cons", "facc")).values()) <= 1e-14
    assert np.array_equal(gpu.gravity_accelerations(), o2.gravity_accelerations())


def test_gravity_rejections(gpu_lib):
    p = _gas_2d(**CASES["constant_kicks"])
    sim = G.GpuSim(p)
    with pytest.raises(G.MvmmError) as e:
        sim.step_cells(p.cells.copy())
    assert e.value.code == -5
