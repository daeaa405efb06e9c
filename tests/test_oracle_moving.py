"""Moving meshes in the CPU oracle (particle motion fluid / steer / steer_pakmor).

The generators drift with the particle velocities of set_particle_velocity
(part.rs:328-372, hydro_kick1 part.rs:87-104) and the host rebuilds the Voronoi
mesh before each step (Space::drift / volume_calculation).  The reference has
no test of this path; it is pinned by properties: a uniform flow carried by
fluid motion stays uniform (Galilean invariance of the moving-mesh scheme: the
faces move with the fluid, so no mass crosses them) while its generators move
by v t, and mass, momentum and energy are conserved to round-off in a periodic
box for every motion.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import ics
from hydro_rs_gb300.moving import MovingMeshStepper
from oracle import oracle as O


def _uniform_problem(nx, v=(0.3, -0.2)):
    p = ics.kelvin_helmholtz_2d(nx, riemann=ics.HLLC, t_end=1.0)
    loc = p.cells.loc
    vel = np.zeros((3, loc.shape[1]))
    vel[0], vel[1] = v
    u = ics.gas_internal_energy_from_pressure(p.params.gamma, 1.0, 1.0)
    p.cells = ics.cells_from_ic(p.mesh, loc, 1.0 * p.mesh.volume, vel, u, p.params.gamma)
    p.params.particle_motion = ics.FLUID
    return p


def test_uniform_flow_fluid_motion():
    p = _uniform_problem(12)
    sim = O.OracleSim(p)
    st = MovingMeshStepper(sim, p.mesh)
    loc0 = p.cells.loc.copy()
    t = 0.0
    for _ in range(6):
        st.step()
        assert sim.error() == 0
    s = sim.state()
    assert np.allclose(s.prim[0], 1.0, rtol=1e-12, atol=0)
    assert np.allclose(s.prim[1], 0.3, rtol=0, atol=1e-12)
    assert np.allclose(s.prim[2], -0.2, rtol=0, atol=1e-12)
    assert np.allclose(s.prim[4], 1.0, rtol=1e-12, atol=0)
    # the generators moved with the flow (periodic unit box); t = last drift time
    t = (sim.ti_old) * p.params.t_end / (1 << 57)
    d = (s.loc[:2] - loc0[:2] - np.array([[0.3], [-0.2]]) * t + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-12
    assert t > 0


@pytest.mark.parametrize("motion", [ics.FLUID, ics.STEER, ics.STEER_PAKMOR])
def test_conservation_moving(motion):
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.HLLC, t_end=1.5)
    p.params.particle_motion = motion
    sim = O.OracleSim(p)
    st = MovingMeshStepper(sim, p.mesh)
    for _ in range(8):
        st.step()
    assert sim.error() == 0
    s = sim.state()
    c0, c1 = p.cells.cons.sum(axis=1), s.cons.sum(axis=1)
    assert abs(c1[0] - c0[0]) <= 1e-13 * c0[0]
    assert abs(c1[4] - c0[4]) <= 1e-13 * c0[4]
    for q in (1, 2):
        assert abs(c1[q] - c0[q]) <= 1e-13 * c0[0]
    # the mesh moved: generators are no longer at the initial positions, and stay in the box
    assert np.abs(s.loc - p.cells.loc).max() > 1e-6
    assert (s.loc[:2] >= 0).all() and (s.loc[:2] < 1).all()
    assert abs(s.volume.sum() - 1.0) < 1e-12


def test_oracle_galilean_invariance_first_cycle():
    """tests/test_gallilean_invariance.rs (commented out in the reference) on the
    oracle: the first gradient estimate and timestep (engine step 0), then the
    drift, new mesh, flux exchange and cons -> prim of the first step with
    dt > 0 (engine step 1), boosted by 10 x, within the reference's 1e-10.  The
    second gradient estimate is not invariant in the reference's arithmetic
    (see tests/test_gpu_boundaries.py); it is recorded here as departing by
    more than the rounding of the states it starts from."""
    from tests.test_gpu_boundaries import _galilean_problem, galilean_differences

    boost = np.array([10.0, 0.0, 0.0])
    pa, pb = _galilean_problem((0.0, 0.0, 0.0)), _galilean_problem(boost)
    a, b = O.OracleSim(pa), O.OracleSim(pb)
    sa, sb = MovingMeshStepper(a, pa.mesh), MovingMeshStepper(b, pb.mesh)
    sa.step()
    sb.step()
    d = galilean_differences(a.state(), b.state(), boost)
    assert a.ti_current == b.ti_current and max(d.values()) <= 1e-10, d
    sa.step()
    sb.step()
    d = galilean_differences(a.state(), b.state(), boost)
    grad = d.pop("grad")
    assert a.ti_current == b.ti_current and max(d.values()) <= 1e-10, d
    assert max(d.values()) < 1e-13 < grad  # states agree to rounding, the limited gradients do not


def test_removal_keep_restates_the_index_shift():
    """space.rs:851-853 removes the collected indices one by one from the
    particle vector: after the first removal each later index names the
    particle after the intended one, and an index past the end panics."""
    from hydro_rs_gb300.moving import RemovalError, removal_keep

    assert removal_keep(10, [3]).tolist() == [0, 1, 2, 4, 5, 6, 7, 8, 9]
    assert removal_keep(10, [3, 7]).tolist() == [0, 1, 2, 4, 5, 6, 7, 9]
    with pytest.raises(RemovalError):
        removal_keep(10, [8, 9])


def _reflect_ref(s, dt, box=(1.0, 1.0), dim=2):
    """Space::drift of a reflective box in numpy, the reference's steps
    (part.rs:107-119, 385-428, 457-469; utils.rs:34-43;
    physical_quantities.rs:239-242): loc, prim and grad after the drift."""
    loc = s.loc.copy()
    for a in range(dim):
        loc[a] = loc[a] + s.v[a] * dt
    prim, grad = s.prim.copy(), s.grad.copy()
    for i in range(loc.shape[1]):
        x = loc[:, i].copy()
        if all(0.0 <= x[a] < box[a] for a in range(dim)):
            continue
        old = x.copy()
        for a in range(dim):
            if x[a] < 0.0:
                x[a] -= 2.0 * x[a]
            if x[a] > box[a]:
                x[a] -= 2.0 * (x[a] - box[a])
        loc[:, i] = x
        sh = x - old
        l2 = sh[0] * sh[0] + sh[1] * sh[1] + sh[2] * sh[2]
        if not l2 > 0.0:
            continue
        n = sh * (1.0 / np.sqrt(l2))
        dot = lambda u, w: u[0] * w[0] + u[1] * w[1] + u[2] * w[2]
        v = prim[1:4, i].copy()
        prim[1:4, i] = v - (2.0 * dot(v, n)) * n
        g = [grad[3 * q:3 * q + 3, i].copy() for q in range(5)]
        g[0] = g[0] - (2.0 * dot(g[0], n)) * n
        g[4] = g[4] - (2.0 * dot(g[0], n)) * n
        dvn = np.array([dot(np.array([g[1][c], g[2][c], g[3][c]]), n) for c in range(3)])
        for q, c in ((1, 0), (2, 1), (3, 2)):
            g[q] = g[q] - (2.0 * dvn) * n[c]
        for q in (1, 2, 3):
            g[q] = g[q] - (2.0 * dot(g[q], n)) * n
        for q in range(5):
            grad[3 * q:3 * q + 3, i] = g[q]
    return loc, prim, grad


@pytest.mark.parametrize("dim", [2, 3])
def test_reflective_drift_restated(dim):
    """A drift long enough to carry generators through the walls: the oracle's
    Particle::box_reflect against the numpy restatement, bit for bit; only
    loc moves (centroid and gradients_centroid are not shifted)."""
    p = ics.wall_flow_2d(16 if dim == 2 else 6, boundary=ics.REFLECTIVE, v=(4.0, 1.0), dim=dim)
    o = O.OracleSim(p)
    st = MovingMeshStepper(o, p.mesh)
    st.step()
    st.step()  # gradients and particle velocities of a stepped state
    s0 = o.state()
    dt = 0.02
    o.drift(dt)
    s1 = o.state()
    loc, prim, grad = _reflect_ref(s0, dt, box=(1.0, 1.0, 1.0), dim=dim)
    ahead = s0.loc[:dim] + s0.v[:dim] * dt
    moved = ((ahead >= 1.0) | (ahead < 0.0)).any(axis=0)
    assert moved.sum() >= 10 and (np.abs(s0.grad[:, moved]) > 0).any()
    assert np.array_equal(s1.loc, loc)
    assert np.array_equal(s1.prim, prim)
    assert np.array_equal(s1.grad, grad)
    assert o.error() == 0
    for a in range(dim):  # centroid drifts by v dt, with no reflection
        assert np.array_equal(s1.centroid[a], s0.centroid[a] + s0.v[a] * dt)


@pytest.mark.parametrize("boundary", [ics.OPEN, ics.VACUUM])
def test_open_box_removes_the_generators_that_left(boundary):
    p = ics.wall_flow_2d(16, boundary=boundary)
    o = O.OracleSim(p)
    st = MovingMeshStepper(o, p.mesh)
    for _ in range(10):
        st.step()
    assert st.removed == 1 and st.sim.mesh.n_cells == p.mesh.n_cells - 1
    assert st.sim.error() == 0 and st.sim.steps == 10
    s = st.sim.state()
    assert (s.loc[0] >= 0).all() and (s.loc[0] < 1).all() and (s.loc[1] >= 0).all() and (s.loc[1] < 1).all()
