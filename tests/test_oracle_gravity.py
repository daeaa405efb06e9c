"""The oracle's gravity solver against an independent numpy restatement of
gravity.rs (the reference has no test of it): KeplerianPotential::acceleration
and circular_velocity (gravity.rs:125-147), the Keplerian timestep
eta * radius_2D / v_circ (:119-123), the constant potential (:81-95),
SelfGravity's direct sum over j > i and its timestep (:22-53), and the kicks:
with a uniform state at rest (no fluxes) a potential only kicks, by grav_kick
(part.rs:303-312) over half of each step's dt twice."""
import numpy as np
import pytest

from hydro_rs_gb300 import ics
from oracle import oracle as O


def _uniform(nx=16, **grav):
    p = ics.kelvin_helmholtz_2d(nx, riemann=ics.HLLC, t_end=0.5)
    n = p.mesh.n_cells
    u = ics.gas_internal_energy_from_pressure(p.params.gamma, 1.0, 1.0)
    p.cells = ics.cells_from_ic(p.mesh, p.cells.loc, 1.0 * p.mesh.volume, np.zeros((3, n)), np.full(n, u),
                                p.params.gamma)
    for k, v in grav.items():
        setattr(p.params, k, v)
    return p


def test_keplerian_formulas():
    pos, soft = np.array([0.5, 0.2, 0.5]), 0.3
    p = _uniform(gravity=ics.GRAVITY_KEPLERIAN, gravity_softening=soft, gravity_position=tuple(pos))
    o = O.OracleSim(p)
    x = p.cells.loc
    dx = x - pos[:, None]
    r2 = (dx * dx).sum(axis=0)
    r = np.sqrt(r2)
    r2s = np.where(r < soft, r2 + soft * soft, r2)
    a_ref = -dx / (r * r2s)
    assert np.allclose(o.gravity_accelerations(), a_ref, rtol=1e-15, atol=0)
    v_circ = np.sqrt(1.0 / np.where(r < soft, r + soft, r))
    dt_ref = 0.5 * np.sqrt(p.mesh.volume / np.pi) / v_circ
    assert np.allclose(o.gravity_timesteps(), dt_ref, rtol=1e-15, atol=0)
    assert (r < soft).any() and (r >= soft).any()  # both branches


def test_constant_potential_kicks_a_uniform_gas():
    g = np.array([0.0, -2.0, 0.0])
    p = _uniform(gravity=ics.GRAVITY_CONSTANT, gravity_acceleration=tuple(g), gravity_accelerations=True)
    o = O.OracleSim(p)
    assert np.all(np.isinf(o.gravity_timesteps()))
    dts = []
    for _ in range(3):
        dts.append(o.state().dt.copy())
        o.step()
    s = o.state()
    m = p.cells.cons[0]
    # kick2 of step k over the dt it starts with, kick1 at its end over the new dt
    t_kicked = sum(0.5 * d for d in dts) + sum(0.5 * d for d in dts[1:]) + 0.5 * s.dt
    # a uniform gas has no pressure gradients: the momentum is the kicks' sum
    mom = s.cons[1:4]
    assert np.allclose(mom[0], 0.0, atol=1e-15) and np.allclose(mom[2], 0.0, atol=1e-15)
    assert np.allclose(mom[1] / m, g[1] * t_kicked, rtol=1e-12)
    assert o.error() == 0


def test_gravity_off_by_default_changes_nothing():
    a = O.OracleSim(_uniform())
    b = O.OracleSim(_uniform(gravity=ics.GRAVITY_SELF, gravity_softening=0.1))
    for _ in range(4):
        a.step()
        b.step()
    x, y = a.state(), b.state()
    assert a.ti_current == b.ti_current
    for k in ("cons", "prim", "dt"):
        assert np.array_equal(getattr(x, k), getattr(y, k))


def _self_gravity_ref(loc, mass, eps):
    """gravity.rs:22-43 term by term in the reference's order: the term of
    particle j is added to every i < j in turn, so each a_i sums j = i+1,
    i+2, ... in index order; |d| = sqrt((dx dx + dy dy) + dz dz) as glam's
    length, r^3 = (r r) r."""
    n = loc.shape[1]
    a = np.zeros((3, n))
    for j in range(1, n):
        d = loc[:, j:j + 1] - loc[:, :j]
        r = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + eps
        r3 = r * r * r
        a[:, :j] = a[:, :j] + (mass[j] * d) / r3
    return a


@pytest.mark.parametrize("case", ["kh2d", "blast3d", "unsoftened"])
def test_self_gravity_accelerations_and_timestep(case):
    if case == "blast3d":
        p = ics.point_blast_3d(5, riemann=ics.HLLC)
    else:
        p = ics.kelvin_helmholtz_2d(12, riemann=ics.HLLC)
    eps = 0.0 if case == "unsoftened" else 0.03
    p.params.gravity, p.params.gravity_softening = ics.GRAVITY_SELF, eps
    o = O.OracleSim(p)
    a_ref = _self_gravity_ref(p.cells.loc, p.cells.cons[0], eps)
    assert np.array_equal(o.gravity_accelerations(), a_ref)
    a2 = a_ref[0] * a_ref[0] + a_ref[1] * a_ref[1] + a_ref[2] * a_ref[2]
    with np.errstate(divide="ignore", invalid="ignore"):
        dt_ref = np.where(a2 == 0.0, np.inf, np.sqrt(eps / np.sqrt(a2)))
    assert np.array_equal(o.gravity_timesteps(), dt_ref)
    assert a2[-1] == 0.0 and (a2[:-1] > 0).all()  # the last particle has nothing after it


def test_self_gravity_kicks_a_uniform_gas():
    """One step of a uniform gas at rest with self-gravity accelerations: no
    pressure gradients, so each cell's momentum is its kicks, a_i m_i (dt_0 / 2
    + dt_1 / 2), with a_i the sum over the cells after it."""
    p = _uniform(gravity=ics.GRAVITY_SELF, gravity_softening=0.05, gravity_accelerations=True)
    o = O.OracleSim(p)
    dt0 = o.state().dt.copy()
    o.step()
    s = o.state()
    a = _self_gravity_ref(p.cells.loc, p.cells.cons[0], 0.05)
    m = p.cells.cons[0]
    for ax in range(2):
        assert np.allclose(s.cons[1 + ax], a[ax] * m * (0.5 * dt0 + 0.5 * s.dt), rtol=1e-12, atol=1e-15)
    assert o.error() == 0
