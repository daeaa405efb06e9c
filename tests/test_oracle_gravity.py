"""The oracle's gravity solver against an independent numpy restatement of
gravity.rs (the reference has no test of it): KeplerianPotential::acceleration
and circular_velocity (gravity.rs:125-147), the Keplerian timestep
eta * radius_2D / v_circ (:119-123), the constant potential (:81-95), and the
kicks: with a uniform state at rest (no fluxes) a constant potential only
kicks, by grav_kick (part.rs:303-312) over half of each step's dt twice."""
import numpy as np

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
