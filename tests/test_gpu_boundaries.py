"""Wall boundaries, the isothermal gas law, near-vacuum exact solves and
Galilean invariance: the CUDA path against the CPU oracle.

* Open and vacuum walls (``flux_exchange_boundary``, ``flux.rs:102-195``, and
  ``Space::get_boundary_part``, ``space.rs:213-229``) on the Sod tube with each
  of the three solvers: the plain FP64 form within 1e-12 after the first dt>0
  step and 1e-9 at t_end, with the same step count, face count and error
  bits; the FP32-face form through its L1 density error; the per-stage
  boundary-face fluxes of both forms.
* ``EquationOfState::Isothermal`` (``gas_law.rs:59-106``) on the Sod tube.  Its
  energy flux is not that of an energy equation, so a cell behind the
  rarefaction goes to negative energy and is reset to vacuum
  (``part.rs:178-193``) as in the reference; the GPU must reset the same cells.
* The FP32-face exact solver on the states its FP32 search is least suited
  to: vacuum-generating pairs and strong rarefactions.
* Galilean invariance of a whole moving-mesh step, restating the reference's
  ``tests/test_gallilean_invariance.rs`` (a 3x3 periodic lattice with a central
  over-pressure, fluid motion, exact solver, boosted by 10 x): extrapolations,
  primitives, gradients, timesteps and conserved quantities of the boosted run,
  de-boosted, equal the unboosted run's within the reference's 1e-10.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from hydro_rs_gb300.mesh import mesh_voronoi
from hydro_rs_gb300.moving import MovingMeshStepper
from oracle import oracle as O
from tests.helpers import compare_cells, rel_err

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0
WALLS = [("open", ics.OPEN), ("vacuum", ics.VACUUM)]
SOLVERS = [("hllc", ics.HLLC), ("exact", ics.EXACT), ("pvrs", ics.PVRS)]


def _lockstep(problem, steps, precision=0):
    orc = O.OracleSim(problem)
    gpu = G.GpuSim(problem, precision=precision)
    for _ in range(steps):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
    return orc, gpu


@pytest.mark.parametrize("wall", WALLS, ids=[w[0] for w in WALLS])
@pytest.mark.parametrize("solver", SOLVERS, ids=[s[0] for s in SOLVERS])
def test_sod_wall_parity(gpu_lib, wall, solver):
    p = ics.sod_1d(400, riemann=solver[1], boundary=wall[1])
    orc, gpu = _lockstep(p, 2)  # engine step 2 is the first with dt > 0
    errs = compare_cells(gpu.state(), orc.state())
    assert max(errs.values()) <= 1e-12, errs
    # boundary faces reached flux_exchange_boundary on both sides
    assert gpu.active_faces == orc.active_faces == 2 * p.mesh.n_faces
    orc.run()
    gpu.run()
    assert gpu.finished and orc.finished
    assert gpu.steps == orc.steps and gpu.active_faces == orc.active_faces
    a, b = gpu.state(), orc.state()
    for q in range(5):
        assert rel_err(a.cons[q], b.cons[q]) <= 1e-9, (q, rel_err(a.cons[q], b.cons[q]))
    assert gpu.error_bits() == orc.error()
    if wall[1] == ics.OPEN:
        # the open walls copy the inner state: no gradient at the ends, so
        # (up to the waves arriving there) nothing leaves the tube
        assert abs(a.cons[0].sum() - p.cells.cons[0].sum()) <= 1e-12
    else:
        # vacuum walls: gas streams out of both ends
        assert a.cons[0].sum() < p.cells.cons[0].sum()


@pytest.mark.parametrize("wall", WALLS, ids=[w[0] for w in WALLS])
def test_sod_wall_fp32_face(gpu_lib, wall):
    p = ics.sod_1d(400, riemann=ics.EXACT, boundary=wall[1])
    orc, gpu = _lockstep(p, 60, precision=1)
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1
    assert gpu.error_bits() == 0


@pytest.mark.parametrize("wall", WALLS, ids=[w[0] for w in WALLS])
@pytest.mark.parametrize("precision", [0, 1])
def test_boundary_face_fluxes_stage(gpu_lib, wall, precision):
    """mvmm_compute_fluxes on a state with gradients and extrapolations: the two
    wall faces (and every other face) against the oracle's FluxInfo rows."""
    p = ics.sod_1d(200, riemann=ics.HLLC, boundary=wall[1])
    orc = O.OracleSim(p)
    for _ in range(30):
        orc.step()
    st = orc.state()
    p2 = ics.Problem(p.name, p.params, p.mesh, st)
    gpu, o2 = G.GpuSim(p2, precision=precision), O.OracleSim(p2)
    gpu.predict(2e-4)
    o2.predict(2e-4)
    active = np.ones(p.mesh.n_cells, dtype=np.uint8)
    fg, ng = gpu.compute_fluxes(active)
    fo, no = o2.compute_fluxes(active)
    assert ng == no
    walls = np.nonzero(p.mesh.right < 0)[0]
    assert walls.size == 2
    tol = 1e-12 if precision == 0 else 2e-5
    for k in range(10):
        assert rel_err(fg[k], fo[k]) <= tol, (k, rel_err(fg[k], fo[k]))
        assert rel_err(fg[k][walls], fo[k][walls]) <= tol, ("wall", k)
    # the wall faces carry a flux: mass leaves through a vacuum wall, momentum through both
    assert np.all(np.abs(fo[1][walls]) > 0)


@pytest.mark.parametrize("solver", [("hllc", ics.HLLC), ("exact", ics.EXACT)], ids=["hllc", "exact"])
def test_isothermal_sod_parity(gpu_lib, solver):
    p = ics.sod_1d(200, riemann=solver[1], iso_u=1.5)
    orc, gpu = _lockstep(p, 2)
    errs = compare_cells(gpu.state(), orc.state())
    assert max(errs.values()) <= 1e-12, errs
    orc.run()
    gpu.run()
    assert gpu.steps == orc.steps and gpu.active_faces == orc.active_faces
    a, b = gpu.state(), orc.state()
    for q in range(5):
        assert rel_err(a.cons[q], b.cons[q]) <= 1e-9, (q, rel_err(a.cons[q], b.cons[q]))
    # pressure is (gamma - 1) iso_u rho everywhere (gas_law.rs:90-97)
    live = b.prim[0] > 0
    assert np.allclose(a.prim[4][live], (GAMMA - 1.0) * 1.5 * a.prim[0][live], rtol=1e-12, atol=0)
    # the same cells were reset to vacuum on both sides
    assert np.array_equal(a.cons[0] == 0.0, b.cons[0] == 0.0)
    assert gpu.error_bits() == orc.error()


def test_isothermal_sod_fp32_face(gpu_lib):
    p = ics.sod_1d(200, riemann=ics.HLLC, iso_u=1.5)
    orc, gpu = _lockstep(p, 40, precision=1)
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1


def _hard_states(rng, n):
    """Vacuum-generating pairs and strong rarefactions (Toro's test 2 family)."""
    L = np.zeros((5, n))
    R = np.zeros((5, n))
    rho = 10 ** rng.uniform(-1, 1, (2, n))
    p = 10 ** rng.uniform(-3, 1, (2, n))
    a = np.sqrt(GAMMA * p / rho)
    # v_R - v_L from 0.5x to 1.5x the vacuum-generation threshold 2/(gamma-1) (a_L + a_R)
    thr = 2.0 / (GAMMA - 1.0) * (a[0] + a[1])
    dv = thr * rng.uniform(0.5, 1.5, n)
    L[0], R[0] = rho
    L[4], R[4] = p
    L[1], R[1] = -0.5 * dv, 0.5 * dv
    nrm = np.zeros((3, n))
    nrm[0] = 1.0
    return L, R, nrm, dv / thr


def test_fp32_exact_near_vacuum(gpu_lib):
    """FP32-face exact solver on vacuum-generating and strong-rarefaction
    states: the FP32 form keeps the FP64 result's vacuum classification and
    meets the form's tolerance on every state; the half-states themselves are
    compared where the star pressure is not far below the side pressures'
    rounding (p* > 1e-6 p_min), since FP32 cannot resolve less."""
    rng = np.random.default_rng(31)
    n = 4096
    L, R, nrm, ratio = _hard_states(rng, n)
    vf = np.zeros((3, n))
    ref, _ = O.riemann_flux(1, GAMMA, L, R, vf, nrm)
    got = G.riemann_flux(1, GAMMA, L, R, vf, nrm, precision=1)
    ok = np.isfinite(ref).all(axis=0)
    assert np.array_equal(np.isfinite(got).all(axis=0), ok)
    vac = ratio >= 1.0  # vacuum generated between the two rarefactions (vacuum.rs)
    assert vac.sum() > n // 4 and (~vac).sum() > n // 4
    # where x/t = 0 lies in the vacuum both forms give exactly zero flux
    assert np.array_equal(got[0] == 0.0, ref[0] == 0.0)
    scale = np.max(np.abs(ref[:, ok]), axis=1) + 1e-300
    err = np.abs(got[:, ok] - ref[:, ok]) / scale[:, None]
    assert np.max(err) <= 1e-5, np.max(err)
    hs_ref, _ = O.riemann_sample(1, GAMMA, L, R, nrm)
    hs = G.riemann_sample(1, GAMMA, L, R, nrm, precision=1)
    strong = (~vac) & (hs_ref[4] > 1e-6 * np.minimum(L[4], R[4]))
    for q in (0, 1, 4):
        rel = np.abs(hs[q, strong] - hs_ref[q, strong]) / (np.abs(hs_ref[q, strong]) + 1e-300)
        assert np.median(rel) <= 1e-6 and np.max(rel) <= 1e-3, (q, np.median(rel), np.max(rel))


def test_fp32_exact_strong_rarefaction_run(gpu_lib):
    """Toro's test 2 (two strong rarefactions, p* ~ 0.0019) run in the FP32-face
    form with the exact solver: L1 density against the FP64 oracle, and the
    faces the FP32 search could not finish are counted as FP64 fallbacks."""
    p = ics.riemann_1d(400, (1.0, -2.0, 0.4), (1.0, 2.0, 0.4), ics.EXACT, t_end=0.15)
    orc, gpu = _lockstep(p, 50, precision=1)
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1
    st = gpu.stats()
    assert 0 <= st["fp64_fallback_faces"] <= st["active_faces"]
    assert gpu.error_bits() == orc.error() == 0


def _galilean_problem(v):
    """get_ic_2d of tests/test_gallilean_invariance.rs: 9 generators on the
    periodic unit square, rho = 1, velocity v, P = 100 at the centre, 1 elsewhere."""
    params = ics.Params(gamma=GAMMA, cfl=0.3, riemann=ics.EXACT, boundary=ics.PERIODIC, dimensionality=2,
                        sync_all=True, t_end=0.5, particle_motion=ics.FLUID)
    x, box, vpp, _ = ics.lattice((1.0, 1.0, 1.0), 9, 2, 0.0, None)
    mesh = mesh_voronoi(x, 2, box, True)
    centre = (np.abs(x[0] - 0.5) < 1e-12) & (np.abs(x[1] - 0.5) < 1e-12)
    assert centre.sum() == 1
    pres = np.where(centre, 100.0, 1.0)
    vel = np.zeros((3, 9))
    vel[:, :] = np.asarray(v, dtype=float)[:, None]
    u = ics.gas_internal_energy_from_pressure(GAMMA, pres, 1.0)
    cells = ics.cells_from_ic(mesh, x, np.full(9, vpp), vel, u, GAMMA)
    return ics.Problem("galilean_2d", params, mesh, cells)


def galilean_differences(x, y, boost):
    """Boosted state y de-boosted and compared with x, field by field (the
    quantities tests/test_gallilean_invariance.rs compares)."""
    m = y.cons[0]
    mom = y.cons[1:4] - m * boost[:, None]
    en = y.cons[4] - (y.cons[1:4] * boost[:, None]).sum(axis=0) + 0.5 * m * (boost @ boost)
    return {
        "extrap": np.abs(x.extrap - y.extrap).max(),
        "rho": np.abs(x.prim[0] - y.prim[0]).max(),
        "v": np.abs(x.prim[1:4] - (y.prim[1:4] - boost[:, None])).max(),
        "P": np.abs(x.prim[4] - y.prim[4]).max(),
        "grad": np.abs(x.grad - y.grad).max(),
        "dt": np.abs(x.dt - y.dt).max(),
        "mass": np.abs(x.cons[0] - m).max(),
        "momentum": np.abs(x.cons[1:4] - mom).max(),
        "energy": np.abs(x.cons[4] - en).max(),
        "volume": np.abs(x.volume - y.volume).max(),
    }


def test_galilean_invariance_moving_mesh(gpu_lib):
    """The reference's scenario, in the order its test checks it: the first
    gradient estimate and timestep (engine step 0), then the drift, the new
    mesh, the flux exchange and cons -> prim of the first step with dt > 0
    (engine step 1), each within the reference's 1e-10.  The reference's test
    goes on to a second gradient estimate, which its own cell-wise limiter
    (gradients.rs:85-102) does not keep invariant on this lattice: four cells
    meet at every Voronoi vertex, pressures that should be equal differ in the
    last bits between the frames (the kinetic energy subtracted in cons -> prim
    is 50x larger when boosted), and the limiter's ratios of those differences
    move dP/dy by ~1e-5 in the reference arithmetic as restated by the oracle
    (the test is commented out in the reference).  Both frames are also
    checked against the oracle over the same two steps; later steps inherit
    the limiter's amplification of last-bit differences on this lattice, where
    the oracle's pow and the GPU's differ by an ulp."""
    boost = np.array([10.0, 0.0, 0.0])
    pa, pb = _galilean_problem((0.0, 0.0, 0.0)), _galilean_problem(boost)
    a, b = G.GpuSim(pa), G.GpuSim(pb)
    oa, ob = O.OracleSim(pa), O.OracleSim(pb)
    steppers = [MovingMeshStepper(s, pa.mesh) for s in (a, b, oa, ob)]
    eps = 1e-10  # float_cmp's epsilon in the reference test
    for step in range(2):
        for s in steppers:
            s.step()
        assert a.ti_current == b.ti_current == oa.ti_current == ob.ti_current, step  # dti == dti_boosted
        d = galilean_differences(a.state(), b.state(), boost)
        if step == 0:
            assert max(d.values()) <= eps, (step, d)
        elif step == 1:
            d.pop("grad")
            assert max(d.values()) <= eps, (step, d)
        for g, o in ((a, oa), (b, ob)):
            errs = compare_cells(g.state(), o.state(), fields=("cons", "prim", "grad", "loc", "volume", "v"))
            assert max(errs.values()) <= 1e-12, (step, errs)
    assert a.error_bits() == 0 and b.error_bits() == 0
