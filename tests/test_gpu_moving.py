"""Moving meshes on the GPU against the oracle: device drift and particle
velocities, host Voronoi rebuild, new faces and geometry uploaded each step
(mvmm_drift, mvmm_get_positions, mvmm_set_mesh, mvmm_step); in boxes with walls
the drift reflects generators (reflective) or the host removes them (open,
vacuum)."""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from hydro_rs_gb300.moving import MovingMeshStepper
from oracle import oracle as O
from tests.helpers import compare_cells, totals

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("motion", [ics.FLUID, ics.STEER, ics.STEER_PAKMOR])
def test_moving_mesh_parity(gpu_lib, motion):
    p = ics.kelvin_helmholtz_2d(32, riemann=ics.HLLC, t_end=1.5)
    p.params.particle_motion = motion
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    so, sg = MovingMeshStepper(orc, p.mesh), MovingMeshStepper(gpu, p.mesh)
    for _ in range(8):
        so.step()
        sg.step()
        assert gpu.ti_current == orc.ti_current
        assert gpu.mesh.n_faces == orc.mesh.n_faces
    a, b = gpu.state(), orc.state()
    errs = compare_cells(a, b, fields=("cons", "prim", "loc", "centroid", "volume", "v", "grad"))
    assert max(errs.values()) <= 1e-10, errs
    assert gpu.error_bits() == 0 and orc.error() == 0
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-13 * abs(t0[0]) and abs(t1[4] - t0[4]) <= 1e-13 * abs(t0[4])


def test_moving_mesh_fp32(gpu_lib):
    p = ics.kelvin_helmholtz_2d(32, riemann=ics.EXACT, t_end=1.5)
    p.params.particle_motion = ics.FLUID
    orc, gpu = O.OracleSim(p), G.GpuSim(p, precision=1)
    so, sg = MovingMeshStepper(orc, p.mesh), MovingMeshStepper(gpu, p.mesh)
    for _ in range(8):
        so.step()
        sg.step()
        assert gpu.ti_current == orc.ti_current
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1
    # generators drift with velocities that include the FP32 gradients: where the
    # cell-wise limiter picks a different bound than in FP64 a cell's slope, and
    # with it its drift, differs locally; on average the positions agree closely
    d = np.abs(a.loc - b.loc)
    assert d.max() <= 1e-4 and d.mean() <= 1e-8, (d.max(), d.mean())


def test_moving_mesh_rejections(gpu_lib):
    p = ics.kelvin_helmholtz_2d(16)
    p.params.particle_motion = ics.STEER
    sim = G.GpuSim(p)
    with pytest.raises(G.MvmmError):
        sim.run(max_steps=2)  # a moving mesh is stepped from the host


@pytest.mark.parametrize("dim", [2, 3])
def test_reflective_drift_bitwise(gpu_lib, dim):
    """The device drift of a reflective box against the oracle's from the same
    state: Particle::box_reflect mirrors the generators that crossed a wall and
    reflects their primitive velocity and gradients, bit for bit."""
    p = ics.wall_flow_2d(16 if dim == 2 else 6, boundary=ics.REFLECTIVE, v=(4.0, 1.0), dim=dim)
    orc = O.OracleSim(p)
    st = MovingMeshStepper(orc, p.mesh)
    st.step()
    st.step()
    s0 = orc.state()
    gpu = G.GpuSim(ics.Problem(p.name, p.params, orc.mesh, s0))
    gpu.ti_current, gpu.ti_old = orc.ti_current, orc.ti_old
    dt = 0.02
    orc.drift(dt)
    gpu.drift(dt)
    a, b = gpu.state(), orc.state()
    ahead = s0.loc[:dim] + s0.v[:dim] * dt
    assert ((ahead >= 1.0) | (ahead < 0.0)).any(axis=0).sum() >= 10
    for f in ("loc", "prim", "grad", "centroid", "gc"):
        assert np.array_equal(a.arrays[f], b.arrays[f]), f
    assert gpu.error_bits() == orc.error() == 0


def test_reflective_box_moving_parity(gpu_lib):
    """Four steps of the wall flow in a reflective box, generators reflected in
    the last drift; the fifth step's state has a negative pressure (the
    reflection flips the primitive velocity but not the momentum), which both
    sides flag."""
    p = ics.wall_flow_2d(16, boundary=ics.REFLECTIVE, v=(4.0, 1.0))
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    so, sg = MovingMeshStepper(orc, p.mesh), MovingMeshStepper(gpu, p.mesh)
    for _ in range(4):
        so.step()
        sg.step()
        assert gpu.ti_current == orc.ti_current and gpu.mesh.n_faces == orc.mesh.n_faces
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim", "loc", "centroid", "volume", "v", "grad"))
    assert max(errs.values()) <= 1e-10, errs
    so.step()
    with pytest.raises(G.MvmmError) as e:
        sg.step()
    assert e.value.code == -3 and e.value.bits == orc.error() == 0x20


@pytest.mark.parametrize("boundary", [ics.OPEN, ics.VACUUM])
def test_open_box_moving_parity(gpu_lib, boundary):
    """Ten steps of the wall flow in an open / vacuum box: a generator leaves
    and is removed (a new context over the 255 kept), as in the oracle."""
    p = ics.wall_flow_2d(16, boundary=boundary)
    orc, gpu = O.OracleSim(p), G.GpuSim(p)
    so, sg = MovingMeshStepper(orc, p.mesh), MovingMeshStepper(gpu, p.mesh)
    for _ in range(10):
        so.step()
        sg.step()
        assert sg.sim.ti_current == so.sim.ti_current and sg.sim.mesh.n_cells == so.sim.mesh.n_cells
    assert sg.removed == so.removed == 1
    a, b = sg.sim.state(), so.sim.state()
    errs = compare_cells(a, b, fields=("cons", "prim", "loc", "centroid", "volume", "v", "grad"))
    assert max(errs.values()) <= 1e-10, errs
    assert sg.sim.error_bits() == so.sim.error() == 0


def test_open_box_fp32_face_form(gpu_lib):
    """The FP32-face form in an open box: the same generator leaves and the
    state stays close to the FP64 oracle."""
    p = ics.wall_flow_2d(16, boundary=ics.OPEN)
    orc, gpu = O.OracleSim(p), G.GpuSim(p, precision=1)
    so, sg = MovingMeshStepper(orc, p.mesh), MovingMeshStepper(gpu, p.mesh)
    for _ in range(10):
        so.step()
        sg.step()
    assert sg.removed == so.removed == 1 and sg.sim.precision == 1
    a, b = sg.sim.state(), so.sim.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1
