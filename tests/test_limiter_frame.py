"""The cell-wise limiter's face offsets, reference frame against flux_exchange's.

The reference's gradient_limit extrapolates to a face at face centroid -
centroid - shift (left cell) / + shift (right cell) (runner/hydrodynamics.rs:119),
while flux_exchange puts the face centroid in the left cell's frame
(flux.rs:33-35): across a periodic seam the offsets are a box length long.
`limiter_frame = 1` takes them in flux_exchange's frame.  CPU: on the oracle the
shear layer then reaches t_end, where with the reference's offsets its timestep
collapses; the two frames agree away from periodic faces (a reflective tube
has none).  GPU (marked): the plain form with the corrected frame against the
oracle at t_end, and the FP32-face form against the plain one at 512^2.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import rel_err, totals

MAX_NR_TIMESTEPS = 1 << 57


def _kh(nx, frame, riemann=ics.EXACT, t_end=1.5):
    p = ics.kelvin_helmholtz_2d(nx, riemann=riemann, t_end=t_end)
    p.params.limiter_frame = frame
    return p


def test_oracle_shear_layer_reaches_t_end_with_flux_frame():
    o = O.OracleSim(_kh(32, 1))
    o.run(max_steps=20000)
    assert o.finished and o.error() == 0


def test_frames_agree_without_periodic_faces():
    """A reflective tube has no face with a shift: both frames give the same bits."""
    a = ics.sod_1d(200)
    b = ics.sod_1d(200)
    b.params.limiter_frame = 1
    oa, ob = O.OracleSim(a), O.OracleSim(b)
    oa.run(max_steps=50)
    ob.run(max_steps=50)
    assert np.array_equal(oa.state().cons, ob.state().cons)


@pytest.mark.gpu
def test_gpu_flux_frame_parity_to_t_end(gpu_lib):
    from hydro_rs_gb300 import gpu as G

    p = _kh(64, 1)
    gpu, orc = G.GpuSim(p), O.OracleSim(p)
    gpu.run()
    orc.run()
    assert gpu.finished and orc.finished and gpu.steps == orc.steps
    a, b = gpu.state(), orc.state()
    for q in range(5):
        assert rel_err(a.cons[q], b.cons[q]) <= 1e-9, (q, rel_err(a.cons[q], b.cons[q]))
    t0, t1 = totals(p.cells), totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-12 * abs(t0[0]) and abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])
    assert gpu.error_bits() == orc.error() == 0


@pytest.mark.gpu
def test_gpu_fp32_face_l1_at_512_with_flux_frame(gpu_lib):
    """Without the seam's runaway gradients the FP32-face form stays on the
    plain form's timeline and within 1e-5 of it (L1, density)."""
    from hydro_rs_gb300 import gpu as G

    p = _kh(512, 1)
    a, b = G.GpuSim(p, precision=0), G.GpuSim(p, precision=1)
    for _ in range(60):
        a.step()
        b.step()
    assert a.ti_current == b.ti_current
    x, y = a.state(), b.state()
    l1 = np.abs(y.prim[0] - x.prim[0]).sum() / np.abs(x.prim[0]).sum()
    assert l1 <= 1e-5, l1
