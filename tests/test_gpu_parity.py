"""GPU parity: the CUDA path, called through the C ABI, against the CPU oracle.

Tolerances: plain FP64 path within 1e-12 (norm-wise relative, per
conserved quantity) after the first dt>0 step and 1e-9 at t_end; the FP32-face
form is checked through its L1 density error against the FP64 oracle.
"""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from oracle import oracle as O
from tests.helpers import compare_cells, rel_err, totals

pytestmark = pytest.mark.gpu

GAMMA = 5.0 / 3.0

# exact.rs:344-398 half-state known answers (gamma = 5/3)
EXACT_HALF = [
    ((0.75, 0.6, 0.8), (0.55, -0.25, 0.5), (0.8927393244785966, 0.35966250129769556, 1.0709476357371466)),
    ((0.75, 0.3, 0.8), (0.55, -0.75, 0.5), (0.9114320476995261, -0.03895103710637815, 1.201228148376388)),
    ((0.75, 0.1, 0.8), (0.55, 0.5, 0.5), (0.5562398903431287, 0.4792910646431622, 0.4861363537732538)),
    ((1.75, -0.1, 0.75), (0.55, 1.5, 0.5), (0.65432665196683, 0.6088656910463873, 0.14554217677392042)),
    ((0.75, -0.5, 0.8), (0.55, -0.1, 0.5), (0.5407985848180775, -0.1207089353568378, 0.4861363537732538)),
    ((1.75, -1.5, 0.75), (1.55, 0.1, 0.5), (0.5687181105004402, -0.5249266813300747, 0.09402548983542296)),
]


def _states(cases):
    n = len(cases)
    L = np.zeros((5, n))
    R = np.zeros((5, n))
    N = np.zeros((3, n))
    N[0] = 1.0
    for k, (l, r, _) in enumerate(cases):
        L[:, k] = [l[0], l[1], 0, 0, l[2]]
        R[:, k] = [r[0], r[1], 0, 0, r[2]]
    return L, R, N


def test_exact_half_state_golden_gpu(gpu_lib):
    L, R, N = _states(EXACT_HALF)
    out = G.riemann_sample(1, GAMMA, L, R, N)
    for k, (_, _, ref) in enumerate(EXACT_HALF):
        for q, idx in enumerate((0, 1, 4)):
            assert abs(out[idx, k] - ref[q]) <= 4 * np.spacing(abs(ref[q])) + 1e-15, (k, q, out[idx, k], ref[q])


def test_vacuum_half_state_golden_gpu(gpu_lib):
    # vacuum.rs:185-220: left state boosted by -0.15, right vacuum
    L = np.array([[1.0], [0.3 - 0.15], [0.0], [0.0], [0.5]])
    R = np.zeros((5, 1))
    N = np.array([[1.0], [0.0], [0.0]])
    out = G.riemann_sample(1, GAMMA, L, R, N)
    ref = (0.4950623323204316, 0.7221531968814576, 0.15490656018956153)
    for q, idx in enumerate((0, 1, 4)):
        assert abs(out[idx, 0] - ref[q]) <= 4 * np.spacing(ref[q]), (q, out[idx, 0], ref[q])


def _random_states(rng, n):
    L = np.zeros((5, n))
    R = np.zeros((5, n))
    for S in (L, R):
        S[0] = 10 ** rng.uniform(-1, 1, n)
        S[1:4] = rng.uniform(-2, 2, (3, n))
        S[4] = 10 ** rng.uniform(-3, 3, n)
    # a few vacuum sides and vacuum-generating states
    L[:, :8] = 0.0
    R[:, 8:16] = 0.0
    L[1, 16:24] = -20.0
    R[1, 16:24] = 20.0
    nrm = rng.normal(size=(3, n))
    nrm /= np.linalg.norm(nrm, axis=0)
    vf = rng.uniform(-0.5, 0.5, (3, n))
    return L, R, vf, nrm


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_riemann_flux_fp64_matches_oracle(gpu_lib, kind):
    rng = np.random.default_rng(10 + kind)
    L, R, vf, nrm = _random_states(rng, 4096)
    ref, _ = O.riemann_flux(kind, GAMMA, L, R, vf, nrm)
    got = G.riemann_flux(kind, GAMMA, L, R, vf, nrm)
    ok = np.isfinite(ref).all(axis=0)
    assert np.array_equal(np.isfinite(got).all(axis=0), ok)
    for q in range(5):
        d = np.abs(got[q, ok] - ref[q, ok])
        s = np.abs(ref[q, ok]) + 1e-300
        # pow() is the only non-correctly-rounded operation on either side
        assert np.max(d / np.maximum(s, np.max(s) * 1e-12)) < 1e-11, (kind, q)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_riemann_flux_fp32_close_to_oracle(gpu_lib, kind):
    rng = np.random.default_rng(20 + kind)
    L, R, vf, nrm = _random_states(rng, 4096)
    # moderate states (FP32 form targets smooth flows): no vacuum cases
    L, R, vf, nrm = L[:, 32:], R[:, 32:], vf[:, 32:], nrm[:, 32:]
    ref, _ = O.riemann_flux(kind, GAMMA, L, R, vf, nrm)
    got = G.riemann_flux(kind, GAMMA, L, R, vf, nrm, precision=1)
    ok = np.isfinite(ref).all(axis=0)
    for q in range(5):
        scale = np.abs(ref[q, ok]).max()
        assert np.median(np.abs(got[q, ok] - ref[q, ok])) / scale < 1e-5, (kind, q)


def _run_both(problem, steps, precision=0):
    orc = O.OracleSim(problem)
    gpu = G.GpuSim(problem, precision=precision)
    for _ in range(steps):
        orc.step()
        gpu.step()
        assert gpu.ti_current == orc.ti_current
    return orc, gpu


def test_sod_first_dt_step_parity(gpu_lib):
    """Config 1 (Sod, N=1000, HLLC): state after engine step 2 (first dt>0) within 1e-12."""
    p = ics.sod_1d(1000)
    orc, gpu = _run_both(p, 2)
    errs = compare_cells(gpu.state(), orc.state())
    for k, v in errs.items():
        assert v <= 1e-12, (k, v)
    assert orc.active_faces == gpu.active_faces == 2 * p.mesh.n_faces


def test_sod_t_end_parity(gpu_lib):
    """Config 1 run to t_end = 0.2: conserved state within 1e-9; totals conserved."""
    p = ics.sod_1d(1000)
    orc = O.OracleSim(p)
    orc.run()
    gpu = G.GpuSim(p)
    gpu.run()
    assert gpu.finished and orc.finished
    assert gpu.steps == orc.steps and gpu.active_faces == orc.active_faces
    a, b = gpu.state(), orc.state()
    for q in range(5):
        assert rel_err(a.cons[q], b.cons[q]) <= 1e-9, q
    t0 = totals(p.cells)
    t1 = totals(a)
    assert abs(t1[0] - t0[0]) <= 1e-13 * abs(t0[0])
    assert abs(t1[4] - t0[4]) <= 1e-13 * abs(t0[4])


@pytest.mark.parametrize("riemann", [ics.HLLC, ics.EXACT, ics.PVRS])
def test_kh_small_parity(gpu_lib, riemann):
    """Config 2 cut down to 32x32 (periodic Voronoi, all three solvers)."""
    p = ics.kelvin_helmholtz_2d(32, riemann=riemann, t_end=1.5)
    orc, gpu = _run_both(p, 12)
    errs = compare_cells(gpu.state(), orc.state(), fields=("cons", "prim", "grad"))
    worst = max(errs.values())
    assert worst <= 1e-10, errs
    assert gpu.active_faces == orc.active_faces


def test_stage_parity(gpu_lib):
    """FiniteVolumeSolver trait entry points one by one on the same state."""
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.EXACT)
    orc = O.OracleSim(p)
    for _ in range(3):
        orc.step()
    st = orc.state()
    p2 = ics.Problem(p.name, p.params, p.mesh, st)
    gpu = G.GpuSim(p2)
    o2 = O.OracleSim(p2)
    rng = np.random.default_rng(0)
    active = (rng.random(p.mesh.n_cells) < 0.7).astype(np.uint8)
    dt = 1e-3
    gpu.predict(dt)
    o2.predict(dt)
    assert max(compare_cells(gpu.state(), o2.state(), fields=("extrap", "prim")).values()) <= 1e-13
    fg, ng = gpu.compute_fluxes(active)
    fo, no = o2.compute_fluxes(active)
    assert ng == no
    for k in range(10):
        assert rel_err(fg[k], fo[k]) <= 1e-12, k
    gpu.apply_fluxes(fo, active)
    o2.apply_fluxes(fo, active)
    assert max(compare_cells(gpu.state(), o2.state(), fields=("cons", "facc")).values()) <= 1e-14
    gpu.convert(active)
    o2.convert(active)
    assert max(compare_cells(gpu.state(), o2.state(), fields=("prim",)).values()) <= 1e-14
    gpu.gradients(active)
    o2.gradients(active)
    assert max(compare_cells(gpu.state(), o2.state(), fields=("grad", "gc")).values()) <= 1e-12
    tg = gpu.compute_timesteps(active)
    to = o2.compute_timesteps(active)
    fin = np.isfinite(to)
    assert np.array_equal(np.isfinite(tg), fin)
    assert rel_err(tg[fin], to[fin]) <= 1e-12


def test_conservation_periodic_kh(gpu_lib):
    """Full-size-independent property: mass, momentum, energy conserved to round-off."""
    p = ics.kelvin_helmholtz_2d(64, riemann=ics.HLLC)
    gpu = G.GpuSim(p)
    gpu.run(max_steps=200)
    t0 = totals(p.cells)
    t1 = totals(gpu.state())
    assert abs(t1[0] - t0[0]) <= 1e-12 * abs(t0[0])
    assert abs(t1[4] - t0[4]) <= 1e-12 * abs(t0[4])
    for q in (1, 2, 3):
        assert abs(t1[q] - t0[q]) <= 1e-12 * abs(t0[0])
    assert gpu.error_bits() == 0


def test_fp32_face_l1(gpu_lib):
    """FP32-face form: L1 relative density error against the FP64 oracle."""
    p = ics.kelvin_helmholtz_2d(32, riemann=ics.EXACT)
    orc = O.OracleSim(p)
    gpu = G.GpuSim(p, precision=1)
    for _ in range(40):
        orc.step()
        gpu.step()
    a, b = gpu.state(), orc.state()
    l1 = np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum()
    assert l1 <= 1e-5, l1


def test_packed_host_block_round_trip(gpu_lib):
    """Upload / download through one packed host block (one copy each way) and
    through separate arrays give the same device state."""
    from hydro_rs_gb300.layout import CELL_ROWS, Cells
    p = ics.kelvin_helmholtz_2d(16)
    n = p.mesh.n_cells
    src = p.cells.copy()
    src.arrays["grad"][:] = np.random.default_rng(1).normal(size=src.grad.shape)
    packed = Cells.packed(n, np.zeros(CELL_ROWS * n), np.zeros(n, dtype=np.int8))
    for k, v in src.arrays.items():
        packed.arrays[k][...] = v
    for precision in (0, 1):
        sim = G.GpuSim(p, precision=precision)
        sim.upload(packed)
        back = sim.state()
        for k, v in src.arrays.items():
            assert np.array_equal(back.arrays[k], v), k
        sim.upload(src)
        out = Cells.packed(n, np.zeros(CELL_ROWS * n), np.zeros(n, dtype=np.int8))
        sim.state(out)
        for k, v in src.arrays.items():
            assert np.array_equal(out.arrays[k], v), k
        sim.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_step_cells_matches_resident_steps(gpu_lib, precision):
    """mvmm_step_cells (host state in, host state out, overlapped copies) gives
    bit-identical states and timelines to resident mvmm_step calls."""
    from hydro_rs_gb300.layout import CELL_ROWS, Cells
    p = ics.kelvin_helmholtz_2d(32, riemann=ics.EXACT)
    n = p.mesh.n_cells
    a = G.GpuSim(p, precision=precision)
    b = G.GpuSim(p, precision=precision)
    host = Cells.packed(n, np.zeros(CELL_ROWS * n), np.zeros(n, dtype=np.int8))
    for k, v in p.cells.arrays.items():
        host.arrays[k][...] = v
    split = p.cells.copy()  # separate arrays: one copy per row group
    for _ in range(6):
        a.step()
        b.step_cells(host)  # in place on one packed block
        assert a.ti_current == b.ti_current and a.active_faces == b.active_faces
    ref = a.state()

    def same_bits(x, y):  # signed zeros and NaN payloads included
        x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
        return x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8))

    for k, v in ref.arrays.items():
        assert same_bits(host.arrays[k], v), k
    c = G.GpuSim(p, precision=precision)
    out = p.cells.copy()
    for _ in range(6):
        c.step_cells(split, out)
        split = out.copy()
    for k, v in ref.arrays.items():
        assert same_bits(out.arrays[k], v), k


def test_step_cells_host_bytes(gpu_lib):
    """Bytes moved per mvmm_step_cells call: all 54 rows and the time bins go up;
    47 rows and the time bins come back out of place (volume, loc and centroid
    never change), and in place only the chunks the step changed, stored into
    pinned and pageable arrays alike with the same result as a full copy."""
    import torch
    from hydro_rs_gb300.layout import CELL_ROWS, Cells
    p = ics.kelvin_helmholtz_2d(64, riemann=ics.EXACT)
    n = p.mesh.n_cells
    sims = [G.GpuSim(p, precision=1) for _ in range(3)]
    pinned = (torch.empty(CELL_ROWS * n, dtype=torch.float64, pin_memory=True),
              torch.empty(n, dtype=torch.int8, pin_memory=True))
    host_pinned = Cells.packed(n, pinned[0].numpy(), pinned[1].numpy())
    host_pageable = p.cells.copy()
    for h in (host_pinned, host_pageable):
        for k, v in p.cells.arrays.items():
            h.arrays[k][...] = v
    src = p.cells.copy()
    for _ in range(4):
        sims[0].step_cells(host_pinned)
        sims[1].step_cells(host_pageable)
        out = p.cells.copy()
        sims[2].step_cells(src, out)
        src = out
    for k, v in out.arrays.items():
        for h in (host_pinned, host_pageable):
            x, y = np.ascontiguousarray(h.arrays[k]), np.ascontiguousarray(v)
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), k
    up, full_back = 4 * (54 * n * 8 + n), 4 * (47 * n * 8 + n)
    st = [s.stats() for s in sims]
    assert all(x["host_bytes_in"] - 54 * n * 8 - n == up for x in st)  # the constructor's upload counts too
    assert st[2]["host_bytes_out"] == full_back
    for x in st[:2]:
        # the z rows of this 2D problem and the rows a step resets stay as they were
        assert 0 < x["host_bytes_out"] < 0.8 * full_back, x


@pytest.mark.parametrize("precision", [0, 1])
def test_step_cells_sees_moved_positions(gpu_lib, precision):
    """Positions and centroids changed on the host between mvmm_step_cells calls
    (a fixed mesh): the FP32 face geometry of the faces next to those cells is
    rebuilt, so the step equals, bit for bit, that of a context that builds all
    of its geometry from the same state."""
    p = ics.kelvin_helmholtz_2d(32, riemann=ics.EXACT)
    a = G.GpuSim(p, precision=precision)
    host = p.cells.copy()
    for _ in range(3):
        a.step_cells(host)
    rng = np.random.default_rng(5)
    moved = rng.choice(p.mesh.n_cells, 40, replace=False)
    host.loc[:2, moved] += rng.uniform(-1e-4, 1e-4, (2, moved.size))
    host.centroid[:2, moved] += rng.uniform(-1e-4, 1e-4, (2, moved.size))
    b = G.GpuSim(p, precision=precision)
    b.upload(host)
    b.ti_current, b.ti_old = a.ti_current, a.ti_old
    out_a, out_b = host.copy(), host.copy()
    a.step_cells(host, out_a)
    b.step_cells(host, out_b)
    assert a.ti_current == b.ti_current
    for k, v in out_b.arrays.items():
        x, y = np.ascontiguousarray(out_a.arrays[k]), np.ascontiguousarray(v)
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), k
