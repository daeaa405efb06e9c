"""The allocation-free entry point against the context-based one.

mvmm_flux_update_noalloc serves callers that cannot call cudaMalloc (a host that
owns the device memory budget, code inside its own graph capture, code that
must avoid cudaMalloc's implicit synchronisation).  Here the test plays such a
caller: it owns every device array (allocated with torch), passes them through
the C ABI, and checks the updated state against mvmm_compute_fluxes +
mvmm_apply_fluxes + mvmm_convert_conserved_to_primitive on a context, on two
calls in a row (the second call reuses the static scratch array the first one
left behind), for the three solvers it supports and every wall boundary, with
the same error bits.  Tolerance: the same 1e-14 as the per-stage parity test.
"""
import ctypes

import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from hydro_rs_gb300.layout import CELL_FIELDS, CCells, CMesh
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

MAX_FACES = 65536


def _lib():
    L = G.load_library()
    fn = L.mvmm_flux_update_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 6
    return fn


def _device_copy(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def _setup(problem, torch):
    """Caller-owned device copies of the mesh and cell state."""
    m = problem.mesh
    keep = {}
    dm = CMesh()
    dm.n_cells, dm.n_faces = m.n_cells, m.n_faces
    for name in ("left", "right", "area", "normal", "centroid", "shift", "csr_off", "csr_face"):
        t = _device_copy(torch, getattr(m, name))
        keep["m_" + name] = t
        setattr(dm, name, t.data_ptr())
    return dm, keep


def _cells_to_device(cells, torch, keep):
    dc = CCells()
    dc.n = cells.n
    for name, _ in CELL_FIELDS:
        t = _device_copy(torch, cells.arrays[name])
        keep["c_" + name] = t
        setattr(dc, name, t.data_ptr())
    t = _device_copy(torch, cells.timebin)
    keep["c_timebin"] = t
    dc.timebin = t.data_ptr()
    return dc


def _params(problem):
    return G.make_params(problem.params, precision=0)


def _state_from_device(keep, like):
    out = like.copy()
    for name, _ in CELL_FIELDS:
        out.arrays[name][...] = keep["c_" + name].cpu().numpy()
    return out


CASES = {
    "sod_reflective_hllc": lambda: ics.sod_1d(400),
    "sod_open_pvrs": lambda: ics.sod_1d(400, riemann=ics.PVRS, boundary=ics.OPEN),
    "sod_vacuum_exact": lambda: ics.sod_1d(400, riemann=ics.EXACT, boundary=ics.VACUUM),
    "sod_vacuum_hllc": lambda: ics.sod_1d(400, riemann=ics.HLLC, boundary=ics.VACUUM),
    "kh_periodic_exact": lambda: ics.kelvin_helmholtz_2d(32, riemann=ics.EXACT),
    "kh_periodic_pvrs": lambda: ics.kelvin_helmholtz_2d(32, riemann=ics.PVRS),
}


def _noalloc_call(fn, prm, dm, dc, d_active, d_err, torch):
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(ctypes.byref(prm), ctypes.byref(dm), ctypes.byref(dc), d_active.data_ptr(),
            None if d_err is None else d_err.data_ptr(), ctypes.c_void_p(stream))
    assert rc == 0, (rc, G.load_library().mvmm_last_error())
    torch.cuda.synchronize()


@pytest.mark.parametrize("which", list(CASES))
def test_noalloc_matches_context_path(gpu_lib, which):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    p = CASES[which]()
    # a state with gradients, extrapolations and pending fluxes
    orc = O.OracleSim(p)
    for _ in range(3):
        orc.step()
    start = orc.state()
    p2 = ics.Problem(p.name, p.params, p.mesh, start)
    rng = np.random.default_rng(7)
    active = (rng.random(p.mesh.n_cells) < 0.8).astype(np.uint8)
    active[0] = active[-1] = 1  # the wall faces of the 1D tubes are exchanged

    # existing entry points on a context
    ctx = G.GpuSim(p2)
    ref = []
    for _ in range(2):
        fl, _ = ctx.compute_fluxes(active)
        ctx.apply_fluxes(fl, active)
        ctx.convert(active)
        ref.append(ctx.state())
    ref_bits = ctx.error_bits()
    ctx.close()

    # the allocation-free entry point on caller-owned device arrays
    fn = _lib()
    dm, keep = _setup(p2, torch)
    dc = _cells_to_device(start, torch, keep)
    d_active = _device_copy(torch, active)
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    prm = _params(p2)
    for call in range(2):
        _noalloc_call(fn, prm, dm, dc, d_active, d_err, torch)
        got = _state_from_device(keep, start)
        for f in ("cons", "prim", "facc", "max_signal_velocity", "max_a_over_r"):
            a, b = got.arrays[f], ref[call].arrays[f]
            if a.ndim == 2:
                for k in range(a.shape[0]):
                    assert rel_err(a[k], b[k]) <= 1e-14, (which, call, f, k)
            else:
                assert rel_err(a, b) <= 1e-14, (which, call, f)
    assert int(d_err.item()) == ref_bits == 0


def test_noalloc_error_bits_match_context(gpu_lib):
    """A cell of zero volume: cons -> prim divides by it (part.rs:249-260), and
    both entry points report the same bits (MVMM_ERR_NONFINITE among them)."""
    torch = pytest.importorskip("torch")
    p = ics.sod_1d(64)
    cells = p.cells.copy()
    cells.volume[10] = 0.0
    p2 = ics.Problem(p.name, p.params, p.mesh, cells)
    active = np.ones(p.mesh.n_cells, dtype=np.uint8)
    ctx = G.GpuSim(p2)
    fl, _ = ctx.compute_fluxes(active)
    ctx.apply_fluxes(fl, active)
    with pytest.raises(G.MvmmError) as ei:
        ctx.convert(active)
    ref_bits = ei.value.bits
    ctx.close()
    assert ref_bits & (1 << 4)  # MVMM_ERR_NONFINITE
    fn = _lib()
    dm, keep = _setup(p2, torch)
    dc = _cells_to_device(cells, torch, keep)
    d_active = _device_copy(torch, active)
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _noalloc_call(fn, _params(p2), dm, dc, d_active, d_err, torch)
    assert int(d_err.item()) == ref_bits


def test_noalloc_reports_bad_indices(gpu_lib):
    """Mesh indices outside their arrays are skipped by the kernels and
    reported as MVMM_ERR_BOUNDS (the arrays are on the device, so the host does
    not validate them as mvmm_ctx_create does)."""
    torch = pytest.importorskip("torch")
    p = ics.sod_1d(64)
    fn = _lib()
    dm, keep = _setup(p, torch)
    n = p.mesh.n_cells
    keep["m_right"][5] = n + 3          # a face whose right cell does not exist
    keep["m_csr_face"][7] = p.mesh.n_faces + 11  # a CSR entry naming no face
    torch.cuda.synchronize()
    dc = _cells_to_device(p.cells, torch, keep)
    d_active = _device_copy(torch, np.ones(n, dtype=np.uint8))
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _noalloc_call(fn, _params(p), dm, dc, d_active, d_err, torch)
    assert int(d_err.item()) & (1 << 7)  # MVMM_ERR_BOUNDS


def test_noalloc_unsupported_solver(gpu_lib):
    p = ics.sod_1d(16, riemann=ics.TSRS)
    fn = _lib()
    dm, dc = CMesh(), CCells()
    dm.n_cells, dm.n_faces, dc.n = 16, 17, 16
    rc = fn(ctypes.byref(_params(p)), ctypes.byref(dm), ctypes.byref(dc), ctypes.c_void_p(1), None, None)
    assert rc == -5  # MVMM_E_UNSUPPORTED, nothing launched
    assert b"HLLC" in G.load_library().mvmm_last_error()


def test_noalloc_rejects_oversized_mesh(gpu_lib):
    fn = _lib()
    p = ics.sod_1d(16)
    prm = _params(p)
    dm = CMesh()
    dm.n_cells = MAX_FACES + 8
    dm.n_faces = MAX_FACES + 1
    dc = CCells()
    dc.n = dm.n_cells
    rc = fn(ctypes.byref(prm), ctypes.byref(dm), ctypes.byref(dc), ctypes.c_void_p(1), None, None)
    assert rc == -1  # MVMM_E_INVALID, nothing launched
    assert b"MVMM_NOALLOC_MAX_FACES" in G.load_library().mvmm_last_error()
