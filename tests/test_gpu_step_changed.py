"""mvmm_step_cells_changed: host-resident state that crosses the link only where
it changed.  Each call must leave the host arrays bit-identical to the state
device-resident steps reach, while storing only the cells the step rewrote."""
import numpy as np
import pytest

from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics
from hydro_rs_gb300.layout import CELL_ROWS, Cells

pytestmark = pytest.mark.gpu

FULL_BYTES_PER_CELL = 47 * 8 + 1  # every row but volume, loc and centroid, and the time bin
EXTRAP_BYTES_PER_CELL = 5 * 8  # the extrapolation rows alone


def _warp_stores(x, n):
    """x as whole warps (32 cells) of full rows plus whole warps of extrapolation rows."""
    for a in range(n // 32 + 1):
        rest = x - 32 * FULL_BYTES_PER_CELL * a
        if rest >= 0 and rest % (32 * EXTRAP_BYTES_PER_CELL) == 0:
            return True
    return False


def _same_bits(x, y):  # signed zeros and NaN payloads included
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    return x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8))


def _assert_same(a: Cells, b: Cells):
    for k, v in b.arrays.items():
        assert _same_bits(a.arrays[k], v), k


def _pinned_cells(n):
    import torch
    block = torch.empty(CELL_ROWS * n, dtype=torch.float64, pin_memory=True)
    tb = torch.empty(n, dtype=torch.int8, pin_memory=True)
    return Cells.packed(n, block.numpy(), tb.numpy()), (block, tb)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("memory", ["pageable", "pinned"])
def test_changed_steps_match_resident_steps(gpu_lib, precision, memory):
    """A hierarchical point blast: every call's host arrays equal the state of
    device-resident steps, and the bytes written back are those of the cells
    the step rewrote (the jittered lattice's density varies, so every cell's
    extrapolation moves each step; the other rows only where cells are active
    or next to an active face), well short of all rows of all cells."""
    p = ics.point_blast_3d(16, riemann=ics.HLLC)
    n = p.mesh.n_cells
    a = G.GpuSim(p, precision=precision)
    b = G.GpuSim(p, precision=precision)
    if memory == "pinned":
        host, keep = _pinned_cells(n)
    else:
        host = Cells.zeros(n)
    for k, v in p.cells.arrays.items():
        host.arrays[k][...] = v
    stored = []
    for s in range(12):
        a.step()
        stored.append(b.step_cells_changed(host, None if s == 0 else []))
        assert a.ti_current == b.ti_current and a.active_faces == b.active_faces
        _assert_same(host, a.state())
    assert all(_warp_stores(x, n) for x in stored), stored
    assert 0 < min(stored[1:]) and max(stored[1:]) < 0.5 * n * FULL_BYTES_PER_CELL, stored


@pytest.mark.parametrize("precision", [0, 1])
def test_changed_cells_are_read(gpu_lib, precision):
    """Cells the host rewrites between calls (pressure and momentum, and for
    some the position and centroid) are read back: the step equals, bit for
    bit, mvmm_step_cells on the same arrays, which uploads every cell."""
    p = ics.point_blast_3d(16, riemann=ics.HLLC)
    n = p.mesh.n_cells
    a = G.GpuSim(p, precision=precision)
    host = p.cells.copy()
    a.step_cells_changed(host)
    for _ in range(3):
        a.step_cells_changed(host, [])
    rng = np.random.default_rng(11)
    edit = rng.choice(n, 60, replace=False)
    host.cons[4, edit] *= 1.5
    host.prim[4, edit] *= 1.5
    kick = edit[:20]  # a small velocity, its kinetic energy added to the energy
    host.cons[1, kick] += 1e-4 * host.cons[0, kick]
    host.cons[4, kick] += 0.5e-8 * host.cons[0, kick]
    host.prim[1, kick] += 1e-4
    moved = edit[:10]
    host.loc[:, moved] += rng.uniform(-1e-4, 1e-4, (3, moved.size))
    host.centroid[:, moved] += rng.uniform(-1e-4, 1e-4, (3, moved.size))
    b = G.GpuSim(p, precision=precision)
    b.upload(host)
    b.ti_current, b.ti_old = a.ti_current, a.ti_old
    out_b = host.copy()
    b.step_cells(host.copy(), out_b)
    a.step_cells_changed(host, np.concatenate([edit, edit[:5]]))  # repeated indices are harmless
    assert a.ti_current == b.ti_current
    _assert_same(host, out_b)


def test_changed_rejects_bad_input(gpu_lib):
    p = ics.point_blast_3d(8, riemann=ics.HLLC)
    n = p.mesh.n_cells
    a = G.GpuSim(p, precision=0)
    host = p.cells.copy()
    a.step_cells_changed(host)
    for bad in ([n], [-1], [0, n + 5]):
        with pytest.raises(G.MvmmError) as e:
            a.step_cells_changed(host, bad)
        assert e.value.code == -1  # MVMM_E_INVALID
