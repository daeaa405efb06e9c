"""Host logic: the integer timeline, the engine loop, host-made failures."""
import numpy as np
import pytest

from hydro_rs_gb300 import ics
from oracle import oracle as O

MAX = 1 << 57


def py_get_integer_timestep(b):
    return 0 if b <= 0 else 1 << (b + 1)


def py_get_time_bin(dti):
    lz = 64 if dti == 0 else 64 - dti.bit_length()
    v = (64 - lz - 2) & 0xFFFFFFFF
    v &= 0xFF
    return v - 256 if v >= 128 else v


def py_get_integer_time_end(ti, b):
    dti = py_get_integer_timestep(b)
    if dti == 0:
        return 0
    m = ti % dti
    return ti if m == 0 else ti - m + dti


def py_make_integer_timestep(dt, old_bin, min_ngb_bin, ti_current, tbi):
    """timeline.rs:103-139 restated independently (Python ints)."""
    x = dt * tbi
    new_dti = 0 if not x > 0 else (2 ** 64 - 1 if x >= 2.0 ** 64 else int(x))
    new_bin = min(py_get_time_bin(new_dti), min_ngb_bin + 2)
    new_dti = py_get_integer_timestep(new_bin)
    cur = py_get_integer_timestep(old_bin)
    if old_bin > 0:
        new_dti = min(new_dti, 2 * cur)
    tl = MAX
    while new_dti < tl:
        tl //= 2
    new_dti = tl
    if new_dti > cur:
        te = py_get_integer_time_end(ti_current, old_bin)
        if (MAX - te) % new_dti != 0:
            new_dti = cur
    return new_dti


def test_make_integer_timestep_matches_restatement():
    rng = np.random.default_rng(3)
    tb = 0.2 / MAX
    for _ in range(3000):
        dt = 10 ** rng.uniform(-9, -1)
        old_bin = int(rng.integers(0, 50))
        ti = int(rng.integers(0, 1 << 20)) << int(rng.integers(2, 36))
        ti = min(ti, MAX)
        got, err = O.make_integer_timestep(dt, old_bin, 56, ti, 1.0 / tb)
        assert got == py_make_integer_timestep(dt, old_bin, 56, ti, 1.0 / tb)
        assert (err != 0) == (got == 0)
    # saturating cast of an infinite timestep (vacuum cell): bin capped at 58
    got, _ = O.make_integer_timestep(float("inf"), 0, 56, 0, 1.0 / tb)
    assert got == py_make_integer_timestep(float("inf"), 0, 56, 0, 1.0 / tb) == MAX


def test_engine_loop_runs_to_t_end():
    """Engine::run: steps at ti = 0, ..., 2^57 inclusive; the first has dt = 0."""
    p = ics.sod_1d(100, t_end=0.05)
    s = O.OracleSim(p)
    s.step()
    st = s.state()
    assert np.array_equal(st.cons, p.cells.cons)  # zero-flux first step
    s.run()
    assert s.finished and s.ti_old == MAX
    assert s.error() == 0


def test_newton_cap_is_reported_not_fatal():
    """A host-made failure: a one-iteration Newton cap turns the reference's
    panic (exact.rs:272-274) into an error bit; the run still returns."""
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.EXACT)
    p.params.max_newton_iter = 1
    s = O.OracleSim(p)
    s.run(max_steps=4)
    assert s.error() & 1


def test_negative_energy_is_reported():
    """convert_conserved_to_primitive asserts E >= 0 (part.rs:221-224)."""
    p = ics.sod_1d(32)
    s = O.OracleSim(p)
    s.step()
    c = s.state()
    c.cons[4][5] = -1.0
    s2 = O.OracleSim(ics.Problem(p.name, p.params, p.mesh, c))
    s2.convert(np.ones(32, np.uint8))
    assert s2.error() & (1 << 3)


def test_max_active_bin_closed_form():
    """The kernels' get_max_active_bin without the bit loop (max_active_bin_bits):
    lowest set bit p >= 2 gives p - 1, else the loop's wrapped shift gives 63 / 64."""
    def closed(ti):
        if ti == 0:
            return 56
        hi = ti & ~3
        if hi:
            return (hi & -hi).bit_length() - 1 - 1
        return 63 if ti & 1 else 64
    rng = np.random.default_rng(0)
    cases = [0, 1, 2, 3, 4, 5, 6, 8, 12, 1 << 57, (1 << 57) - 4, (1 << 63), (1 << 64) - 1]
    cases += [int(x) << int(s) for x, s in zip(rng.integers(1, 1 << 20, 300), rng.integers(0, 44, 300))]
    for ti in cases:
        assert closed(ti) == O.get_max_active_bin(ti), ti


def test_cells_pointer_struct_follows_the_arrays():
    """Cells.cview keeps its C struct of pointers while the same arrays are in
    place, and rebuilds it when an array is replaced or n changes."""
    from hydro_rs_gb300.layout import CELL_ROWS, Cells
    n = 64
    c = Cells.packed(n, np.zeros(CELL_ROWS * n), np.zeros(n, dtype=np.int8))
    a = c.cview()
    assert c.cview() is a
    assert a.prim == c.prim.ctypes.data and a.timebin == c.timebin.ctypes.data
    c.arrays["prim"] = np.ones((5, n))
    b = c.cview()
    assert b is not a and b.prim == c.prim.ctypes.data and b.cons == a.cons
    c.arrays["timebin"] = np.zeros(n, dtype=np.int8)
    assert c.cview().timebin == c.timebin.ctypes.data
    d = c.copy()
    assert d.cview().prim == d.prim.ctypes.data != c.prim.ctypes.data
