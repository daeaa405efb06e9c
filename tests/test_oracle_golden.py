"""The CPU oracle pinned against the reference's own known answers.

Every case below is a unit test of the reference (file:line cited), restated:
if the oracle reproduces them, the restatement follows the reference's
arithmetic; the GPU parity tests then compare the CUDA path with the oracle.
float_cmp's default ``assert_approx_eq!`` margin (float-cmp 0.9) is
``|a-b| <= f64::EPSILON`` or at most 4 ulps apart; tests with an explicit
epsilon keep it.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GAMMA = 5.0 / 3.0
HERE = os.path.dirname(os.path.abspath(__file__))


def approx_eq(a, b, ulps=4, eps=None):
    if eps is not None:
        return abs(a - b) <= eps
    if a == b or abs(a - b) <= np.finfo(np.float64).eps:
        return True
    return abs(a - b) <= ulps * np.spacing(max(abs(a), abs(b)))


def prim(rho, vx, p, vy=0.0, vz=0.0):
    return np.array([rho, vx, vy, vz, p], dtype=np.float64)


def boost(s, v):
    s = s.copy()
    if s[0] > 0:
        s[1:4] += v
    return s


def flux(kind, l, r, iv, n=(1.0, 0.0, 0.0), gamma=GAMMA):
    out, err = O.riemann_flux(kind, gamma, l.reshape(5, 1), r.reshape(5, 1), np.reshape(iv, (3, 1)),
                              np.reshape(n, (3, 1)))
    assert err == 0
    return out[:, 0]


def sample(kind, l, r, n=(1.0, 0.0, 0.0), gamma=GAMMA):
    out, err = O.riemann_sample(kind, gamma, l.reshape(5, 1), r.reshape(5, 1), np.reshape(n, (3, 1)))
    assert err == 0
    return out[:, 0]


EXACT_HALF = [  # riemann_solver/exact.rs:344-398
    ((0.75, 0.6, 0.8), (0.55, -0.25, 0.5), (0.8927393244785966, 0.35966250129769556, 1.0709476357371466)),
    ((0.75, 0.3, 0.8), (0.55, -0.75, 0.5), (0.9114320476995261, -0.03895103710637815, 1.201228148376388)),
    ((0.75, 0.1, 0.8), (0.55, 0.5, 0.5), (0.5562398903431287, 0.4792910646431622, 0.4861363537732538)),
    ((1.75, -0.1, 0.75), (0.55, 1.5, 0.5), (0.65432665196683, 0.6088656910463873, 0.14554217677392042)),
    ((0.75, -0.5, 0.8), (0.55, -0.1, 0.5), (0.5407985848180775, -0.1207089353568378, 0.4861363537732538)),
    ((1.75, -1.5, 0.75), (1.55, 0.1, 0.5), (0.5687181105004402, -0.5249266813300747, 0.09402548983542296)),
]


@pytest.mark.parametrize("case", range(6))
def test_exact_half_state(case):
    (rl, vl, pl), (rr, vr, pr), ref = EXACT_HALF[case]
    h = sample(O.lib and 1, prim(rl, vl, pl), prim(rr, vr, pr))
    assert approx_eq(h[0], ref[0]) and approx_eq(h[1], ref[1]) and approx_eq(h[4], ref[2]), (h, ref)


@pytest.mark.parametrize("kind", [0, 1])
def test_symmetry(kind):
    """exact.rs:312-342 and hllc.rs:139-166."""
    iv = np.array([-0.3, 0.0, 0.0])
    left = prim(1.0, 0.0, 1.0)
    right = prim(1.0, -0.6, 1.0)
    right_rev = prim(1.0, 0.6, 1.0)
    f = flux(kind, boost(left, -iv), boost(right, -iv), iv)
    fr = flux(kind, boost(right_rev, iv), boost(left, iv), -iv)
    assert approx_eq(f[0], -fr[0]) and approx_eq(f[1], fr[1]) and approx_eq(f[4], -fr[4])
    assert approx_eq(f[2], fr[2]) and approx_eq(f[3], fr[3])


def test_vacuum_symmetry():
    """vacuum.rs:151-183 (through the exact solver's vacuum branch)."""
    iv = np.array([0.15, 0.0, 0.0])
    left = prim(1.0, 0.3, 0.5)
    left_rev = prim(1.0, -0.3, 0.5)
    vac = np.zeros(5)
    f = flux(1, boost(left, -iv), vac, iv)
    fr = flux(1, vac, boost(left_rev, iv), -iv)
    assert approx_eq(f[0], -fr[0]) and approx_eq(f[1], fr[1]) and approx_eq(f[4], -fr[4])


def test_vacuum_half_state():
    """vacuum.rs:185-220."""
    h = sample(1, boost(prim(1.0, 0.3, 0.5), np.array([-0.15, 0, 0])), np.zeros(5))
    ref = (0.4950623323204316, 0.7221531968814576, 0.15490656018956153)
    assert approx_eq(h[0], ref[0]) and approx_eq(h[1], ref[1]) and approx_eq(h[4], ref[2])


# vacuum.rs:222-260 asserts the same relation for a left state next to vacuum,
# but there x/t = 0 (lab) and x/t = 0.3 (the face frame's origin) both lie
# inside the rarefaction fan at different positions, so the two sides sample
# different states and the relation does not hold; that case is not restated.
# The fan sampler is pinned by vacuum.rs:185-220 (test_vacuum_half_state).
@pytest.mark.parametrize("kind,iv,left,right", [
    (1, -0.1, (1.5, 0.2, 1.2), (0.7, -0.4, 0.1)),    # exact.rs:400-438
    (2, -0.17, (1.5, 0.2, 1.2), (0.7, -0.4, 0.1)),   # pvrs.rs:64-101
])
def test_galilean_invariance(kind, iv, left, right):
    L = prim(*left)
    R = np.zeros(5) if right is None else prim(*right)
    ivv = np.array([iv, 0.0, 0.0])
    w = sample(kind, L, R)
    roe = w[4] * (1.0 / (GAMMA - 1.0)) + 0.5 * w[0] * (w[1] ** 2 + w[2] ** 2 + w[3] ** 2)
    lab = flux(kind, L, R, np.zeros(3)) - np.array(
        [w[0] * iv, w[0] * w[1] * iv, w[0] * w[2] * iv, w[0] * w[3] * iv, roe * iv])
    face = flux(kind, boost(L, -ivv), boost(R, -ivv) if right is not None else R, ivv)
    assert approx_eq(lab[0], face[0]) and approx_eq(lab[1], face[1]) and approx_eq(lab[4], face[4]), (lab, face)


def test_hllc_close_to_exact():
    """hllc.rs:168-195: HLLC within 5e-2 of the exact flux."""
    iv = np.array([0.15, 0.0, 0.0])
    L = boost(prim(1.0, 0.2, 0.5), -iv)
    R = boost(prim(0.5, 0.1, 0.1), -iv)
    a = flux(0, L, R, iv)
    b = flux(1, L, R, iv)
    for q in (0, 1, 4):
        assert approx_eq(a[q], b[q], eps=5e-2)


def test_swift_regression_does_not_fail():
    """exact.rs:440-460: a near-vacuum state from SWIFT must not panic."""
    out, err = O.exact_star(GAMMA, 2.1669723793e-9, 1.4698121886e-10, 3.3622390032e-01, 1.7172516742e-09,
                            1.1778487907e-10, 3.3810544014e-01, -1.5249514580e+00, 4.9803251028e-01)
    assert err == 0 and np.all(np.isfinite(out))


def test_conversions_round_trip():
    """physical_quantities.rs:318-339."""
    p = prim(0.75, 0.4, 0.8)
    c = O.cons_from_primitives(GAMMA, p, 0.1)
    p2 = O.prim_from_conserved(GAMMA, c, 0.1)
    for q in range(5):
        assert approx_eq(p[q], p2[q]), (q, p, p2)


def test_timeline_round_trip():
    """timeline.rs:149-155 plus the bin / integer-time helpers."""
    assert O.get_time_bin(O.get_integer_timestep(8)) == 8
    for b in range(1, 57):
        assert O.get_time_bin(O.get_integer_timestep(b)) == b
    assert O.get_integer_timestep(0) == 0 and O.get_integer_timestep(56) == 1 << 57
    assert O.get_max_active_bin(0) == 56
    assert O.get_max_active_bin(1 << 10) == 9
    assert O.get_max_active_bin(3 << 10) == 9


def _python_golden():
    with open(os.path.join(HERE, "golden", "riemann_python.json")) as f:
        return json.load(f)


def test_python_reference_p_star():
    """Toro's p* known answers from the reference's Python solver (1e-4, riemann_solver.py:1094-1110)."""
    g = _python_golden()
    for c in g["p_star"]:
        rl, ul, pl, rr, ur, pr = c["state"]
        gamma = c["gamma"]
        al = np.sqrt(gamma * pl / rl)
        ar = np.sqrt(gamma * pr / rr)
        out, err = O.exact_star(gamma, rl, pl, al, rr, pr, ar, ul, ur)
        assert err == 0
        assert abs(out[3] - c["p_star_known"]) < 1e-4 * abs(out[3] + c["p_star_known"])
        assert abs(out[3] - c["p_star"]) <= 1e-5 * abs(c["p_star"])


def test_python_reference_samples():
    """Sampled x/t=0 states: the oracle vs the reference's Python exact solver.

    In vacuum-generating states the Python script's fan velocity uses
    2/(gamma-1) * u (python/riemann_solver.py, sample_vacuum_generation) where
    the Rust reference's sample_rarefaction_fan (riemann_solver.rs:120-134)
    uses (gamma-1)/2 * u, Toro's (4.56); the Rust code is the reference for
    this path, so for those states only density and pressure are compared.
    """
    g = _python_golden()
    worst = 0.0
    n_vacgen = 0
    for c in g["samples"]:
        rl, ul, pl, rr, ur, pr = c["state"]
        gamma = c["gamma"]
        h = sample(1, prim(rl, ul, pl), prim(rr, ur, pr), gamma=gamma)
        ref = c["sample"]
        al, ar = np.sqrt(gamma * pl / rl), np.sqrt(gamma * pr / rr)
        vacgen = 2.0 / (gamma - 1.0) * (al + ar) <= ur - ul
        n_vacgen += vacgen
        pairs = ((h[0], ref[0]), (h[4], ref[2])) if vacgen else ((h[0], ref[0]), (h[1], ref[1]), (h[4], ref[2]))
        for a, b in pairs:
            scale = max(abs(b), 1e-12)
            worst = max(worst, abs(a - b) / scale if abs(b) > 1e-10 else abs(a - b))
        if "known" in c:
            for a, b in ((h[0], c["known"][0]), (h[1], c["known"][1]), (h[4], c["known"][2])):
                assert a == b or abs(a - b) < 1e-4 * abs(a + b)
    assert worst < 1e-5, worst
    assert n_vacgen <= 8  # a handful of the 406 seeded states
