"""Generates tests/golden/riemann_python.json from the reference's Python solver.

The reference ships a standalone exact Riemann solver with Toro's known
answers (python/riemann_solver.py, self-tests at :1094-1134).  This script
imports it from the reference checkout (argument 1, the directory that holds
python/riemann_solver.py) and records, for Toro's cases and for seeded random
states at gamma 5/3 and 1.4, the state it samples at x/t = 0.  The JSON is
committed; tests compare the CPU oracle (and through it the GPU path) with it.
Run:  python tests/golden/make_riemann_golden.py <reference checkout>
"""
import json
import os
import sys

import numpy as np


def main(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "python"))
    import riemann_solver as R  # noqa: E402  (reference code, read-only)

    cases = []
    toro_p = [  # gamma 1.4, p* known answers (riemann_solver.py:1104-1110)
        (1.0, 0.0, 1.0, 0.125, 0.0, 0.1, 0.30313),
        (1.0, -2.0, 0.4, 1.0, 2.0, 0.4, 0.001894),
        (1.0, 0.0, 1000.0, 1.0, 0.0, 0.01, 460.894),
        (1.0, 0.0, 0.01, 1.0, 0.0, 100.0, 46.095),
        (5.99924, 19.5975, 460.894, 5.99242, -6.19633, 46.0950, 1691.64),
    ]
    s14 = R.RiemannSolver(1.4)
    for c in toro_p:
        u, p = s14.solve_middle_state(*c[:6])
        cases.append({"gamma": 1.4, "state": c[:6], "p_star_known": c[6], "p_star": float(p), "u_star": float(u)})
    toro_s = [  # gamma 5/3, sampled known answers (riemann_solver.py:1113-1131)
        (1.0, 0.0, 1.0, 0.125, 0.0, 0.1, 0.47969, 0.841194, 0.293945, -1),
        (1.0, -2.0, 0.4, 1.0, 2.0, 0.4, 0.00617903, 0.0, 8.32249e-05, -1),
        (1.0, 0.0, 1000.0, 1.0, 0.0, 0.01, 0.615719, 18.2812, 445.626, -1),
        (1.0, 0.0, 0.01, 1.0, 0.0, 100.0, 0.61577, -5.78011, 44.5687, 1),
        (5.99924, 19.5975, 460.894, 5.99242, -6.19633, 46.0950, 12.743, 8.56045, 1841.82, -1),
        (1.0, -1.0, 1.0e-6, 1.0, 1.0, 1.0005e-6, 0.0, 0.0, 0.0, 0),
    ]
    s53 = R.RiemannSolver(5.0 / 3.0)
    samples = []
    for c in toro_s:
        rho, u, p, flag = s53.solve(*c[:6])
        samples.append({"gamma": 5.0 / 3.0, "state": c[:6], "known": c[6:9], "flag_known": c[9],
                        "sample": [float(np.ravel(rho)[0]), float(np.ravel(u)[0]), float(np.ravel(p)[0])]})
    rng = np.random.default_rng(1234)
    for gamma, solver in ((5.0 / 3.0, s53), (1.4, s14)):
        for _ in range(200):
            rl, rr = 10 ** rng.uniform(-1, 1, 2)
            pl, pr = 10 ** rng.uniform(-2, 2, 2)
            ul, ur = rng.uniform(-1.5, 1.5, 2)
            rho, u, p, flag = solver.solve(rl, ul, pl, rr, ur, pr)
            samples.append({"gamma": gamma, "state": [rl, ul, pl, rr, ur, pr],
                            "sample": [float(np.ravel(rho)[0]), float(np.ravel(u)[0]), float(np.ravel(p)[0])],
                            "flag": int(np.ravel(flag)[0])})
    out = {"source": "python/riemann_solver.py of the reference (SWIFT exact solver)", "p_star": cases,
           "samples": samples}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "riemann_python.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst, len(cases), "p* cases,", len(samples), "samples")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_riemann_golden.py <path to the mvmm_hydro source tree>")
    main(sys.argv[1])
