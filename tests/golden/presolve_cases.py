"""Models of the presolve (Ruiz scaling) parity cases, shared by the fixture
generator (make_presolve_golden.py) and tests/test_presolve.py.

Each case is (name, LP, lb, ub, integer flags, max_iterations). The first two are
the models of the reference's own unit tests (tests/unit/test_scaling.cpp:17-33
and :108-118); the others are seeded LPs with mixed bounds and integer columns."""
import numpy as np


def _lp(sk, m, n, cols, b, c):
    """CSC LP from per-column (row, value) lists."""
    cp, ri, va = [0], [], []
    for col in cols:
        for r, v in sorted(col):
            ri.append(r)
            va.append(v)
        cp.append(len(ri))
    return sk.LP(m, n, cp, ri, va, b, c)


def _mixed_bounds(n, seed):
    rng = np.random.default_rng(seed)
    lb = rng.uniform(-5.0, 5.0, n)
    ub = lb + rng.uniform(0.5, 10.0, n)
    lb[rng.random(n) < 0.2] = -np.inf
    ub[rng.random(n) < 0.3] = np.inf
    integer = (np.arange(n) % 7 == 3).astype(np.uint8)
    return lb, ub, integer


def cases(sk, large=False):
    out = []
    # test_scaling.cpp:17-33: x0 in [10, 20] (c 1), x1 >= 0 (c 2); rows (1e6, 1e-4) and (1e-4, 1e6), rhs 1e3
    lp = _lp(sk, 2, 2, [[(0, 1e6), (1, 1e-4)], [(0, 1e-4), (1, 1e6)]], [1e3, 1e3], [1.0, 2.0])
    out.append(("scaling_conditioning", lp, np.array([10.0, 0.0]), np.array([20.0, np.inf]),
                np.zeros(2, np.uint8), 20))
    # test_scaling.cpp:108-118: binary x0 (c 1), continuous x1 (c 2); row (100, 100), rhs 50
    lp = _lp(sk, 1, 2, [[(0, 100.0)], [(0, 100.0)]], [50.0], [1.0, 2.0])
    out.append(("scaling_integer", lp, np.array([0.0, 0.0]), np.array([1.0, np.inf]),
                np.array([1, 0], np.uint8), 10))
    lp = sk.random_lp(60, 150, 0.06, 11)
    lb, ub, it = _mixed_bounds(lp.n, 5)
    out.append(("random_60x150", lp, lb, ub, it, 10))
    lp = sk.generate(0, 0)
    lb, ub, it = _mixed_bounds(lp.n, 6)
    out.append(("family0_0", lp, lb, ub, it, 10))
    lp = sk.random_lp(300, 700, 0.015, 13)
    out.append(("random_300x700_3passes", lp, np.zeros(lp.n), np.full(lp.n, np.inf), np.zeros(lp.n, np.uint8), 3))
    if large:
        lp = sk.generate(1, 0)
        out.append(("family1_0", lp, np.zeros(lp.n), np.full(lp.n, np.inf), np.zeros(lp.n, np.uint8), 10))
    return out
