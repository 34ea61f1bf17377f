"""Variable bounds (the reference's IPM ignores them): the host standard form
(sk_lp_standard_form) solved by the CPU oracle against an independent solver
(SciPy's HiGHS) on seeded bounded LPs."""
import numpy as np
import pytest

from bounded_cases import bounded_case, highs_objective


@pytest.mark.parametrize("seed", [3, 4, 5])
def test_standard_form_matches_independent_solver(sk, oracle, seed):
    pytest.importorskip("scipy.optimize")
    lp, lb, ub, A = bounded_case(sk, seed)
    ref = highs_objective(lp, lb, ub, A)
    slp, off = sk.standard_form(lp, lb, ub)
    nbox = int(np.sum(np.isfinite(lb) & np.isfinite(ub)))
    nfree = int(np.sum(~np.isfinite(lb) & ~np.isfinite(ub)))
    assert (slp.m, slp.n) == (lp.m + nbox, lp.n + nfree + nbox)
    r, xs, ys, ss = oracle.ipm_solve(slp)
    assert r["status"] == 0
    assert abs(r["objective"] + off - ref) / (1 + abs(ref)) <= 1e-8
    # map x' back and check the original constraints and bounds
    x = np.where(np.isfinite(lb), lb + xs[:lp.n], np.where(np.isfinite(ub), ub - xs[:lp.n], xs[:lp.n]))
    free = np.flatnonzero(~np.isfinite(lb) & ~np.isfinite(ub))
    x[free] -= xs[lp.n:lp.n + len(free)]
    assert np.max(np.abs(A @ x - lp.b)) <= 1e-7 * (1 + np.max(np.abs(lp.b)))
    assert np.all(x >= lb - 1e-7) and np.all(x <= ub + 1e-7)
    assert abs(lp.c @ x - ref) / (1 + abs(ref)) <= 1e-8


def test_standard_form_rejects_crossed_bounds(sk):
    lp = sk.random_lp(10, 30, 0.2, 1)
    lb = np.zeros(lp.n)
    ub = np.ones(lp.n)
    ub[3] = -1.0
    with pytest.raises(RuntimeError, match="bounds"):
        sk.standard_form(lp, lb, ub)
