"""Device convex QP (sk_qp_solve, the reference's qp::QPSolver interface) against
the reference's own QP solver: its unit-test problems with their analytic answers
(tests/unit/test_qp_solver.cpp) and the golden runs of the reference's compiled
solver (tests/golden/reference_qp.json). A diagonal H follows the reference's
iteration step for step, so the iteration counts agree exactly; a coupled H is
solved through its lifting (w = F x, H = F^T F) and must reach the same optimum."""
import json
import os

import numpy as np
import pytest

import qp_cases as qc

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def golden():
    with open(os.path.join(HERE, "golden", "reference_qp.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("name", sorted(qc.REFERENCE_CASES))
def test_reference_known_answers_on_device(gpu, name):
    H, c, A, b, lb, ub, xs, obj, margin = qc.REFERENCE_CASES[name]
    st, info, x, y, z = gpu.qp_solve(H, c, A, b, lb, ub)
    assert st == 0, gpu.QP_STATUS[st]
    assert np.max(np.abs(x - np.array(xs))) <= margin
    assert abs(info["objective"] - obj) <= margin
    assert info["primal_residual"] < 1e-6 and info["dual_residual"] < 1e-6 and info["iterations"] > 0


def test_status_contract_on_device(gpu):
    st, *_ = gpu.qp_solve(*qc.INFEASIBLE_CASE)
    assert st in (1, 3, 4)                          # Infeasible / IterationLimit / NumericalFailure
    st, *_ = gpu.qp_solve(*qc.INDEFINITE_CASE, convexity=gpu.QP_NONCONVEX)
    assert st == 5
    st, *_ = gpu.qp_solve(*qc.INDEFINITE_CASE, convexity=gpu.QP_CONVEXITY_UNKNOWN)
    assert st == 5
    st, info, *_ = gpu.qp_solve(*qc.ITERLIMIT_CASE, max_iterations=2)
    assert st == 3 and info["iterations"] == 2


@pytest.mark.parametrize("case", golden(), ids=lambda c: c["name"])
def test_matches_reference_qp_solver(gpu, case):
    H = np.array(case["H"])
    n = H.shape[0]
    A = np.array(case["A"]).reshape(-1, n)
    st, info, x, y, z = gpu.qp_solve(H, case["c"], A, case["b"], case["lb"], case["ub"],
                                     max_iterations=case["max_iter"])
    diagonal = not np.any(H - np.diag(np.diag(H)))
    if case["status"] in (0, 3):
        assert st == case["status"]
        if diagonal:      # the reference's iteration itself, step for step
            assert info["iterations"] == case["iterations"]
    if case["status"] == 0:
        ref = case["objective"]
        assert abs(info["objective"] - ref) <= 1e-5 * (1 + abs(ref))
        # both stop at the reference's 1e-6 tolerances: x agrees to that order
        assert np.max(np.abs(x - np.array(case["x"]))) <= 1e-3
        if diagonal:
            assert np.max(np.abs(x - np.array(case["x"]))) <= 1e-9 * (1 + np.max(np.abs(x)))
        assert np.max(np.abs(A @ x - np.array(case["b"]))) <= 1e-6
    elif case["status"] != 3:
        assert st != 0


def test_tighter_tolerances_converge_to_the_optimum(gpu):
    # a separable QP solved to 1e-10 agrees with a dense KKT solve of its active set
    H, c, A, b, lb, ub = qc.random_qp(30, 80, 0.08, 42, coupled=False, bounded=False)
    st, info, x, y, z = gpu.qp_solve(H, c, A, b, lb, ub, feasibility_tol=1e-10, dual_tol=1e-10, grad_tol=1e-12)
    assert st == 0
    # KKT: H x + c - A^T y - z = 0, A x = b, x >= 0, z >= 0, x z ~ 0
    assert np.max(np.abs(H @ x + c - A.T @ y - z)) <= 1e-9
    assert np.max(np.abs(A @ x - b)) <= 1e-9
    assert np.min(x) >= -1e-12 and np.min(z) >= -1e-12
    assert np.max(np.abs(x * z)) <= 1e-9
