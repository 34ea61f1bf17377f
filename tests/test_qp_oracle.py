"""The QP oracle (oracle/qp_oracle.py, a restatement of the reference's
src/qp/qp_solver.cpp) against the reference's own QP unit tests
(tests/unit/test_qp_solver.cpp: analytic answers) and, where the reference was
compiled here, against the reference's QPSolver run on the same QPs
(tests/golden/reference_qp.json)."""
import json
import os

import numpy as np
import pytest

import qp_cases as qc

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def qo():
    import qp_oracle
    return qp_oracle


@pytest.mark.parametrize("name", sorted(qc.REFERENCE_CASES))
def test_reference_known_answers(qo, name):
    H, c, A, b, lb, ub, xs, obj, margin = qc.REFERENCE_CASES[name]
    r = qo.solve(H, c, A, b, lb, ub)
    assert r["status"] == qo.OPTIMAL
    assert np.max(np.abs(r["x"] - np.array(xs))) <= margin
    assert abs(r["objective"] - obj) <= margin
    assert r["primal_residual"] < 1e-6 and r["dual_residual"] < 1e-6 and r["iterations"] > 0


def test_reference_status_cases(qo):
    assert qo.solve(*qc.INFEASIBLE_CASE)["status"] != qo.OPTIMAL
    assert qo.solve(*qc.INDEFINITE_CASE, convexity=qo.NONCONVEX)["status"] == qo.UNSUPPORTED_NONCONVEX
    assert qo.solve(*qc.INDEFINITE_CASE, convexity=qo.CONVEX_UNKNOWN)["status"] == qo.UNSUPPORTED_NONCONVEX
    r = qo.solve(*qc.ITERLIMIT_CASE, max_iter=2)
    assert r["status"] == qo.ITERATION_LIMIT and r["iterations"] == 2


def test_lifting_keeps_the_solution(qo):
    # H = F^T F lifted into w = F x (free, unit Hessian) with F x - w = 0: the
    # lifted QP has a diagonal Hessian and the same x
    H, c, A, b, lb, ub = qc.random_qp(12, 30, 0.2, 5, coupled=True)
    F = qo.lift(H)
    assert np.max(np.abs(F.T @ F - H)) <= 1e-12 * np.max(np.abs(H))
    r = F.shape[0]
    m, n = A.shape
    A2 = np.block([[A, np.zeros((m, r))], [F, -np.eye(r)]])
    H2 = np.diag(np.concatenate([np.zeros(n), np.ones(r)]))
    c2 = np.concatenate([c, np.zeros(r)])
    b2 = np.concatenate([b, np.zeros(r)])
    lb2 = np.concatenate([lb, np.full(r, -qc.INF)])
    ub2 = np.concatenate([ub, np.full(r, qc.INF)])
    r1 = qo.solve(H, c, A, b, lb, ub, feas_tol=1e-9, dual_tol=1e-9, grad_tol=1e-9)
    r2 = qo.solve(H2, c2, A2, b2, lb2, ub2, feas_tol=1e-9, dual_tol=1e-9, grad_tol=1e-9)
    assert r1["status"] == qo.OPTIMAL and r2["status"] == qo.OPTIMAL
    assert np.max(np.abs(r1["x"] - r2["x"][:n])) <= 1e-5
    assert abs(r1["objective"] - r2["objective"]) <= 1e-7 * (1 + abs(r1["objective"]))


def test_oracle_matches_reference_build():
    path = os.path.join(HERE, "golden", "reference_qp.json")
    with open(path) as f:
        cases = json.load(f)["cases"]
    import qp_oracle as qo
    for case in cases:
        H = np.array(case["H"]); A = np.array(case["A"]).reshape(-1, H.shape[0])
        r = qo.solve(H, case["c"], A, case["b"], case["lb"], case["ub"], max_iter=case["max_iter"])
        assert r["status"] == case["status"], case["name"]
        assert r["iterations"] == case["iterations"], case["name"]
        if case["status"] == qo.OPTIMAL:
            assert abs(r["objective"] - case["objective"]) <= 1e-9 * (1 + abs(case["objective"])), case["name"]
            assert np.max(np.abs(r["x"] - np.array(case["x"]))) <= 1e-8, case["name"]
