"""Pins the CPU oracle against the reference: the golden vectors of the
reference's own tests and, where the reference's CPU code is built here
(oracle/_ref), its outputs on the same inputs."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def csr(m, rp, ci, vals=None):
    rp = np.array(rp, dtype=np.int32)
    ci = np.array(ci, dtype=np.int32)
    v = np.ones(len(ci)) if vals is None else np.array(vals, dtype=np.float64)
    return rp, ci, v


# tests/unit/test_ipm_symbolic.cpp:10-78 (star graph)
def test_symbolic_star_graph(oracle):
    rp, ci, _ = csr(5, [0, 4, 5, 6, 7, 8], [0, 1, 2, 3, 0, 1, 2, 3])
    P = oracle.min_degree(5, 5, rp, ci)
    assert P.tolist() == [1, 2, 3, 0, 4]
    Pinv, parent, Lrp, Lci = oracle.symbolic(5, 5, rp, ci, P)
    assert all(Pinv[P[i]] == i for i in range(5))
    assert Lrp[5] == 4
    assert parent.tolist() == [3, 3, 3, 4, -1]


# tests/unit/test_ipm_symbolic.cpp:80-151 (4-cycle + isolated row)
def test_symbolic_cycle_fill(oracle):
    rp, ci, _ = csr(5, [0, 2, 4, 6, 8, 9], [0, 3, 0, 1, 1, 2, 2, 3, 4])
    P = oracle.min_degree(5, 5, rp, ci)
    assert P.tolist() == [4, 0, 1, 2, 3]
    Pinv, parent, Lrp, Lci = oracle.symbolic(5, 5, rp, ci, P)
    assert Lrp.tolist() == [0, 0, 0, 1, 2, 5]
    assert Lci.tolist() == [1, 2, 1, 2, 3]
    assert parent.tolist() == [-1, 2, 3, 4, -1]


KKT_A = ([0, 3, 5, 7], [0, 3, 4, 1, 3, 2, 4], [2.0, 1.0, 1.0, 2.0, 1.0, 2.0, 1.0])


# tests/unit/test_gpu_kkt.cu:14-123: ordering {1,0,2}, solution (1,2,3)
def test_kkt_golden_solution(oracle):
    rp, ci, v = csr(3, *KKT_A)
    P = oracle.min_degree(3, 5, rp, ci)
    assert P.tolist() == [1, 0, 2]
    ok, dy = oracle.kkt_solve(3, 5, rp, ci, v, np.ones(5), np.array([11.0, 11.0, 16.0]), P=P, tol=1e-10)
    assert ok
    np.testing.assert_allclose(dy, [1.0, 2.0, 3.0], atol=1e-6)
    M = np.array([[6, 1, 1], [1, 5, 0], [1, 0, 5]], dtype=float)
    assert np.linalg.norm(M @ dy - [11, 11, 16]) < 1e-6


# tests/unit/test_gpu_kkt.cu:138-195: x1e4 right-hand side, relative physical residual
def test_kkt_golden_relative_contract(oracle):
    rp, ci, v = csr(3, *KKT_A)
    P = oracle.min_degree(3, 5, rp, ci)
    scale = 1e4
    ok, dy = oracle.kkt_solve(3, 5, rp, ci, v, np.ones(5), scale * np.array([11.0, 11.0, 16.0]), P=P, tol=1e-10,
                              rel=True)
    assert ok
    np.testing.assert_allclose(dy, scale * np.array([1.0, 2.0, 3.0]), rtol=1e-8)
    M = np.array([[6, 1, 1], [1, 5, 0], [1, 0, 5]], dtype=float)
    assert np.max(np.abs(M @ dy - scale * np.array([11, 11, 16]))) / (16 * scale) < 1e-8


def textbook_lp(sk):
    # tests/unit/test_mehrotra.cu:29-67: min -3x1-5x2, x1+x2+x3=4, 2x1+3x2+x4=12 -> -20
    cp = [0, 2, 4, 5, 6]
    ri = [0, 1, 0, 1, 0, 1]
    va = [1.0, 2.0, 1.0, 3.0, 1.0, 1.0]
    return sk.LP(2, 4, cp, ri, va, [4.0, 12.0], [-3.0, -5.0, 0.0, 0.0], "textbook")


def test_oracle_textbook_lp(sk, oracle):
    lp = textbook_lp(sk)
    for crit in (0, 1):
        r, x, y, s = oracle.ipm_solve(lp, criteria=crit)
        assert r["status"] == 0
        assert r["iterations"] > 0
        assert abs(r["objective"] + 20.0) <= 1e-4
        assert np.all(np.isfinite(x)) and np.all(np.isfinite(y))
    r, x, y, s = oracle.ipm_solve(lp, criteria=1)
    assert r["primal_residual"] < 1e-6 and r["dual_residual"] < 1e-6 and r["duality_gap"] < 1e-6


def test_oracle_c_api_fixture(sk, oracle):
    # tests/unit/test_c_api.c:61-67 (fixture objective -2)
    lp = sk.LP(2, 4, [0, 1, 2, 3, 4], [0, 1, 0, 1], [1.0, 1.0, 1.0, 1.0], [1.0, 1.0], [-1.0, -1.0, 0.0, 0.0])
    r, x, y, s = oracle.ipm_solve(lp)
    assert r["status"] == 0 and abs(r["objective"] + 2.0) < 1e-7


def golden_cases():
    with open(os.path.join(HERE, "golden", "reference_lp_objectives.json")) as f:
        return json.load(f)["cases"]


def make_case(sk, name):
    if name.startswith("family0_"):
        return sk.generate(0, int(name.split("_")[1]))
    dims, seeds = {"random_60x150": (60, 150, 0.06, 11), "random_200x450": (200, 450, 0.02, 12),
                   "random_300x700": (300, 700, 0.015, 13)}, None
    m, n, d, seed = dims[name]
    return sk.random_lp(m, n, d, seed)


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_oracle_matches_reference_simplex(sk, oracle, case):
    lp = make_case(sk, case["name"])
    dg = case["digest"]
    assert (lp.m, lp.n, lp.nnz) == (dg["m"], dg["n"], dg["nnz"])
    assert abs(float(np.sum(lp.vals)) - dg["sum_vals"]) <= 1e-9 * (1 + abs(dg["sum_vals"]))
    r, x, y, s = oracle.ipm_solve(lp)
    assert case["ref_status"] == 0
    assert r["status"] == 0
    ref = case["ref_objective"]
    assert abs(r["objective"] - ref) / (1 + abs(ref)) <= 1e-8
    assert max(r["rel_pinf"], r["rel_dinf"], r["rel_gap"]) <= 1e-8


def test_oracle_symbolic_matches_reference_build(sk, oracle):
    if not oracle.have_reference():
        pytest.skip("oracle/_ref not built here (reference sources absent)")
    for (m, n, d, seed) in [(25, 50, 0.1, 1), (90, 200, 0.04, 2), (250, 500, 0.015, 3)]:
        lp = sk.random_lp(m, n, d, seed)
        rp, ci, _ = lp.csr()
        P_ref = oracle.ref_min_degree(m, n, rp, ci)
        assert np.array_equal(oracle.min_degree(m, n, rp, ci), P_ref)
        a = oracle.symbolic(m, n, rp, ci, P_ref)
        b = oracle.ref_symbolic(m, n, rp, ci, P_ref)
        for u, v in zip(a, b):
            assert np.array_equal(u, v)


def test_oracle_objective_matches_reference_build(sk, oracle):
    if not oracle.have_reference():
        pytest.skip("oracle/_ref not built here (reference sources absent)")
    lp = sk.random_lp(80, 190, 0.05, 77)
    st, obj, _ = oracle.ref_simplex(lp)
    r, x, y, s = oracle.ipm_solve(lp)
    assert st == 0 and r["status"] == 0
    assert abs(r["objective"] - obj) / (1 + abs(obj)) <= 1e-8


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c["name"])
def test_oracle_mehrotra_start_matches_reference_simplex(sk, oracle, case):
    lp = make_case(sk, case["name"])
    r, x, y, s = oracle.ipm_solve(lp, start=1)
    r0, _, _, _ = oracle.ipm_solve(lp)
    assert r["status"] == 0
    ref = case["ref_objective"]
    assert abs(r["objective"] - ref) / (1 + abs(ref)) <= 1e-8
    assert max(r["rel_pinf"], r["rel_dinf"], r["rel_gap"]) <= 1e-8
    assert r["iterations"] <= r0["iterations"] + 2
