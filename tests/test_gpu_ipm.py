"""Device Mehrotra IPM through the C ABI against the reference's known answers,
the reference's simplex objectives (golden fixtures) and the CPU oracle."""
import ctypes
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-8   # relative objective and relative pinf / dinf / gap


def textbook(sk):
    return sk.LP(2, 4, [0, 2, 4, 5, 6], [0, 1, 0, 1, 0, 1], [1.0, 2.0, 1.0, 3.0, 1.0, 1.0], [4.0, 12.0],
                 [-3.0, -5.0, 0.0, 0.0], "textbook")


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("criteria", [0, 1])
def test_textbook_lp(gpu, precision, criteria):
    # tests/unit/test_mehrotra.cu:29-67
    sk = gpu
    info, x, y, s = sk.solve(textbook(sk), precision=precision, criteria=criteria)
    assert info["status"] == 0 and info["iterations"] > 0
    assert abs(info["objective"] + 20.0) <= 1e-4
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(y)) and x.shape == (4,) and y.shape == (2,)
    if criteria == 1:
        assert info["primal_residual"] < 1e-6 and info["dual_residual"] < 1e-6 and info["duality_gap"] < 1e-6


def test_c_api_fixture_solves_on_gpu(gpu):
    # tests/unit/test_c_api.c:24-67 (objective -2), now through the device IPM
    lib = ctypes.CDLL(gpu.LIB_PATH)
    env, model = ctypes.c_void_p(), ctypes.c_void_p()
    assert lib.sankhya_create_env(ctypes.byref(env)) == 0
    assert lib.sankhya_load_model(env, b"fixture", ctypes.byref(model)) == 0
    assert lib.sankhya_solve(model) == 0
    obj = ctypes.c_double()
    assert lib.sankhya_get_objval(model, ctypes.byref(obj)) == 0
    assert -2.001 < obj.value < -1.999
    lib.sankhya_free_model(model)
    lib.sankhya_free_env(env)


def golden():
    with open(os.path.join(HERE, "golden", "reference_lp_objectives.json")) as f:
        return json.load(f)["cases"]


def make_case(sk, name):
    if name.startswith("family0_"):
        return sk.generate(0, int(name.split("_")[1]))
    m, n, d, seed = {"random_60x150": (60, 150, 0.06, 11), "random_200x450": (200, 450, 0.02, 12),
                     "random_300x700": (300, 700, 0.015, 13)}[name]
    return sk.random_lp(m, n, d, seed)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", golden(), ids=lambda c: c["name"])
def test_matches_reference_simplex_objective(gpu, oracle, case, precision):
    sk = gpu
    lp = make_case(sk, case["name"])
    assert lp.nnz == case["digest"]["nnz"]
    info, x, y, s = sk.solve(lp, precision=precision)
    assert info["status"] == 0, info
    ref = case["ref_objective"]
    assert abs(info["objective"] - ref) / (1 + abs(ref)) <= TOL
    meas = oracle.kkt_measures(lp, x, y, s)     # independent FP64 check of (x, y, s)
    assert meas["rel_pinf"] <= TOL and meas["rel_dinf"] <= TOL and meas["rel_gap"] <= TOL
    assert meas["min_x"] > 0 and meas["min_s"] > 0


def test_reference_criteria_follow_the_oracle(gpu, oracle):
    # Same algorithm, same stopping rule (scaled 2-norms < 1e-6): the device path
    # and the CPU restatement take the same number of iterations (+-1) and agree
    # on the objective to the accuracy that rule delivers.
    sk = gpu
    lp = sk.generate(0, 0)
    info, x, y, s = sk.solve(lp, precision=0, criteria=1)
    r, xo, yo, so = oracle.ipm_solve(lp, criteria=1)
    assert info["status"] == 0 and r["status"] == 0
    assert abs(info["iterations"] - r["iterations"]) <= 1
    assert abs(info["objective"] - r["objective"]) / (1 + abs(r["objective"])) <= 1e-6


def test_relative_criteria_iterations_match_oracle(gpu, oracle):
    sk = gpu
    lp = sk.random_lp(200, 450, 0.02, 12)
    info, x, y, s = sk.solve(lp, precision=0)
    r, *_ = oracle.ipm_solve(lp)
    assert abs(info["iterations"] - r["iterations"]) <= 1
    assert abs(info["objective"] - r["objective"]) / (1 + abs(r["objective"])) <= TOL


def test_batch_equals_single_solves(gpu):
    sk = gpu
    lps = [sk.random_lp(80 + 30 * i, 200 + 50 * i, 0.04, 100 + i) for i in range(5)]
    solver = sk.Solver(lps, precision=1)
    solver.run()
    for i, lp in enumerate(lps):
        info_b, xb, yb, sb = solver.result(i)
        info_s, xs, ys, ss = sk.solve(lp, precision=1)
        assert info_b["status"] == 0 and info_s["status"] == 0
        assert abs(info_b["objective"] - info_s["objective"]) / (1 + abs(info_s["objective"])) <= TOL
    solver.close()


def test_solver_rerun_is_repeatable(gpu):
    sk = gpu
    solver = sk.Solver([sk.generate(0, 2)], precision=1)
    solver.run()
    a = solver.result(0)
    solver.run()
    b = solver.result(0)
    assert a[0]["status"] == 0 and b[0]["status"] == 0
    assert a[0]["iterations"] == b[0]["iterations"]
    np.testing.assert_array_equal(a[1], b[1])     # deterministic reductions and assembly
    solver.close()


def test_ill_conditioned_fallback_case(gpu):
    # tests/unit/test_phase1.cpp:483-530 ("Test 11"): 1e-7 entries; the reference
    # either solves it or reports IterationLimit. Here it must end with a valid answer.
    sk = gpu
    lp = sk.LP(2, 2, [0, 2, 4], [0, 1, 0, 1], [1e-7, 1.0, 1.0, 1e-7], [1.0, 1.0], [1.0, 1.0])
    info, x, y, s = sk.solve(lp, precision=0)
    if info["status"] == 0:
        assert abs(info["objective"] - 2.0 / (1.0 + 1e-7)) <= 1e-6
    else:
        assert info["status"] == 3


def test_non_finite_input_rejected(gpu):
    sk = gpu
    lp = sk.random_lp(20, 40, 0.2, 3)
    c = lp.c.copy()
    c[3] = np.nan
    bad = sk.LP(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, c)
    with pytest.raises(RuntimeError, match="code 1"):
        sk.solve(bad)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", golden(), ids=lambda c: c["name"])
def test_mehrotra_start_reaches_reference_objective(gpu, oracle, case, precision):
    # Mehrotra's heuristic start (SK_START_MEHROTRA) changes the path, not the answer.
    sk = gpu
    lp = make_case(sk, case["name"])
    info, x, y, s = sk.solve(lp, precision=precision, start=1)
    assert info["status"] == 0, info
    ref = case["ref_objective"]
    assert abs(info["objective"] - ref) / (1 + abs(ref)) <= TOL
    meas = oracle.kkt_measures(lp, x, y, s)
    assert meas["rel_pinf"] <= TOL and meas["rel_dinf"] <= TOL and meas["rel_gap"] <= TOL
    o, _, _, _ = oracle.ipm_solve(lp, start=1)
    assert o["status"] == 0 and abs(info["iterations"] - o["iterations"]) <= 2


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("seed", [3, 4])
def test_bounded_lp_on_device(gpu, seed, precision):
    # Variable bounds through sk_ipm_solve_bounded (host standard form, device solve,
    # mapped back) against an independent solver (SciPy's HiGHS).
    pytest.importorskip("scipy.optimize")
    from bounded_cases import bounded_case, highs_objective
    sk = gpu
    lp, lb, ub, A = bounded_case(sk, seed)
    ref = highs_objective(lp, lb, ub, A)
    info, x, y, s = sk.solve_bounded(lp, lb, ub, precision=precision)
    assert info["status"] == 0
    assert abs(info["objective"] - ref) / (1 + abs(ref)) <= TOL
    assert np.max(np.abs(A @ x - lp.b)) <= 1e-7 * (1 + np.max(np.abs(lp.b)))
    assert np.all(x >= lb - 1e-7) and np.all(x <= ub + 1e-7)
    np.testing.assert_allclose(s, lp.c - A.T @ y, atol=1e-9)


def test_cli_honours_mps_bounds(gpu, tmp_path):
    # An MPS file with LO / UP / MI / FR bounds through the CLI with --bounds.
    pytest.importorskip("scipy.optimize")
    import subprocess
    from bounded_cases import bounded_case, highs_objective, write_mps
    sk = gpu
    lp, lb, ub, A = bounded_case(sk, 5)
    ref = highs_objective(lp, lb, ub, A)
    path = tmp_path / "bounded.mps"
    write_mps(str(path), lp, lb, ub)
    cli = os.path.join(os.path.dirname(sk.LIB_PATH), "sankhya_cli")
    out = subprocess.run([cli, str(path), "--bounds"], capture_output=True, text=True, check=True).stdout
    res = json.loads(out)
    assert res["status"] == "Optimal"
    assert abs(res["objective"] - ref) / (1 + abs(ref)) <= TOL
