"""Presolve (Ruiz equilibration of a model, sk_presolve_ruiz) on the host:
the reference's own unit-test assertions (tests/unit/test_scaling.cpp), bit-exact
parity with the CPU restatement (oracle/presolve_oracle.py) and with the
reference's compiled presolve::apply_ruiz_scaling through the committed fixture
tests/golden/reference_presolve.json (and live when oracle/_ref is built)."""
import hashlib
import json
import os

import numpy as np
import pytest

import presolve_oracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = ("vals", "b", "c", "lb", "ub", "row_scale", "col_scale")


@pytest.fixture(scope="module")
def cases(sk):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import presolve_cases
    return presolve_cases.cases(sk, large=True)


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "reference_presolve.json")) as f:
        return {c["name"]: c for c in json.load(f)["cases"]}


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def _maxabs_rows_cols(m, n, cp, ri, v):
    r = np.zeros(m)
    np.maximum.at(r, ri, np.abs(v))
    col_of = np.repeat(np.arange(n), np.diff(cp))
    c = np.zeros(n)
    np.maximum.at(c, col_of, np.abs(v))
    return r, c


def test_reference_unit_test_conditioning_and_reversibility(sk, cases):
    # tests/unit/test_scaling.cpp:17-104
    name, lp, lb, ub, it, iters = cases[0]
    assert name == "scaling_conditioning"
    out = sk.presolve_ruiz(lp, lb=lb, ub=ub, integer=it, max_iter=iters)
    before = np.abs(lp.vals)
    after = np.abs(out["vals"])
    assert after.max() / after[after > 0].min() < before.max() / before[before > 0].min()
    r, c = _maxabs_rows_cols(lp.m, lp.n, lp.col_ptrs, lp.row_idx, out["vals"])
    assert np.all(np.abs(c - 1.0) < 1e-2) and np.all(np.abs(r - 1.0) < 1e-2)
    assert abs(out["b"][0] - out["row_scale"][0] * 1e3) < 1e-9
    assert abs(out["b"][1] - out["row_scale"][1] * 1e3) < 1e-9
    assert abs(out["lb"][0] - 10.0 / out["col_scale"][0]) < 1e-9
    assert abs(out["c"][0] - 1.0 * out["col_scale"][0]) < 1e-9
    assert out["ub"][1] == np.inf


def test_reference_unit_test_integer_column_unchanged(sk, cases):
    # tests/unit/test_scaling.cpp:106-124
    name, lp, lb, ub, it, iters = cases[1]
    assert name == "scaling_integer"
    out = sk.presolve_ruiz(lp, lb=lb, ub=ub, integer=it, max_iter=iters)
    assert out["col_scale"][0] == 1.0
    assert out["col_scale"][1] != 1.0


def test_product_matches_oracle_bit_for_bit(sk, cases):
    for name, lp, lb, ub, it, iters in cases:
        got = sk.presolve_ruiz(lp, lb=lb, ub=ub, integer=it, max_iter=iters)
        want = po.ruiz(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, lp.c, lb, ub, it, iters)
        for k in KEYS:
            assert np.array_equal(got[k], want[k]), (name, k)


def test_product_matches_reference_fixture_bit_for_bit(sk, cases, golden):
    assert set(golden) == {c[0] for c in cases}
    for name, lp, lb, ub, it, iters in cases:
        g = golden[name]
        assert (g["m"], g["n"], g["nnz"], g["max_iterations"]) == (lp.m, lp.n, lp.nnz, iters)
        got = sk.presolve_ruiz(lp, lb=lb, ub=ub, integer=it, max_iter=iters)
        for k in KEYS:
            assert _digest(got[k]) == g["digest"][k], (name, k)
        if "arrays" in g:
            for k in KEYS:
                want = np.array([float(x) for x in g["arrays"][k]])
                assert np.array_equal(got[k], want), (name, k)


def test_product_matches_live_reference(sk, oracle, cases):
    if not oracle.have_reference():
        pytest.skip("oracle/_ref not built here (the reference sources are absent)")
    for name, lp, lb, ub, it, iters in cases:
        got = sk.presolve_ruiz(lp, lb=lb, ub=ub, integer=it, max_iter=iters)
        ref = oracle.ref_ruiz(lp, lb, ub, it, iters)
        for k in KEYS:
            assert np.array_equal(got[k], ref[k]), (name, k)


def test_scales_accumulate_and_edge_cases(sk):
    lp = sk.random_lp(40, 90, 0.08, 3)
    one = sk.presolve_ruiz(lp, max_iter=2)
    # a second call continues from the first call's scaled model and scale vectors
    lp2 = sk.LP(lp.m, lp.n, lp.col_ptrs, lp.row_idx, one["vals"], lp.b, lp.c)
    two = sk.presolve_ruiz(lp2, max_iter=2, row_scale=one["row_scale"], col_scale=one["col_scale"])
    want = po.ruiz(lp.m, lp.n, lp.col_ptrs, lp.row_idx, one["vals"], lp.b, lp.c, max_iter=2,
                   row_scale=one["row_scale"], col_scale=one["col_scale"])
    for k in ("vals", "row_scale", "col_scale", "b", "c"):
        assert np.array_equal(two[k], want[k]), k
    # zero iterations: values untouched, rhs / objective scaled by the given vectors (ones)
    z = sk.presolve_ruiz(lp, max_iter=0)
    assert np.array_equal(z["vals"], lp.vals) and np.array_equal(z["b"], lp.b)
    # an empty column and an all-zero row keep factor 1
    e = sk.LP(3, 3, [0, 2, 2, 3], [0, 2, 2], [4.0, 0.5, 9.0], [1.0, 2.0, 3.0], [1.0, 1.0, 1.0])
    out = sk.presolve_ruiz(e)
    assert out["col_scale"][1] == 1.0 and out["row_scale"][1] == 1.0
    want = po.ruiz(3, 3, e.col_ptrs, e.row_idx, e.vals, e.b, e.c)
    for k in ("vals", "row_scale", "col_scale"):
        assert np.array_equal(out[k], want[k]), k


def test_invalid_input_rejected(sk):
    lp = sk.random_lp(10, 20, 0.2, 1)
    bad = sk.LP(lp.m, lp.n, lp.col_ptrs, np.where(lp.row_idx == 0, 99, lp.row_idx), lp.vals, lp.b, lp.c)
    with pytest.raises(RuntimeError):
        sk.presolve_ruiz(bad)
    with pytest.raises(RuntimeError):
        sk.presolve_ruiz(lp, max_iter=-1)


def test_cpp_api_source_compatible(sk, cases, tmp_path):
    """The C++ entry point presolve::apply_ruiz_scaling, called as the reference's
    own unit test calls it (Model built with add_variable / add_constraint /
    finalize), gives the same bits as the C ABI on the same two models."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    root = os.path.dirname(HERE)
    pkg = os.path.join(root, "soverign-gpu-accelerator-_gb300")
    exe = str(tmp_path / "presolve_api")
    src = [os.path.join(HERE, "cpp", "presolve_api.cpp"), os.path.join(pkg, "csrc", "presolve", "scaling.cpp"),
           os.path.join(pkg, "csrc", "core", "problem.cpp"), os.path.join(pkg, "csrc", "core", "sparse_matrix.cpp")]
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(root, "include"), "-I" + os.path.join(pkg, "csrc"),
                    "-o", exe] + src, check=True, capture_output=True)
    res = json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    for key, (name, lp, lb, ub, it, iters) in zip(("conditioning", "integer"), cases[:2]):
        want = sk.presolve_ruiz(lp, lb=lb, ub=ub, integer=it, max_iter=iters)
        got = res[key]
        assert np.array_equal(np.array(got["vals"]), want["vals"]), key
        assert np.array_equal(np.array(got["rhs"]), want["b"]), key
        assert np.array_equal(np.array(got["obj"]), want["c"]), key
        assert np.array_equal(np.array(got["row_scale"]), want["row_scale"]), key
        assert np.array_equal(np.array(got["col_scale"]), want["col_scale"]), key
        assert got["lb0"] == want["lb"][0], key
