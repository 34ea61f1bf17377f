"""Host-side logic without a GPU: generators, MPS input, C ABI surface."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("include/sankhya/sk_ipm.h", "include/sankhya/sankhya.h"):
        txt = open(os.path.join(ROOT, h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for mt in re.finditer(r"^\s*(?:const\s+)?[a-zA-Z_][\w\s\*]*?\b(s(?:k|ankhya)_\w+)\s*\(", txt, flags=re.M):
            names.add(mt.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(sk):
    lib = ctypes.CDLL(sk.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_generators_are_deterministic_and_consistent(sk):
    a = sk.generate(0, 0)
    b = sk.generate(0, 0)
    assert np.array_equal(a.vals, b.vals) and np.array_equal(a.b, b.b)
    assert (a.m, a.n) == (500, 1000)
    counts = np.diff(a.col_ptrs)
    assert counts.min() >= 2
    assert np.all(np.bincount(a.row_idx, minlength=a.m) >= 1)
    assert np.all(np.abs(a.vals) >= 0.1) and np.all(np.abs(a.vals) <= 10)
    c = sk.generate(0, 1)
    assert not np.array_equal(a.vals, c.vals)


def test_block_angular_family_shape(sk):
    lp = sk.generate(1, 0)
    assert (lp.m, lp.n) == (22000, 48000)
    assert abs(lp.nnz / lp.n - 6.0) < 0.01
    # column j of block k touches only block k rows and linking rows
    j = 5 * 1200 + 7
    rows = lp.row_idx[lp.col_ptrs[j]:lp.col_ptrs[j + 1]]
    assert np.sum((rows >= 5 * 500) & (rows < 6 * 500)) == 5 and np.sum(rows >= 20000) == 1


def test_batch_family_sizes(sk):
    ms = []
    for i in range(6):
        lp = sk.generate(3, i)
        assert 200 <= lp.m <= 5000
        assert 2 * lp.m <= lp.n <= 3 * lp.m + 1
        ms.append(lp.m)
    assert len(set(ms)) > 1


def test_mps_reader_reference_fixture(sk, tmp_path):
    # tests/unit/test_mps_reader.cpp:10-67 fixture
    p = tmp_path / "t.mps"
    p.write_text("""NAME          TESTPROB
ROWS
 N  COST
 L  LIM1
 G  LIM2
 E  MYEQN
COLUMNS
    XONE      COST                 1   LIM1                 1
    XONE      LIM2                 1
    YTWO      COST                 4   LIM1                 1
    YTWO      MYEQN               -1
    ZTHREE    COST                 9   LIM2                 1
    ZTHREE    MYEQN                1
RHS
    RHS1      LIM1                 5   LIM2                10
    RHS1      MYEQN                7
BOUNDS
 UP BND1      XONE                 4
 LO BND1      YTWO                -1
 UP BND1      YTWO                 1
ENDATA
""")
    lp = sk.read_mps(str(p))
    assert (lp.m, lp.n) == (3, 5)
    assert lp.c.tolist() == [1.0, 4.0, 9.0, 0.0, 0.0]
    assert lp.b.tolist() == [5.0, 10.0, 7.0]
    dense = np.zeros((3, 5))
    for j in range(5):
        for q in range(lp.col_ptrs[j], lp.col_ptrs[j + 1]):
            dense[lp.row_idx[q], j] = lp.vals[q]
    assert dense.tolist() == [[1, 1, 0, 1, 0], [1, 0, 1, 0, -1], [0, -1, 1, 0, 0]]


def test_mps_reader_rejects_ranges(sk, tmp_path):
    p = tmp_path / "r.mps"
    p.write_text("NAME X\nROWS\n N C\n E R\nCOLUMNS\n    X C 1 R 1\nRANGES\n    S R 1\nENDATA\n")
    with pytest.raises(RuntimeError):
        sk.read_mps(str(p))


def test_c_api_fixture_load_without_gpu(sk):
    lib = ctypes.CDLL(sk.LIB_PATH)
    env = ctypes.c_void_p()
    model = ctypes.c_void_p()
    assert lib.sankhya_create_env(ctypes.byref(env)) == 0
    assert lib.sankhya_load_model(env, b"fixture", ctypes.byref(model)) == 0
    assert lib.sankhya_load_model(env, None, ctypes.byref(model)) == 1
    assert lib.sankhya_load_model(env, b"/nonexistent.mps", ctypes.byref(ctypes.c_void_p())) == 2
    lib.sankhya_free_model(model)
    lib.sankhya_free_env(env)


def test_invalid_lp_arrays_rejected_before_device(sk):
    lp = sk.random_lp(10, 20, 0.2, 1)
    bad = sk.LP(lp.m, lp.n, lp.col_ptrs.copy(), lp.row_idx.copy(), lp.vals.copy(), lp.b, lp.c)
    bad.col_ptrs[0] = 1
    with pytest.raises(RuntimeError):
        sk.solve(bad)


def _cuda_visible():
    try:
        rt = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def test_spmv_plan_rejects_bad_arguments_before_the_device(sk):
    L = sk.lib()
    out = ctypes.c_void_p()
    vp = ctypes.c_void_p
    # negative sizes, missing row pointers, missing output handle: SK_ERR_INVALID (1)
    assert L.sk_spmv_plan_create(-1, 5, 0, vp(8), None, None, None, ctypes.byref(out)) == 1
    assert L.sk_spmv_plan_create(5, 5, 3, None, vp(8), vp(8), None, ctypes.byref(out)) == 1
    assert L.sk_spmv_plan_create(5, 5, 3, vp(8), vp(8), vp(8), None, None) == 1
    assert L.sk_spmv_plan_execute(None, vp(8), 1.0, 0.0, vp(8), None) == 1
    assert L.sk_spmv_plan_set_group(None, 4, 0) == 1
    # a well-formed empty plan (no rows: no device memory is read): SK_ERR_NO_DEVICE (4) without a
    # device, no fallback; with a device it is created and destroyed
    rc = L.sk_spmv_plan_create(0, 5, 0, vp(8), None, None, None, ctypes.byref(out))
    if _cuda_visible():
        assert rc == 0
        L.sk_spmv_plan_destroy(out)
    else:
        assert rc == 4


def test_presolve_and_spmv_plan_symbols_declared(sk):
    names = declared_symbols()
    for n in ("sk_presolve_ruiz", "sk_spmv_plan_create", "sk_spmv_plan_execute", "sk_spmv_plan_info",
              "sk_spmv_plan_set_group", "sk_spmv_plan_destroy"):
        assert n in names


def test_dependent_rows_entry_checks_arguments_and_needs_a_device(sk):
    assert "sk_presolve_dependent_rows" in declared_symbols()
    lp = sk.random_lp(30, 60, 0.1, 5)
    keep = np.ones(lp.m, dtype=np.int32)
    cnt, inc = ctypes.c_int(0), ctypes.c_double(0.0)
    L = sk.lib()
    # bad column pointers: SK_ERR_INVALID (1) before any device work
    bad_cp = lp.col_ptrs.copy()
    bad_cp[0] = 1
    assert L.sk_presolve_dependent_rows(lp.m, lp.n, bad_cp, lp.row_idx, lp.vals, lp.b, keep, ctypes.byref(cnt),
                                        ctypes.byref(inc)) == 1
    assert L.sk_presolve_dependent_rows(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, keep, None, None) == 1
    rc = L.sk_presolve_dependent_rows(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, keep, ctypes.byref(cnt),
                                      ctypes.byref(inc))
    if _cuda_visible():
        assert rc == 0 and cnt.value == 0
    else:
        assert rc == 4            # SK_ERR_NO_DEVICE: no CPU fallback


def test_dependent_rows_option_is_validated(sk):
    lp = sk.random_lp(30, 60, 0.1, 5)
    with pytest.raises(RuntimeError, match="dependent_rows"):
        sk.solve(lp, dependent_rows=2)
