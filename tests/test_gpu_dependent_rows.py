"""Linearly dependent rows of A (sk_presolve_dependent_rows, sk_options.dependent_rows).

Staircase transportation LPs (family 2's structure: per stage, every arc has +1 in one
supply row and +1 in one demand row, so the supply rows minus the demand rows of a
stage sum to zero) are rank deficient by one row per connected stage. The device
detection (FP64 factor of A A^T, pivots L_kk^2 <= 1e-9) must find exactly m - rank(A)
rows (numpy's SVD rank on small members), keep a full-rank set, flag an inconsistent
b, and the IPM with the rows dropped must reach the same objective and a certificate
on the original LP (y of the dropped rows 0)."""
import numpy as np
import pytest

import sankhya_gb300 as sk_mod

pytestmark = pytest.mark.gpu
TOL = 1e-8


def _dense(lp):
    A = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        A[lp.row_idx[lp.col_ptrs[j]:lp.col_ptrs[j + 1]], j] = lp.vals[lp.col_ptrs[j]:lp.col_ptrs[j + 1]]
    return A


def _from_dense(A, b, c, name):
    cp, ri, va = [0], [], []
    for j in range(A.shape[1]):
        nz = np.nonzero(A[:, j])[0]
        ri.extend(nz.tolist())
        va.extend(A[nz, j].tolist())
        cp.append(len(ri))
    return sk_mod.LP(A.shape[0], A.shape[1], cp, ri, va, b, c, name)


@pytest.mark.parametrize("stages,seed", [(1, 3), (3, 7)])
def test_staircase_rank_matches_numpy(gpu, stages, seed):
    sk = gpu
    lp = sk.staircase(seed, stages, 60, 60, 120, 480)
    A = _dense(lp)
    rank = np.linalg.matrix_rank(A)
    assert rank < lp.m                                   # the structure guarantees a deficiency
    keep, cnt, inc = sk.dependent_rows(lp)
    assert cnt == lp.m - rank, (cnt, lp.m - rank)
    assert inc <= 1e-9
    assert int(keep.sum()) == rank
    assert np.linalg.matrix_rank(A[keep == 1]) == rank   # the kept rows are independent


def test_full_rank_and_duplicated_rows(gpu):
    sk = gpu
    lp = sk.random_lp(150, 400, 0.04, 11)
    keep, cnt, inc = sk.dependent_rows(lp)
    assert cnt == 0 and keep.all()
    A = _dense(lp)
    A2 = np.vstack([A, 2.0 * A[5], A[7] - A[9]])
    b2 = np.concatenate([lp.b, [2.0 * lp.b[5], lp.b[7] - lp.b[9]]])
    dup = _from_dense(A2, b2, lp.c, "dup")
    keep, cnt, inc = sk.dependent_rows(dup)
    assert cnt == 2 and inc <= 1e-9 and int(keep.sum()) == lp.m
    assert np.linalg.matrix_rank(A2[keep == 1]) == lp.m
    # an inconsistent right-hand side: the dependent rows are reported but kept
    b3 = b2.copy()
    b3[-1] += 1.0
    bad = _from_dense(A2, b3, lp.c, "inconsistent")
    keep, cnt, inc = sk.dependent_rows(bad)
    assert cnt == 2 and inc > 1e-6 and keep.all()


@pytest.mark.parametrize("stages,sizes", [(3, (60, 60, 120, 480)), (6, (1000, 1000, 2000, 8000))])
def test_solve_with_dependent_rows_dropped(gpu, oracle, stages, sizes):
    sk = gpu
    lp = sk.staircase(0xC2, stages, *sizes)
    keep, cnt, inc = sk.dependent_rows(lp)
    assert cnt == stages and inc <= 1e-9
    for prec in (sk.PREC_MIXED, sk.PREC_FP64):
        base, *_ = sk.solve(lp, precision=prec)
        info, x, y, s = sk.solve(lp, precision=prec, dependent_rows=1)
        assert base["status"] == 0 and info["status"] == 0, (base, info)
        assert info["dependent_rows"] == stages and base["dependent_rows"] == 0
        assert np.all(y[keep == 0] == 0.0)
        assert abs(info["objective"] - base["objective"]) / (1 + abs(base["objective"])) <= TOL
        meas = oracle.kkt_measures(lp, x, y, s)          # on the original LP, dropped rows included
        assert max(meas["rel_pinf"], meas["rel_dinf"], meas["rel_gap"]) <= TOL, meas


def test_batch_solver_maps_dropped_rows(gpu):
    sk = gpu
    lps = [sk.staircase(5, 2, 60, 60, 120, 480), sk.random_lp(120, 300, 0.05, 3)]
    solver = sk.Solver(lps, precision=sk.PREC_MIXED, dependent_rows=1)
    solver.run()
    i0, x0, y0, s0 = solver.result(0)
    i1, *_ = solver.result(1)
    solver.close()
    assert i0["status"] == 0 and i1["status"] == 0
    assert i0["dependent_rows"] == 2 and i1["dependent_rows"] == 0
    assert len(y0) == lps[0].m
