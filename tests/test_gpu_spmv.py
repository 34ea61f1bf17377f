"""Autotuned SpMV plans (sk_spmv_plan_*) against an FP64 numpy reference: every
lane-group width, the autotuner's choice, reuse of the kept width, and the edge
cases of the reference's SpMV call sites (empty rows, one very long row, no rows).
The reference computes these products with cusparseSpMV (FP64, CSR, int32
indices; src/ipm/mehrotra_device.cu:508-530); there is no bit pattern to match,
so results are compared at 1e-12 relative to the row's absolute sum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ref(rp, ci, v, x):
    out = np.zeros(len(rp) - 1)
    scale = np.zeros(len(rp) - 1)
    for i in range(len(rp) - 1):
        a, b = rp[i], rp[i + 1]
        out[i] = np.dot(v[a:b], x[ci[a:b]])
        scale[i] = np.dot(np.abs(v[a:b]), np.abs(x[ci[a:b]]))
    return out, scale


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


def _check(sk, rows, cols, rp, ci, v, seed=0, widths=None):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(cols)
    y0 = rng.standard_normal(rows)
    d_rp, d_ci, d_v, d_x = _dev(rp), _dev(ci), _dev(v), _dev(x)
    plan = sk.SpmvPlan(rows, cols, len(v), d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr())
    info = plan.info()
    assert info["group"] in sk.SPMV_GROUPS and info["heuristic_group"] in sk.SPMV_GROUPS
    ref, scale = _ref(rp, ci, v, x)
    want = 2.0 * ref - 0.5 * y0
    runs = [(None, None)] + [(g, w) for g in (widths or sk.SPMV_GROUPS) for w in (False, True)]
    by_group = {}
    for g, w in runs:
        if g is not None:
            plan.set_group(g, windowed=w)
        d_y = _dev(y0.copy())
        plan.execute(d_x.data_ptr(), d_y.data_ptr(), alpha=2.0, beta=-0.5)
        torch.cuda.synchronize()
        got = d_y.cpu().numpy()
        err = np.abs(got - want) / (1.0 + 2.0 * scale + 0.5 * np.abs(y0))
        assert err.max() <= 1e-12, (g, w, err.max())
        if g is not None:
            # shared-memory windows change where x is read from, not the order of the additions
            if g in by_group:
                assert np.array_equal(by_group[g], got), g
            by_group[g] = got
    plan.close()
    return info


def _random_csr(rows, cols, per_row, seed):
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, 2 * per_row, size=rows)
    rp = np.zeros(rows + 1, dtype=np.int32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate([np.sort(rng.choice(cols, size=k, replace=False)) for k in lens]).astype(np.int32)
    return rp, ci, rng.uniform(-10.0, 10.0, size=len(ci))


def test_plan_matches_numpy_for_every_width(gpu):
    sk = gpu
    # a shape no other test or solver uses in this process, so the plan times it
    rp, ci, v = _random_csr(1777, 2333, 9, 21)
    info = _check(sk, 1777, 2333, rp, ci, v, seed=1)
    assert all(t > 0 for t in info["ms_per_group"].values())             # every width was timed
    assert all(t > 0 for t in info["ms_windowed_per_group"].values())    # plain and windowed
    lp = sk.generate(0, 3)
    rp, ci, v = lp.csr()
    _check(sk, lp.m, lp.n, rp, ci, v, seed=1)
    # A^T (CSR of A^T = CSC of A)
    _check(sk, lp.n, lp.m, lp.col_ptrs, lp.row_idx, lp.vals, seed=2)


def test_kept_width_is_reused_for_the_same_shape(gpu):
    sk = gpu
    rp, ci, v = _random_csr(1999, 2999, 6, 22)
    d_rp, d_ci, d_v = _dev(rp), _dev(ci), _dev(v)
    p1 = sk.SpmvPlan(1999, 2999, len(v), d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr())
    p2 = sk.SpmvPlan(1999, 2999, len(v), d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr())
    i1, i2 = p1.info(), p2.info()
    assert i1["group"] == i2["group"] and i1["windowed"] == i2["windowed"]
    assert any(t > 0.0 for t in i1["ms_per_group"].values())    # the first plan timed ...
    assert all(t == 0.0 for t in i2["ms_per_group"].values())   # ... the second did not
    p1.close()
    p2.close()


def test_ragged_and_empty_rows(gpu):
    sk = gpu
    rng = np.random.default_rng(7)
    rows, cols = 3000, 5000
    lens = rng.integers(0, 4, size=rows)
    lens[::7] = 0                       # empty rows
    lens[1234] = 4000                   # one very long row
    rp = np.zeros(rows + 1, dtype=np.int32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate([np.sort(rng.choice(cols, size=k, replace=False)) for k in lens]).astype(np.int32)
    v = rng.uniform(0.1, 10.0, size=len(ci)) * rng.choice([-1.0, 1.0], size=len(ci))
    _check(sk, rows, cols, rp, ci, v, seed=3)


def test_wide_and_narrow_rows_mixed(gpu):
    # rows spanning more columns than one shared-memory window (24576) gather from
    # global memory; the rows around them use windows
    sk = gpu
    rng = np.random.default_rng(11)
    rows, cols = 4000, 70000
    rp, ci = [0], []
    for r in range(rows):
        if r % 97 == 5:                                   # wide row over the whole range
            c = np.sort(rng.choice(cols, size=300, replace=False))
        elif r % 13 == 0:
            c = np.zeros(0, dtype=np.int64)               # empty row
        else:                                             # narrow row inside a moving band
            lo = (r * 17) % (cols - 2000)
            c = np.sort(rng.choice(np.arange(lo, lo + 2000), size=int(rng.integers(1, 40)), replace=False))
        ci.extend(c.tolist())
        rp.append(len(ci))
    rp = np.array(rp, dtype=np.int32)
    ci = np.array(ci, dtype=np.int32)
    v = rng.uniform(-5.0, 5.0, size=len(ci))
    _check(sk, rows, cols, rp, ci, v, seed=4)


def test_plan_edge_sizes_and_errors(gpu):
    sk = gpu
    rp = np.zeros(1, dtype=np.int32)
    d_rp = _dev(rp)
    plan = sk.SpmvPlan(0, 5, 0, d_rp.data_ptr(), 0, 0)      # no rows: a no-op plan
    plan.execute(0, 0)
    plan.close()
    lp = sk.generate(0, 3)
    r, c, v = lp.csr()
    d_r, d_c, d_v = _dev(r), _dev(c), _dev(v)
    plan = sk.SpmvPlan(lp.m, lp.n, lp.nnz, d_r.data_ptr(), d_c.data_ptr(), d_v.data_ptr())
    with pytest.raises(RuntimeError):
        plan.set_group(3)
    assert sk.lib().sk_spmv_plan_set_group(plan.h, 4, 2) != 0      # windowed must be 0 or 1
    plan.close()
    with pytest.raises(RuntimeError):
        sk.SpmvPlan(-1, 5, 0, d_rp.data_ptr(), 0, 0)


def test_solver_spmv_widths_keep_solves_exact(gpu, oracle):
    """The solver's A x / A^T y widths come from the autotuner: the result still
    matches the FP64 oracle to 1e-8 and two solver instances on the same LP in one
    process give identical bits (the kept width is reused)."""
    sk = gpu
    lp = sk.random_lp(150, 330, 0.03, 99)
    ref, *_ = oracle.ipm_solve(lp)
    out = []
    for _ in range(2):
        s = sk.Solver([lp], precision=sk.PREC_MIXED)
        s.run()
        info, x, y, z = s.result(0)
        s.close()
        assert info["status"] == 0
        assert abs(info["objective"] - ref["objective"]) / (1.0 + abs(ref["objective"])) <= 1e-8
        out.append(x)
    assert np.array_equal(out[0], out[1])
