"""Seeded LPs with variable bounds (lower only, boxed, upper only, free), feasible and
bounded by construction, for the standard-form tests."""
import numpy as np


def bounded_case(sk, seed, m=40, n=90, d=0.1):
    import scipy.sparse as sp
    base = sk.random_lp(m, n, d, seed)
    rng = np.random.default_rng(seed)
    A = sp.csc_matrix((base.vals, base.row_idx, base.col_ptrs), shape=(m, n))
    kind = rng.choice(4, n, p=[0.5, 0.25, 0.15, 0.1])   # 0 lower only, 1 box, 2 upper only, 3 free
    lo = rng.uniform(-1, 1, n)
    lb = np.where((kind == 0) | (kind == 1), lo, -np.inf)
    ub = np.where(kind == 1, lo + rng.uniform(0.5, 2, n), np.where(kind == 2, rng.uniform(-1, 1, n), np.inf))
    x0 = np.select([kind == 0, kind == 1, kind == 2], [lo + rng.uniform(0.1, 1, n), lo + 0.25,
                                                      ub - rng.uniform(0.1, 1, n)], rng.normal(0, 1, n))
    y0 = rng.normal(0, 1, m)
    # reduced costs of the sign that keeps the LP bounded: >= 0 on lower-bounded, <= 0 on
    # upper-bounded-only and 0 on free columns
    s0 = np.select([kind == 0, kind == 1, kind == 2], [rng.uniform(0.1, 1, n), rng.normal(0, 1, n),
                                                      -rng.uniform(0.1, 1, n)], 0.0)
    b = A @ x0
    c = A.T @ y0 + s0
    lp = sk.LP(m, n, base.col_ptrs, base.row_idx, base.vals, b, c, "bounded%d" % seed)
    return lp, lb, ub, A


def highs_objective(lp, lb, ub, A):
    from scipy.optimize import linprog
    res = linprog(lp.c, A_eq=A, b_eq=lp.b, bounds=list(zip(lb, ub)), method="highs")
    assert res.status == 0
    return res.fun


def write_mps(path, lp, lb, ub):
    """Free-format MPS of min c^T x, A x = b (rows E), with a BOUNDS section."""
    lines = ["NAME BOUNDED", "ROWS", " N COST"] + [" E R%d" % i for i in range(lp.m)] + ["COLUMNS"]
    for j in range(lp.n):
        lines.append(" X%d COST %.17g" % (j, lp.c[j]))
        for q in range(lp.col_ptrs[j], lp.col_ptrs[j + 1]):
            lines.append(" X%d R%d %.17g" % (j, lp.row_idx[q], lp.vals[q]))
    lines.append("RHS")
    lines += [" RHS R%d %.17g" % (i, lp.b[i]) for i in range(lp.m)]
    lines.append("BOUNDS")
    for j in range(lp.n):
        lo, hi = lb[j], ub[j]
        if np.isinf(lo) and np.isinf(hi):
            lines.append(" FR BND X%d" % j)
            continue
        if np.isinf(lo):
            lines.append(" MI BND X%d" % j)
        elif lo != 0.0:
            lines.append(" LO BND X%d %.17g" % (j, lo))
        if not np.isinf(hi):
            lines.append(" UP BND X%d %.17g" % (j, hi))
    lines.append("ENDATA")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
