"""CPU restatement of the reference's presolve (Ruiz equilibration), for tests only.

TEST INFRASTRUCTURE: only tests/ may import this module, as the checker of the
product's presolve (sk_presolve_ruiz / presolve::apply_ruiz_scaling); nothing in
the product calls it.

Follows src/presolve/scaling.cpp with the same floating-point operations in the
same order, so the results are bit-identical:
  :32-35   stopping tolerance 1e-4 on |max - 1|
  :45-53   row maxima of |a_ij|
  :55-66   row factor 1/sqrt(max) for rows whose max exceeds 1e-15; row_scale *= factor
  :69-71   A <- diag(row factor) A
  :77-88   column maxima of the row-scaled matrix
  :90-109  column factor 1/sqrt(max) (integer columns and columns with max <= 1e-15 keep 1);
           col_scale *= factor
  :112-119 A <- A diag(column factor)
  :122-124 stop when both deviations are below the tolerance
  :130-146 b <- row_scale .* b; c <- col_scale .* c; finite lb, ub <- bound / col_scale
"""
import numpy as np

TOL = 1e-4     # scaling.cpp:32
ZERO = 1e-15   # scaling.cpp:58, 101


def ruiz(m, n, col_ptrs, row_idx, vals, b=None, c=None, lb=None, ub=None, integer=None, max_iter=10,
         row_scale=None, col_scale=None):
    """Returns dict(vals, b, c, lb, ub, row_scale, col_scale, passes); inputs are not modified."""
    cp = np.asarray(col_ptrs, dtype=np.int64)
    ri = np.asarray(row_idx, dtype=np.int64)
    v = np.array(vals, dtype=np.float64)
    rs = np.ones(m) if row_scale is None else np.array(row_scale, dtype=np.float64)
    cs = np.ones(n) if col_scale is None else np.array(col_scale, dtype=np.float64)
    isint = np.zeros(n, dtype=bool) if integer is None else np.asarray(integer, dtype=bool)
    col_of = np.repeat(np.arange(n), np.diff(cp))
    passes = 0
    if m > 0 and n > 0:
        for _ in range(max_iter):
            passes += 1
            r = np.zeros(m)
            np.maximum.at(r, ri, np.abs(v))                           # :45-53
            live = r > ZERO
            sr = np.ones(m)
            sr[live] = 1.0 / np.sqrt(r[live])                         # :55-66
            dev_r = np.max(np.abs(r[live] - 1.0)) if live.any() else 0.0
            rs[live] *= sr[live]
            v *= sr[ri]                                               # :69-71
            cm = np.zeros(n)
            np.maximum.at(cm, col_of, np.abs(v))                      # :77-88
            livec = (cm > ZERO) & ~isint
            sc = np.ones(n)
            sc[livec] = 1.0 / np.sqrt(cm[livec])                      # :90-109
            dev_c = np.max(np.abs(cm[livec] - 1.0)) if livec.any() else 0.0
            cs[livec] *= sc[livec]
            v *= sc[col_of]                                           # :112-119
            if dev_r < TOL and dev_c < TOL:                           # :122-124
                break
    out = {"vals": v, "row_scale": rs, "col_scale": cs, "passes": passes}
    out["b"] = None if b is None else np.asarray(b, dtype=np.float64) * rs          # :130-133
    out["c"] = None if c is None else np.asarray(c, dtype=np.float64) * cs          # :138-139
    for key, bound, keep in (("lb", lb, lambda x: x > -np.inf), ("ub", ub, lambda x: x < np.inf)):
        if bound is None:
            out[key] = None
            continue
        bd = np.array(bound, dtype=np.float64)
        k = keep(bd)
        bd[k] = bd[k] / cs[k]                                                        # :141-146
        out[key] = bd
    return out
