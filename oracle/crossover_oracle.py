"""CPU restatement of the reference's crossover (basis purification), for tests only.

TEST INFRASTRUCTURE: only tests/ may import this module, as the checker of the
device crossover (sk_crossover); nothing in the product calls it.

Follows src/ipm/crossover.cu step by step with plain loops in the reference's order
(first index wins ties, strict comparisons):
  purify_step_kernel        :53-290  (one step of a strictly interior, non-basic column)
  purify_bound_step_kernel  :292-320 (second pass: fill rows whose artificial is basic)
  generate_crossover_basis  :322-460 (driver, statuses, errors)
B^-1 A_q is computed by a dense solve with the current basis matrix ([A | I] columns),
numerically independent of the device's explicit inverse. Small cases only (m <= ~300).
"""
import numpy as np

AT_BOUND = 1e-6     # crossover.cu:68-70, 446
PIVOT_TOL = 1e-7    # crossover.cu:100-109, 200-218; device_ftran.cu:143
DIR_TOL = 1e-9      # crossover.cu:165, 170
NO_BOUND = 1e30     # crossover.cu:137-140

BASIC, AT_LOWER, AT_UPPER = 0, 1, 2


def _dense(m, n, cp, ri, v):
    A = np.zeros((m, n))
    for j in range(n):
        for k in range(cp[j], cp[j + 1]):
            A[ri[k], j] += v[k]
    return A


def crossover(m, n, cp, ri, v, x, lb=None, ub=None, inverse="solve", trace=None):
    """Returns (rc, basic, status, x): rc 0, 'invalid_pivot' or 'rank_deficient'.
    inverse="solve": B^-1 A_q by a dense solve with the current basis matrix;
    inverse="explicit": an explicit B^-1 with the product-form update E B^-1 (the
    device's arithmetic). trace: a list that receives one record per decision."""
    A = _dense(m, n, cp, ri, v)
    full = np.hstack([A, np.eye(m)])             # artificial columns n..n+m-1
    lb = np.zeros(n) if lb is None else np.asarray(lb, dtype=float)
    ub = np.full(n, np.inf) if ub is None else np.asarray(ub, dtype=float)
    x = np.array(x, dtype=float)
    basis = [n + i for i in range(m)]             # init_ws_kernel :45-53
    is_basic = [False] * n

    binv = np.eye(m)

    def ftran(q):
        if inverse == "explicit":
            return binv @ full[:, q]
        return np.linalg.solve(full[:, basis], full[:, q])

    def exchange(row, d):
        if inverse == "explicit":
            r = binv[row, :] / d[row]
            binv[:, :] = binv - np.outer(d, r)
            binv[row, :] = r

    def best_artificial(d):
        best, row = PIVOT_TOL, -1
        for i in range(m):
            if basis[i] >= n and abs(d[i]) > best:
                best, row = abs(d[i]), i
        return row

    def step(q):
        """One purify_step_kernel call: returns (pivoted, error)."""
        if x[q] <= lb[q] + AT_BOUND or x[q] >= ub[q] - AT_BOUND or is_basic[q]:
            return False, False
        d = ftran(q)
        row = best_artificial(d)
        if row >= 0:                                   # :113-127
            if trace is not None:
                trace.append(("art", q, row))
            exchange(row, d)
            basis[row] = q
            is_basic[q] = True
            return True, False
        pos_t, pos_leave = NO_BOUND, -1                # :135-177
        neg_t, neg_leave = NO_BOUND, -1
        if ub[q] - x[q] < pos_t:
            pos_t, pos_leave = ub[q] - x[q], q
        if x[q] - lb[q] < neg_t:
            neg_t, neg_leave = x[q] - lb[q], q
        for i in range(m):
            bv = basis[i]
            if bv >= n:
                continue
            vi = -d[i]
            dub, dlb = ub[bv] - x[bv], x[bv] - lb[bv]
            if vi > DIR_TOL:
                t = dub / vi
                if t < pos_t:
                    pos_t, pos_leave = t, bv
                t = dlb / vi
                if t < neg_t:
                    neg_t, neg_leave = t, bv
            elif vi < -DIR_TOL:
                t = dlb / (-vi)
                if t < pos_t:
                    pos_t, pos_leave = t, bv
                t = dub / (-vi)
                if t < neg_t:
                    neg_t, neg_leave = t, bv

        def leave_row(var):                            # :179-197
            if var == -1 or var == q:
                return -1
            r = -1
            for i in range(m):
                if basis[i] == var:
                    r = i
            return r if r != -1 and abs(d[r]) > PIVOT_TOL else -1
        r1, r2 = leave_row(pos_leave), leave_row(neg_leave)
        if r1 != -1:                                   # :200-248
            theta, row = pos_t, r1
        elif r2 != -1:
            theta, row = -neg_t, r2
        elif pos_leave == q:
            theta, row = pos_t, -1
        elif neg_leave == q:
            theta, row = -neg_t, -1
        else:
            return False, True
        if trace is not None:
            trace.append(("ratio", q, row, theta, pos_t, neg_t))
        if row != -1:
            exchange(row, d)
            is_basic[basis[row]] = False
            basis[row] = q
            is_basic[q] = True
        x[q] += theta                                  # :251-260, over the updated basis
        for i in range(m):
            bv = basis[i]
            if bv < n:
                x[bv] += theta * (-d[i])
        return True, False

    failed = False
    for q in range(n):                                 # :406-416
        while True:
            pivoted, err = step(q)
            if err:
                failed = True
                break
            if not pivoted:
                break
        if failed:
            break
    if not failed:
        for q in range(n):                             # :418-423
            if is_basic[q]:
                continue
            d = ftran(q)
            row = best_artificial(d)
            if row >= 0:
                if trace is not None:
                    trace.append(("bound", q, row))
                exchange(row, d)
                basis[row] = q
                is_basic[q] = True
    status = [AT_LOWER] * n                            # :433-449
    deficient = False
    for i in range(m):
        if basis[i] < n:
            status[basis[i]] = BASIC
        else:
            deficient = True
    for j in range(n):
        if status[j] != BASIC and abs(x[j] - ub[j]) < AT_BOUND:
            status[j] = AT_UPPER
    rc = "invalid_pivot" if failed else ("rank_deficient" if deficient else 0)
    return rc, np.array(basis), np.array(status), x
