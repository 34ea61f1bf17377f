"""CPU oracle of the convex QP interior-point method -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's qp::QPSolver::solve_with_diagnostics
(src/qp/qp_solver.cpp:151-560, interface src/qp/qp_solver.hpp:47-66, model
src/qp/qp_model.hpp:32-72): minimise 1/2 x^T H x + c^T x subject to A x = b and
lb <= x <= ub with the reference's primal-dual path-following steps, so that the
device QP solver can be checked iterate for iterate. Used only by tests/ as the
checker; the product never imports it.

Steps restated (reference lines):
  * start x_j = (lo + hi) / 2 with lo = lb or -10, hi = ub or 10; y = 0; zl, zu = 1 on
    finite bounds (:190-208); a bound is finite when lb > -1e15 / ub < 1e15 (:196-197)
  * residuals rp = A x - b, rd = H x + c - A^T y - zl + zu; mu over the finite
    bounds (:222-258); stop when ||rp||_inf < feas_tol, ||rd||_inf < dual_tol and
    mu < grad_tol (:269-281); Infeasible when ||y||_inf > 1e15, Unbounded when the
    objective < -1e15 (:284-292)
  * D_j = zl/max(x - lb, 1e-12) + zu/max(ub - x, 1e-12), floored at 1e-12; W = H + D
    (:295-325); Cholesky failure -> NumericalFailure (:328-333)
  * sigma = 0.2; rhs_x = -rd + sum of (sigma mu - z gap)/gap terms (:335-352)
  * S = A W^-1 A^T, rhs_y = -A W^-1 rhs_x - rp, S dy = rhs_y, dx = W^-1 (A^T dy + rhs_x)
    (:354-430); dzl, dzu from the complementarity rows (:432-446); fraction to the
    boundary 0.995 with separate primal and dual steps (:448-477); z floored at
    1e-14 on finite bounds (:479-491); m = 0 solves W dx = rhs_x alone (:493-545)
  * IterationLimit after max_iterations with iterations = max_iterations (:548-560)
"""
import numpy as np

OPTIMAL, INFEASIBLE, UNBOUNDED, ITERATION_LIMIT, NUMERICAL_FAILURE, UNSUPPORTED_NONCONVEX, INVALID_MODEL = range(7)
CONVEX_UNKNOWN, CONVEX_PSD, NONCONVEX = 0, 1, 2
INF = 1e30


def _chol(W):
    """Dense Cholesky with the reference's pivot test (sum <= 1e-14 fails; :27-51)."""
    n = W.shape[0]
    L = np.zeros_like(W)
    for j in range(n):
        s = W[j, j] - np.dot(L[j, :j], L[j, :j])
        if s <= 1e-14:
            return None
        L[j, j] = np.sqrt(s)
        if j + 1 < n:
            L[j + 1:, j] = (W[j + 1:, j] - L[j + 1:, :j] @ L[j, :j]) / L[j, j]
    return L


def _chol_solve(L, b):
    import scipy.linalg as sl
    y = sl.solve_triangular(L, b, lower=True)
    return sl.solve_triangular(L.T, y, lower=False)


def solve(H, c, A, b, lb, ub, convexity=CONVEX_PSD, feas_tol=1e-6, dual_tol=1e-6, grad_tol=1e-6, max_iter=200,
          trace=None):
    """Dense H (n x n, symmetric), A (m x n). Returns dict(status, objective, iterations,
    primal_residual, dual_residual, complementarity, x, y, z) with z = zl - zu.
    `trace` (a list) receives (x, y, zl, zu) after every iteration's update."""
    H = np.asarray(H, dtype=float)
    A = np.asarray(A, dtype=float).reshape(-1, H.shape[0]) if np.size(A) else np.zeros((0, H.shape[0]))
    c, b = np.asarray(c, dtype=float), np.asarray(b, dtype=float)
    lb, ub = np.asarray(lb, dtype=float), np.asarray(ub, dtype=float)
    res = {"status": INVALID_MODEL, "objective": 0.0, "iterations": 0, "primal_residual": 0.0,
           "dual_residual": 0.0, "complementarity": 0.0, "x": None, "y": None, "z": None}
    if convexity == NONCONVEX:
        res["status"] = UNSUPPORTED_NONCONVEX
        return res
    n, m = H.shape[0], A.shape[0]
    if H.shape != (n, n) or lb.shape != (n,) or ub.shape != (n,) or np.any(lb > ub):
        return res
    if convexity == CONVEX_UNKNOWN:
        res["status"] = UNSUPPORTED_NONCONVEX
        return res
    if n == 0:
        return res
    has_lb, has_ub = lb > -1e15, ub < 1e15
    lo = np.where(has_lb, lb, -10.0)
    hi = np.where(has_ub, ub, 10.0)
    x = (lo + hi) / 2.0
    y = np.zeros(m)
    zl = np.where(has_lb, 1.0, 0.0)
    zu = np.where(has_ub, 1.0, 0.0)
    ncomp = int(has_lb.sum() + has_ub.sum())
    sigma, eta = 0.2, 0.995
    for it in range(max_iter):
        res["iterations"] = it
        Hx = H @ x
        rp = A @ x - b
        rd = Hx + c - A.T @ y - zl + zu
        mu = float(np.sum(np.where(has_lb, (x - lb) * zl, 0.0)) + np.sum(np.where(has_ub, (ub - x) * zu, 0.0)))
        if ncomp > 0:
            mu /= ncomp
        nrp = float(np.max(np.abs(rp))) if m else 0.0
        nrd = float(np.max(np.abs(rd)))
        res.update(primal_residual=nrp, dual_residual=nrd, complementarity=mu)
        obj = float(np.sum(0.5 * x * Hx + c * x))
        res["objective"] = obj
        if nrp < feas_tol and nrd < dual_tol and mu < grad_tol:
            res.update(status=OPTIMAL, x=x.copy(), y=y.copy(), z=zl - zu)
            return res
        if m and float(np.max(np.abs(y))) > 1e15:
            res["status"] = INFEASIBLE
            return res
        if obj < -1e15:
            res["status"] = UNBOUNDED
            return res
        gl = np.maximum(x - lb, 1e-12)
        gu = np.maximum(ub - x, 1e-12)
        D = np.where(has_lb, zl / gl, 0.0) + np.where(has_ub, zu / gu, 0.0)
        D = np.maximum(D, 1e-12)
        L = _chol(H + np.diag(D))
        if L is None:
            res["status"] = NUMERICAL_FAILURE
            return res
        comp = np.where(has_lb, (sigma * mu - zl * gl) / gl, 0.0) - np.where(has_ub, (sigma * mu - zu * gu) / gu, 0.0)
        rhs_x = -rd + comp
        if m > 0:
            WinvAT = _chol_solve(L, A.T)
            S = A @ WinvAT
            rhs_y = -(A @ _chol_solve(L, rhs_x)) - rp
            Ls = _chol(S)
            if Ls is None:
                res["status"] = NUMERICAL_FAILURE
                return res
            dy = _chol_solve(Ls, rhs_y)
            dx = _chol_solve(L, A.T @ dy + rhs_x)
        else:
            dy = np.zeros(0)
            dx = _chol_solve(L, rhs_x)
        dzl = np.where(has_lb, (sigma * mu - zl * gl - zl * dx) / gl, 0.0)
        dzu = np.where(has_ub, (sigma * mu - zu * gu + zu * dx) / gu, 0.0)
        ap, ad = 1.0, 1.0
        with np.errstate(divide="ignore", invalid="ignore"):
            sel = has_lb & (dx < 0)
            if sel.any():
                ap = min(ap, float(np.min(-(x - lb)[sel] / dx[sel])))
            sel = has_ub & (dx > 0)
            if sel.any():
                ap = min(ap, float(np.min((ub - x)[sel] / dx[sel])))
            sel = has_lb & (dzl < 0) & (zl > 0)
            if sel.any():
                ad = min(ad, float(np.min(-zl[sel] / dzl[sel])))
            sel = has_ub & (dzu < 0) & (zu > 0)
            if sel.any():
                ad = min(ad, float(np.min(-zu[sel] / dzu[sel])))
        ap = min(1.0, eta * ap)
        ad = min(1.0, eta * ad)
        x = x + ap * dx
        zl = np.where(has_lb, np.maximum(zl + ad * dzl, 1e-14), zl + ad * dzl)
        zu = np.where(has_ub, np.maximum(zu + ad * dzu, 1e-14), zu + ad * dzu)
        y = y + ad * dy
        if trace is not None:
            trace.append((x.copy(), y.copy(), zl.copy(), zu.copy()))
    res.update(status=ITERATION_LIMIT, iterations=max_iter, x=x.copy(), y=y.copy(), z=zl - zu)
    return res


def lift(H, tol=1e-14):
    """Pivoted Cholesky of a PSD H: F (r x n) with H = F^T F up to rounding; pivots
    below tol * max(diag H) end the factorisation (the remaining part of H is treated
    as zero). Returns F."""
    H = np.array(H, dtype=float)
    n = H.shape[0]
    d = np.diag(H).copy()
    stop = tol * max(1.0, float(np.max(d))) if n else 0.0
    rows = []
    Lc = np.zeros((0, n))
    for _ in range(n):
        p = int(np.argmax(d))
        if d[p] <= stop:
            break
        col = H[:, p] - Lc.T @ Lc[:, p]
        f = col / np.sqrt(d[p])
        rows.append(f)
        Lc = np.vstack([Lc, f])
        d = d - f * f
        d[p] = 0.0
    return np.array(rows).reshape(-1, n)
