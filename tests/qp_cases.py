"""Convex QP cases: the reference's own unit-test problems
(tests/unit/test_qp_solver.cpp:161-404, analytic answers) and seeded random
separable / coupled QPs built on the LP generator's sparsity."""
import numpy as np

INF = 1e30

# name: (H dense, c, A dense (m x n), b, lb, ub, expected x or None, expected objective or None, margin)
REFERENCE_CASES = {
    "diagonal": (np.array([[2.0, 0.0], [0.0, 4.0]]), [-4.0, -6.0], [[1.0, 1.0]], [3.0], [0.0, 0.0], [INF, INF],
                 [5.0 / 3.0, 4.0 / 3.0], -25.0 / 3.0, 1e-4),                         # :161-190
    "coupled_psd": (np.array([[2.0, 1.0], [1.0, 2.0]]), [-1.0, -1.0], [[1.0, 1.0]], [1.0], [0.0, 0.0], [INF, INF],
                    [0.5, 0.5], -0.25, 1e-4),                                         # :197-229
    "active_bounds": (np.diag([1.0, 1.0, 0.0]), [-2.0, 0.0, 0.0], [[1.0, 1.0, 1.0]], [1.5], [0.0, 0.0, 0.0],
                      [1.0, 1.0, INF], [1.0, 0.0, 0.5], -1.5, 2e-3),                  # :236-271
    "qplib_tridiagonal": (np.array([[4.0, 1.0, 0.0], [1.0, 4.0, 1.0], [0.0, 1.0, 4.0]]), [-8.0, -12.0, -8.0],
                          [[1.0, 1.0, 1.0]], [6.0], [0.0, 0.0, 0.0], [INF, INF, INF],
                          [1.75, 2.5, 1.75], -24.5, 1e-3),                            # :350-404
}
INFEASIBLE_CASE = (np.array([[1.0]]), [0.0], [[1.0]], [2.0], [0.0], [1.0])             # :276-298
INDEFINITE_CASE = (np.array([[1.0, 0.0], [0.0, -1.0]]), [0.0, 0.0], [[1.0, 1.0]], [1.0], [0.0, 0.0], [INF, INF])
ITERLIMIT_CASE = (np.array([[2.0, 0.0], [0.0, 2.0]]), [-1.0, -1.0], [[1.0, 1.0]], [1.0], [0.0, 0.0], [INF, INF])


def random_qp(m, n, density, seed, coupled=False, bounded=True):
    """A feasible, bounded convex QP: A sparse (each column density*m entries,
    +-U[0.1,10]), b = A x0 with x0 in the box, H diagonal U[0.1, 2] (coupled: plus
    a sparse PSD part G^T G with G having 2 entries per row), c ~ N(0, 1);
    lb = 0, ub = U[2, 4] on a third of the columns (bounded) else +inf."""
    rng = np.random.default_rng(seed)
    A = np.zeros((m, n))
    k = max(2, int(round(density * m)))
    for j in range(n):
        rows = rng.choice(m, size=min(k, m), replace=False)
        A[rows, j] = rng.uniform(0.1, 10.0, len(rows)) * rng.choice([-1.0, 1.0], len(rows))
    for i in range(m):
        if not A[i].any():
            A[i, rng.integers(n)] = rng.uniform(0.1, 10.0)
    lb = np.zeros(n)
    ub = np.full(n, INF)
    if bounded:
        sel = rng.random(n) < 1.0 / 3.0
        ub[sel] = rng.uniform(2.0, 4.0, sel.sum())
    x0 = rng.uniform(0.5, 1.5, n)
    b = A @ x0
    H = np.diag(rng.uniform(0.1, 2.0, n))
    if coupled:
        G = np.zeros((n // 2, n))
        for r in range(n // 2):
            cols = rng.choice(n, size=2, replace=False)
            G[r, cols] = rng.standard_normal(2)
        H = H + G.T @ G
    c = rng.standard_normal(n)
    return H, c, A, b, lb, ub
