"""CPU checks of the learned-start network's oracle: its analytic gradient
against central finite differences, and its BF16 rounding."""
import numpy as np
import pytest
import scipy.sparse as sp

import gnn_oracle as go


def small_graph(seed, m=6, n=11):
    rng = np.random.default_rng(seed)
    A = (rng.random((m, n)) < 0.4) * rng.uniform(-2, 2, (m, n))
    for j in range(n):
        if not A[:, j].any():
            A[rng.integers(m), j] = 1.0
    S = sp.csr_matrix(A)
    b, c = rng.standard_normal(m), rng.standard_normal(n)
    t = (rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(m))
    return m, n, S.indptr, S.indices, S.data, b, c, t


@pytest.mark.parametrize("seed", [0, 1])
def test_oracle_gradient_matches_finite_differences(seed):
    m, n, rp, ci, v, b, c, t = small_graph(seed)
    p = go.glorot_params(seed + 7).astype(np.float64)
    *_, loss, cache = go.forward(p, m, n, rp, ci, v, b, c, t, bf16=False)
    g = go.backward(cache)
    rng = np.random.default_rng(seed)
    idx = np.concatenate([rng.choice(p.size, 80, replace=False), np.flatnonzero(g)[:40]])
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        lp = go.forward(p + e, m, n, rp, ci, v, b, c, t, bf16=False)[3]
        lm = go.forward(p - e, m, n, rp, ci, v, b, c, t, bf16=False)[3]
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * (1.0 + abs(fd)), (i, fd, g[i])


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e38, np.inf], dtype=np.float32)
    r = go.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0                 # tie -> even mantissa
    assert r[2] == 1.0 + 2.0 ** -6                      # tie -> even mantissa (up)
    assert r[3] == -2.5 and np.isinf(r[5])
    assert r[4] == np.float32(3.0e38).astype(np.float64) or abs(r[4] / 3.0e38 - 1) < 2 ** -7
