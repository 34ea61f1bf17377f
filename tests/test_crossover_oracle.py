"""The crossover oracle against the reference's known-answer tests
(tests/unit/test_crossover.cu:15-134): the 2-row example's basis properties and the
rank-deficient case."""
import numpy as np

import crossover_oracle as xo


def ref_example():
    # min -x1 - x2  s.t.  x1 + 2 x2 + x3 = 4,  2 x1 + x2 + x4 = 4,  x >= 0  (test_crossover.cu:15-35)
    cp = [0, 2, 4, 5, 6]
    ri = [0, 1, 0, 1, 0, 1]
    v = [1.0, 2.0, 2.0, 1.0, 1.0, 1.0]
    return 2, 4, cp, ri, v, np.array([4.0, 4.0])


def test_reference_example_basis():
    m, n, cp, ri, v, b = ref_example()
    rc, basic, status, x = xo.crossover(m, n, cp, ri, v, [1.0, 1.0, 1.0, 1.0])
    assert rc == 0
    assert len(basic) == 2 and all(0 <= k < 4 for k in basic)                 # A, B
    assert int(np.sum(status == xo.BASIC)) == 2                                # C
    A = np.zeros((2, 4))
    for j in range(4):
        for k in range(cp[j], cp[j + 1]):
            A[ri[k], j] = v[k]
    B = A[:, basic]
    assert abs(np.linalg.det(B)) > 1e-7                                        # D
    xb = np.linalg.solve(B, b)                                                 # E
    xf = np.zeros(4)
    xf[basic] = xb
    assert np.max(np.abs(A @ xf - b)) <= 1e-6
    assert np.min(xf) >= -1e-6                                                 # F
    for j in range(4):                                                         # G
        if j not in basic:
            assert status[j] == xo.AT_LOWER and abs(xf[j]) <= 1e-6


def test_reference_rank_deficient_case():
    # x1 + x2 = 2, 2 x1 + 2 x2 = 4 (test_crossover.cu:118-134)
    rc, basic, status, x = xo.crossover(2, 2, [0, 2, 4], [0, 1, 0, 1], [1.0, 2.0, 1.0, 2.0], [1.0, 1.0])
    assert rc == "rank_deficient"
    assert np.sum(basic >= 2) == 1
