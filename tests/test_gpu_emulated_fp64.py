"""FP64 trailing updates on the tensor cores (k_oz_digits + k_update_oz: BF16
digits of each FP64 panel row, exact FP32 tensor-core sums per digit level, an
integer epilogue) against the same factorisation on the FP64 pipe (k_update<double>),
on dense and multifrontal plans, and through whole mixed-precision solves."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _factor(sk, lp, theta, mode):
    rp, ci, v = lp.csr()
    k = sk.Kkt(lp.m, lp.n, rp, ci, v, precision=sk.PREC_FP64)
    k.set_fp64_update(mode)
    assert k.factorize(theta) == 0, sk.last_error()
    L, D = k.factor_dense()
    rhs = np.random.default_rng(1).standard_normal(lp.m)
    rc, x = k.solve(rhs, tol=1e-12)
    k.close()
    return L, D, rc, x


@pytest.mark.parametrize("m,n,d,seed", [(300, 700, 0.03, 1),        # one dense front, partial last panel
                                        (700, 1600, 0.012, 2),       # dense, 11 panels
                                        (1200, 3000, 0.003, 3)])     # multifrontal: many fronts and levels
def test_factor_matches_fp64_pipe(gpu, m, n, d, seed):
    sk = gpu
    lp = sk.random_lp(m, n, d, seed)
    rng = np.random.default_rng(seed)
    theta = np.exp(rng.uniform(-6.0, 6.0, n))        # a late-iteration spread of x / s
    Ln, Dn, rcn, xn = _factor(sk, lp, theta, sk.FP64_UPDATE_NATIVE)
    Lt, Dt, rct, xt = _factor(sk, lp, theta, sk.FP64_UPDATE_TENSOR)
    np.testing.assert_array_equal(Dn, Dt)            # equilibration is not part of the update
    scale = np.max(np.abs(Ln))
    err = np.max(np.abs(Lt - Ln)) / scale
    assert err <= 1e-14, err                          # both are FP64-accurate factors of the same matrix
    assert rcn == 0 and rct == 0
    assert np.max(np.abs(xt - xn)) <= 1e-9 * (1.0 + np.max(np.abs(xn)))


def test_mixed_solves_agree_with_either_fp64_update(gpu, oracle):
    sk = gpu
    for lp in [sk.generate(1, 0), sk.generate(3, 0), sk.generate(3, 17)]:
        res = {}
        for mode in (sk.FP64_UPDATE_NATIVE, sk.FP64_UPDATE_TENSOR):
            info, x, y, s = sk.solve(lp, precision=sk.PREC_MIXED, fp64_update=mode)
            assert info["status"] == 0, (lp.name, mode, info)
            meas = oracle.kkt_measures(lp, x, y, s)
            assert max(meas["rel_pinf"], meas["rel_dinf"], meas["rel_gap"]) <= 1e-8, (lp.name, mode, meas)
            res[mode] = info
        a, b = res[sk.FP64_UPDATE_NATIVE]["objective"], res[sk.FP64_UPDATE_TENSOR]["objective"]
        assert abs(a - b) / (1.0 + abs(a)) <= 1e-8, (lp.name, a, b)
