"""Device KKT engine (sk_kkt_*) and SpMV against the reference's golden vectors,
the CPU oracle and an FP64 numpy reference."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KKT_A = (np.array([0, 3, 5, 7], dtype=np.int32), np.array([0, 3, 4, 1, 3, 2, 4], dtype=np.int32),
         np.array([2.0, 1.0, 1.0, 2.0, 1.0, 2.0, 1.0]))
M0 = np.array([[6.0, 1.0, 1.0], [1.0, 5.0, 0.0], [1.0, 0.0, 5.0]])


@pytest.mark.parametrize("precision", [0, 1])
def test_kkt_golden_factor_and_solve(gpu, precision):
    sk = gpu
    rp, ci, v = KKT_A
    P = sk.amd_ordering(3, 5, rp, ci)
    assert P.tolist() == [1, 0, 2]                       # test_gpu_kkt.cu:35
    k = sk.Kkt(3, 5, rp, ci, v, P=P, precision=precision)
    assert k.factorize(np.ones(5)) == 0
    L, D = k.factor_dense()
    PMP = M0[np.ix_(P, P)]
    recon = (L @ L.T) / np.outer(D, D)                   # undo the equilibration
    tol = 1e-6 if precision == 0 else 1e-5
    assert np.linalg.norm(recon - PMP) < tol             # test_gpu_kkt.cu:76-97
    rc, x = k.solve(np.array([11.0, 11.0, 16.0]), tol=1e-10)
    assert rc == 0
    np.testing.assert_allclose(x, [1.0, 2.0, 3.0], atol=1e-6)   # :112-114
    assert np.linalg.norm(M0 @ x - [11, 11, 16]) < 1e-6
    k.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_kkt_relative_contract(gpu, precision):
    sk = gpu
    rp, ci, v = KKT_A
    P = sk.amd_ordering(3, 5, rp, ci)
    k = sk.Kkt(3, 5, rp, ci, v, P=P, precision=precision)
    assert k.factorize(np.ones(5)) == 0
    scale = 1e4
    rc, x = k.solve(scale * np.array([11.0, 11.0, 16.0]), tol=1e-10)
    assert rc == 0                                       # test_gpu_kkt.cu:176-177
    np.testing.assert_allclose(x, scale * np.array([1.0, 2.0, 3.0]), rtol=1e-8)
    assert np.max(np.abs(M0 @ x - scale * np.array([11, 11, 16]))) / (16 * scale) < 1e-8


@pytest.mark.parametrize("m,n,d,seed", [(60, 150, 0.06, 3), (300, 700, 0.015, 4), (900, 2000, 0.004, 5)])
@pytest.mark.parametrize("precision", [0, 1])
def test_kkt_random_vs_oracle(gpu, oracle, m, n, d, seed, precision):
    sk = gpu
    lp = sk.random_lp(m, n, d, seed)
    rp, ci, v = lp.csr()
    rng = np.random.default_rng(seed)
    theta = np.exp(rng.uniform(-3, 3, n))
    rhs = rng.standard_normal(m)
    k = sk.Kkt(m, n, rp, ci, v, precision=precision)
    assert k.factorize(theta) == 0
    rc, x = k.solve(rhs, tol=1e-11)
    assert rc == 0
    ok, xo = oracle.kkt_solve(m, n, rp, ci, v, theta, rhs, tol=1e-11, rel=True)
    assert ok
    assert np.max(np.abs(x - xo)) <= 1e-8 * (1 + np.max(np.abs(xo)))
    # FP64 numpy check of the physical residual
    A = np.zeros((m, n))
    for i in range(m):
        A[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    M = (A * theta) @ A.T
    assert np.max(np.abs(M @ x - rhs)) <= 1e-11 * max(1.0, np.max(np.abs(rhs)))
    k.close()


def test_spmv_matches_numpy(gpu):
    torch = pytest.importorskip("torch")
    sk = gpu
    lp = sk.generate(0, 3)
    rp, ci, v = lp.csr()
    dev = torch.device("cuda:0")
    t_rp = torch.from_numpy(rp).to(dev)
    t_ci = torch.from_numpy(ci).to(dev)
    t_v = torch.from_numpy(v).to(dev)
    x = np.random.default_rng(1).standard_normal(lp.n)
    y0 = np.random.default_rng(2).standard_normal(lp.m)
    t_x = torch.from_numpy(x).to(dev)
    t_y = torch.from_numpy(y0.copy()).to(dev)
    L = sk.lib()
    rc = L.sk_spmv_csr(lp.m, ctypes.c_void_p(t_rp.data_ptr()), ctypes.c_void_p(t_ci.data_ptr()),
                       ctypes.c_void_p(t_v.data_ptr()), ctypes.c_void_p(t_x.data_ptr()), 2.0, -0.5,
                       ctypes.c_void_p(t_y.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    ref = np.zeros(lp.m)
    for i in range(lp.m):
        ref[i] = np.dot(v[rp[i]:rp[i + 1]], x[ci[rp[i]:rp[i + 1]]])
    ref = 2.0 * ref - 0.5 * y0
    np.testing.assert_allclose(t_y.cpu().numpy(), ref, rtol=1e-12, atol=1e-12)
