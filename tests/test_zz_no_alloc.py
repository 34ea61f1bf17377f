"""Allocation-free KKT solve (sk_kkt_solve_noalloc) through the C ABI against the
KKT engine's sk_kkt_factorize_device + sk_kkt_solve_device on the same device
inputs. The file name sorts last so that the entry point is exercised after every
other GPU test of a run, and it passes in a fresh process on its own as well."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
vp = ctypes.c_void_p
TOL = 1e-11
SK_ERR_TOO_LARGE = 7


def _bind(sk):
    L = sk.lib()
    L.sk_kkt_solve_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_double, vp]
    L.sk_kkt_solve_noalloc.restype = ctypes.c_int
    return L


def _dense(m, n, rp, ci, v):
    A = np.zeros((m, n))
    for i in range(m):
        A[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    return A


@pytest.mark.parametrize("m,n,d,seed", [(60, 150, 0.06, 3), (200, 450, 0.02, 12), (256, 600, 0.02, 21)])
def test_noalloc_matches_kkt_engine(gpu, m, n, d, seed):
    torch = pytest.importorskip("torch")
    sk = gpu
    L = _bind(sk)
    lp = sk.random_lp(m, n, d, seed)
    rp, ci, v = lp.csr()
    rng = np.random.default_rng(seed)
    theta = np.exp(rng.uniform(-3, 3, n))
    rhs = rng.standard_normal(m)
    dev = torch.device("cuda:0")
    t_rp, t_ci, t_v, t_th = (torch.from_numpy(a).to(dev) for a in (rp, ci, v, theta))

    # existing entry point: KKT engine, FP64 factor
    k = sk.Kkt(m, n, rp, ci, v, precision=sk.PREC_FP64)
    t_ref = torch.from_numpy(rhs.copy()).to(dev)
    torch.cuda.synchronize()
    assert L.sk_kkt_factorize_device(k.h, vp(t_th.data_ptr())) == 0, sk.last_error()
    assert L.sk_kkt_solve_device(k.h, vp(t_ref.data_ptr()), TOL) == 0, sk.last_error()
    ref = t_ref.cpu().numpy()
    k.close()

    # the allocation-free entry point, two calls in a row on the same inputs
    outs = []
    for _ in range(2):
        t_rhs = torch.from_numpy(rhs.copy()).to(dev)
        torch.cuda.synchronize()
        rc = L.sk_kkt_solve_noalloc(m, n, vp(t_rp.data_ptr()), vp(t_ci.data_ptr()), vp(t_v.data_ptr()),
                                    vp(t_th.data_ptr()), vp(t_rhs.data_ptr()), TOL, None)
        assert rc == 0, sk.last_error()
        outs.append(t_rhs.cpu().numpy())

    scale = 1.0 + np.max(np.abs(ref))
    for x in outs:
        assert np.max(np.abs(x - ref)) <= 1e-8 * scale
    np.testing.assert_array_equal(outs[0], outs[1])    # one block, fixed summation order
    M = (_dense(m, n, rp, ci, v) * theta) @ _dense(m, n, rp, ci, v).T
    assert np.max(np.abs(M @ outs[0] - rhs)) <= TOL * max(1.0, np.max(np.abs(rhs)))


def test_noalloc_rejects_rows_beyond_limit(gpu):
    torch = pytest.importorskip("torch")
    sk = gpu
    L = _bind(sk)
    lp = sk.random_lp(257, 600, 0.02, 5)
    rp, ci, v = lp.csr()
    dev = torch.device("cuda:0")
    t_rp, t_ci, t_v = (torch.from_numpy(a).to(dev) for a in (rp, ci, v))
    t_th = torch.ones(600, dtype=torch.float64, device=dev)
    t_rhs = torch.ones(257, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = L.sk_kkt_solve_noalloc(257, 600, vp(t_rp.data_ptr()), vp(t_ci.data_ptr()), vp(t_v.data_ptr()),
                                vp(t_th.data_ptr()), vp(t_rhs.data_ptr()), TOL, None)
    assert rc == SK_ERR_TOO_LARGE
    assert "256" in sk.last_error()
    assert torch.all(t_rhs == 1.0)                      # untouched
