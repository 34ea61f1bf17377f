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


def _small_case(sk, torch, seed=3):
    lp = sk.random_lp(60, 150, 0.06, seed)
    rp, ci, v = lp.csr()
    rng = np.random.default_rng(seed)
    theta = np.exp(rng.uniform(-3, 3, 150))
    rhs = rng.standard_normal(60)
    return rp, ci, v, theta, rhs


def _call(L, torch, m, n, rp, ci, v, theta, rhs, stream=None):
    dev = torch.device("cuda:0")
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (rp, ci, v, theta, rhs)]
    torch.cuda.synchronize()
    rc = L.sk_kkt_solve_noalloc(m, n, *(vp(x.data_ptr()) for x in t), TOL, vp(stream) if stream else None)
    return rc, t[4].cpu().numpy()


SK_ERR_INVALID, SK_ERR_NUMERICAL = 1, 3


@pytest.mark.parametrize("fault", ["unsorted_columns", "column_out_of_range", "negative_theta", "nan_theta",
                                   "nan_rhs", "nan_value", "decreasing_row_ptrs"])
def test_noalloc_rejects_bad_input_and_leaves_rhs(gpu, fault):
    # malformed input is caught by the kernel's own checks before any write: no device fault
    torch = pytest.importorskip("torch")
    sk = gpu
    L = _bind(sk)
    rp, ci, v, theta, rhs = (a.copy() for a in _small_case(sk, torch))
    if fault == "unsorted_columns":
        q = int(np.argmax(np.diff(rp) >= 2))
        ci[rp[q]], ci[rp[q] + 1] = ci[rp[q] + 1], ci[rp[q]]
    elif fault == "column_out_of_range":
        ci[rp[5]] = 150
    elif fault == "negative_theta":
        theta[7] = -1.0
    elif fault == "nan_theta":
        theta[7] = np.nan
    elif fault == "nan_rhs":
        rhs[3] = np.nan
    elif fault == "nan_value":
        v[11] = np.inf
    elif fault == "decreasing_row_ptrs":
        assert rp[10] >= 1
        rp[11] = rp[10] - 1          # row 10 ends before it starts; every pointer stays within [0, nnz]
    rc, out = _call(L, torch, 60, 150, rp, ci, v, theta, rhs)
    assert rc == SK_ERR_INVALID, (rc, sk.last_error())
    assert "bad input" in sk.last_error()
    np.testing.assert_array_equal(np.nan_to_num(out, nan=1234.5), np.nan_to_num(rhs, nan=1234.5))


def test_noalloc_empty_row_is_a_numerical_failure(gpu):
    # a row of A without entries makes A Theta A^T singular: the regularised factor
    # exists, but the refinement cannot reach the tolerance for that row
    torch = pytest.importorskip("torch")
    sk = gpu
    L = _bind(sk)
    rp, ci, v, theta, rhs = _small_case(sk, torch)
    k = 20
    drop = rp[k + 1] - rp[k]
    ci2 = np.concatenate([ci[:rp[k]], ci[rp[k + 1]:]]).astype(np.int32)
    v2 = np.concatenate([v[:rp[k]], v[rp[k + 1]:]])
    rp2 = rp.copy()
    rp2[k + 1:] -= drop
    rc, out = _call(L, torch, 60, 150, rp2, ci2, v2, theta, rhs)
    assert rc == SK_ERR_NUMERICAL, (rc, sk.last_error())
    assert "above tolerance" in sk.last_error()


def test_noalloc_on_a_non_default_stream(gpu):
    torch = pytest.importorskip("torch")
    sk = gpu
    L = _bind(sk)
    rp, ci, v, theta, rhs = _small_case(sk, torch, seed=9)
    rc0, ref = _call(L, torch, 60, 150, rp, ci, v, theta, rhs)
    assert rc0 == 0, sk.last_error()
    s = torch.cuda.Stream()
    rc, out = _call(L, torch, 60, 150, rp, ci, v, theta, rhs, stream=s.cuda_stream)
    assert rc == 0, sk.last_error()
    np.testing.assert_array_equal(out, ref)
