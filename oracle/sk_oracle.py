"""ctypes binding of the CPU oracle (oracle/lib/libsk_oracle.so) and of the
reference's own CPU code (oracle/_ref/libsankhya_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker or the timed CPU baseline,
never as part of the product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "lib", "libsk_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsankhya_ref.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class IpmOpts(C.Structure):
    _fields_ = [("criteria", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int), ("verbose", C.c_int),
                ("start", C.c_int), ("strict", C.c_int)]


class IpmResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("objective", C.c_double),
                ("primal_residual", C.c_double), ("dual_residual", C.c_double), ("duality_gap", C.c_double),
                ("rel_pinf", C.c_double), ("rel_dinf", C.c_double), ("rel_gap", C.c_double), ("solves", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build(reference_root=None):
    """Builds the oracle library, and oracle/_ref when the reference sources are
    given (argument, else the SK_REFERENCE_ROOT environment variable: the
    directory that holds the reference's src/ and include/)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    reference_root = reference_root or os.environ.get("SK_REFERENCE_ROOT")
    if reference_root and os.path.isdir(os.path.join(reference_root, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + reference_root], check=True)


_o = None
_r = None


def oracle():
    global _o
    if _o is None:
        if not os.path.exists(ORACLE_LIB):
            build()
        L = C.CDLL(ORACLE_LIB)
        L.oracle_min_degree.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p]
        L.oracle_symbolic.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, C.c_int]
        L.oracle_kkt_solve.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, C.c_void_p, _f64p, C.c_double,
                                       C.c_int, _f64p]
        L.oracle_ipm_solve.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.POINTER(IpmOpts),
                                       _f64p, _f64p, _f64p, C.POINTER(IpmResult)]
        L.oracle_kkt_measures.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                          _f64p]
        L.oracle_lp_family.argtypes = [C.c_int, C.c_int, C.c_void_p]
        L.oracle_lp_random.argtypes = [C.c_int, C.c_int, C.c_double, C.c_ulonglong, C.c_void_p]
        L.oracle_lp_block_angular.argtypes = [C.c_ulonglong] + [C.c_int] * 5 + [C.c_void_p]
        L.oracle_lp_free.argtypes = [C.c_void_p]
        L.oracle_lp_family3_shape.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                              C.POINTER(C.c_double)]
        _o = L
    return _o


class OracleLP(C.Structure):
    _fields_ = [("m", C.c_int), ("n", C.c_int), ("nnz", C.c_int), ("col_ptrs", C.POINTER(C.c_int)),
                ("row_idx", C.POINTER(C.c_int)), ("vals", C.POINTER(C.c_double)), ("b", C.POINTER(C.c_double)),
                ("c", C.POINTER(C.c_double))]


class LP:
    """A generated LP (min c^T x, A x = b, x >= 0; A in CSC) as numpy arrays, built by
    the oracle's restatement of the seeded generator (no product code involved)."""

    def __init__(self, m, n, col_ptrs, row_idx, vals, b, c, name="lp"):
        self.m, self.n = int(m), int(n)
        self.col_ptrs, self.row_idx, self.vals, self.b, self.c = col_ptrs, row_idx, vals, b, c
        self.name = name

    @property
    def nnz(self):
        return int(self.col_ptrs[-1])


def _take_lp(h, name):
    def arr(p, k, dt):
        return np.ctypeslib.as_array(p, shape=(k,)).astype(dt, copy=True) if k > 0 else np.zeros(0, dtype=dt)
    lp = LP(h.m, h.n, arr(h.col_ptrs, h.n + 1, np.int32), arr(h.row_idx, h.nnz, np.int32),
            arr(h.vals, h.nnz, np.float64), arr(h.b, h.m, np.float64), arr(h.c, h.n, np.float64), name)
    oracle().oracle_lp_free(C.byref(h))
    return lp


def generate(family, instance=0):
    """Seeded LP of family 0, 1 or 3, identical to the product's generator."""
    h = OracleLP()
    assert oracle().oracle_lp_family(family, instance, C.byref(h)) == 0, (family, instance)
    return _take_lp(h, "family%d/%d" % (family, instance))


def generate_dims(family, instance):
    """(m, n) of a family-3 member without building it."""
    assert family == 3
    m, n, d = C.c_int(), C.c_int(), C.c_double()
    oracle().oracle_lp_family3_shape(instance, C.byref(m), C.byref(n), C.byref(d))
    return m.value, n.value


def random_lp(m, n, density, seed):
    h = OracleLP()
    assert oracle().oracle_lp_random(m, n, density, seed, C.byref(h)) == 0
    return _take_lp(h, "random%dx%d" % (m, n))


def block_angular(seed, blocks, block_rows=500, block_cols=1200, link_rows=2000, nnz_per_col=5):
    h = OracleLP()
    assert oracle().oracle_lp_block_angular(seed, blocks, block_rows, block_cols, link_rows, nnz_per_col,
                                            C.byref(h)) == 0
    return _take_lp(h, "block_angular%dx%d" % (blocks, link_rows))


def have_reference():
    return os.path.exists(REF_LIB)


def reference():
    global _r
    if _r is None:
        L = C.CDLL(REF_LIB)
        L.ref_min_degree.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p]
        L.ref_symbolic.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, C.c_int]
        L.ref_simplex_solve.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                        C.POINTER(C.c_double)]
        L.ref_verify_optimal.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p, _f64p]
        if hasattr(L, "ref_qp_solve"):
            L.ref_qp_solve.argtypes = [C.c_int, C.c_int] + [_f64p] * 6 + [C.c_int] + [_f64p] * 4
        if hasattr(L, "ref_ruiz_scaling"):
            _u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
            L.ref_ruiz_scaling.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p, _f64p, _u8p,
                                           C.c_int] + [_f64p] * 7
        _r = L
    return _r


def min_degree(m, n, rp, ci):
    P = np.zeros(m, dtype=np.int32)
    assert oracle().oracle_min_degree(m, n, rp, ci, P) == 0
    return P


def symbolic(m, n, rp, ci, P):
    cap = max(1, m * (m - 1) // 2)
    Pinv = np.zeros(m, dtype=np.int32)
    parent = np.zeros(m, dtype=np.int32)
    Lrp = np.zeros(m + 1, dtype=np.int32)
    Lci = np.zeros(cap, dtype=np.int32)
    nnz = oracle().oracle_symbolic(m, n, rp, ci, np.ascontiguousarray(P, dtype=np.int32), Pinv, parent, Lrp, Lci, cap)
    assert nnz >= 0
    return Pinv, parent, Lrp, Lci[:nnz].copy()


def kkt_solve(m, n, rp, ci, vals, theta, rhs, P=None, tol=1e-10, rel=True):
    dy = np.zeros(m, dtype=np.float64)
    Pp = None if P is None else np.ascontiguousarray(P, dtype=np.int32)
    ok = oracle().oracle_kkt_solve(m, n, rp, ci, vals, np.ascontiguousarray(theta, dtype=np.float64),
                                   None if Pp is None else Pp.ctypes.data_as(C.c_void_p),
                                   np.ascontiguousarray(rhs, dtype=np.float64), tol, 1 if rel else 0, dy)
    return bool(ok), dy


def ipm_solve(lp, criteria=0, tol=1e-8, max_iter=200, verbose=0, strict=0, start=0):
    o = IpmOpts(criteria, tol, max_iter, verbose, start, strict)
    x = np.zeros(lp.n)
    y = np.zeros(lp.m)
    s = np.zeros(lp.n)
    r = IpmResult()
    oracle().oracle_ipm_solve(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, lp.c, C.byref(o), x, y, s,
                              C.byref(r))
    return r.as_dict(), x, y, s


def kkt_measures(lp, x, y, s):
    out = np.zeros(6)
    oracle().oracle_kkt_measures(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, lp.c,
                                 np.ascontiguousarray(x, dtype=np.float64), np.ascontiguousarray(y, dtype=np.float64),
                                 np.ascontiguousarray(s, dtype=np.float64), out)
    return {"rel_pinf": out[0], "rel_dinf": out[1], "rel_gap": out[2], "objective": out[3], "min_x": out[4],
            "min_s": out[5]}


def ref_min_degree(m, n, rp, ci):
    P = np.zeros(m, dtype=np.int32)
    assert reference().ref_min_degree(m, n, rp, ci, P) == 0
    return P


def ref_symbolic(m, n, rp, ci, P):
    cap = max(1, m * (m - 1) // 2)
    Pinv = np.zeros(m, dtype=np.int32)
    parent = np.zeros(m, dtype=np.int32)
    Lrp = np.zeros(m + 1, dtype=np.int32)
    Lci = np.zeros(cap, dtype=np.int32)
    nnz = reference().ref_symbolic(m, n, rp, ci, np.ascontiguousarray(P, dtype=np.int32), Pinv, parent, Lrp, Lci,
                                   cap)
    assert nnz >= 0
    return Pinv, parent, Lrp, Lci[:nnz].copy()


def ref_simplex(lp):
    """Reference CPU Phase-I + primal simplex: (status, objective, x)."""
    x = np.zeros(lp.n)
    obj = C.c_double()
    st = reference().ref_simplex_solve(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, lp.c, x, C.byref(obj))
    return st, obj.value, x


def ref_ruiz(lp, lb, ub, integer, max_iter=10):
    """The reference's presolve::apply_ruiz_scaling on the LP with bounds and integer
    flags: dict(vals, b, c, lb, ub, row_scale, col_scale)."""
    L = reference()
    out = {k: np.zeros(n) for k, n in (("vals", lp.nnz), ("b", lp.m), ("c", lp.n), ("lb", lp.n), ("ub", lp.n),
                                        ("row_scale", lp.m), ("col_scale", lp.n))}
    rc = L.ref_ruiz_scaling(lp.m, lp.n, lp.col_ptrs, lp.row_idx, lp.vals, lp.b, lp.c,
                            np.ascontiguousarray(lb, dtype=np.float64), np.ascontiguousarray(ub, dtype=np.float64),
                            np.ascontiguousarray(integer, dtype=np.uint8), max_iter, out["vals"], out["b"], out["c"],
                            out["lb"], out["ub"], out["row_scale"], out["col_scale"])
    assert rc == 0, rc
    return out


def ref_qp(H, c, A, b, lb, ub, max_iter=200):
    """The reference's qp::QPSolver on a dense QP: dict(status, objective, iterations,
    primal_residual, dual_residual, complementarity, x, y, z)."""
    H = np.ascontiguousarray(H, dtype=np.float64)
    n = H.shape[0]
    A = np.ascontiguousarray(np.asarray(A, dtype=np.float64).reshape(-1, n))
    m = A.shape[0]
    f = lambda v: np.ascontiguousarray(v, dtype=np.float64)
    x, y, z, info = np.zeros(n), np.zeros(max(m, 1)), np.zeros(n), np.zeros(5)
    st = reference().ref_qp_solve(n, m, H.ravel(), f(c), A.ravel() if m else np.zeros(1), f(b) if m else np.zeros(1),
                                  f(lb), f(ub), max_iter, x, y, z, info)
    return {"status": st, "objective": info[0], "iterations": int(info[1]), "primal_residual": info[2],
            "dual_residual": info[3], "complementarity": info[4], "x": x, "y": y[:m], "z": z}
