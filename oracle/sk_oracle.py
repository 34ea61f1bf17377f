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


def build(reference_root="/root/reference"):
    """Builds the oracle library, and oracle/_ref when the reference sources exist."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if os.path.isdir(os.path.join(reference_root, "src")):
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
        _o = L
    return _o


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
