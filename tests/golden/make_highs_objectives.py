"""Independent objectives of the large generated LPs from SciPy's bundled HiGHS.

The FP64 CPU oracle cannot factor these sizes in reasonable time (family 2:
1.8e12 flops per factorisation), so the device results at these sizes are
checked against HiGHS (a third-party solver, cross-check only) plus their own
FP64 residuals. Run once where SciPy is installed:
    python tests/golden/make_highs_objectives.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "soverign-gpu-accelerator-_gb300"))

import sankhya_gb300 as sk  # noqa: E402


def digest(lp):
    return {"m": lp.m, "n": lp.n, "nnz": lp.nnz, "sum_vals": float(np.sum(lp.vals)), "sum_b": float(np.sum(lp.b)),
            "sum_c": float(np.sum(lp.c))}


def highs(lp, method):
    import scipy.sparse as spx
    from scipy.optimize import linprog
    A = spx.csc_matrix((lp.vals, lp.row_idx, lp.col_ptrs), shape=(lp.m, lp.n))
    t = time.time()
    res = linprog(lp.c, A_eq=A, b_eq=lp.b, bounds=(0, None), method=method,
                  options={"primal_feasibility_tolerance": 1e-10, "dual_feasibility_tolerance": 1e-10})
    return res, time.time() - t


def record(out, case):
    """Adds one case to the fixture under an exclusive lock (several runs may share it)."""
    import fcntl
    with open(out + ".lock", "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        cases = json.load(open(out))["cases"] if os.path.exists(out) else []
        cases = [c for c in cases if c["name"] != case["name"]] + [case]
        with open(out, "w") as f:
            json.dump({"generator": "tests/golden/make_highs_objectives.py",
                       "source": "scipy.optimize.linprog (HiGHS), tolerances 1e-10", "cases": cases}, f, indent=1)


def main():
    """Usage: make_highs_objectives.py [case names...] (default: all cases)."""
    out = os.path.join(HERE, "highs_large_objectives.json")
    todo = [("family1_0", lambda: sk.generate(1, 0), "highs-ipm"),
            ("staircase_13", lambda: sk.staircase(0xC2, 13), "highs-ipm"),
            ("family2_0", lambda: sk.generate(2, 0), "highs-ipm")]
    want = set(sys.argv[1:]) or {t[0] for t in todo}
    for name, make, method in todo:
        if name not in want:
            continue
        method = os.environ.get("HIGHS_METHOD", method)
        lp = make()
        res, secs = highs(lp, method)
        print(name, res.status, repr(res.fun), "%.1f s" % secs, flush=True)
        if res.status != 0:
            continue
        record(out, {"name": name, "digest": digest(lp), "method": method, "objective": float(res.fun),
                     "seconds": secs})


if __name__ == "__main__":
    main()
