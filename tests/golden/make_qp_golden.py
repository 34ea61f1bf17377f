"""Records the reference's own convex QP solver (qp::QPSolver, src/qp/qp_solver.cpp,
built from its sources into oracle/_ref by `make -C oracle ref`) on the reference's
QP unit-test problems and on seeded random separable and coupled QPs
(tests/qp_cases.py), with all inputs, into tests/golden/reference_qp.json.

Run where the reference is mounted:
    SK_REFERENCE_ROOT=<reference root> python tests/golden/make_qp_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import qp_cases as qc  # noqa: E402
import sk_oracle as so  # noqa: E402


def main():
    so.build()
    assert so.have_reference(), "oracle/_ref not built (set SK_REFERENCE_ROOT)"
    problems = []
    for name, (H, c, A, b, lb, ub, *_rest) in sorted(qc.REFERENCE_CASES.items()):
        problems.append((name, H, c, A, b, lb, ub, 200))
    problems.append(("infeasible",) + qc.INFEASIBLE_CASE + (200,))
    problems.append(("iteration_limit",) + qc.ITERLIMIT_CASE + (2,))
    for k, (m, n, d, coupled, bounded) in enumerate([(10, 24, 0.25, False, True), (20, 50, 0.1, False, True),
                                                     (30, 80, 0.08, True, True), (15, 40, 0.15, True, False),
                                                     (40, 120, 0.05, False, False), (25, 70, 0.1, True, True)]):
        H, c, A, b, lb, ub = qc.random_qp(m, n, d, 700 + k, coupled=coupled, bounded=bounded)
        problems.append(("random_%s_%dx%d" % ("coupled" if coupled else "separable", m, n), H, c, A, b, lb, ub, 200))
    cases = []
    for name, H, c, A, b, lb, ub, it in problems:
        H = np.asarray(H, dtype=float)
        A = np.asarray(A, dtype=float).reshape(-1, H.shape[0])
        r = so.ref_qp(H, c, A, b, lb, ub, max_iter=it)
        cases.append({"name": name, "H": H.tolist(), "c": list(map(float, c)), "A": A.ravel().tolist(),
                      "m": A.shape[0], "b": list(map(float, b)), "lb": list(map(float, lb)),
                      "ub": list(map(float, ub)), "max_iter": it, "status": r["status"],
                      "iterations": r["iterations"], "objective": r["objective"], "x": r["x"].tolist(),
                      "y": r["y"].tolist(), "z": r["z"].tolist(), "primal_residual": r["primal_residual"],
                      "dual_residual": r["dual_residual"], "complementarity": r["complementarity"]})
        print(name, r["status"], r["iterations"], r["objective"])
    with open(os.path.join(HERE, "reference_qp.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_qp_golden.py", "source": "reference qp::QPSolver",
                   "cases": cases}, f)


if __name__ == "__main__":
    main()
