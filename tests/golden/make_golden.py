"""Generates tests/golden/*.json from the reference's own CPU code (oracle/_ref,
built from the reference sources by `make -C oracle ref`).

Run in a container where the reference is mounted:
    python tests/golden/make_golden.py
The fixtures let the GPU tests (which run where the reference is absent) check
against the reference's results: simplex objectives of small LPs and the
reference's ordering / elimination tree / L pattern for a few patterns.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "soverign-gpu-accelerator-_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import sankhya_gb300 as sk  # noqa: E402
import sk_oracle as so  # noqa: E402


def lp_digest(lp):
    return {"m": lp.m, "n": lp.n, "nnz": lp.nnz, "sum_vals": float(np.sum(lp.vals)), "sum_b": float(np.sum(lp.b)),
            "sum_c": float(np.sum(lp.c)), "sum_rows": int(np.sum(lp.row_idx, dtype=np.int64))}


def main():
    so.build()
    assert so.have_reference(), "oracle/_ref not built (needs the reference sources)"
    cases = []
    for name, lp in [("family0_0", sk.generate(0, 0)), ("family0_1", sk.generate(0, 1)),
                     ("random_60x150", sk.random_lp(60, 150, 0.06, 11)),
                     ("random_200x450", sk.random_lp(200, 450, 0.02, 12)),
                     ("random_300x700", sk.random_lp(300, 700, 0.015, 13))]:
        st, obj, x = so.ref_simplex(lp)
        cases.append({"name": name, "digest": lp_digest(lp), "ref_status": st, "ref_objective": obj})
        print(name, st, repr(obj))
    sym = []
    for (m, n, d, seed) in [(40, 90, 0.08, 21), (120, 260, 0.03, 22)]:
        lp = sk.random_lp(m, n, d, seed)
        rp, ci, _ = lp.csr()
        P = so.ref_min_degree(m, n, rp, ci)
        Pinv, parent, Lrp, Lci = so.ref_symbolic(m, n, rp, ci, P)
        sym.append({"m": m, "n": n, "density": d, "seed": seed, "digest": lp_digest(lp), "P": P.tolist(),
                    "parent": parent.tolist(), "L_row_ptrs": Lrp.tolist(), "L_cols": Lci.tolist()})
    with open(os.path.join(HERE, "reference_lp_objectives.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "source": "reference CPU Phase-I + primal simplex",
                   "cases": cases}, f, indent=1)
    with open(os.path.join(HERE, "reference_symbolic.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "source": "reference compute_amd_ordering + compute_symbolic_factorization", "cases": sym}, f)


if __name__ == "__main__":
    main()
