"""Writes tests/golden/reference_presolve.json from the reference's own
presolve::apply_ruiz_scaling (src/presolve/scaling.cpp), compiled from the
reference sources into oracle/_ref by `make -C oracle ref`.

Run in a container where the reference is mounted:
    python tests/golden/make_presolve_golden.py
Small cases keep every output array; larger ones keep a SHA-256 digest of each
array's little-endian FP64 bytes (the product must match them bit for bit)."""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "soverign-gpu-accelerator-_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import presolve_cases  # noqa: E402
import sankhya_gb300 as sk  # noqa: E402
import sk_oracle as so  # noqa: E402

KEYS = ("vals", "b", "c", "lb", "ub", "row_scale", "col_scale")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def main():
    so.build()
    assert so.have_reference(), "oracle/_ref not built (needs the reference sources)"
    out = []
    for name, lp, lb, ub, integer, it in presolve_cases.cases(sk, large=True):
        r = so.ref_ruiz(lp, lb, ub, integer, it)
        case = {"name": name, "m": lp.m, "n": lp.n, "nnz": lp.nnz, "max_iterations": it,
                "digest": {k: digest(r[k]) for k in KEYS}}
        if lp.nnz <= 1000:
            case["arrays"] = {k: [float(x) if np.isfinite(x) else repr(float(x)) for x in r[k]] for k in KEYS}
        out.append(case)
        print(name, lp.m, lp.n, lp.nnz)
    with open(os.path.join(HERE, "reference_presolve.json"), "w") as f:
        json.dump({"source": "reference presolve::apply_ruiz_scaling (src/presolve/scaling.cpp), oracle/_ref",
                   "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
