"""Records the reference's own CPU simplex objective (oracle/_ref, built from the
reference sources by `make -C oracle ref`; reference src/simplex/phase1.cpp:124-449
`simplex::solve_with_phase1`) for the members of the 512-LP family-3 batch
(m ~ logUniform[200, 5000], n = ceil(m U[2, 3]), density 0.5-2 %, instances
0..511) whose row count is at most --max-m. Each member runs in its own process
under a per-instance time cap; members that hit the cap are recorded as DNF.

Run where the reference is mounted (it cannot run on the GPU host):
    SK_REFERENCE_ROOT=<reference root> python tests/golden/make_family3_golden.py [--max-m 800] [--cap 240] [-j 6]
Writes tests/golden/reference_family3_objectives.json. With --add-highs the
existing file gets, per member, the objective of SciPy's HiGHS dual simplex at
1e-10 feasibility tolerances (a third-party cross-check: the reference's simplex
stops within its own tolerances, about 1e-6, of the optimum on some members).
"""
import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "soverign-gpu-accelerator-_gb300")
ORACLE = os.path.join(ROOT, "oracle")
OUT = os.path.join(HERE, "reference_family3_objectives.json")

_ONE = r"""
import json, sys, time
sys.path.insert(0, %r); sys.path.insert(0, %r); sys.path.insert(0, %r)
import sankhya_gb300 as sk, sk_oracle as so
from make_golden import lp_digest
k = int(sys.argv[1])
lp = sk.generate(3, k)
t = time.perf_counter()
st, obj, _ = so.ref_simplex(lp)
print(json.dumps({"instance": k, "m": lp.m, "n": lp.n, "digest": lp_digest(lp), "ref_status": st,
                  "ref_objective": obj, "ref_seconds": time.perf_counter() - t}))
""" % (PKG, ORACLE, HERE)


def run_one(k, cap):
    t = time.perf_counter()
    try:
        p = subprocess.run([sys.executable, "-c", _ONE, str(k)], capture_output=True, text=True, timeout=cap)
    except subprocess.TimeoutExpired:
        return {"instance": k, "ref_status": "DNF", "cap_s": cap}
    if p.returncode != 0:
        return {"instance": k, "ref_status": "error", "stderr": p.stderr[-400:], "wall_s": time.perf_counter() - t}
    return json.loads(p.stdout.strip().splitlines()[-1])


def add_highs():
    import scipy.optimize as so_
    import scipy.sparse as sp
    sys.path.insert(0, PKG)
    import sankhya_gb300 as sk
    with open(OUT) as f:
        d = json.load(f)
    for c in d["cases"]:
        lp = sk.generate(3, c["instance"])
        A = sp.csc_matrix((lp.vals, lp.row_idx, lp.col_ptrs), shape=(lp.m, lp.n))
        tols = {"primal_feasibility_tolerance": 1e-10, "dual_feasibility_tolerance": 1e-10}
        r = so_.linprog(lp.c, A_eq=A, b_eq=lp.b, bounds=(0, None), method="highs-ds", options=tols)
        c["highs_objective"] = float(r.fun) if r.status == 0 else None
        r2 = so_.linprog(lp.c, A_eq=A, b_eq=lp.b, bounds=(0, None), method="highs-ipm", options=tols)
        c["highs_ipm_objective"] = float(r2.fun) if r2.status == 0 else None
        # consensus: a value on which two of the three solvers agree to 1e-9 relative
        vals = [v for v in (c["ref_objective"] if c["ref_status"] == 0 else None, c["highs_objective"],
                            c["highs_ipm_objective"]) if v is not None]
        c["consensus_objective"] = None
        for a_ in range(len(vals)):
            for b_ in range(a_ + 1, len(vals)):
                if c["consensus_objective"] is None and \
                        abs(vals[a_] - vals[b_]) <= 1e-9 * (1.0 + abs(vals[b_])):
                    c["consensus_objective"] = vals[a_]
        if c["ref_status"] == 0 and c["consensus_objective"] is not None:
            c["ref_vs_consensus"] = abs(c["ref_objective"] - c["consensus_objective"]) / \
                (1.0 + abs(c["consensus_objective"]))
        print(c["instance"], c.get("consensus_objective"), c.get("ref_vs_consensus"), flush=True)
    d["highs"] = ("scipy.optimize.linprog(method='highs-ds' and 'highs-ipm'), primal / dual feasibility "
                  "tolerances 1e-10; consensus = a value two of reference, highs-ds, highs-ipm agree on to 1e-9")
    with open(OUT, "w") as f:
        json.dump(d, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--add-highs", action="store_true")
    ap.add_argument("--max-m", type=int, default=800)
    ap.add_argument("--cap", type=float, default=240.0)
    ap.add_argument("-j", type=int, default=max(1, (os.cpu_count() or 2) - 2))
    a = ap.parse_args()
    if a.add_highs:
        add_highs()
        return
    sys.path.insert(0, PKG)
    sys.path.insert(0, ORACLE)
    import sankhya_gb300 as sk
    import sk_oracle as so
    so.build()
    assert so.have_reference(), "oracle/_ref not built (needs the reference sources)"
    sizes = {k: sk.generate(3, k).m for k in range(512)}
    todo = sorted((k for k in sizes if sizes[k] <= a.max_m), key=lambda k: sizes[k])
    cases = []
    with cf.ThreadPoolExecutor(max_workers=a.j) as ex:
        for r in ex.map(lambda k: run_one(k, a.cap), todo):
            r.setdefault("m", sizes[r["instance"]])
            cases.append(r)
            print(r["instance"], r["m"], r["ref_status"], r.get("ref_objective"), "%.1fs" % r.get("ref_seconds", -1),
                  flush=True)
    cases.sort(key=lambda r: r["instance"])
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_family3_golden.py",
                   "source": "reference CPU Phase-I + primal simplex (simplex::solve_with_phase1)",
                   "family": 3, "instances": "0..511", "max_m": a.max_m, "cap_s": a.cap,
                   "attempted": len(todo), "solved": sum(1 for c in cases if c["ref_status"] == 0),
                   "dnf": [c["instance"] for c in cases if c["ref_status"] == "DNF"],
                   "not_attempted": "members with m > %d" % a.max_m, "cases": cases}, f, indent=1)


if __name__ == "__main__":
    main()
