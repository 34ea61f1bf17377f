"""Members of the 512-LP family-3 batch pinned to the reference's own CPU simplex.

tests/golden/reference_family3_objectives.json holds, for every member with
m <= 800 (216 of 512), the objective that the reference's Phase-I + primal simplex
(src/simplex/phase1.cpp:124-449, built from its sources into oracle/_ref by
oracle/Makefile) reached, and SciPy's HiGHS dual simplex and interior-point
objectives at 1e-10 tolerances as third-party cross-checks
(tests/golden/make_family3_golden.py). The "consensus" objective is a value on
which two of the three agree to 1e-9 relative (215 of 216 members; on member 257
the three differ by 1.4e-9 to 3.1e-9 and HiGHS's dual simplex value stands in).
The reference's simplex stops within its own tolerances (1e-6) of the optimum:
on 31 of its 213 solved members its objective differs from the consensus by more
than 1e-8 relative (up to 7e-7), and 3 members end at its iteration limit; on
member 373 HiGHS's dual simplex is the outlier (2.8e-8 from the other two).

Those members are solved together in one batch on the device, in mixed precision
with the learned start and in plain FP64. Every LP must
  * reach the consensus objective within 1e-8 relative, with a host FP64
    certificate (relative primal / dual infeasibility and gap <= 1e-8, x, s > 0);
  * reach the reference's objective within 1e-8 relative wherever the reference
    agrees with the consensus to 1e-9 (171 members), and within the reference's
    own 1e-6 everywhere it finished."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-8
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "reference_family3_objectives.json")
WEIGHTS = os.path.join(os.path.dirname(HERE), "soverign-gpu-accelerator-_gb300", "weights",
                       "learned_start_family3.npy")


def solved_cases():
    with open(FIXTURE) as f:
        return [c for c in json.load(f)["cases"] if c.get("highs_objective") is not None]


def test_fixture_covers_the_small_members():
    with open(FIXTURE) as f:
        d = json.load(f)
    assert d["family"] == 3 and d["max_m"] >= 800
    assert d["solved"] >= 150
    assert all(c["m"] <= d["max_m"] for c in d["cases"])
    agree = [c for c in d["cases"] if c.get("ref_vs_consensus") is not None and c["ref_vs_consensus"] <= 1e-9]
    assert len(agree) >= 150
    assert sum(c.get("consensus_objective") is not None for c in d["cases"]) >= 200


@pytest.mark.parametrize("arm", ["mixed_learned", "plain_fp64"])
def test_batch_matches_reference_simplex(gpu, oracle, arm):
    sk = gpu
    cases = solved_cases()
    lps = []
    for c in cases:
        lp = sk.generate(3, c["instance"])
        assert (lp.m, lp.n, lp.nnz) == (c["digest"]["m"], c["digest"]["n"], c["digest"]["nnz"])
        assert abs(float(np.sum(lp.vals)) - c["digest"]["sum_vals"]) <= 1e-9 * (1 + abs(c["digest"]["sum_vals"]))
        lps.append(lp)
    if arm == "mixed_learned":
        solver = sk.Solver(lps, precision=sk.PREC_MIXED, start=sk.START_LEARNED)
        net = sk.Gnn(1)
        net.load(WEIGHTS)
        solver.set_gnn(net)
    else:
        net = None
        solver = sk.Solver(lps, precision=sk.PREC_FP64, start=sk.START_UNIT)
    solver.run()
    bad = []
    pinned = 0
    for k, (lp, c) in enumerate(zip(lps, cases)):
        info, x, y, s = solver.result(k)
        obj = info["objective"]
        target = c["consensus_objective"] if c.get("consensus_objective") is not None else c["highs_objective"]
        err_h = abs(obj - target) / (1 + abs(target))
        err_r = abs(obj - c["ref_objective"]) / (1 + abs(c["ref_objective"])) if c["ref_status"] == 0 else 0.0
        tol_r = TOL if c.get("ref_vs_consensus", 1.0) <= 1e-9 else 1e-6
        pinned += c["ref_status"] == 0 and tol_r == TOL
        meas = oracle.kkt_measures(lp, x, y, s)
        cert = max(meas["rel_pinf"], meas["rel_dinf"], meas["rel_gap"])
        if (info["status"] != 0 or err_h > TOL or err_r > tol_r or cert > TOL or meas["min_x"] <= 0 or
                meas["min_s"] <= 0):
            bad.append((c["instance"], info["status"], err_h, err_r, cert))
    solver.close()
    if net is not None:
        net.close()
    assert not bad, bad[:10]
    assert pinned >= 150
