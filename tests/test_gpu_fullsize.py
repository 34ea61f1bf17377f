"""Full-size workloads checked through size-independent properties: the KKT
certificate (rel. primal / dual infeasibility and gap <= 1e-8, x, s > 0) and
agreement of the FP64 and mixed-precision paths."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-8


def test_block_angular_full_size(gpu, oracle):
    sk = gpu
    lp = sk.generate(1, 0)        # m=22000, n=48000
    info_m, x, y, s = sk.solve(lp, precision=1)
    assert info_m["status"] == 0, info_m
    meas = oracle.kkt_measures(lp, x, y, s)
    assert meas["rel_pinf"] <= TOL and meas["rel_dinf"] <= TOL and meas["rel_gap"] <= TOL
    assert meas["min_x"] > 0 and meas["min_s"] > 0
    info_d, xd, yd, sd = sk.solve(lp, precision=0)
    assert info_d["status"] == 0, info_d
    assert abs(info_d["objective"] - info_m["objective"]) / (1 + abs(info_d["objective"])) <= TOL


def test_batch_members_full_certificate(gpu, oracle):
    sk = gpu
    lps = [sk.generate(3, i) for i in range(8)]
    solver = sk.Solver(lps, precision=1)
    solver.run()
    for i, lp in enumerate(lps):
        info, x, y, s = solver.result(i)
        assert info["status"] == 0, (i, info)
        meas = oracle.kkt_measures(lp, x, y, s)
        assert max(meas["rel_pinf"], meas["rel_dinf"], meas["rel_gap"]) <= TOL, (i, meas)
    solver.close()


def test_staircase_rows_beyond_the_large_lp_threshold(gpu, oracle):
    # 13 stages of the family-2 staircase (m = 52000 >= 50000): the automatic ordering
    # picks the row order or nested dissection by flops; certificate, FP64 / mixed
    # agreement and, when recorded, the HiGHS objective (third-party cross-check fixture)
    import json
    import os
    sk = gpu
    lp = sk.staircase(0xC2, 13)
    info_m, x, y, s = sk.solve(lp, precision=1, start=sk.START_MEHROTRA)
    assert info_m["status"] == 0, info_m
    meas = oracle.kkt_measures(lp, x, y, s)
    assert max(meas["rel_pinf"], meas["rel_dinf"], meas["rel_gap"]) <= TOL, meas
    assert meas["min_x"] > 0 and meas["min_s"] > 0
    info_d, *_ = sk.solve(lp, precision=0)
    assert info_d["status"] == 0, info_d
    assert abs(info_d["objective"] - info_m["objective"]) / (1 + abs(info_d["objective"])) <= TOL
    # The primal-dual certificate above (feasibility and gap <= 1e-8, measured on the host in
    # FP64) already bounds the objective's distance from the optimum; a HiGHS objective, when
    # tests/golden/make_highs_objectives.py has recorded one for this LP, cross-checks it.
    fixture = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "highs_large_objectives.json")
    cases = []
    if os.path.exists(fixture):
        with open(fixture) as f:
            cases = [c for c in json.load(f)["cases"] if c["name"] == "staircase_13"]
    for case in cases:
        assert case["digest"]["nnz"] == lp.nnz and case["digest"]["m"] == lp.m
        assert abs(info_m["objective"] - case["objective"]) / (1 + abs(case["objective"])) <= TOL
