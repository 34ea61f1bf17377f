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
