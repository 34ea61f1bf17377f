"""Product symbolic analysis (C ABI) against the reference: bit-exact ordering,
elimination tree and L pattern (golden fixtures from the reference build, and the
reference build itself when present)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_reference_golden_vectors(sk):
    # tests/unit/test_ipm_symbolic.cpp (star, cycle) and test_gpu_kkt.cu ordering
    rp = np.array([0, 4, 5, 6, 7, 8], dtype=np.int32)
    ci = np.array([0, 1, 2, 3, 0, 1, 2, 3], dtype=np.int32)
    P = sk.amd_ordering(5, 5, rp, ci)
    assert P.tolist() == [1, 2, 3, 0, 4]
    Pinv, parent, Lrp, Lci = sk.symbolic(5, 5, rp, ci, P)
    assert parent.tolist() == [3, 3, 3, 4, -1] and Lrp[5] == 4
    rp = np.array([0, 2, 4, 6, 8, 9], dtype=np.int32)
    ci = np.array([0, 3, 0, 1, 1, 2, 2, 3, 4], dtype=np.int32)
    P = sk.amd_ordering(5, 5, rp, ci)
    assert P.tolist() == [4, 0, 1, 2, 3]
    Pinv, parent, Lrp, Lci = sk.symbolic(5, 5, rp, ci, P)
    assert Lrp.tolist() == [0, 0, 0, 1, 2, 5]
    assert Lci.tolist() == [1, 2, 1, 2, 3]
    assert parent.tolist() == [-1, 2, 3, 4, -1]
    rp = np.array([0, 3, 5, 7], dtype=np.int32)
    ci = np.array([0, 3, 4, 1, 3, 2, 4], dtype=np.int32)
    assert sk.amd_ordering(3, 5, rp, ci).tolist() == [1, 0, 2]


def test_symbolic_matches_reference_fixtures(sk):
    with open(os.path.join(HERE, "golden", "reference_symbolic.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        lp = sk.random_lp(c["m"], c["n"], c["density"], c["seed"])
        assert lp.nnz == c["digest"]["nnz"]
        rp, ci, _ = lp.csr()
        P = sk.amd_ordering(lp.m, lp.n, rp, ci)
        assert P.tolist() == c["P"]
        Pinv, parent, Lrp, Lci = sk.symbolic(lp.m, lp.n, rp, ci, P)
        assert parent.tolist() == c["parent"]
        assert Lrp.tolist() == c["L_row_ptrs"]
        assert Lci.tolist() == c["L_cols"]


def test_symbolic_matches_oracle_and_reference_build(sk, oracle):
    for (m, n, d, seed) in [(30, 60, 0.1, 5), (150, 320, 0.03, 6), (500, 1000, 0.01, 0xC0)]:
        lp = sk.random_lp(m, n, d, seed)
        rp, ci, _ = lp.csr()
        P = sk.amd_ordering(m, n, rp, ci)
        assert np.array_equal(P, oracle.min_degree(m, n, rp, ci))
        a = sk.symbolic(m, n, rp, ci, P)
        b = oracle.symbolic(m, n, rp, ci, P)
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
        if oracle.have_reference():
            assert np.array_equal(P, oracle.ref_min_degree(m, n, rp, ci))
            for u, v in zip(a, oracle.ref_symbolic(m, n, rp, ci, P)):
                assert np.array_equal(u, v)


def test_fill_ordering_is_permutation_and_competitive(sk):
    lp = sk.random_lp(400, 900, 0.012, 9)
    rp, ci, _ = lp.csr()
    Pf = sk.fill_ordering(lp.m, lp.n, rp, ci)
    assert sorted(Pf.tolist()) == list(range(lp.m))
    Pr = sk.amd_ordering(lp.m, lp.n, rp, ci)
    nf = len(sk.symbolic(lp.m, lp.n, rp, ci, Pf)[3])
    nr = len(sk.symbolic(lp.m, lp.n, rp, ci, Pr)[3])
    assert nf <= 1.15 * nr


def test_symbolic_rejects_bad_permutation(sk):
    rp = np.array([0, 1, 2], dtype=np.int32)
    ci = np.array([0, 1], dtype=np.int32)
    with pytest.raises(RuntimeError):
        sk.symbolic(2, 2, rp, ci, np.array([0, 0], dtype=np.int32))


def test_dissection_ordering_is_permutation(sk):
    # several components (the staircase has coupling rows without arcs) and a random LP
    for lp in (sk.staircase(3, 4, 100, 100, 200, 800), sk.random_lp(600, 1400, 0.008, 4)):
        rp, ci, _ = lp.csr()
        P = sk.dissection_ordering(lp.m, lp.n, rp, ci)
        assert sorted(P.tolist()) == list(range(lp.m))
        st = sk.plan_stats(lp, sk.ORDER_DISSECTION)
        assert st["ordering_used"] == 4 and st["consistent"] == 1


def test_dissection_beats_minimum_degree_on_staircase(sk):
    # 8 stages of 250 supply + 250 demand + 500 capacity rows: the coupling rows of
    # each stage separate the stages, which greedy minimum degree interleaves
    lp = sk.staircase(7, 8, 250, 250, 500, 2000)
    nd = sk.plan_stats(lp, sk.ORDER_DISSECTION)
    md = sk.plan_stats(lp, sk.ORDER_MINDEG)
    assert nd["consistent"] == 1 and md["ordering_used"] == 0
    assert nd["flops_factor"] < 0.75 * md["flops_factor"]


def test_auto_ordering_of_a_large_staircase(sk):
    # >= 50000 rows: the automatic choice takes the cheaper of the row order and
    # nested dissection (13 stages, m = 52000)
    lp = sk.staircase(0xC2, 13)
    auto = sk.plan_stats(lp, sk.ORDER_AUTO)
    nat = sk.plan_stats(lp, sk.ORDER_NATURAL)
    assert auto["ordering_used"] in (2, 4) and auto["consistent"] == 1
    assert auto["flops_factor"] <= nat["flops_factor"] * (1 + 1e-12)


def _row_spans(lp):
    rp, ci, _ = lp.csr()
    lo = np.minimum.reduceat(ci, rp[:-1])
    hi = np.maximum.reduceat(ci, rp[:-1])
    return rp, ci, hi - lo + 1


def test_linking_rows_are_ordered_last(sk):
    # block-angular LP: rows spanning more than a quarter of the columns (the linking rows)
    # come last; the blocks before them are ordered by minimum degree
    lp = sk.block_angular(0xB1, 12, 150, 360, 200, 4)
    rp, ci, span = _row_spans(lp)
    wide = span * 4 > lp.n
    assert 0 < wide.sum() <= lp.m // 4
    P = sk.fill_ordering(lp.m, lp.n, rp, ci)
    assert sorted(P.tolist()) == list(range(lp.m))
    nw = int(wide.sum())
    assert wide[P[-nw:]].all() and not wide[P[:-nw]].any()
    assert P[-nw:].tolist() == sorted(P[-nw:].tolist())      # in their given order


def test_constrained_ordering_is_repeatable_and_not_worse(sk):
    # the blocks are ordered on worker threads; the result must not depend on scheduling,
    # and the constraint must not cost fill against the natural order
    lp = sk.block_angular(0xB2, 16, 120, 300, 160, 4)
    rp, ci, _ = _row_spans(lp)
    first = sk.fill_ordering(lp.m, lp.n, rp, ci)
    for _ in range(5):
        assert np.array_equal(sk.fill_ordering(lp.m, lp.n, rp, ci), first)
    auto = sk.plan_stats(lp, ordering=sk.ORDER_MINDEG)
    natural = sk.plan_stats(lp, ordering=sk.ORDER_NATURAL)
    assert auto["consistent"] == 1.0
    assert auto["flops_factor"] <= natural["flops_factor"]


def test_family1_ordering_flops(sk):
    # the family-1 LP (40 blocks + 2000 linking rows): the constrained minimum degree keeps
    # the factorisation at or below the 2.121e10 flops of the unconstrained ordering
    lp = sk.generate(1, 0)
    st = sk.plan_stats(lp)
    assert st["consistent"] == 1.0
    assert st["flops_factor"] <= 2.121e10 * 1.0001


def test_family1_plan_is_pinned(sk):
    # The automatic plan of the family-1 LP as the GB300 runs were measured with (constrained
    # minimum degree, relaxed supernodes, Khatri-Rao map): the parallel host analysis must give
    # exactly these integers whatever the thread count.
    st = sk.plan_stats(sk.generate(1, 0))
    want = {"supernodes": 2222, "levels": 8, "nnz_factor": 19714304, "flops_factor": 20996637444,
            "front_entries": 170729700, "slots": 718906, "khatri_rao_entries": 1008000, "max_front_rows": 2000}
    assert {k: int(st[k]) for k in want} == want
