"""The oracle's restatement of the seeded LP generator (oracle/lpgen_oracle.c)
gives the same arrays as the product's generator (csrc/gen/lpgen.cpp), so the
CPU baselines can build the benchmark's LPs without loading the product."""
import numpy as np
import pytest

KEYS = ("col_ptrs", "row_idx", "vals", "b", "c")


def _same(a, b):
    assert (a.m, a.n) == (b.m, b.n)
    for k in KEYS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.parametrize("family,instance", [(0, 0), (0, 3), (1, 0)] + [(3, k) for k in (0, 3, 33, 100, 257, 511)])
def test_family_members_identical(sk, oracle, family, instance):
    _same(sk.generate(family, instance), oracle.generate(family, instance))


def test_random_and_block_angular_identical(sk, oracle):
    _same(sk.random_lp(120, 260, 0.04, 2024), oracle.random_lp(120, 260, 0.04, 2024))
    _same(sk.block_angular(0xC1, 1, 500, 1200, 50, 5), oracle.block_angular(0xC1, 1, 500, 1200, 50, 5))
