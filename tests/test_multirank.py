"""The N > 1 host path on CPU: two gloo ranks (127.0.0.1), as torchrun would start
them on two GPUs. A batch of independent LPs is sharded over the ranks
(sharding.shard_lps), each rank solves its shard, and the per-LP results meet on
rank 0 in one gather; the bench's max-over-ranks timing (bench.barrier_max) is the
only other collective. The GPU solve is replaced by the CPU oracle here (this
is a test of the host logic; the device solve of each shard is the single-GPU
path the other tests cover)."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "soverign-gpu-accelerator-_gb300")

torch = pytest.importorskip("torch")


def _paths():
    for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), HERE):
        if p not in sys.path:
            sys.path.insert(0, p)


def _small_batch(sk):
    sizes = [(60, 150, 0.06), (90, 200, 0.05), (40, 100, 0.08), (120, 260, 0.04), (70, 160, 0.06),
             (50, 120, 0.07), (100, 230, 0.045)]
    return [sk.random_lp(m, n, d, 300 + k) for k, (m, n, d) in enumerate(sizes)]


def _rank_main(rank, world, port, outdir):
    _paths()
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import sankhya_gb300 as sk
        import sharding
        import sk_oracle
        lps = _small_batch(sk)
        shards = sharding.shard_lps([sharding.lp_cost(lp.m, lp.n, lp.nnz) for lp in lps], world)
        mine = {}
        for k in shards[rank]:
            r, *_ = sk_oracle.ipm_solve(lps[k])
            mine[k] = (r["status"], r["objective"])
        merged = sharding.gather_results(mine, dist, rank, world)
        slowest = bench.barrier_max(dist, 1.5 + rank)
        with open(os.path.join(outdir, "rank%d.txt" % rank), "w") as f:
            f.write("%r\n%r\n%r\n" % (shards, merged, slowest))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_lps_covers_every_lp_once_and_balances():
    _paths()
    import sharding
    costs = [sharding.lp_cost(m, 2 * m, 20 * m) for m in (200, 5000, 800, 1500, 300, 4000, 2500, 900, 600)]
    for world in (1, 2, 3, 4, 8, 12):
        shards = sharding.shard_lps(costs, world)
        assert len(shards) == world
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(costs)))
        assert shards == sharding.shard_lps(costs, world)          # every rank computes the same split
        loads = [sum(costs[i] for i in s) for s in shards]
        assert max(loads) - min(loads) <= max(costs)               # longest-first bound
    assert sharding.shard_lps([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        sharding.shard_lps(costs, 0)
    # dense (family-3-like) members cost m^3/3; a sparse proxy otherwise
    assert sharding.lp_cost(1000, 2500, 30000) == pytest.approx(1000 ** 3 / 3.0)
    assert sharding.lp_cost(100000, 250000, 400000) == pytest.approx(400000.0 ** 2 / 100000)


def test_gather_rejects_an_lp_solved_twice():
    _paths()
    import sharding

    class FakeDist:   # two ranks that both claim LP 3, seen from rank 0
        @staticmethod
        def gather_object(obj, bucket, dst=0):
            bucket[0] = obj
            bucket[1] = {3: "x"}

    with pytest.raises(RuntimeError):
        sharding.gather_results({3: "y"}, FakeDist, 0, 2)
    assert sharding.gather_results({1: "a"}, None, 0, 1) == {1: "a"}


def test_two_gloo_ranks_shard_solve_and_gather(tmp_path):
    _paths()
    import sankhya_gb300 as sk
    import sk_oracle
    sk.lib()
    sk_oracle.oracle()
    world = 2
    torch.multiprocessing.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    import ast
    texts = [open(os.path.join(str(tmp_path), "rank%d.txt" % r)).read().splitlines() for r in range(world)]
    shards = ast.literal_eval(texts[0][0])
    merged = ast.literal_eval(texts[0][1])
    assert ast.literal_eval(texts[1][1]) is None                   # only rank 0 receives the results
    assert shards == ast.literal_eval(texts[1][0])                 # both ranks agree on the split
    assert all(len(s) > 0 for s in shards)
    lps = _small_batch(sk)
    assert sorted(merged) == list(range(len(lps)))
    for k, lp in enumerate(lps):                                   # same results as one process solving all
        r, *_ = sk_oracle.ipm_solve(lp)
        assert merged[k] == (r["status"], r["objective"])
    assert float(texts[0][2]) == float(texts[1][2]) == 2.5         # max over ranks on both ranks
