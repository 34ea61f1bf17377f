"""Sharding of a batch of independent LPs over the ranks of a job (one process per GPU).

A batch of LPs has no exchange step: every LP is solved by exactly one rank, and
the only communication is one gather of the per-LP results to rank 0 after the
solves. The LPs are assigned longest-first to the least-loaded rank by their
estimated factorisation cost (m^3 / 3 when A A^T is dense, as for the uneven
family-3 batches; otherwise nnz(A)^2 / m as a sparse proxy), so
ranks finish at about the same time. The assignment depends only on the sizes and
the world size, so every rank computes the same shards without talking.
"""


def lp_cost(m, n, nnz):
    """Estimated flops of one factorisation of A Theta A^T for an m x n LP with nnz entries."""
    m, n = max(1, int(m)), max(1, int(n))
    d = nnz / float(m * n)
    if n * d * d >= 0.2:      # two rows share a column with probability ~ n d^2: A A^T is dense
        return m ** 3 / 3.0
    return float(nnz) ** 2 / m


def shard_lps(costs, world):
    """Indices of the LPs each rank solves: longest-first to the least-loaded rank (lowest rank
    on ties). Returns `world` lists of indices, each in increasing order."""
    if world < 1:
        raise ValueError("world size must be positive")
    load = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def gather_results(results, dist, rank, world):
    """Gathers each rank's {lp_index: result} dict to rank 0 (the one communication of a
    sharded batch). Rank 0 gets the merged dict, other ranks None. Works on any
    torch.distributed backend (gloo on CPU, nccl on GPUs)."""
    if dist is None or world == 1:
        return dict(results)
    bucket = [None] * world if rank == 0 else None
    dist.gather_object(dict(results), bucket, dst=0)
    if rank != 0:
        return None
    merged = {}
    for part in bucket:
        for k, v in part.items():
            if k in merged:
                raise RuntimeError("LP %r solved by two ranks" % (k,))
            merged[k] = v
    return merged
