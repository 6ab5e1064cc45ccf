"""Path sharding across processes (one per GPU).

Monte Carlo paths are independent, and a path's normals depend only on
(seed, global path index, step).  So a run over M paths splits into
contiguous path blocks, one per rank, with no data exchange during pricing.
The one exchange is at the end: a sum of the per-output (sum x, sum x^2)
pairs, 2 x out FP64 values (torch.distributed, gloo or NCCL), after which
every rank applies the reference's mean / standard-error formula
(rBergLib/rBergomiMT.cpp:404-409) through the library's C++ merge,
rbg_merge_sums.  The merged result equals a single-process run over all M
paths up to the order of the final FP64 additions, when the shard
boundaries fall on the payoff chunks (multiples of 256 G paths).
"""
from __future__ import annotations

import numpy as np


def shard_range(M: int, world_size: int, rank: int) -> tuple[int, int]:
    """(first global path, path count) of `rank`'s contiguous block of M."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("bad world size / rank")
    base, extra = divmod(int(M), world_size)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def merge_sums(s1, s2, M: int):
    """(price, stat) from summed payoffs, by the library's C-ABI merge
    (rbg_merge_sums): price = sum x / M, stat = sqrt(sum x^2 / M - price^2) /
    sqrt(M), as the reference computes them.  s1, s2: [out] after an
    all-reduce, or [n_shards, out] gathered per shard (merged in shard order)."""
    from . import merge_sums as _merge

    return _merge(s1, s2, M)


def allreduce_sums(s1, s2, group=None):
    """Sums (s1, s2) over all ranks of the default torch.distributed group
    (gloo on CPU, NCCL on GPUs); one all-reduce of 2 x out FP64 values."""
    import torch
    import torch.distributed as dist

    both = np.concatenate([np.asarray(s1, np.float64), np.asarray(s2, np.float64)])
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.from_numpy(both).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    t = t.cpu().numpy()
    n = len(both) // 2
    return t[:n], t[n:]


def price_rt_sharded(xi, H, eta, rho, T, K, N, M, seed=0, group=None, **opts):
    """RT prices over M paths with this rank pricing its own path block on
    its GPU (rbg_price_rt_sums), then one all-reduce and the reference's
    moment formula.  Every rank returns the same (price, stat)."""
    import torch.distributed as dist

    from . import price_rt_sums

    ws, rank = dist.get_world_size(group), dist.get_rank(group)
    start, count = shard_range(M, ws, rank)
    if count > 0:
        s1, s2 = price_rt_sums(xi, H, eta, rho, T, K, N, count, seed=seed, path_offset=start, **opts)
    else:
        out = len(H) * len(T)
        s1, s2 = np.zeros(out), np.zeros(out)
    s1, s2 = allreduce_sums(s1, s2, group)
    return merge_sums(s1, s2, M)
