"""Path sharding across ranks (the multi-GPU form of the pricer), tested on
CPU with a world-size-2 gloo group: each rank prices its contiguous block of
paths (here with the oracle standing in for its GPU), one all-reduce merges
the (sum x, sum x^2) pairs, and the merged price equals a single-process run
over all paths."""
import os
import socket

import numpy as np
import pytest

XI, H, ETA, RHO = 0.235 ** 2, [0.07, 0.2], [1.9, 1.2], [-0.9, -0.6]
T, K = [0.5, 1.0], [0.9, 1.1]
N, M, SEED = 32, 3001, 17


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from oracle import oracle as O
    from rbergomi_gb300 import shards

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    start, count = shards.shard_range(M, ws, rank)
    pay = O.payoffs_rt(XI, H, ETA, RHO, T, K, O.normals_f64(SEED, count, N, 2, path0=start))
    s1, s2 = shards.allreduce_sums(pay.sum(0), (pay * pay).sum(0))
    price, stat = shards.merge_sums(s1, s2, M)
    q.put((rank, price, stat))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_ranges_cover_paths_once():
    from rbergomi_gb300.shards import shard_range
    for M_, ws in ((10, 3), (7, 8), (1 << 20, 4), (0, 2)):
        blocks = [shard_range(M_, ws, r) for r in range(ws)]
        assert sum(c for _, c in blocks) == M_
        pos = 0
        for s, c in blocks:
            assert s == pos
            pos += c
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_two_rank_merge_equals_single_process(oracle):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    pay = oracle.payoffs_rt(XI, H, ETA, RHO, T, K, oracle.normals_f64(SEED, M, N, 2))
    want_p, want_s = oracle.reduce(pay)
    for _, price, stat in got:
        np.testing.assert_allclose(price, want_p, rtol=1e-13, atol=0)
        np.testing.assert_allclose(stat, want_s, rtol=1e-9, atol=0)


@pytest.mark.gpu
def test_sharded_single_rank_matches_direct():
    """On one GPU: the sharded call over a one-rank group equals the direct call."""
    import torch.distributed as dist

    import rbergomi_gb300 as R
    from rbergomi_gb300 import shards

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{_free_port()}", rank=0, world_size=1)
    try:
        for prec in (R.FP64, R.MIXED):
            p, s = shards.price_rt_sharded(XI, H, ETA, RHO, T, K, 256, 1 << 15, seed=SEED, precision=prec)
            dp, ds, _ = R.price_rt(XI, H, ETA, RHO, T, K, 256, 1 << 15, seed=SEED, precision=prec)
            np.testing.assert_allclose(p, dp, rtol=1e-12, atol=0)
            np.testing.assert_allclose(s, ds, rtol=1e-8, atol=0)
    finally:
        dist.destroy_process_group()
