"""Path sharding across ranks (the multi-GPU form of the pricer).

On CPU, a world-size-2 gloo group: each rank prices its contiguous block of
paths (here with the oracle standing in for its GPU), one all-reduce merges
the (sum x, sum x^2) pairs, the library's C-ABI merge (rbg_merge_sums)
applies the moment formula, and the merged price equals a single-process run
over all paths.  On the GPU, two gloo ranks both price their blocks with the
real pricer (rbg_price_rt_sums) on cuda:0 -- their kernels never wait on
each other -- and the merge equals one call over all paths."""
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


def test_merge_sums_c_abi_matches_reference_formula():
    """rbg_merge_sums (host-only): shard-order merge of gathered sums and the
    reference's moment formula, against the same arithmetic in numpy."""
    import rbergomi_gb300 as R
    rng = np.random.default_rng(5)
    pay = rng.lognormal(-2.0, 0.7, size=(4, 1000, 6))  # 4 shards x 1000 paths x 6 outputs
    s1, s2 = pay.sum(1), (pay * pay).sum(1)
    M = 4000
    price, stat = R.merge_sums(s1, s2, M)
    want_p = s1.sum(0) / M
    want_s = np.sqrt(s2.sum(0) / M - want_p ** 2) / np.sqrt(M)
    np.testing.assert_allclose(price, want_p, rtol=1e-14, atol=0)
    np.testing.assert_allclose(stat, want_s, rtol=1e-10, atol=0)
    # one shard after an all-reduce: the same numbers
    p1, st1 = R.merge_sums(s1.sum(0), s2.sum(0), M)
    np.testing.assert_allclose(p1, price, rtol=1e-15, atol=0)
    np.testing.assert_allclose(st1, stat, rtol=1e-12, atol=0)
    with pytest.raises(R.RbgError):
        R.merge_sums(s1, s2, 0)


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


def _gpu_rank(rank, ws, port, prec, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist

    import rbergomi_gb300 as R
    from rbergomi_gb300 import shards

    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        price, stat = shards.price_rt_sharded(XI, H, ETA, RHO, T, K, 256, GPU_M, seed=SEED, precision=prec)
        q.put((rank, price, stat, R.launch_count()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


GPU_M = 1 << 16  # two blocks of 2^15 paths: whole payoff chunks on both ranks


@pytest.mark.gpu
@pytest.mark.parametrize("prec_name", ["FP64", "MIXED"])
def test_two_rank_gpu_shards_equal_one_call(prec_name):
    """Two gloo ranks, both on cuda:0, each price their contiguous path block
    through rbg_price_rt_sums; one all-reduce plus rbg_merge_sums equals one
    call over all paths (FP64 and mixed) to FP64 roundoff."""
    import torch.multiprocessing as mp

    import rbergomi_gb300 as R
    prec = getattr(R, prec_name)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gpu_rank, args=(r, 2, port, prec, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=600) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    want_p, want_s, _ = R.price_rt(XI, H, ETA, RHO, T, K, 256, GPU_M, seed=SEED, precision=prec)
    for _, price, stat, launches in got:
        assert launches > 0  # each rank ran its own kernels
        np.testing.assert_allclose(price, want_p, rtol=1e-13, atol=0)
        np.testing.assert_allclose(stat, want_s, rtol=1e-9, atol=0)
