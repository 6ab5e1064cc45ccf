"""The continuously batched serving loop on the GPU: every request's result
is the same alone (rbg_price_rt) and in a concurrent mix of other requests --
bitwise, since normals are counter-based and each request keeps its own sums
-- with and without CUDA graphs, whether it ran on its own slot or inside a
shared (job-table) launch with other requests; repeated (H, N) requests hit
the device table cache; malformed requests fail without disturbing the
others."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


def make_requests(n, seed=7):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        nk = int(rng.integers(1, 17))
        N = int([64, 100, 256, 512, 700, 1024][i % 6])
        M = int(rng.choice([1 << 12, 5000, 1 << 14, 1 << 16]))
        H = float(rng.uniform(0.03, 0.45))
        if i % 5 == 0:  # every fifth request repeats one (H, N): device table cache hits
            H, N = 0.1, 256
        reqs.append(dict(xi=float(rng.uniform(0.01, 0.1)), H=[H], eta=[float(rng.uniform(0.5, 3.0))],
                         rho=[float(rng.uniform(-0.99, -0.3))], T=[float(rng.uniform(0.05, 3.0))] * nk,
                         K=list(np.sort(rng.uniform(0.5, 1.5, nk))), N=N, M=M, seed=i))
    return reqs


def alone(R, r):
    return R.price_rt(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"], seed=r["seed"],
                      precision=R.MIXED)


@pytest.mark.parametrize("graphs", [1, 0])
def test_results_same_alone_and_in_mix(R, graphs):
    reqs = make_requests(30)
    want = [alone(R, r) for r in reqs]
    with R.Server(use_graphs=graphs, slots=6, high_priority_slots=3) as srv:
        tickets = [srv.submit(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"], seed=r["seed"])
                   for r in reqs]
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for (wp, ws, wi), (gp, gs, gi, lat) in zip(want, got):
        np.testing.assert_allclose(gp, wp, rtol=1e-12, atol=0)
        np.testing.assert_allclose(gs, ws, rtol=1e-12, atol=0)
        assert lat > 0
    if graphs:  # one graph per shared launch or per request on its own slot
        assert st["graph_launches"] == st["batches"] + len(reqs) - st["batched_requests"]
    assert st["table_cache_hits"] >= 1


def small_requests(n, seed=5):
    """One-pass requests (N <= 512, one H) that the server prices in shared launches."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nk = int(rng.integers(1, 17))
        out.append(dict(xi=float(rng.uniform(0.01, 0.1)), H=[float(rng.uniform(0.03, 0.45))],
                        eta=[float(rng.uniform(0.5, 3.0))], rho=[float(rng.uniform(-0.99, -0.3))],
                        T=[float(rng.uniform(0.05, 3.0))] * nk, K=list(np.sort(rng.uniform(0.5, 1.5, nk))),
                        N=int([64, 100, 256, 512, 37, 480][i % 6]), M=int(rng.choice([1 << 12, 5000, 1 << 14])),
                        seed=100 + i))
    return out


@pytest.mark.parametrize("split", [0, 2])
def test_shared_launches(R, split):
    """Requests pending together go through job-table launches: fewer kernel
    launches than requests, and each result bit-identical to the same request
    priced alone (its own call) -- the job-table kernels run each request's
    paths and sums exactly as the per-request kernels do."""
    reqs = small_requests(48)
    want = [R.price_rt(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"], seed=r["seed"],
                       precision=R.MIXED, split=split) for r in reqs]
    n0 = R.launch_count()
    # a batching window long enough for the whole burst to be pending together
    with R.Server(batch_slots=1, slots=2, high_priority_slots=1, batch_wait_us=2e5, max_batch_jobs=64) as srv:
        tickets = [srv.submit(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"], seed=r["seed"],
                              split=split) for r in reqs]
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    launches = R.launch_count() - n0
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batched_requests"] == len(reqs)
    assert st["batches"] <= 2  # the burst, and at most a tail that missed the window
    assert launches <= 8 < len(reqs)  # path, payoff, merge, finalize per shared launch
    for (wp, ws, wi), (gp, gs, gi, _) in zip(want, got):
        np.testing.assert_array_equal(gp, wp)
        np.testing.assert_array_equal(gs, ws)
        np.testing.assert_array_equal(gi, wi)


def test_shared_launch_of_one_equals_batch(R):
    """A request alone in a server (a shared launch of one) and the same
    request among many give the same bits."""
    reqs = small_requests(12, seed=9)
    with R.Server(batch_slots=1) as srv:
        t = srv.submit(**{k: v for k, v in reqs[3].items() if k not in ("seed",)}, seed=reqs[3]["seed"])
        one = srv.wait(t)
    with R.Server(batch_slots=1) as srv:
        ts = [srv.submit(**{k: v for k, v in r.items() if k != "seed"}, seed=r["seed"]) for r in reqs]
        many = [srv.wait(t) for t in ts]
    np.testing.assert_array_equal(one[0], many[3][0])
    np.testing.assert_array_equal(one[1], many[3][1])


def test_concurrent_submitters_and_budget(R):
    """Two threads submit while a third waits; a tight HBM budget forces
    admission to wait for memory; results still match the alone runs."""
    reqs = make_requests(16, seed=11)
    want = [alone(R, r) for r in reqs]
    got = [None] * len(reqs)
    budget = max(r["M"] * r["N"] * 4 for r in reqs) + (8 << 20)
    with R.Server(hbm_budget=budget, slots=8, high_priority_slots=4) as srv:
        tickets = [None] * len(reqs)

        def sub(idx):
            for i in idx:
                r = reqs[i]
                tickets[i] = srv.submit(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"],
                                        seed=r["seed"])

        th = [threading.Thread(target=sub, args=(range(k, len(reqs), 2),)) for k in (0, 1)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for i, t in enumerate(tickets):
            got[i] = srv.wait(t)
    for (wp, _, _), (gp, _, _, _) in zip(want, got):
        np.testing.assert_allclose(gp, wp, rtol=1e-12, atol=0)


def test_bad_request_is_rejected_at_submit(R):
    with R.Server() as srv:
        with pytest.raises(R.RbgError):
            srv.submit(0.04, [1.5], [1.0], [-0.5], [1.0], [1.0], 64, 1024)  # H outside (0, 1)
        t = srv.submit(0.04, [0.1], [1.0], [-0.5], [1.0], [1.0], 64, 1024, seed=1)
        p, s, iv, lat = srv.wait(t)
        assert p[0] > 0
