"""GPU checks of the mixed-precision form (tcgen05 split GEMM, FP32 path
state, FP32 payoffs, FP64 cross-path sums).

Stage by stage on identical inputs:
  normals   the fused kernel's Philox/Box-Muller output equals the exported
            FP32 stream bit for bit;
  GEMM      X = Y2 + a1 W1 + a2 W1perp against an FP64 convolution of those
            normals: BF16x3 error <= 4e-5 of the term magnitude, FP16x3 <= 1e-6,
            TF32 with one compensation term (normals rounded to TF32, 2^-11
            relative each) <= 5e-4;
  epilogue  (Ivdt, IsvdW) against FP64 on the same normals;
  prices    against the FP64 form fed the same FP32 normals: at most 1e-4
            relative and below 0.2 Monte Carlo standard errors.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


CFG2 = dict(xi=0.235 ** 2, H=[0.1], eta=[1.9], rho=[-0.9], T=[1.0] * 21, K=list(np.linspace(0.6, 1.4, 21)))
GRID = dict(xi=0.04, H=[0.05, 0.1, 0.1, 0.3, 0.1], eta=[1.0, 1.5, 1.5, 2.5, 1.5],
            rho=[-0.95, -0.7, -0.5, -0.7, -0.3], T=[0.25, 0.25, 0.5, 1.0, 1.0, 2.0], K=[0.9, 1.1, 1.0, 0.8, 1.3, 2.0])


def fp64_x(W1, W1p, H, N):
    """X_j = sum_{k<j} W1_k Gamma_{j-k} + a1 W1_j + a2 W1perp_j in FP64 and
    the magnitude sum_{k<j} |W1_k Gamma_{j-k}| (rBergLib/rBergomiMT.cpp:83-109),
    both as FP64 FFT convolutions (roundoff ~1e-15 of the magnitude)."""
    from oracle import oracle as O
    G = O.gamma(H, N).copy()
    G[0] = 0.0
    s2H = np.sqrt(2 * H)
    rhoH = s2H / (H + 0.5)
    a1, a2 = rhoH / s2H, np.sqrt(1 - rhoH ** 2) / s2H
    L = 1 << int(np.ceil(np.log2(2 * N)))
    W = W1[:, :N]

    def conv(a, g):
        return np.fft.irfft(np.fft.rfft(a, L) * np.fft.rfft(g, L)[None, :], L)[:, :N]

    Y = conv(W, G)
    A = conv(np.abs(W), np.abs(G))
    return Y + a1 * W + a2 * W1p[:, :N], A


@pytest.mark.parametrize("N,M", [(100, 300), (512, 256), (33, 129), (700, 200), (1024, 130), (1500, 100),
                                 (4096, 40)])
def test_fused_normals_are_the_exported_stream(R, N, M):
    w, _, _ = R.debug_mixed_paths(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], N, M, seed=11, path_offset=7)
    Z = R.generate_normals(11, M, N, precision=R.MIXED, path_offset=7)
    np.testing.assert_array_equal(w[:, :, :N].astype(np.float64), Z)
    assert np.all(w[:, :, N:] == 0)


@pytest.mark.parametrize("split,tol", [(0, 4e-5), (1, 1e-6), (2, 5e-4)])
@pytest.mark.parametrize("N", [64, 100, 512, 513, 700, 1024, 1025, 1500, 2048, 3001, 4096])
def test_toeplitz_gemm_columns(R, split, tol, N):
    """Columns of one TMEM pass (N <= 512); for 512 < N <= 1024, of 256-column
    passes in two TMEM buffers whose far-field comes from cached A tiles (the
    16-bit splits) or of two 512-column passes fed by redrawn A tiles (TF32);
    and of up to eight (N > 1024: redrawn chunks read their strip window,
    copied into the stage, every later pass) against the FP64 convolution."""
    H = 0.1
    M = 256
    w, x, _ = R.debug_mixed_paths(0.04, [H], [1.5], [-0.7], [1.0], [1.0], N, M, seed=3, split=split)
    Xf, A = fp64_x(w[:, 0, :].astype(np.float64), w[:, 1, :].astype(np.float64), H, N)
    err = np.abs(x[:, :N].astype(np.float64) - Xf)
    assert np.max(err / (A + 1.0)) < tol


def test_epilogue_integrals(R, oracle):
    g = GRID
    N, M = 64, 384
    w, _, iv = R.debug_mixed_paths(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=9, split=1)
    Z = w[:, :, :N].astype(np.float64)
    # FP64 reference of (Ivdt, IsvdW) per output through the oracle's payoff
    # machinery: recover them from the FP64 form's per-group sums instead of
    # re-deriving, by pricing each output with both and comparing payoffs.
    pay64 = oracle.payoffs_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z)
    _, _, groups = R.plan_info(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N)
    O = len(g["T"])
    for i in range(pay64.shape[1]):
        rho, K = g["rho"][i // O], g["K"][i % O]
        Iv, Iw = iv[groups[i], :, 0].astype(np.float64), iv[groups[i], :, 1].astype(np.float64)
        vol = np.sqrt((1 - rho * rho) * Iv)
        spot = np.exp(-0.5 * rho * rho * Iv + rho * Iw)
        from scipy.special import erfc
        d1 = (np.log(spot / K) + 0.5 * vol * vol) / vol
        pay = 0.5 * erfc(-d1 / np.sqrt(2)) * spot - 0.5 * erfc(-(d1 - vol) / np.sqrt(2)) * K
        assert np.max(np.abs(pay - pay64[:, i])) < 2e-5 * max(1.0, np.abs(pay64[:, i]).max())


@pytest.mark.parametrize("split", [0, 1, 2])
def test_mixed_prices_vs_fp64_identical_normals(R, split):
    """Workload-2 shape (N = 512, 21 strikes) at reduced M: error vs the FP64
    form on the same FP32 normals <= 1e-4 relative and < 0.2 standard errors."""
    c = CFG2
    N, M = 512, 1 << 16
    mp, ms, miv = R.price_rt(c["xi"], c["H"], c["eta"], c["rho"], c["T"], c["K"], N, M, seed=11,
                             precision=R.MIXED, split=split)
    fp, fs, fiv = R.price_rt(c["xi"], c["H"], c["eta"], c["rho"], c["T"], c["K"], N, M, seed=11,
                             normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)
    assert np.all(np.abs(ms / fs - 1) < 1e-3)


def test_mixed_grid_multi_pass(R):
    g = GRID
    N, M = 64, 1 << 14
    mp, ms, _ = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=21,
                           precision=R.MIXED, split=1)
    fp, fs, _ = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=21,
                           normals=R.NORMALS_F32)
    big = fp > 1e-4
    assert np.all(np.abs(mp - fp)[big] <= 1e-4 * fp[big])
    assert np.all(np.abs(mp - fp) < 0.2 * np.maximum(fs, 1e-12) + 1e-9)


def test_gemm_backend_rejects_longer_horizon(R):
    with pytest.raises(R.RbgError):
        R.price_rt(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 4097, 256, precision=R.MIXED, conv=R.CONV_GEMM)


@pytest.mark.parametrize("N", [544, 1024, 1056, 1500, 2048, 4096])
def test_multi_pass_gemm_prices_vs_fp64_identical_normals(R, N):
    """Long-horizon shape on the multi-pass GEMM (two passes up to N = 1024,
    up to eight with streamed strip windows above): error vs the FP64 form on
    the same FP32 normals <= 1e-4 relative and < 0.2 standard errors."""
    H, eta, rho, xi, T = [0.1], [1.5], [-0.7], 0.04, 2.0
    K = list(np.linspace(0.5, 1.5, 11))
    M = 1 << 13
    mp, ms, _ = R.price_rt(xi, H, eta, rho, [T] * 11, K, N, M, seed=3, precision=R.MIXED, conv=R.CONV_GEMM)
    fp, fs, _ = R.price_rt(xi, H, eta, rho, [T] * 11, K, N, M, seed=3, normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)


@pytest.mark.parametrize("N,split", [(544, 1), (768, 0), (1024, 1)])
def test_cached_tile_passes_many_tiles_per_cta(R, N, split):
    """512 < N <= 1024 with the 16-bit splits: 256-column passes alternate two
    TMEM buffers across the tiles of a CTA (three passes at N <= 768, so a
    tile's first pass lands in either buffer) and the per-CTA A-tile cache is
    rewritten by every tile.  M = three waves of 128-path tiles over every SM
    plus a ragged tail; error vs the FP64 form on the same FP32 normals
    <= 1e-4 relative and < 0.2 standard errors."""
    H, eta, rho, xi, T = [0.1], [1.5], [-0.7], 0.04, 2.0
    K = list(np.linspace(0.5, 1.5, 11))
    M = 3 * 160 * 128 + 77
    mp, ms, _ = R.price_rt(xi, H, eta, rho, [T] * 11, K, N, M, seed=5, precision=R.MIXED, split=split,
                           conv=R.CONV_GEMM)
    fp, fs, _ = R.price_rt(xi, H, eta, rho, [T] * 11, K, N, M, seed=5, normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)
    assert np.all(np.abs(ms / fs - 1) < 1e-3)


@pytest.mark.parametrize("N,split", [(800, 1), (2500, 1), (700, 2), (2500, 2)])
def test_multi_pass_gemm_multi_group_grid(R, N, split):
    """Several variance groups and Volterra passes at N = 800 (two TMEM
    passes) and N = 2500 (five, strip windows streamed)."""
    g = GRID
    M = 1 << 12
    mp, ms, _ = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=23,
                           precision=R.MIXED, split=split, conv=R.CONV_GEMM)
    fp, fs, _ = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=23,
                           normals=R.NORMALS_F32)
    big = fp > 1e-4
    assert np.all(np.abs(mp - fp)[big] <= 1e-4 * fp[big])
    assert np.all(np.abs(mp - fp) < 0.2 * np.maximum(fs, 1e-12) + 1e-9)


# ------------------------------------------------------------ FFT backend
@pytest.mark.parametrize("N,M", [(64, 130), (100, 64), (700, 96), (1024, 64), (4096, 8)])
def test_fft_backend_columns(R, N, M):
    """Batched FFT convolution (two paths per complex transform, radix-4/2
    Stockham, FP32): X within 1e-5 of the FP64 convolution's term magnitude."""
    H = 0.07
    w, x, _ = R.debug_mixed_paths(0.04, [H], [1.5], [-0.7], [1.0], [1.0], N, M, seed=4, conv=R.CONV_FFT)
    Z = R.generate_normals(4, M, N, precision=R.MIXED)
    np.testing.assert_array_equal(w[:, :, :N].astype(np.float64), Z)
    Xf, A = fp64_x(Z[:, 0, :], Z[:, 1, :], H, N)
    err = np.abs(x[:, :N].astype(np.float64) - Xf)
    assert np.max(err / (A + 1.0)) < 1e-5


@pytest.mark.parametrize("N", [512, 1024])
def test_fft_and_gemm_backends_agree(R, N):
    c = CFG2
    M = 1 << 14
    pg, sg, _ = R.price_rt(c["xi"], c["H"], c["eta"], c["rho"], c["T"], c["K"], N, M, seed=5, precision=R.MIXED,
                           conv=R.CONV_GEMM, split=1)
    pf, sf, _ = R.price_rt(c["xi"], c["H"], c["eta"], c["rho"], c["T"], c["K"], N, M, seed=5, precision=R.MIXED,
                           conv=R.CONV_FFT)
    assert np.all(np.abs(pg - pf) <= 2e-5 * pg)


@pytest.mark.parametrize("N", [1024, 2048])
def test_fft_prices_vs_fp64_identical_normals(R, N):
    H, eta, rho, xi, T = [0.1], [1.5], [-0.7], 0.04, 2.0
    K = list(np.linspace(0.5, 1.5, 11))
    M = 1 << 12
    mp, ms, _ = R.price_rt(xi, H, eta, rho, [T] * 11, K, N, M, seed=3, precision=R.MIXED, conv=R.CONV_FFT)
    fp, fs, _ = R.price_rt(xi, H, eta, rho, [T] * 11, K, N, M, seed=3, normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)


def test_mixed_extreme_strikes(R):
    """FP32 conditional BS (Chebyshev erfc tails, put-call parity for ITM)
    against the FP64 form on identical normals, deep in both wings."""
    K = [0.2, 0.4, 0.6, 0.8, 1.0, 1.25, 1.6, 2.2, 3.0]
    N, M = 128, 1 << 15
    mp, ms, _ = R.price_rt(0.04, [0.1], [2.5], [-0.9], [1.5] * len(K), K, N, M, seed=8, precision=R.MIXED, split=1)
    fp, fs, _ = R.price_rt(0.04, [0.1], [2.5], [-0.9], [1.5] * len(K), K, N, M, seed=8, normals=R.NORMALS_F32)
    rel = np.abs(mp - fp) / fp
    assert np.all(rel[fp > 1e-5] < 1e-4)
    assert np.all(np.abs(mp - fp) < 0.2 * fs)


def test_repeated_calls_reuse_the_plan(R):
    """A mixed call with the inputs of the last one (another seed or path
    offset) skips planning and uploads; its results equal a call that plans
    afresh, including after other calls changed what the device holds."""
    a = (CFG2["xi"], CFG2["H"], CFG2["eta"], CFG2["rho"], CFG2["T"], CFG2["K"], 512, 20000)
    b = (GRID["xi"], GRID["H"], GRID["eta"], GRID["rho"], GRID["T"], GRID["K"], 300, 9000)
    first = R.price_rt(*a, seed=5, precision=R.MIXED)
    again = R.price_rt(*a, seed=5, precision=R.MIXED)                 # same inputs: the cached plan
    other_seed = R.price_rt(*a, seed=6, precision=R.MIXED)            # cached plan, another stream
    R.price_rt(*b, seed=5, precision=R.MIXED)                         # another plan and images
    after_other = R.price_rt(*a, seed=5, precision=R.MIXED)
    R.price_rt(*a, seed=5, precision=R.FP64)                          # the FP64 form's tables
    after_fp64 = R.price_rt(*a, seed=5, precision=R.MIXED)
    shard = R.price_rt(*a, seed=5, precision=R.MIXED, path_offset=20000)
    for r in (again, after_other, after_fp64):
        for x, y in zip(first, r):
            np.testing.assert_array_equal(x, y)
    assert np.all(other_seed[0] != first[0]) and np.all(shard[0] != first[0])
    # another seed through a freshly planned call gives the cached call's bits
    R.price_rt(*b, seed=5, precision=R.MIXED)
    fresh = R.price_rt(*a, seed=6, precision=R.MIXED)
    for x, y in zip(other_seed, fresh):
        np.testing.assert_array_equal(x, y)


def test_calls_on_two_streams_from_two_threads(R):
    """Host threads pricing on different CUDA streams hold separate library
    contexts (buffers, tables, plan cache, lock) and run side by side; each
    result equals the same call made alone."""
    import threading

    import torch

    a = (CFG2["xi"], CFG2["H"], CFG2["eta"], CFG2["rho"], CFG2["T"], CFG2["K"], 512, 30000)
    b = (GRID["xi"], GRID["H"], GRID["eta"], GRID["rho"], GRID["T"], GRID["K"], 300, 20000)
    want_a = R.price_rt(*a, seed=3, precision=R.MIXED)
    want_b = R.price_rt(*b, seed=4, precision=R.MIXED)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    got = {}

    def run(key, args, seed, stream):
        torch.cuda.set_device(0)
        got[key] = [R.price_rt(*args, seed=seed, precision=R.MIXED, stream=stream.cuda_stream) for _ in range(3)]

    th = [threading.Thread(target=run, args=("a", a, 3, s1)), threading.Thread(target=run, args=("b", b, 4, s2))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for key, want in (("a", want_a), ("b", want_b)):
        assert len(got[key]) == 3
        for r in got[key]:
            for x, y in zip(r, want):
                np.testing.assert_array_equal(x, y)


def test_prepared_pricer_equals_price_rt(R):
    """RtPricer (arguments marshalled once) gives price_rt's results call by
    call, seed and path offset changed between calls."""
    a = (CFG2["xi"], CFG2["H"], CFG2["eta"], CFG2["rho"], CFG2["T"], CFG2["K"], 512, 20000)
    pr = R.RtPricer(*a, precision=R.MIXED)
    for seed, off in ((5, 0), (6, 0), (6, 20000), (5, 0)):
        got = [x.copy() for x in pr(seed=seed, path_offset=off)]
        want = R.price_rt(*a, seed=seed, path_offset=off, precision=R.MIXED)
        for x, y in zip(got, want):
            np.testing.assert_array_equal(x, y)
