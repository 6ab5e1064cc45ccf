"""Sobol' quasi-Monte Carlo on the GPU against the oracle (FP64 form).

Direction integers: the reference's own (rBergomi/sobol.cpp), recovered from
its points in tests/golden/sobol.npz (valid for point indices below 2^24).
Normals: CUDA's FP64 normcdfinv against the oracle's quantile, a few ulps.
Prices: the FP64 pipeline on identical normals, 1e-12 relative; the mixed
form (producer-drawn or materialized points, with or without the bridge, on
either backend) within its 1e-4 relative / 0.2 standard-error bounds."""
import os

import numpy as np
import pytest

from tests._golden import rel_err

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sobol.npz")
NORMAL_TOL = 2e-14  # absolute, |z| < 9.1 on Sobol' points
PRICE_TOL = 1e-12
STAT_TOL = 1e-8

GRID = dict(xi=0.04, H=[0.05, 0.1, 0.1, 0.3], eta=[1.0, 1.5, 1.5, 2.5], rho=[-0.95, -0.7, -0.5, -0.7],
            T=[0.25, 0.5, 1.0, 2.0], K=[0.9, 1.1, 1.0, 0.8])


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


@pytest.fixture(scope="module")
def V(oracle):
    return oracle.sobol_directions_from_points(np.load(GOLD)["gray_points"])


@pytest.mark.parametrize("N,M,off,bridge", [(64, 3000, 0, False), (37, 1000, 12345, False), (64, 2000, 777, True),
                                            (1, 50, 0, True), (512, 300, 99, True)])
def test_normals_match_oracle(R, oracle, V, N, M, off, bridge):
    Z = R.sobol_normals(V, N, M, path_offset=off, bridge=bridge)
    Zo = oracle.sobol_normals(V, N, M, path0=off, bridge=bridge)
    assert np.max(np.abs(Z - Zo)) < NORMAL_TOL * (4 if bridge else 1)


@pytest.mark.parametrize("N,M,off", [(64, 4000, 0), (300, 500, 70000)])
def test_fp32_normals_match_oracle(R, oracle, V, N, M, off):
    """The mixed form's FP32 Sobol' normals (top 32 bits of the point, fitted
    FP32 quantile, relative error <= 6e-7) against the oracle's FP64 normals."""
    Z = R.sobol_normals(V, N, M, path_offset=off, precision=R.MIXED)
    Zo = oracle.sobol_normals(V, N, M, path0=off)
    assert np.all(Z.astype(np.float32).astype(np.float64) == Z)
    assert np.max(np.abs(Z - Zo) / (1e-6 * np.abs(Zo) + 1e-7)) <= 1.0


def test_normals_offset_is_a_suffix(R, V):
    a = R.sobol_normals(V, 32, 150)
    b = R.sobol_normals(V, 32, 100, path_offset=50)
    np.testing.assert_array_equal(a[50:], b)


@pytest.mark.parametrize("N,M,bridge", [(64, 4096, False), (64, 4096, True), (100, 2500, False)])
def test_prices_match_oracle_on_identical_normals(R, oracle, V, N, M, bridge):
    g = GRID
    price, stat, iv = R.price_rt_sobol(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, V, bridge=bridge)
    Z = oracle.sobol_normals(V, N, M, bridge=bridge)
    op, os_ = oracle.reduce(oracle.payoffs_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z))
    assert np.all(rel_err(price, op) < PRICE_TOL)
    assert np.all(rel_err(stat, os_) < STAT_TOL)
    O = len(g["T"])
    ivo = np.array([oracle.iv_call(p, g["K"][i % O], g["T"][i % O]) for i, p in enumerate(op)])
    ok = ~np.isnan(ivo)
    assert np.all(rel_err(iv[ok], ivo[ok]) < 1e-10)


def test_qmc_agrees_with_monte_carlo(R, V):
    """The QMC estimate (point set 1..2^16) and a 2^21-path Philox estimate of
    the same prices agree within 4 combined standard errors (the QMC run's
    `stat`, the Monte Carlo formula the reference reports, bounds its error
    from above)."""
    args = (0.04, [0.1], [1.5], [-0.7], [0.5, 1.0], [1.0, 1.1], 128)
    pq, sq, _ = R.price_rt_sobol(*args, 1 << 16, V)
    pm, sm, _ = R.price_rt(*args, 1 << 21, seed=3, precision=R.FP64)
    assert np.all(np.abs(pq - pm) < 4 * np.hypot(sq, sm))


@pytest.mark.parametrize("N,M", [(37, 3001), (512, 20000), (544, 8192)])
def test_mixed_form_matches_fp64_form(R, V, N, M):
    """The tensor-core form on the same Sobol' points (FP32 quantile, BF16x3
    Volterra GEMM, one and two TMEM passes): within 1e-4 relative and 0.2
    standard errors of the FP64 form, the mixed form's bound on Philox normals."""
    g = GRID
    a = (g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, V)
    p64, s64, _ = R.price_rt_sobol(*a, precision=R.FP64)
    p32, s32, _ = R.price_rt_sobol(*a, precision=R.MIXED)
    assert np.all(rel_err(p32, p64) < 1e-4)
    assert np.all(np.abs(p32 - p64) < 0.2 * s64)
    assert np.all(rel_err(s32, s64) < 1e-3)


def test_mixed_form_path_offset(R, V):
    """Shifting the point range moves the QMC estimate; the same shifted
    range in the FP64 form agrees."""
    a = (0.04, [0.1], [1.5], [-0.7], [1.0, 1.0], [1.0, 1.2], 64, 5000, V)
    p0, _, _ = R.price_rt_sobol(*a, precision=R.MIXED)
    p1, s1, _ = R.price_rt_sobol(*a, precision=R.MIXED, path_offset=100000)
    q1, _, _ = R.price_rt_sobol(*a, precision=R.FP64, path_offset=100000)
    assert np.all(p0 != p1)
    assert np.all(np.abs(p1 - q1) < 0.2 * s1)
    # offsets that are not multiples of 16 take the producer's general walk
    for off in (100003, 7):
        p2, s2, _ = R.price_rt_sobol(*a, precision=R.MIXED, path_offset=off)
        q2, _, _ = R.price_rt_sobol(*a, precision=R.FP64, path_offset=off)
        assert np.all(rel_err(p2, q2) < 1e-4)
        assert np.all(np.abs(p2 - q2) < 0.2 * s2)


@pytest.mark.parametrize("N,M", [(64, 4096), (256, 8192)])
def test_mixed_bridge_matches_fp64_bridge(R, V, N, M):
    """The Brownian bridge in the mixed form: the FP64 form's bridged
    normals, materialized on the device and read in FP32 by the tensor-core
    path kernel, price within the mixed form's bounds of the FP64 bridge."""
    g = GRID
    a = (g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, V)
    p64, s64, _ = R.price_rt_sobol(*a, bridge=True, precision=R.FP64)
    p32, s32, _ = R.price_rt_sobol(*a, bridge=True, precision=R.MIXED)
    assert np.all(rel_err(p32, p64) < 1e-4)
    assert np.all(np.abs(p32 - p64) < 0.2 * s64)
    # the bridge changes the estimate: not the unbridged points' prices
    q32, _, _ = R.price_rt_sobol(*a, precision=R.MIXED)
    assert np.all(p32 != q32)


@pytest.mark.parametrize("N", [100, 512])
def test_mixed_sobol_on_the_fft_backend(R, V, N):
    """The FFT backend on Sobol' points: the same FP32 normals the GEMM
    producer draws, materialized; both backends within the mixed bounds of
    the FP64 form and of each other."""
    g = GRID
    a = (g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, 6000, V)
    p64, s64, _ = R.price_rt_sobol(*a, precision=R.FP64)
    pg, _, _ = R.price_rt_sobol(*a, precision=R.MIXED)
    pf, sf, _ = R.price_rt_sobol(*a, precision=R.MIXED, conv=R.CONV_FFT)
    for p in (pg, pf):
        assert np.all(rel_err(p, p64) < 1e-4)
        assert np.all(np.abs(p - p64) < 0.2 * s64)
    assert np.all(rel_err(pf, pg) < 1e-4)


def synthetic_directions(dims, seed=5):
    """Any 62-bit integers define a digital point set by the same Gray-code
    rule (not a low-discrepancy one): enough to check that both forms price
    the same points beyond the reference table's 1111 dimensions and 2^24
    points."""
    rng = np.random.default_rng(seed)
    hi = rng.integers(0, 1 << 31, size=(dims, 62), dtype=np.uint64)
    lo = rng.integers(0, 1 << 31, size=(dims, 62), dtype=np.uint64)
    return (hi << np.uint64(31)) | lo


@pytest.mark.parametrize("N,M,off", [(1536, 3000, 0), (64, 4096, (1 << 32) + 5)])
def test_mixed_sobol_materialized_matches_fp64(R, N, M, off):
    """Past the GEMM producer's range -- more than 1024 steps (multi-pass
    tiles), point indices beyond 2^32 -- the mixed form materializes the
    points' FP32 normals and prices them within its bounds of the FP64 form."""
    Vs = synthetic_directions(2 * N)
    a = (0.04, [0.1, 0.3], [1.5, 2.0], [-0.7, -0.9], [1.0, 2.0], [1.0, 0.9], N, M, Vs)
    p64, s64, _ = R.price_rt_sobol(*a, precision=R.FP64, path_offset=off)
    p32, _, _ = R.price_rt_sobol(*a, precision=R.MIXED, path_offset=off)
    assert np.all(rel_err(p32, p64) < 1e-4)
    assert np.all(np.abs(p32 - p64) < 0.2 * s64)


def test_rejects_bad_requests(R, V):
    args = (0.04, [0.1], [1.5], [-0.7], [1.0], [1.0])
    with pytest.raises(R.RbgError, match="fewer than 2N"):
        R.price_rt_sobol(*args, 600, 16, V)       # 1111 dimensions < 1200
    with pytest.raises(R.RbgError, match="power of two"):
        R.price_rt_sobol(*args, 48, 16, V, bridge=True)
    with pytest.raises(R.RbgError, match="fewer than 2N"):
        R.sobol_normals(V[:10], 8, 4)
