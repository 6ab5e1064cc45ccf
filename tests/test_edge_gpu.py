"""GPU parity at the corners of the parameter space the reference accepts:
rho = -1 and +1 (zero conditional variance: the conditional Black-Scholes call
becomes the intrinsic value), eta = 0 (flat variance), H = 1/2 (the Volterra
kernel is flat), H = 0.9 (a growing kernel), H = 0.01 (near-singular), a short
maturity, deep in- and out-of-the-money strikes, and a single path.

FP64 form against the oracle on identical normals (1e-12 relative on prices;
NaN implied vols in the same places), and the mixed form against the FP64
form fed the same FP32 normals (1e-4 relative, 0.2 standard errors)."""
import numpy as np
import pytest

from tests._golden import rel_err

pytestmark = pytest.mark.gpu

PRICE_TOL = 1e-12
STAT_TOL = 1e-8

CORNERS = dict(xi=0.04, H=[0.5, 0.5, 0.9, 0.01, 0.3], eta=[1.0, 1.0, 1.2, 3.0, 0.0], rho=[-1.0, 1.0, -0.5, 0.0, -0.7],
               T=[0.01, 1.0, 1.0], K=[1.0, 0.5, 2.0])


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


@pytest.mark.parametrize("N,M", [(40, 1500), (7, 1), (33, 2)])
def test_fp64_corners_vs_oracle(R, oracle, N, M):
    g = CORNERS
    price, stat, iv = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=17)
    Z = R.generate_normals(17, M, N, precision=R.FP64)
    op, os_ = oracle.reduce(oracle.payoffs_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z))
    assert np.all(np.isfinite(price))
    assert np.all(np.abs(price - op) <= PRICE_TOL * np.maximum(np.abs(op), 1e-3))
    assert np.all(np.abs(stat - os_) <= STAT_TOL * np.maximum(np.abs(os_), 1e-6))
    if M == 1:
        assert np.all(stat == 0.0)
    O = len(g["T"])
    ivo = np.array([oracle.iv_call(p, g["K"][i % O], g["T"][i % O]) for i, p in enumerate(op)])
    ok = ~np.isnan(ivo)
    np.testing.assert_array_equal(np.isnan(iv), ~ok)
    assert np.all(rel_err(iv[ok], ivo[ok]) < 1e-10)


def test_fp64_zero_conditional_variance_is_intrinsic(R):
    """rho = +-1: each payoff is the intrinsic value of the conditional spot
    (rBergLib/rBergomiMT.cpp:598-602 with vol = 0)."""
    N, M = 16, 64
    Z = R.generate_normals(23, M, N, precision=R.FP64)
    for rho in (-1.0, 1.0):
        pay = R.computeIVRT_tensor_quadrature(0.04, [0.5], [1.0], [rho], [1.0, 1.0], [0.9, 1.1], Z)
        assert pay.shape == (M, 2)
        assert np.all(pay >= 0.0)
        # the payoff is max(S - K, 0) of one conditional spot S per sample
        s = pay[:, 0] + 0.9
        both = pay[:, 0] > 0.2
        np.testing.assert_allclose(pay[both, 1], s[both] - 1.1, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("conv", ["gemm", "fft"])
def test_mixed_corners_vs_fp64_identical_normals(R, conv):
    g = CORNERS
    N, M = 96, 1 << 14
    mp, ms, _ = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=31,
                           precision=R.MIXED, conv={"gemm": R.CONV_GEMM, "fft": R.CONV_FFT}[conv])
    fp, fs, _ = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=31,
                           normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    big = fp > 1e-5
    assert np.all(err[big] <= 1e-4 * fp[big])
    assert np.all(err <= 0.2 * fs + 1e-12)
    assert np.all(np.abs(ms[big] / fs[big] - 1) < 1e-3)


def test_implied_vol_sweep_vs_oracle(R, oracle):
    """The GPU implied-vol search (FP32 bracketing, FP64 check, Halley and
    Newton steps on the log price, FP64 fallback) against the oracle's FP64
    root on 4,000 call prices from K in [0.3, 3], T in [0.01, 5] and vols in
    [0.01, 3], out-of-the-money values down to 1e-12 -- where FP32 cannot
    resolve the price the search falls back to FP64 -- plus prices with no
    volatility (NaN in both)."""
    from scipy.stats import norm

    rng = np.random.default_rng(4)
    n = 4000
    K = np.exp(rng.uniform(np.log(0.3), np.log(3.0), n))
    T = np.exp(rng.uniform(np.log(0.01), np.log(5.0), n))
    sig = np.exp(rng.uniform(np.log(0.01), np.log(3.0), n))
    d1 = (np.log(1.0 / K) + 0.5 * sig * sig * T) / (sig * np.sqrt(T))
    d2 = d1 - sig * np.sqrt(T)
    otm = np.where(K < 1.0, K * norm.cdf(-d2) - norm.cdf(-d1), norm.cdf(d1) - K * norm.cdf(d2))
    keep = otm > 1e-12
    K, T, sig, otm = K[keep], T[keep], sig[keep], otm[keep]
    price = np.where(K < 1.0, otm + 1.0 - K, otm)  # call prices
    # and a few with no volatility: below intrinsic, at or above the spot
    price = np.concatenate([price, [0.3, 1.0, 1.5, 0.05]])
    K = np.concatenate([K, [0.5, 1.0, 0.9, 1.2]])
    T = np.concatenate([T, [1.0, 1.0, 1.0, 0.0]])
    iv = R.implied_vol(price, K, T)
    ivo = np.array([oracle.iv_call(p, k, t) for p, k, t in zip(price, K, T)])
    ok = ~np.isnan(ivo)
    np.testing.assert_array_equal(np.isnan(iv), ~ok)
    assert ok.sum() >= len(sig) - 5
    assert np.all(rel_err(iv[ok], ivo[ok]) < 1e-10)
    # the generating vols, where the call price carries the OTM value to many digits
    m = len(sig)
    good = ok[:m] & (otm > 1e-6)
    assert np.all(rel_err(iv[:m][good], sig[good]) < 1e-6)
