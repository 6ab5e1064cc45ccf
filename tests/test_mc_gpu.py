"""GPU parity of the plain Monte Carlo estimator (the reference's
computeIV_tensor, rBergLib/cinterface.cpp:10-46 over rBergomiMT.cpp:174-289):
third normal stream, S_T from the log-Euler sum, payoff max(S_T - K, 0), S
recomputed only on the rho trigger.  FP64 form: 1e-12 relative on prices
against the reference's own output and the oracle on identical normals.
Mixed form: against the FP64 form on identical FP32 normals."""
import numpy as np
import pytest

from tests._golden import dropin, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


def test_mc_payoffs_vs_reference_fixture(R, oracle):
    """The reference's computeIV_tensor(num_threads = 1) output, replayed on
    its own mt19937 normals through the GPU's per-path MC payoffs."""
    c = dropin("mc")
    args = (float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"])
    pay = R.payoffs_mc(*args, c["Z"])
    price, stat = oracle.reduce(pay)
    assert np.all(rel_err(price, c["ref_price"]) < 1e-12)
    assert np.all(rel_err(stat, c["ref_stat"]) < 1e-8)
    want = oracle.payoffs_mc(*args, c["Z"])
    assert np.max(np.abs(pay - want)) < 1e-12 * max(1.0, np.abs(want).max())


def test_mc_prices_vs_oracle_on_philox_normals(R, oracle):
    xi, H, eta, rho = 0.05, [0.07, 0.2], [1.9, 1.2], [-0.9, -0.6]
    T, K = [0.5, 0.5, 1.5], [0.9, 1.1, 1.0]
    N, M, seed = 48, 6000, 31
    p, s, iv = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=seed)
    Z = R.generate_normals(seed, M, N, streams=3)
    Zo = oracle.normals_f64(seed, M, N, 3)
    assert np.max(np.abs(Z - Zo)) < 1e-13
    op, os_ = oracle.reduce(oracle.payoffs_mc(xi, H, eta, rho, T, K, Z))
    assert np.all(rel_err(p, op) < 1e-12)
    assert np.all(rel_err(s, os_) < 1e-8)


def test_mc_rho_trigger_keeps_stale_state(R, oracle):
    """rho moving by 5e-11 (< the 1e-10 trigger) keeps the earlier S: the
    second tuple prices exactly like the first, in the oracle and on the GPU."""
    xi, H, eta, rho = 0.04, [0.1, 0.1], [1.5, 1.5], [-0.7, -0.7 + 5e-11]
    N, M, seed = 32, 2048, 3
    p, _, _ = R.price_mc(xi, H, eta, rho, [1.0], [1.0], N, M, seed=seed)
    assert p[1] == p[0]
    Z = R.generate_normals(seed, M, N, streams=3)
    op, _ = oracle.reduce(oracle.payoffs_mc(xi, H, eta, rho, [1.0], [1.0], Z))
    assert np.all(rel_err(p, op) < 1e-12)


def test_computeIV_tensor_dropin(R):
    """Drop-in ABI: same prices as the extended call with the folded seed,
    and the reference's eta_tot / rho_tot swap (cinterface.cpp:45)."""
    xi, H, eta, rho = 0.07, [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85]
    T, K = [0.5, 1.0], [0.8, 1.0]
    res = R.computeIV_tensor(xi, H, eta, rho, T, K, 64, 1 << 14, [123], num_threads=4)
    p, s, iv = R.price_mc(xi, H, eta, rho, T, K, 64, 1 << 14, seed=123)
    np.testing.assert_array_equal(res.price, p)
    np.testing.assert_array_equal(res.stat, s)
    np.testing.assert_array_equal(res.iv, iv)
    np.testing.assert_array_equal(res.eta, np.repeat(rho, 2))
    np.testing.assert_array_equal(res.rho, np.repeat(eta, 2))
    np.testing.assert_array_equal(res.H, np.repeat(H, 2))
    np.testing.assert_array_equal(res.T, np.tile(T, 2))


def test_mc_and_rt_estimate_the_same_price(R):
    """Plain MC and the Romano-Touzi conditional estimator target the same
    expectation: independent-stream agreement within 4 combined SEs."""
    xi, H, eta, rho = 0.235 ** 2, [0.07], [1.9], [-0.9]
    T, K = [1.0] * 5, [0.8, 0.9, 1.0, 1.1, 1.2]
    pm, sm, _ = R.price_mc(xi, H, eta, rho, T, K, 100, 1 << 18, seed=42)
    pr, sr, _ = R.price_rt(xi, H, eta, rho, T, K, 100, 1 << 18, seed=43)
    assert np.all(np.abs(pm - pr) < 4 * np.sqrt(sm ** 2 + sr ** 2))
    assert np.all(sr < sm)  # conditioning on W1 reduces the variance


@pytest.mark.parametrize("N", [100, 512, 700])
def test_mc_mixed_vs_fp64_identical_normals(R, N):
    """Mixed plain MC (third Philox stream in the fused tcgen05 kernel, FP32
    payoffs) against the FP64 form on the same FP32 normals: <= 1e-4
    relative and < 0.2 standard errors; one- and two-pass GEMM."""
    xi, H, eta, rho = 0.235 ** 2, [0.07, 0.2], [1.9, 1.2], [-0.9, -0.6]
    T, K = [0.5, 0.5, 1.5], [0.9, 1.1, 1.0]
    M = 1 << 15
    mp, ms, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=9, precision=R.MIXED)
    fp, fs, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=9, normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)
    assert np.all(np.abs(ms / fs - 1) < 1e-3)


@pytest.mark.parametrize("N,conv", [(1500, "fft"), (700, "fft"), (1500, "auto"), (2048, "gemm")])
def test_mc_mixed_long_horizon_vs_fp64(R, N, conv):
    """Mixed plain MC on the batched-FFT backend and on the multi-pass GEMM
    (three and four TMEM passes with streamed strip windows)."""
    xi, H, eta, rho = 0.05, [0.1], [1.5], [-0.7]
    T, K = [2.0, 2.0], [0.9, 1.2]
    M = 1 << 13
    cv = {"fft": R.CONV_FFT, "auto": R.CONV_AUTO, "gemm": R.CONV_GEMM}[conv]
    mp, ms, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=4, precision=R.MIXED, conv=cv)
    fp, fs, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=4, normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)


def test_computeIV_tensor_mixed_env(R, monkeypatch):
    monkeypatch.setenv("RBG_PRECISION", "mixed")
    xi, H, eta, rho, T, K = 0.05, [0.1], [1.5], [-0.7], [1.0], [1.0]
    res = R.computeIV_tensor(xi, H, eta, rho, T, K, 128, 1 << 14, [5])
    p, s, _ = R.price_mc(xi, H, eta, rho, T, K, 128, 1 << 14, seed=5, precision=R.MIXED)
    np.testing.assert_array_equal(res.price, p)


def test_mc_mixed_tf32_split_vs_fp64(R):
    """Plain MC on the TF32 split (normals rounded to TF32, Gamma in TF32 hi + lo)."""
    xi, H, eta, rho = 0.05, [0.1], [1.5], [-0.7]
    T, K = [1.0, 1.0], [0.9, 1.2]
    N, M = 512, 1 << 14
    mp, ms, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=6, precision=R.MIXED, split=R.SPLIT_TF32X2)
    fp, fs, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=6, normals=R.NORMALS_F32)
    err = np.abs(mp - fp)
    assert np.all(err <= 1e-4 * fp)
    assert np.all(err < 0.2 * fs)
