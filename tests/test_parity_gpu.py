"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference's golden fixtures.  FP64 form: 1e-12 relative on prices, 1e-8 on
standard errors (the reference's E[X^2]-E[X]^2 formula cancels), implied vols
within the reference's own 2^-10 root-finder tolerance."""
import numpy as np
import pytest

from tests._golden import QUAD_CASES, debug8, dropin, quad, rel_err

pytestmark = pytest.mark.gpu

PRICE_TOL = 1e-12   # FP64 form vs reference on identical normals (relative)
STAT_TOL = 1e-8
IV_REF_TOL = 2.0 ** -10


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


def test_normals_match_oracle(R, oracle):
    Z = R.generate_normals(42, 300, 37, precision=R.FP64, path_offset=12345)
    Zo = oracle.normals_f64(42, 300, 37, 2, path0=12345)
    assert np.max(np.abs(Z - Zo)) < 1e-13
    Z32 = R.generate_normals(42, 300, 37, precision=R.MIXED, path_offset=12345)
    assert np.all(Z32.astype(np.float32).astype(np.float64) == Z32)
    # the FP32 transform runs on hardware approximations (lg2/sqrt/sin/cos
    # .approx): ~1e-6 relative except near r = 0, where log2(u) ~ 0 loses bits
    d = np.abs(Z32 - Zo)
    assert np.max(d) < 1e-3
    assert np.mean(d < 1e-5 * (1 + np.abs(Zo))) > 0.999


@pytest.mark.parametrize("name", QUAD_CASES)
def test_quadrature_vs_reference_fixture(R, name):
    c = quad(name)
    pay = R.computeIVRT_tensor_quadrature(float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"])
    ref = c["payoff"]
    assert pay.shape == ref.shape
    # per-sample payoffs: FFT (reference) vs direct sum, roundoff only
    assert np.max(np.abs(pay - ref) / np.maximum(np.abs(ref), 1e-3)) < 1e-11
    # prices (sample means): relative, with prices below 1e-3 held to 1e-15 absolute
    gp, rp = pay.mean(0), ref.mean(0)
    assert np.all(np.abs(gp - rp) <= PRICE_TOL * np.maximum(np.abs(rp), 1e-3))


def test_debug8_on_gpu(R):
    d = debug8()
    p = d["params"]
    i = np.arange(p["N"], dtype=float)
    Z = np.stack([np.stack([np.cos(i * float(m)), np.cos(i * float(m))]) for m in d["m"]])
    pay = R.computeIVRT_tensor_quadrature(p["xi"], [p["H"]], [p["eta"]], [p["rho"]], [p["T"]], [p["K"]], Z)[:, 0]
    want = np.array(d["payoff"])
    nz = want != 0
    assert np.all(rel_err(pay[nz], want[nz]) < 6e-6)


def test_dropin_rt_fixture(R, oracle):
    """GPU payoffs on the reference's own mt19937 normals reproduce
    computeIVRT_tensor(num_threads=1): price, stat, and IV to its tolerance."""
    c = dropin("rt")
    pay = R.computeIVRT_tensor_quadrature(float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"])
    price, stat = oracle.reduce(pay)
    assert np.all(rel_err(price, c["ref_price"]) < PRICE_TOL)
    assert np.all(rel_err(stat, c["ref_stat"]) < STAT_TOL)
    O = len(c["T"])
    Kt, Tt = np.tile(c["K"], len(c["H"])), np.tile(c["T"], len(c["H"]))
    iv = R.implied_vol(c["ref_price"], Kt, Tt)
    assert np.all(rel_err(iv, c["ref_iv"]) < IV_REF_TOL)
    assert np.all(rel_err(iv, [oracle.iv_call(p, k, t) for p, k, t in zip(c["ref_price"], Kt, Tt)]) < 1e-10)
    assert O == 2


GRID = dict(xi=0.04, H=[0.05, 0.1, 0.1, 0.3, 0.1], eta=[1.0, 1.5, 1.5, 2.5, 1.5],
            rho=[-0.95, -0.7, -0.5, -0.7, -0.3], T=[0.25, 0.25, 0.5, 1.0, 1.0, 2.0], K=[0.9, 1.1, 1.0, 0.8, 1.3, 2.0])


@pytest.mark.parametrize("N,M", [(64, 1000), (100, 4096), (1, 77)])
def test_fp64_prices_vs_oracle(R, oracle, N, M):
    """FP64 form, GPU reductions and IV, against the oracle on identical normals."""
    g = GRID
    price, stat, iv = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, seed=99)
    Z = R.generate_normals(99, M, N, precision=R.FP64)
    op, os_ = oracle.reduce(oracle.payoffs_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z))
    assert np.all(rel_err(price, op) < PRICE_TOL)
    assert np.all(rel_err(stat, os_) < STAT_TOL)
    O = len(g["T"])
    ivo = np.array([oracle.iv_call(p, g["K"][i % O], g["T"][i % O]) for i, p in enumerate(op)])
    ok = ~np.isnan(ivo)
    assert np.all(np.isnan(iv[~ok]))
    assert np.all(rel_err(iv[ok], ivo[ok]) < 1e-10)


def test_path_offset_and_batching_invariance(R):
    g = GRID
    s_all, q_all = R.price_rt_sums(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], 32, 3000, seed=5)
    s_a, q_a = R.price_rt_sums(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], 32, 1000, seed=5)
    s_b, q_b = R.price_rt_sums(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], 32, 2000, seed=5,
                               path_offset=1000)
    assert np.all(rel_err(s_a + s_b, s_all) < 1e-13)
    assert np.all(rel_err(q_a + q_b, q_all) < 1e-13)


def test_dropin_abi_vs_oracle(R, oracle):
    """computeIVRT_tensor through the C ABI: seed folding, layout, prices."""
    H, eta, rho, T, K = [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0], [0.8, 1.0]
    seed = [123, 452, 567]
    r = R.computeIVRT_tensor(0.07, H, eta, rho, T, K, 64, 2048, seed, num_threads=8)
    key = oracle.fold_seed(seed)
    Z = R.generate_normals(key, 2048, 64)
    op, os_ = oracle.reduce(oracle.payoffs_rt(0.07, H, eta, rho, T, K, Z))
    assert np.all(rel_err(r.price, op) < PRICE_TOL)
    assert np.all(rel_err(r.stat, os_) < STAT_TOL)
    np.testing.assert_array_equal(r.H, np.repeat(H, 2))
    np.testing.assert_array_equal(r.eta, np.repeat(eta, 2))
    np.testing.assert_array_equal(r.rho, np.repeat(rho, 2))
    np.testing.assert_array_equal(r.T, np.tile(T, 2))
    np.testing.assert_array_equal(r.K, np.tile(K, 2))


def test_reference_unit_test_prices(R):
    """testRBergLib/tests.cpp:16-44: |price - truePrice| < 0.005 + stat and
    |iv - IV(truePrice)| < 0.005 at the test's own N = 256, M = 10 * 256^2."""
    true = np.array([0.2149403, 0.08461882, 0.2157838, 0.07758564])
    H, eta, rho, T, K = [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0], [0.8, 1.0]
    r = R.computeIVRT_tensor(0.07, H, eta, rho, T, K, 256, 10 * 256 * 256, [123, 452, 567, 248], num_threads=8)
    assert np.all(np.abs(r.price - true) < 0.005 + r.stat)
    true_iv = R.implied_vol(true, np.tile(K, 2), np.tile(T, 2))
    assert np.all(np.abs(r.iv - true_iv) < 0.005)


def test_independent_stream_vs_reference_published(R):
    """rBergomiR/resRT_C.RData (computeIVRT_tensor, 4 threads): N=256,
    M=655,360 price 0.05817106 +- 6.9e-5.  Independent Philox stream must agree
    within 3 combined standard errors."""
    p, s, _ = R.price_rt(0.04, [0.06], [2.5], [-0.8], [0.8], [1.0], 256, 1 << 20, seed=17)
    ref, ref_se = 0.05817106, 6.9e-5
    assert abs(p[0] - ref) < 3 * np.hypot(s[0], ref_se)
