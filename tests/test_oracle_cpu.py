"""The CPU oracle pinned against the reference's own golden vectors (no GPU)."""
import numpy as np
import pytest

from tests._golden import QUAD_CASES, debug8, dropin, dropin_cv, quad, rel_err


def test_philox_known_answers(oracle):
    # Random123 published known-answer vectors for Philox4x32-10
    assert list(oracle.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                                       0x6D5451FD]
    assert list(oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_normals_moments_and_layout(oracle):
    Z = oracle.normals_f64(42, 4096, 64, 2)
    assert abs(Z.mean()) < 0.01 and abs(Z.std() - 1) < 0.01
    # a later block of paths is the tail of a longer draw (counter = global path index)
    Zb = oracle.normals_f64(42, 96, 64, 2, path0=4000)
    np.testing.assert_array_equal(Zb, Z[4000:])
    # a shorter horizon is the prefix of a longer one (counter = step group)
    Zs = oracle.normals_f64(42, 16, 37, 2)
    np.testing.assert_array_equal(Zs, oracle.normals_f64(42, 16, 64, 2)[:, :, :37])


def test_debug8_known_answer(oracle):
    """rBergomi/testing/debug8.txt~: per-path RT payoffs printed to 6 digits."""
    d = debug8()
    p = d["params"]
    N = p["N"]
    i = np.arange(N, dtype=float)
    Z = np.stack([np.stack([np.cos(i * float(m)), np.cos(i * float(m))]) for m in d["m"]])
    pay = oracle.payoffs_rt(p["xi"], [p["H"]], [p["eta"]], [p["rho"]], [p["T"]], [p["K"]], Z)[:, 0]
    want = np.array(d["payoff"])
    nz = want != 0
    assert np.all(rel_err(pay[nz], want[nz]) < 6e-6)
    assert np.all(np.abs(pay[~nz]) < 1e-6)


@pytest.mark.parametrize("name", QUAD_CASES)
def test_quadrature_fixtures(oracle, name):
    """Oracle payoffs == reference computeIVRT_tensor_quadrature on identical normals."""
    c = quad(name)
    pay = oracle.payoffs_rt(float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"])
    assert pay.shape == c["payoff"].shape
    # FFT (reference) vs direct causal sum (oracle): roundoff only
    assert np.max(np.abs(pay - c["payoff"]) / np.maximum(np.abs(c["payoff"]), 1e-3)) < 1e-11


def test_dropin_rt_fixture(oracle):
    """computeIVRT_tensor(num_threads=1) replayed on its own mt19937_64 normals."""
    c = dropin("rt")
    pay = oracle.payoffs_rt(float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"])
    price, stat = oracle.reduce(pay)
    assert np.all(rel_err(price, c["ref_price"]) < 1e-12)
    assert np.all(rel_err(stat, c["ref_stat"]) < 1e-8)
    out = len(price)
    P, O = len(c["H"]), len(c["T"])
    assert out == P * O
    iv = np.array([oracle.iv_call(price[i], c["K"][i % O], c["T"][i % O]) for i in range(out)])
    # the reference inverts to 2^(1-11) relative bracket width and returns the midpoint
    assert np.all(rel_err(iv, c["ref_iv"]) < 2.0 ** -10)
    np.testing.assert_array_equal(c["ref_H"], np.repeat(c["H"], O))
    np.testing.assert_array_equal(c["ref_eta"], np.repeat(c["eta"], O))
    np.testing.assert_array_equal(c["ref_rho"], np.repeat(c["rho"], O))
    np.testing.assert_array_equal(c["ref_T"], np.tile(c["T"], P))
    np.testing.assert_array_equal(c["ref_K"], np.tile(c["K"], P))


def test_dropin_mc_fixture(oracle):
    """computeIV_tensor(num_threads=1) replayed; its eta_tot/rho_tot are swapped."""
    c = dropin("mc")
    pay = oracle.payoffs_mc(float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"])
    price, stat = oracle.reduce(pay)
    assert np.all(rel_err(price, c["ref_price"]) < 1e-12)
    assert np.all(rel_err(stat, c["ref_stat"]) < 1e-8)
    O = len(c["T"])
    np.testing.assert_array_equal(c["ref_eta"], np.repeat(c["rho"], O))  # quirk: rBergLib/cinterface.cpp:45
    np.testing.assert_array_equal(c["ref_rho"], np.repeat(c["eta"], O))


def test_reference_unit_test_prices(oracle):
    """testRBergLib/tests.cpp:16-22 truePrice, |price - true| < 0.005 + stat, on
    the project's Philox stream (RT estimator, N = 256)."""
    true = np.array([0.2149403, 0.08461882, 0.2157838, 0.07758564])
    price, stat = oracle.price_rt_philox(0.07, [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0], [0.8, 1.0],
                                         256, 1 << 14, 2024)
    assert np.all(np.abs(price - true) < 0.005 + stat)


def test_iv_roundtrip(oracle):
    for K in (0.6, 0.9, 1.0, 1.1, 1.4):
        for T in (0.1, 1.0, 3.0):
            for s in (0.05, 0.2, 0.8):
                p = oracle.bs_call(1.0, K, T, s)
                if p - max(1 - K, 0) < 1e-8:  # ITM time value lost to cancellation
                    continue
                assert abs(oracle.iv_call(p, K, T) / s - 1) < 1e-8
    assert np.isnan(oracle.iv_call(0.0, 1.2, 1.0))
    assert np.isnan(oracle.iv_call(1.5, 1.0, 1.0))


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).ref_available(),
                    reason="reference build (oracle/_ref) only exists where the reference sources are mounted")
def test_live_reference_random_grid(oracle):
    rng = np.random.default_rng(5)
    H = rng.uniform(0.03, 0.45, 3)
    eta = rng.uniform(0.5, 3.0, 3)
    rho = rng.uniform(-0.99, -0.3, 3)
    T = np.sort(rng.uniform(0.05, 3.0, 4))
    K = rng.uniform(0.5, 1.5, 4)
    Z = oracle.normals_f64(99, 50, 80, 2)
    a = oracle.payoffs_rt(0.06, H, eta, rho, T, K, Z)
    b = oracle.ref_payoffs_rt(0.06, H, eta, rho, T, K, Z)
    assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-3)) < 1e-11


@pytest.mark.parametrize("name", ["base", "qmax"])
def test_cv_oracle_vs_reference_fixture(oracle, name):
    """The control-variate estimator (ML_console_ST's ComputeIVRTVarRed,
    compiled from its own sources) replayed on the pilot and main normals it
    drew: price 1e-12, stat 1e-8; the qmax case takes the Q_max branch."""
    d = dropin_cv(name)
    price, stat, alpha, Q, cnt = oracle.price_rt_cv(d["xi"], d["H"], d["eta"], d["rho"], d["T"], d["K"],
                                                    d["Zc"], d["Z"])
    assert np.all(rel_err(price, d["ref_price"]) < 1e-12)
    assert np.all(rel_err(stat, d["ref_stat"]) < 1e-8)
    if name == "qmax":
        assert cnt.sum() > 0
    else:
        assert cnt.sum() == 0
