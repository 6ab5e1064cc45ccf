"""GPU parity of the control-variate Romano-Touzi estimator (ML_console_ST's
RBergomi::ComputeIVRTVarRed, ML_console_ST/RBergomi.cpp:218-306 and 478-540):
pilot Q and alpha, antithetic main paths, closed-form adjustment.  FP64:
1e-12 relative on prices against the reference's own output on the normals
it drew, and against the oracle on the Philox stream; the mixed form within
1e-4 relative and 0.2 standard errors of the FP64 form on the same normals."""
import numpy as np
import pytest

from tests._golden import dropin_cv, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


@pytest.mark.parametrize("name", ["base", "qmax"])
def test_cv_vs_reference_fixture(R, oracle, name):
    d = dropin_cv(name)
    price, stat, iv = R.price_rt_cv_normals(d["xi"], d["H"], d["eta"], d["rho"], d["T"], d["K"], d["Zc"], d["Z"])
    assert np.all(rel_err(price, d["ref_price"]) < 1e-12)
    assert np.all(rel_err(stat, d["ref_stat"]) < 1e-8)
    # the reference inverts with Newton to 2^-10; ours is the FP64 bracketing search
    ivo = np.array([oracle.iv_call(p, k, t) for p, k, t in zip(price, d["K"], d["T"])])
    assert np.all(rel_err(iv, ivo) < 1e-10)
    assert np.all(np.abs(iv - d["ref_iv"]) < 2.0 ** -9 * d["ref_iv"])


def test_cv_philox_vs_oracle(R, oracle):
    xi, H, eta, rho = [0.04, 0.06, 0.05], [0.07, 0.2, 0.35], [1.9, 1.2, 2.4], [-0.9, -0.5, -0.7]
    T, K = [1.0, 0.5, 2.0], [1.05, 0.95, 1.2]
    N, M, Mc, seed = 48, 3000, 700, 13
    price, stat, _ = R.price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=Mc, seed=seed)
    Zc = R.generate_normals(seed, Mc, N, path_offset=1 << 62)
    Z = R.generate_normals(seed, M, N)
    op, os_, _, _, _ = oracle.price_rt_cv(xi, H, eta, rho, T, K, Zc, Z)
    assert np.all(rel_err(price, op) < 1e-12)
    assert np.all(rel_err(stat, os_) < 1e-8)


def test_cv_reduces_the_standard_error(R):
    """The control variate and antithetics leave the estimate unbiased (two
    independent seeds agree) and cut the standard error well below the plain
    Romano-Touzi estimator's on the same number of paths."""
    xi, H, eta, rho, T, K = 0.235 ** 2, [0.07], [1.9], [-0.9], [1.0], [1.0]
    N, M = 100, 1 << 15
    p1, s1, _ = R.price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=4000, seed=1)
    p2, s2, _ = R.price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=4000, seed=2)
    assert abs(p1[0] - p2[0]) < 4 * np.hypot(s1[0], s2[0])
    _, srt, _ = R.price_rt(xi, H, eta, rho, T, K, N, M, seed=1)
    assert s1[0] < 0.5 * srt[0]


@pytest.mark.parametrize("N,M,Mc,conv", [(100, 1 << 14, 2000, "auto"), (512, 1 << 14, 2000, "auto"),
                                         (1536, 8192, 1500, "auto"), (64, 1 << 14, 40, "auto"),
                                         (700, 8192, 1500, "fft")])
def test_mixed_cv_matches_fp64_cv_on_the_same_normals(R, N, M, Mc, conv):
    """The mixed form of the control-variate estimator -- FP64 pilot, main
    paths through the tensor-core kernel as is and with the exponent negated
    (the antithetic paths), FP32 payoffs -- against the FP64 form on the same
    FP32 normals (RBG_NORMALS_F32): the same pilot alpha and Q, prices within
    1e-4 relative and 0.2 of their standard error.  One tuple xi each; one and
    three TMEM passes and the FFT backend; M_control = 40 sends paths through
    the Q_max branch."""
    xi, H, eta, rho = [0.04, 0.06, 0.05, 0.03], [0.07, 0.2, 0.35, 0.1], [1.9, 1.2, 2.4, 1.5], [-0.9, -0.5, -0.7, -0.8]
    T, K = [1.0, 0.5, 2.0, 0.25], [1.05, 0.95, 1.2, 1.0]
    p64, s64, iv64 = R.price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=Mc, seed=21, normals=R.NORMALS_F32)
    p32, s32, iv32 = R.price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=Mc, seed=21, precision=R.MIXED,
                                   conv=R.CONV_FFT if conv == "fft" else R.CONV_AUTO)
    assert np.all(rel_err(p32, p64) < 1e-4)
    assert np.all(np.abs(p32 - p64) < 0.2 * s64)
    assert np.all(rel_err(s32, s64) < 1e-2)
    assert np.all(rel_err(iv32, iv64) < 1e-3)


def test_cv_rejects_bad_input(R):
    with pytest.raises(R.RbgError):
        R.price_rt_cv(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 32, 256, M_control=1)
    with pytest.raises(R.RbgError):  # no such precision
        R.price_rt_cv(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 32, 256, M_control=100, precision=7)
