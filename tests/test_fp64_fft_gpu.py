"""The FP64 form's FFT Volterra convolution (k_path_fp64_fft): Stockham
radix-4/2 transforms in FP64, two paths per complex transform, used by AUTO
from 200 steps.  Against the oracle (a direct causal sum) on identical
normals at the same 1e-12 as the direct kernel, and against the direct
kernel itself, for RT, plain Monte Carlo, the control-variate form (the
antithetic variant) and the per-path quadrature."""
import numpy as np
import pytest

from tests._golden import rel_err

pytestmark = pytest.mark.gpu

PRICE_TOL = 1e-12
STAT_TOL = 1e-8

GRID = dict(xi=0.04, H=[0.05, 0.1, 0.1, 0.3, 0.1], eta=[1.0, 1.5, 1.5, 2.5, 1.5],
            rho=[-0.95, -0.7, -0.5, -0.7, -0.3], T=[0.25, 0.25, 0.5, 1.0, 1.0, 2.0], K=[0.9, 1.1, 1.0, 0.8, 1.3, 2.0])


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


# L = 512 (radix 2 + 4 x radix 4), 1024, 2048 (odd: radix-2 first), 4096; N = 3, 37 force the FFT at L = 256
@pytest.mark.parametrize("N,M,conv", [(256, 600, "auto"), (300, 401, "auto"), (512, 300, "auto"),
                                      (700, 160, "auto"), (1500, 41, "auto"), (3, 999, "fft"), (37, 500, "fft")])
def test_fp64_fft_prices_vs_oracle(R, oracle, N, M, conv):
    g = GRID
    kw = dict(seed=7) if conv == "auto" else dict(seed=7, conv=R.CONV_FFT)
    price, stat, iv = R.price_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M, **kw)
    Z = R.generate_normals(7, M, N, precision=R.FP64)
    op, os_ = oracle.reduce(oracle.payoffs_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z))
    assert np.all(np.abs(price - op) <= PRICE_TOL * np.maximum(np.abs(op), 1e-3))
    assert np.all(np.abs(stat - os_) <= STAT_TOL * np.maximum(np.abs(os_), 1e-6))
    O = len(g["T"])
    ivo = np.array([oracle.iv_call(p, g["K"][i % O], g["T"][i % O]) for i, p in enumerate(op)])
    ok = ~np.isnan(ivo)
    np.testing.assert_array_equal(np.isnan(iv), ~ok)
    assert np.all(rel_err(iv[ok], ivo[ok]) < 1e-10)


@pytest.mark.parametrize("N", [256, 1024, 2048])
def test_fp64_fft_matches_direct_sum(R, N):
    g = GRID
    M = 2001  # odd: the last transform pairs a path with nothing
    a = (g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], N, M)
    pf, sf, _ = R.price_rt(*a, seed=3, conv=R.CONV_FFT)
    pd, sd, _ = R.price_rt(*a, seed=3, conv=R.CONV_DIRECT)
    assert np.all(np.abs(pf - pd) <= PRICE_TOL * np.maximum(np.abs(pd), 1e-3))
    assert np.all(np.abs(sf - sd) <= STAT_TOL * np.maximum(np.abs(sd), 1e-6))


def test_fp64_fft_plain_mc_vs_oracle(R, oracle):
    xi, H, eta, rho = 0.05, [0.07, 0.2], [1.9, 1.2], [-0.9, -0.6]
    T, K = [0.5, 0.5, 1.5], [0.9, 1.1, 1.0]
    N, M, seed = 300, 801, 31
    p, s, _ = R.price_mc(xi, H, eta, rho, T, K, N, M, seed=seed)
    Z = R.generate_normals(seed, M, N, streams=3)
    op, os_ = oracle.reduce(oracle.payoffs_mc(xi, H, eta, rho, T, K, Z))
    assert np.all(rel_err(p, op) < PRICE_TOL)
    assert np.all(rel_err(s, os_) < STAT_TOL)


def test_fp64_fft_control_variate_vs_oracle(R, oracle):
    """The antithetic path pass (ANTI) through the FFT kernel."""
    xi, H, eta, rho = [0.04, 0.06], [0.07, 0.35], [1.9, 2.4], [-0.9, -0.7]
    T, K = [1.0, 2.0], [1.05, 1.2]
    N, M, Mc, seed = 256, 600, 300, 13
    price, stat, _ = R.price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=Mc, seed=seed)
    Zc = R.generate_normals(seed, Mc, N, path_offset=1 << 62)
    Z = R.generate_normals(seed, M, N)
    op, os_, _, _, _ = oracle.price_rt_cv(xi, H, eta, rho, T, K, Zc, Z)
    assert np.all(rel_err(price, op) < PRICE_TOL)
    assert np.all(rel_err(stat, os_) < STAT_TOL)


def test_fp64_fft_quadrature_payoffs(R, oracle):
    g = GRID
    N, M = 333, 257
    Z = np.random.default_rng(5).standard_normal((M, 2, N))
    pay = R.computeIVRT_tensor_quadrature(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z)
    want = oracle.payoffs_rt(g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"], Z)
    assert np.max(np.abs(pay - want) / np.maximum(np.abs(want), 1e-3)) < 1e-11


def test_fp64_backend_errors(R):
    g = GRID
    a = (g["xi"], g["H"], g["eta"], g["rho"], g["T"], g["K"])
    with pytest.raises(R.RbgError, match="GEMM"):
        R.price_rt(*a, 64, 16, conv=R.CONV_GEMM)
    with pytest.raises(R.RbgError, match="2048"):
        R.price_rt(*a, 2049, 16, conv=R.CONV_FFT)
