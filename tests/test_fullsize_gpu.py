"""Parity at the workloads' full sizes (the shapes the benchmarks run).

At these sizes the oracle would take minutes, so each check is a property
that holds at any size:
  - the mixed form against the FP64 form on identical FP32 normals (the FP64
    form's RBG_NORMALS_F32 option), <= 1e-4 relative and < 0.2 standard
    errors per price;
  - the FP64 form against the oracle where the oracle is quick (N=100, 2^16
    paths);
  - the counter-based stream's causal prefix: the first n steps of an N-step
    draw are the n-step draw, which is what lets one Gaussian draw serve all
    maturities of a grid."""
import numpy as np
import pytest

from tests._golden import rel_err

pytestmark = pytest.mark.gpu

REL, SE = 1e-4, 0.2


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


def assert_mixed_matches(R, args, seed, **opts):
    fp, fs, _ = R.price_rt(*args, seed=seed, normals=R.NORMALS_F32, **opts)
    mp, _, _ = R.price_rt(*args, seed=seed, precision=R.MIXED, **opts)
    assert np.all(rel_err(mp, fp) < REL), np.max(rel_err(mp, fp))
    assert np.all(np.abs(mp - fp) < SE * fs), np.max(np.abs(mp - fp) / fs)


def test_workload0_fp64_vs_oracle(R, oracle):
    """N=100, 2^16 paths, five strikes, seed 42: FP64 form against the oracle
    on the same Philox normals."""
    xi, H, eta, rho, T, K = 0.235 ** 2, [0.07], [1.9], [-0.9], [1.0] * 5, [0.8, 0.9, 1.0, 1.1, 1.2]
    price, stat, _ = R.price_rt(xi, H, eta, rho, T, K, 100, 1 << 16, seed=42)
    Z = R.generate_normals(42, 1 << 16, 100)
    op, os_ = oracle.reduce(oracle.payoffs_rt(xi, H, eta, rho, T, K, Z))
    assert np.all(rel_err(price, op) < 1e-12)
    assert np.all(rel_err(stat, os_) < 1e-8)


def test_workload1_grid_mixed_vs_fp64(R):
    """The full ParamTot grid: 48 (H, eta, rho) tuples x 4 maturities x 11
    strikes, 256 steps per unit time, 2^20 paths, seed 7."""
    Hs, etas, rhos = [0.05, 0.1, 0.2, 0.3], [1.0, 1.5, 2.0, 2.5], [-0.95, -0.7, -0.5]
    H = [h for h in Hs for _ in etas for _ in rhos]
    eta = [e for _ in Hs for e in etas for _ in rhos]
    rho = [r for _ in Hs for _ in etas for r in rhos]
    K = list(np.round(np.linspace(0.7, 1.3, 11), 10))
    for T in (0.25, 0.5, 1.0, 2.0):
        assert_mixed_matches(R, (0.235 ** 2, H, eta, rho, [T] * 11, K, int(256 * T), 1 << 20), 7)


def test_workload2_headline_mixed_vs_fp64(R):
    """N=512, 2^22 paths, 21 strikes on [0.6, 1.4], seed 11."""
    K = list(np.round(np.linspace(0.6, 1.4, 21), 10))
    assert_mixed_matches(R, (0.235 ** 2, [0.1], [1.9], [-0.9], [1.0] * 21, K, 512, 1 << 22), 11)


@pytest.mark.parametrize("N", [1024, 2048])
def test_workload3_long_horizon_mixed_vs_fp64(R, N):
    """N=1024 (two-pass tensor-core GEMM) and N=2048 (four passes, strip
    windows streamed), 2^20 paths, three H, 11 strikes on [0.5, 1.5], seed 3."""
    K = list(np.round(np.linspace(0.5, 1.5, 11), 10))
    assert_mixed_matches(R, (0.04, [0.03, 0.1, 0.4], [1.5] * 3, [-0.7] * 3, [2.0] * 11, K, N, 1 << 20), 3)


def test_causal_prefix_of_the_stream(R):
    a = R.generate_normals(7, 4096, 512)
    for n in (64, 128, 256, 37):
        np.testing.assert_array_equal(R.generate_normals(7, 4096, n), a[:, :, :n])
