"""Unordered parameter lists (the reference's ParamTotUnordered +
ComputeIVRTMTunstructured, rBergomi/ParamTot.h:57-75 and
rBergomi/rBergomiMT.cpp:837-957): every index recomputes its own chain, so
output i must equal a one-tuple ParamTot call on the same normals."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


def tuples(n, seed):
    rng = np.random.default_rng(seed)
    H = rng.choice([0.07, 0.1, 0.3], n)
    eta = rng.choice([1.5, 2.2], n)
    rho = rng.uniform(-0.95, -0.4, n)
    T = rng.choice([0.25, 1.0, 1.7], n)
    K = rng.uniform(0.7, 1.3, n)
    H[3], eta[3], T[3], rho[3], K[3] = H[0], eta[0], T[0], rho[0], K[0]  # an exact duplicate
    return H, eta, rho, T, K


def test_unordered_fp64_vs_oracle_per_tuple(R, oracle):
    xi, N, M, seed = 0.05, 64, 4096, 17
    H, eta, rho, T, K = tuples(12, 1)
    p, s, iv = R.price_rt_unordered(xi, H, eta, rho, T, K, N, M, seed=seed)
    for i in range(len(H)):
        op, os_ = oracle.price_rt_philox(xi, [H[i]], [eta[i]], [rho[i]], [T[i]], [K[i]], N, M, seed)
        assert abs(p[i] - op[0]) <= 1e-12 * abs(op[0])
        assert abs(s[i] - os_[0]) <= 1e-8 * abs(os_[0])
    assert p[3] == p[0] and s[3] == s[0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_unordered_equals_tensor_grid(R, precision):
    """A ParamTot grid without near-duplicate values, flattened to tuples,
    prices bit for bit like the ordered call."""
    prec = R.FP64 if precision == "fp64" else R.MIXED
    xi, N, M = 0.04, 100, 1 << 13
    H, eta, rho = [0.05, 0.1, 0.1, 0.3], [1.0, 1.5, 2.0, 2.5], [-0.9, -0.7, -0.5, -0.8]
    T, K = [0.25, 0.5, 0.5, 1.0, 2.0], [0.9, 1.0, 1.1, 1.0, 1.2]
    p0, s0, _ = R.price_rt(xi, H, eta, rho, T, K, N, M, seed=5, precision=prec)
    P, O = len(H), len(T)
    flat = lambda a, b: (np.repeat(a, O), np.tile(b, P))
    Hu, Tu = flat(H, T)
    eu, Ku = flat(eta, K)
    ru = np.repeat(rho, O)
    p1, s1, _ = R.price_rt_unordered(xi, Hu, eu, ru, Tu, Ku, N, M, seed=5, precision=prec)
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(s1, s0)


def test_unordered_mixed_vs_fp64(R):
    xi, N, M = 0.06, 700, 1 << 13
    H, eta, rho, T, K = tuples(10, 2)
    mp, ms, _ = R.price_rt_unordered(xi, H, eta, rho, T, K, N, M, seed=8, precision=R.MIXED)
    fp, fs, _ = R.price_rt_unordered(xi, H, eta, rho, T, K, N, M, seed=8, normals=R.NORMALS_F32)
    big = fp > 1e-4
    assert np.all(np.abs(mp - fp)[big] <= 1e-4 * fp[big])
    assert np.all(np.abs(mp - fp) < 0.2 * fs)


def test_unordered_rejects_bad_input(R):
    with pytest.raises(R.RbgError):
        R.price_rt_unordered(0.04, [0.1, 1.2], [1.5, 1.5], [-0.7, -0.7], [1.0, 1.0], [1.0, 1.0], 64, 256)
    with pytest.raises(ValueError):
        R.price_rt_unordered(0.04, [0.1], [1.5, 1.5], [-0.7], [1.0], [1.0], 64, 256)
