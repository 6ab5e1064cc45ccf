"""Sobol' quasi-Monte Carlo, CPU side: the oracle restatement pinned to the
reference's own generator (rBergomi/sobol.cpp i8_sobol, rBergomi/qmc.cpp
normalQMC_sample, rBergomi/aux.h hierarchical2increments) through the
committed fixture tests/golden/sobol.npz, and live against oracle/_ref when the
reference was compiled in this checkout."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sobol.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def V(gold, oracle):
    return oracle.sobol_directions_from_points(gold["gray_points"])


def test_direction_integers_are_sobol(V):
    # column k holds m_k 2^(61 - k) with m_k odd and below 2^(k+1); dimension 0
    # is the van der Corput sequence (all m_k = 1)
    K = 24
    for k in range(K):
        m = V[:, k] >> np.uint64(61 - k)
        assert np.all(m % 2 == 1) and np.all(m < (1 << (k + 1)))
        assert np.all(V[:, k] == m << np.uint64(61 - k))
    assert np.all(V[0, :K] >> np.uint64(61 - np.arange(K)) == 1)


def test_oracle_points_match_reference_fixture(gold, V, oracle):
    run = gold["run_points"]  # i8_sobol points 1..64, 128 dimensions
    for s in range(1, 65):
        np.testing.assert_array_equal(oracle.sobol_point(V, s, 128), run[s - 1])


def test_oracle_normals_match_reference_fixture(gold, V, oracle):
    """normalQMC_sample(Z, 128, i) of the reference (quantile from the oracle's
    Boost stand-in) against the oracle's point + quantile."""
    for i, z in zip(gold["sample_index"], gold["samples"]):
        np.testing.assert_allclose(oracle.inv_normal(oracle.sobol_point(V, int(i), 128)), z, rtol=0, atol=1e-14)


def test_oracle_bridge_matches_reference_fixture(gold, oracle):
    np.testing.assert_allclose(oracle.hier(gold["hier_in"]), gold["hier_out"], rtol=0, atol=1e-15)


def test_bridge_properties(oracle):
    rng = np.random.default_rng(3)
    for n in (1, 2, 4, 64, 512):
        z = rng.standard_normal(n)
        w = oracle.hier(z)
        # orthonormal (Haar synthesis): norms kept; the increments sum to the
        # endpoint sqrt(n) Z[0]
        assert np.isclose(np.linalg.norm(w), np.linalg.norm(z), rtol=1e-13)
        assert np.isclose(w.sum(), np.sqrt(n) * z[0], rtol=1e-12, atol=1e-12)
    with pytest.raises(ValueError):
        oracle.hier(np.zeros(6))


def test_quantile_accuracy(oracle):
    from scipy.special import ndtri

    p = np.concatenate([np.logspace(np.log10(2.0 ** -62), -1, 400), np.linspace(0.01, 0.99, 197),
                        1 - np.logspace(-16, -1, 100)])
    np.testing.assert_allclose(oracle.inv_normal(p), ndtri(p), rtol=0, atol=4e-15 * 9)


def test_oracle_normals_layout(V, oracle):
    """Path m takes point path0 + m + 1; W1 = even coordinates, W1perp = odd."""
    N = 8
    Z = oracle.sobol_normals(V, N, 5, path0=10)
    for m in range(5):
        x = oracle.inv_normal(oracle.sobol_point(V, 10 + m + 1, 2 * N))
        np.testing.assert_array_equal(Z[m, 0], x[0::2])
        np.testing.assert_array_equal(Z[m, 1], x[1::2])
    Zb = oracle.sobol_normals(V, N, 5, path0=10, bridge=True)
    for m in range(5):
        np.testing.assert_allclose(Zb[m, 0], oracle.hier(Z[m, 0]), rtol=0, atol=0)
    with pytest.raises(ValueError):
        oracle.sobol_normals(V, 6, 2, bridge=True)


def test_live_reference_generator(oracle, V):
    if not oracle.qmc_ref_available():
        pytest.skip("reference Sobol' build not present (needs the reference sources)")
    seeds = np.unique(np.concatenate([np.arange(1, 2000), np.random.default_rng(5).integers(2000, 1 << 17, 200)]))
    ref = oracle.qmc_ref_points(1111, seeds)
    for s, x in zip(seeds, ref):
        np.testing.assert_array_equal(oracle.sobol_point(V, int(s)), x)
    rng = np.random.default_rng(9)
    for n in (2, 32, 256):
        z = rng.standard_normal(n)
        np.testing.assert_array_equal(oracle.hier(z), oracle.qmc_ref_hier(z))


def test_sobol_entry_takes_every_mixed_form():
    """The mixed form takes the bridge and the FFT backend on Sobol' points
    (the normals are materialized); no host-side refusal precedes the device
    work, which this container cannot run.  A malformed table is refused
    before any call."""
    import rbergomi_gb300 as R

    V = np.zeros((8, 62), np.uint64)
    a = (0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 4, 16, V)
    for kw in (dict(bridge=True, precision=R.MIXED), dict(precision=R.MIXED, conv=R.CONV_FFT)):
        with pytest.raises(R.RbgError) as e:
            R.price_rt_sobol(*a, **kw)
        assert "FP64 form only" not in str(e.value) and "GEMM backend" not in str(e.value)
    with pytest.raises(ValueError):
        R.price_rt_sobol(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 4, 16, np.zeros((8, 63), np.uint64))


def test_fp32_quantile_coefficients():
    """The FP32 quantile of the mixed form's Sobol' normals
    (rbg_device.cuh normal_quantile_lower_f32), evaluated in float32 with the
    coefficients parsed from the CUDA source: relative error <= 6e-7 of the
    exact quantile of its float32 input on [2^-32, 1/2]."""
    import re

    from scipy.special import ndtri

    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "rbergomi_gb300", "csrc",
                            "rbg_device.cuh")).read()
    body = src[src.index("normal_quantile_lower_f32(float u)"):]
    cen, tail = [np.array([float(v.rstrip("f")) for v in m.split(",")], np.float32)
                 for m in re.findall(r"const float c\[9\] = \{([^}]*)\}", body)[:2]]
    f32 = np.float32
    u = np.concatenate([np.logspace(np.log10(2.0 ** -32), np.log10(0.5), 100000),
                        np.linspace(0.3, 0.5, 50000)]).astype(f32)
    x = f32(2) * u - f32(1)
    w = (-np.log(f32(4) * u * (f32(1) - u))).astype(f32)
    t, s = (w - f32(2.5)).astype(f32), (np.sqrt(w) - f32(3)).astype(f32)
    p, q = np.full_like(u, cen[0]), np.full_like(u, tail[0])
    for a, b in zip(cen[1:], tail[1:]):
        p, q = (p * t + a).astype(f32), (q * s + b).astype(f32)
    z = (f32(1.41421356) * x * np.where(w < 5, p, q)).astype(np.float64)
    zt = ndtri(u.astype(np.float64))
    m = np.abs(zt) > 1e-6
    assert np.max(np.abs(z[m] - zt[m]) / np.abs(zt[m])) < 6e-7
