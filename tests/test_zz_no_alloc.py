"""The allocation-free entry point rbg_price_rt_static, through the C ABI.

It serves callers that cannot call cudaMalloc (a host that pre-reserved all
device memory for its own pool, or a latency-critical loop that cannot take
cudaMalloc's device-wide synchronisation).  Its results must match the
regular entry point rbg_price_rt on the same inputs, on two calls in a row
(the shared static scratch keeps the previous call's contents, so a second
call checks that everything that must start at zero is cleared).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same kernels, same batching of the Philox stream: roundoff only
# 512 < N <= 1024 (16-bit splits): rbg_price_rt runs 256-column TMEM passes
# whose far-field reads A tiles back from a per-CTA device cache (tens of MB),
# which does not fit the static scratch, so the static entry runs the two-pass
# kernel that draws those tiles again.  Same products, another FP32
# accumulation order in TMEM, and W1 in the epilogue as drawn in FP32 instead
# of read back as the 16-bit hi + lo pair: prices agree to about 1e-6.
RTOL_TWO_PASS = (2e-6, 2e-5)  # prices; standard errors and implied vols


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    L = R.lib()
    L.rbg_price_rt_static.argtypes = [C.POINTER(R.RbgParams), C.POINTER(R.RbgOptions), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.rbg_price_rt_static.restype = C.c_int
    L.rbg_static_last_error.restype = C.c_char_p
    L.rbg_static_scratch_bytes.restype = C.c_size_t
    return R


def static_price(R, xi, H, eta, rho, T, K, N, M, **opts):
    p = R._Params(xi, H, eta, rho, T, K, N, M)
    o = R.options(precision=R.MIXED, **opts)
    price, stat, iv = np.empty(p.out), np.empty(p.out), np.empty(p.out)
    dp = C.POINTER(C.c_double)
    rc = R.lib().rbg_price_rt_static(C.byref(p.s), C.byref(o), price.ctypes.data_as(dp), stat.ctypes.data_as(dp),
                                     iv.ctypes.data_as(dp))
    if rc != 0:
        raise R.RbgError(f"static entry point status {rc}: {R.lib().rbg_static_last_error().decode()}")
    return price, stat, iv


CASES = [
    # workload-2 shape, reduced M
    dict(xi=0.235 ** 2, H=[0.1], eta=[1.9], rho=[-0.9], T=[1.0] * 21, K=list(np.linspace(0.6, 1.4, 21)), N=512,
         M=(1 << 18) + 77, seed=11),
    # two Volterra passes, several variance groups, N = 1024 (the two-pass kernel in the static entry)
    dict(xi=0.04, H=[0.07, 0.3], eta=[1.5, 2.0], rho=[-0.7, -0.5], T=[0.5, 2.0], K=[0.9, 1.2], N=1024, M=5000,
         seed=3),
    # longer horizon: three TMEM passes with streamed strip windows, and the batched-FFT backend
    dict(xi=0.05, H=[0.1], eta=[1.5], rho=[-0.7], T=[2.0, 2.0, 2.0], K=[0.8, 1.0, 1.2], N=1500, M=3001, seed=4),
    dict(xi=0.05, H=[0.1], eta=[1.5], rho=[-0.7], T=[2.0, 2.0, 2.0], K=[0.8, 1.0, 1.2], N=1500, M=3001, seed=4,
         conv=2),
    # eight variance groups over 300,001 paths: the (Ivdt, IsvdW) buffer (8 B per group and path, 19.2 MB)
    # does not fit the 16 MiB array, so the paths run in smaller batches than rbg_price_rt's single one
    dict(xi=0.04, H=[0.1], eta=[1.9], rho=[-0.9], T=[0.25, 0.5, 0.75, 1.0, 1.25, 1.5, 1.75, 2.0],
         K=[0.8, 0.9, 1.0, 1.1, 1.2, 1.0, 0.95, 1.05], N=128, M=300001, seed=5),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_static_entry_point_matches_regular(R, case):
    c = dict(CASES[case])
    seed = c.pop("seed")
    conv = c.pop("conv", 0)
    args = (c["xi"], c["H"], c["eta"], c["rho"], c["T"], c["K"], c["N"], c["M"])
    want_p, want_s, want_iv = R.price_rt(*args, seed=seed, precision=R.MIXED, conv=conv)
    rp, rs = (RTOL, 1e-9) if not (512 < c["N"] <= 1024 and conv == 0) else RTOL_TWO_PASS
    for _ in range(2):  # second call runs on the contents the first call left behind
        p, s, iv = static_price(R, *args, seed=seed, conv=conv)
        np.testing.assert_allclose(p, want_p, rtol=rp, atol=0)
        np.testing.assert_allclose(s, want_s, rtol=rs, atol=0)
        np.testing.assert_allclose(iv, want_iv, rtol=rs, atol=0)


def test_static_entry_point_rejects_oversize(R):
    assert R.lib().rbg_static_scratch_bytes() == 16 << 20
    with pytest.raises(R.RbgError, match="4096 outputs"):
        static_price(R, 0.04, [0.1] * 70, [1.5] * 70, [-0.7] * 70, [1.0] * 60, [1.0] * 60, 64, 1024)
