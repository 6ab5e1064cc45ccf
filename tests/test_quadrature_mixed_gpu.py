"""Per-path payoffs for caller-supplied normals in the mixed form (the
quadrature entry points rbg_payoffs_rt / rbg_payoffs_mc with precision MIXED,
and computeIVRT_tensor_quadrature under RBG_PRECISION=mixed): the caller's
FP64 normals go through the tensor-core path kernel (FP32 path state), and
each path's payoff comes out of the FP32 Black-Scholes formula.

Against the reference's own payoffs (the fixtures tests/golden/quad_*.npz,
rBergLib computeIVRT_tensor_quadrature) and against the FP64 form on the same
normals.  Per path: |mixed - FP64| <= PATH_TOL * max(|FP64|, 0.01) (plain
MC: PATH_TOL_MC); over the paths: the means within 1e-4 relative, the mixed
form's price bound."""
import os

import numpy as np
import pytest

from tests._golden import QUAD_CASES, quad, rel_err

pytestmark = pytest.mark.gpu

PATH_TOL = 2e-4
PATH_TOL_MC = 1e-3  # plain MC exponentiates the whole N-step sum in FP32
MEAN_TOL = 1e-4


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    R.lib()
    return R


def check(pay, ref, path_tol=PATH_TOL):
    assert pay.shape == ref.shape
    err = np.abs(pay - ref) / np.maximum(np.abs(ref), 0.01)
    assert np.max(err) < path_tol, f"per-path {np.max(err):.3g}"
    gm, rm = pay.mean(0), ref.mean(0)
    big = np.abs(rm) > 1e-3
    assert np.all(rel_err(gm[big], rm[big]) < MEAN_TOL), f"mean {np.max(rel_err(gm[big], rm[big])):.3g}"


@pytest.mark.parametrize("name", QUAD_CASES)
def test_mixed_quadrature_vs_reference_fixture(R, name):
    c = quad(name)
    pay = R.payoffs_rt(float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"], precision=R.MIXED)
    check(pay, c["payoff"])


@pytest.mark.parametrize("N,M,conv", [(512, 20000, 0), (700, 5000, 0), (1500, 3000, 0), (1500, 3000, 2),
                                      (100, 4099, 2)])
def test_mixed_quadrature_vs_fp64(R, N, M, conv):
    """One TMEM pass (N=512), two passes (N=700), three passes with streamed
    strip windows (N=1500), the FFT backend (N=1500 and N=100 forced); ragged
    path counts."""
    xi, H, eta, rho = 0.04, [0.05, 0.1, 0.3], [1.0, 1.5, 2.5], [-0.95, -0.7, -0.5]
    T, K = [0.25, 1.0, 2.0], [0.9, 1.0, 1.3]
    Z = R.generate_normals(5, M, N)
    p64 = R.payoffs_rt(xi, H, eta, rho, T, K, Z)
    p32 = R.payoffs_rt(xi, H, eta, rho, T, K, Z, precision=R.MIXED, conv=conv)
    check(p32, p64)


@pytest.mark.parametrize("N", [256, 1500])
def test_mixed_quadrature_plain_mc(R, N):
    xi, H, eta, rho, T, K = 0.04, [0.1, 0.2], [1.5, 2.0], [-0.7, -0.3], [0.5, 1.0], [1.0, 1.1]
    Z = R.generate_normals(6, 3000, N, streams=3)
    p64 = R.payoffs_mc(xi, H, eta, rho, T, K, Z)
    p32 = R.payoffs_mc(xi, H, eta, rho, T, K, Z, precision=R.MIXED)
    check(p32, p64, PATH_TOL_MC)


def test_dropin_quadrature_honours_mixed_precision(R):
    c = quad("testparams")
    args = (float(c["xi"]), c["H"], c["eta"], c["rho"], c["T"], c["K"], c["Z"])
    old = os.environ.get("RBG_PRECISION")
    try:
        os.environ["RBG_PRECISION"] = "mixed"
        pay = R.computeIVRT_tensor_quadrature(*args)
    finally:
        if old is None:
            os.environ.pop("RBG_PRECISION", None)
        else:
            os.environ["RBG_PRECISION"] = old
    check(pay, c["payoff"])
    p64 = R.computeIVRT_tensor_quadrature(*args)
    assert np.max(np.abs(p64 - c["payoff"])) < 1e-11   # back to FP64 without the variable
    assert not np.array_equal(pay, p64)


@pytest.mark.parametrize("shift", [0, 1])
def test_mixed_quadrature_device_buffers(R, shift):
    """Device pointers (a caller's own CUDA buffers): the same payoffs as the
    host-buffer call, also when the normals start only 8-byte aligned (one
    double into an allocation)."""
    torch = pytest.importorskip("torch")
    xi, H, eta, rho, T, K = 0.04, [0.1], [1.5], [-0.7], [0.5, 1.0], [0.9, 1.1]
    M, N = 3001, 37
    Z = R.generate_normals(8, M, N)
    want = R.payoffs_rt(xi, H, eta, rho, T, K, Z, precision=R.MIXED)
    buf = torch.zeros(shift + Z.size, dtype=torch.float64, device="cuda")
    buf[shift:] = torch.from_numpy(Z.ravel()).cuda()
    out = torch.full((M, len(T)), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()  # the library runs on its own stream
    R.payoffs_rt(xi, H, eta, rho, T, K, buf.data_ptr() + 8 * shift, device_ptrs=True, M=M, N=N,
                 precision=R.MIXED, out_ptr=out.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("N", [512, 1500])
def test_mixed_quadrature_tf32_split(R, N):
    """Caller normals through the TF32 split (one and three TMEM passes)."""
    xi, H, eta, rho = 0.04, [0.1, 0.3], [1.5, 2.5], [-0.7, -0.5]
    T, K = [0.5, 2.0], [0.9, 1.2]
    Z = R.generate_normals(8, 3000, N)
    p64 = R.payoffs_rt(xi, H, eta, rho, T, K, Z)
    p32 = R.payoffs_rt(xi, H, eta, rho, T, K, Z, precision=R.MIXED, split=R.SPLIT_TF32X2)
    # per path the normals carry TF32's rounding (<= 2^-11 relative each) into X, which v = xi exp(eta X)
    # amplifies by eta (2.5 here): a few 1e-3 on the worst paths; the means stay within MEAN_TOL
    check(p32, p64, 5e-3)
