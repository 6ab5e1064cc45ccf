"""Failure detection without a GPU fault: a bounded device-side wait that runs
out (an mbarrier nothing arrives on) returns an error status the host reads,
and the CUDA context stays usable.  The pricing kernels' pipeline waits use
the same helper with a 2 s limit and report RBG_ERR_TIMEOUT the same way."""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RBG_ERR_TIMEOUT = 5


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    L = R.lib()
    L.rbg_debug_wait_timeout.argtypes = [C.POINTER(C.c_uint)]
    L.rbg_debug_wait_timeout.restype = C.c_int
    return R


def test_bounded_wait_expires_and_context_survives(R):
    before = R.price_rt(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 64, 4096, seed=1, precision=R.MIXED)
    site = C.c_uint(0)
    t0 = time.perf_counter()
    rc = R.lib().rbg_debug_wait_timeout(C.byref(site))
    dt = time.perf_counter() - t0
    assert rc == RBG_ERR_TIMEOUT
    assert site.value == 99
    assert "bounded wait expired" in R.lib().rbg_last_error().decode()
    assert 0.02 <= dt < 1.0
    after = R.price_rt(0.04, [0.1], [1.5], [-0.7], [1.0], [1.0], 64, 4096, seed=1, precision=R.MIXED)
    for a, b in zip(before, after):
        np.testing.assert_array_equal(a, b)

