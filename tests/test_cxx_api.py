"""The reference's C++ interface (rBergLib/interface.h:23-62), exported by
librbergomi_gb300.so through include/rbergomi_gb300.hpp.

tests/cxx/test_interface.cpp is a C++ caller written like the reference's
unit test (testRBergLib/tests.cpp:14-70): the same parameters, reference
prices, implied vols and tolerances, for ComputeIV[RT]_{single,multi}Thread.
On CPU it must compile and link against the library; on the GPU it runs, its
own checks pass, and its prices equal the drop-in C calls (computeIV_tensor,
computeIVRT_tensor) with the same seed words bit for bit.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "test_interface.cpp")


def _cuda_lib_dir():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def _build(tmp_path):
    import rbergomi_gb300 as R
    if not os.path.exists(R.LIB_PATH):
        from rbergomi_gb300 import build
        build.build()
    exe = str(tmp_path / "test_interface")
    libdir = os.path.dirname(R.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", libdir,
           "-lrbergomi_gb300", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath-link,{_cuda_lib_dir()}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cxx_interface_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_cxx_interface_runs_reference_unit_test(tmp_path):
    import rbergomi_gb300 as R
    exe = _build(tmp_path)
    env = dict(os.environ)
    env.pop("RBG_PRECISION", None)
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = {}
    for line in r.stdout.split("\n"):
        if line.strip():
            f = line.split()
            rows.setdefault(f[0], []).append([float(x) for x in f[2:]])
    xi, H, eta, rho, T, K = 0.07, [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0], [0.8, 1.0]
    N, M, seed = 256, 10 * 256 * 256, [123, 452, 567, 248, 9436, 675, 194, 6702]
    for name, fn in (("IV", R.computeIV_tensor), ("IVRT", R.computeIVRT_tensor)):
        got = np.array(rows[name])
        want = fn(xi, H, eta, rho, T, K, N, M, seed, num_threads=8)
        np.testing.assert_array_equal(got[:, 0], want.price)
        np.testing.assert_array_equal(got[:, 1], want.stat)
        np.testing.assert_array_equal(got[:, 2], want.iv)
        # echoed parameters are not swapped in the C++ interface (interface.cpp:36-49)
        np.testing.assert_array_equal(got[:, 3], np.repeat(H, 2))
        np.testing.assert_array_equal(got[:, 4], np.repeat(eta, 2))
        np.testing.assert_array_equal(got[:, 5], np.repeat(rho, 2))
        np.testing.assert_array_equal(got[:, 6], np.tile(T, 2))
        np.testing.assert_array_equal(got[:, 7], np.tile(K, 2))
