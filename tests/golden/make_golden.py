"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout that has the reference sources mounted (it reads
/root/reference and compiles oracle/_ref from them):

    python tests/golden/make_golden.py

Outputs (all small, committed):
  debug8.json          the reference dump rBergomi/testing/debug8.txt~
                       (200 per-path RT payoffs for W1 = W1perp = cos(i*m))
  quad_*.npz           computeIVRT_tensor_quadrature(num_threads = 1) of the
                       compiled reference on the stored normals Z
  dropin_rt.npz        computeIVRT_tensor(num_threads = 1) of the compiled
                       reference plus the mt19937_64 normals it drew
  dropin_mc.npz        computeIV_tensor(num_threads = 1), same
  cv_*.npz             RBergomi::ComputeIVRTVarRed of ML_console_ST (the
                       control-variate Romano-Touzi estimator) with a small
                       pilot, plus the pilot and main normals it drew
  sobol.npz            the reference's Sobol' generator (rBergomi/sobol.cpp
                       i8_sobol, 1111 dimensions): its points at indices
                       2^(k+1) - 1, k < 24 (from which the direction integers
                       follow), a run of points 1..64 in 128 dimensions, a few
                       normalQMC_sample outputs (rBergomi/qmc.cpp) and one
                       hierarchical2increments input/output pair (aux.h)
The GPU machine has no reference; tests read only these files there.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

REF = "/root/reference"


def write_debug8():
    path = os.path.join(REF, "rBergomi", "testing", "debug8.txt~")
    d = np.loadtxt(path)
    doc = {
        "source": "rBergomi/testing/debug8.txt~ (printed by rBergomi/text/tests.cpp:283-291)",
        "params": {"xi": 0.07, "H": 0.07, "eta": 2.2, "rho": -0.9, "T": 0.5, "K": 0.8, "N": 256},
        "inputs": "W1[i] = W1perp[i] = cos(i*m), i < N (rBergomi/aux.h:198-201)",
        "m": [int(x) for x in d[:, 0]],
        "payoff": [float(x) for x in d[:, 1]],
    }
    with open(os.path.join(HERE, "debug8.json"), "w") as f:
        json.dump(doc, f, indent=0)


def quad_case(name, xi, H, eta, rho, T, K, N, M, seed):
    Z = O.normals_f64(seed, M, N, 2)
    pay = O.ref_payoffs_rt(xi, H, eta, rho, T, K, Z)
    np.savez_compressed(os.path.join(HERE, f"quad_{name}.npz"), xi=xi, H=np.array(H, float),
                        eta=np.array(eta, float), rho=np.array(rho, float), T=np.array(T, float),
                        K=np.array(K, float), N=N, M=M, seed=seed, Z=Z, payoff=pay)


def dropin_case(name, fn, nstreams, xi, H, eta, rho, T, K, N, M, seed):
    r = O.ref_compute(fn, xi, H, eta, rho, T, K, N, M, seed, 1)
    Z = O.ref_st_normals(seed, M, N, nstreams)
    np.savez_compressed(os.path.join(HERE, f"dropin_{name}.npz"), xi=xi, H=np.array(H, float),
                        eta=np.array(eta, float), rho=np.array(rho, float), T=np.array(T, float),
                        K=np.array(K, float), N=N, M=M, seed=np.array(seed, np.uint64), Z=Z,
                        **{f"ref_{k}": v for k, v in r.items()})


def cv_case(name, xi, H, eta, rho, T, K, N, M, Mc, seed):
    p, s, iv, Zc, Z = O.ml_ref_price_rt_cv(xi, H, eta, rho, T, K, N, M, Mc, seed)
    np.savez_compressed(os.path.join(HERE, f"cv_{name}.npz"), xi=np.array(xi, float), H=np.array(H, float),
                        eta=np.array(eta, float), rho=np.array(rho, float), T=np.array(T, float),
                        K=np.array(K, float), N=N, M=M, Mc=Mc, seed=np.array(seed, np.uint64), Zc=Zc, Z=Z,
                        ref_price=p, ref_stat=s, ref_iv=iv)


def sobol_case():
    D, K = 1111, 24
    gray_pts = O.qmc_ref_points(D, [(1 << (k + 1)) - 1 for k in range(K)])
    run = O.qmc_ref_points(128, np.arange(1, 65))
    samp_idx = np.array([1, 2, 3, 17, 1000, 4099, 65536], np.int64)
    samples = np.stack([O.qmc_ref_normal_sample(128, i) for i in samp_idx])
    z = np.random.default_rng(11).standard_normal(256)
    np.savez_compressed(os.path.join(HERE, "sobol.npz"), gray_points=gray_pts, run_points=run,
                        sample_index=samp_idx, samples=samples, hier_in=z, hier_out=O.qmc_ref_hier(z))


def main():
    O.build(ref=True)
    write_debug8()
    xi0 = 0.235 ** 2
    # workload 0 shape: one (H, eta, rho), five strikes at T = 1, N = 100
    quad_case("cfg0", xi0, [0.07], [1.9], [-0.9], [1.0] * 5, [0.8, 0.9, 1.0, 1.1, 1.2], 100, 128, 42)
    # trigger-heavy grid: repeated and non-monotone H, repeated T, deep OTM strike
    quad_case("grid", 0.04, [0.05, 0.1, 0.1, 0.3, 0.1], [1.0, 1.5, 1.5, 2.5, 1.5],
              [-0.95, -0.7, -0.5, -0.7, -0.3], [0.25, 0.25, 0.5, 1.0, 1.0, 2.0],
              [0.9, 1.1, 1.0, 0.8, 1.3, 2.0], 64, 64, 7)
    # the reference unit-test parameters (testRBergLib/tests.cpp:16-21)
    quad_case("testparams", 0.07, [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0], [0.8, 1.0], 256, 32, 3)
    # tiny and ragged shapes
    quad_case("n1", 0.05, [0.2], [1.0], [-0.5], [1.0], [1.0], 1, 8, 5)
    quad_case("n3", 0.05, [0.2, 0.45], [1.0, 3.0], [0.0, -0.99], [0.05, 3.0], [0.5, 1.5], 3, 9, 6)
    quad_case("n37", 0.1, [0.03], [2.9], [-0.6], [0.3, 0.3, 2.5], [0.7, 1.0, 1.4], 37, 40, 8)
    dropin_case("rt", "computeIVRT_tensor", 2, 0.07, [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0],
                [0.8, 1.0], 64, 256, [123, 452, 567])
    dropin_case("mc", "computeIV_tensor", 3, 0.07, [0.07, 0.1], [2.2, 2.4], [-0.9, -0.85], [0.5, 1.0],
                [0.8, 1.0], 64, 256, [123, 452, 567])
    # control variate: unordered tuples with their own xi; a 256-path pilot,
    # and a 4-path pilot whose Q is exceeded on some main paths (Qmax branch)
    cv_case("base", [0.04, 0.05, 0.04, 0.235 ** 2], [0.1, 0.2, 0.1, 0.07], [1.5, 1.9, 1.5, 1.9],
            [-0.7, -0.9, -0.7, -0.9], [1.0, 0.5, 1.0, 1.0], [1.0, 0.9, 1.1, 1.2], 16, 256, 256, [5, 7])
    cv_case("qmax", [0.04, 0.06], [0.1, 0.3], [2.5, 1.2], [-0.8, -0.4], [1.5, 0.75], [1.0, 1.05], 16, 128, 4, [9])
    sobol_case()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
