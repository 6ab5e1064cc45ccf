"""Derivation of the FP32 normal-quantile coefficients in rbg_device.cuh
(normal_quantile_lower_f32).

The form is M. Giles, "Approximating the erfinv function" (GPU Computing Gems,
Jade Edition, 2011): erfinv(x) = x P(w), w = -ln(1 - x^2), with P a
polynomial in w - 2.5 for w < 5 and in sqrt(w) - 3 above.  The coefficients
here are fitted afresh: weighted least squares on the relative error against
scipy's double-precision erfinv, re-weighted toward the worst points, on
w in [0, 5) and [5, 22.5] (the Sobol' normals' range, u >= 2^-32).

    python rbergomi_gb300/csrc/fit_normal_quantile.py

prints the two coefficient lists (highest degree first) in the literal
format the CUDA source uses.  Not part of the build.
"""
import numpy as np
from scipy.special import erfinv


def target(w):
    x = np.sqrt(-np.expm1(-w))
    return erfinv(x) / x


def fit(lo, hi, var, deg=8, n=4000, passes=30):
    k = np.arange(n)
    w = 0.5 * (lo + hi) + 0.5 * (hi - lo) * np.cos(np.pi * (k + 0.5) / n)
    t, f = var(w), target(w)
    wt = 1.0 / f
    for _ in range(passes):
        A = np.vander(t, deg + 1) * wt[:, None]
        c, *_ = np.linalg.lstsq(A, f * wt, rcond=None)
        err = np.abs(np.polyval(c, t) - f) / f
        wt = wt * (1 + 5 * err / err.max())
    return c, err.max()


def literal(v):
    return ("%.9e" % v).replace("e-0", "e-").replace("e+0", "e+") + "f"


if __name__ == "__main__":
    central, e1 = fit(1e-12, 5.0, lambda w: w - 2.5)
    tail, e2 = fit(5.0, 22.5, lambda w: np.sqrt(w) - 3.0)
    print(f"central (w < 5), max relative error {e1:.2e}:\n  " + ", ".join(literal(v) for v in central))
    print(f"tail (w >= 5), max relative error {e2:.2e}:\n  " + ", ".join(literal(v) for v in tail))
