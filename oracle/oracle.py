"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/librbg_oracle.so`` (the C restatement of the reference
arithmetic, built by ``make -C oracle``) and, when it was built in this
checkout, ``oracle/_ref/librbergomi_ref.so`` (the reference rBergLib compiled
from its own sources against the shims in ``oracle/shims``).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module, and only as the checker or the timed CPU baseline.  The
product package ``rbergomi_gb300`` never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "librbg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "librbergomi_ref.so")
ML_REF_SO = os.path.join(HERE, "_ref", "libml_ref.so")
QMC_REF_SO = os.path.join(HERE, "_ref", "libqmc_ref.so")
REF_SRC_DIR = "/root/reference"

_dp = C.POINTER(C.c_double)
_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and, when the reference sources exist, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref is None:
        ref = os.path.isdir(os.path.join(REF_SRC_DIR, "rBergLib"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_SRC_DIR}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        L.rbgo_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.rbgo_fold_seed.argtypes = [_u64p, C.c_int]
        L.rbgo_fold_seed.restype = C.c_uint64
        L.rbgo_normals_f64.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int, C.c_int, _dp]
        L.rbgo_bs_call.argtypes = [C.c_double] * 4
        L.rbgo_bs_call.restype = C.c_double
        L.rbgo_iv_call.argtypes = [C.c_double] * 3
        L.rbgo_iv_call.restype = C.c_double
        L.rbgo_gamma.argtypes = [C.c_double, C.c_int, _dp]
        sig = [C.c_double, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int64, _dp, C.c_int, _dp]
        L.rbgo_payoffs_rt.argtypes = sig
        L.rbgo_payoffs_rt.restype = C.c_int
        L.rbgo_payoffs_mc.argtypes = sig
        L.rbgo_payoffs_mc.restype = C.c_int
        L.rbgo_reduce.argtypes = [_dp, C.c_int64, C.c_long, _dp, _dp]
        L.rbgo_price_rt_philox.argtypes = [C.c_double, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int, C.c_int,
                                           C.c_int64, C.c_uint64, C.c_int, _dp, _dp, _dp, _dp]
        L.rbgo_price_rt_philox.restype = C.c_int
        L.rbgo_max_threads.restype = C.c_int
        L.rbgo_price_rt_cv.argtypes = [C.c_long] + [_dp] * 6 + [C.c_int, C.c_int64, _dp, C.c_int64, _dp,
                                                                  C.c_double, C.c_int, _dp, _dp, _dp, _dp,
                                                                  C.POINTER(C.c_int64)]
        L.rbgo_price_rt_cv.restype = C.c_int
        L.rbgo_inv_normal.argtypes = [C.c_double]
        L.rbgo_inv_normal.restype = C.c_double
        L.rbgo_sobol_point.argtypes = [_u64p, C.c_int, C.c_uint64, _dp]
        L.rbgo_hier.argtypes = [_dp, C.c_int, _dp]
        L.rbgo_hier.restype = C.c_int
        L.rbgo_sobol_normals.argtypes = [_u64p, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int, _dp]
        L.rbgo_sobol_normals.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def price_rt_cv(xi, H, eta, rho, T, K, Zc, Z, Qmax=10000.0, nthreads: int = 0):
    """The control-variate Romano-Touzi estimator (ML_console_ST) on the
    pilot normals Zc [Mc, 2, N] and main normals Z [M, 2, N]: per tuple
    (price, stat, alpha, Q, exception count)."""
    arrs = [np.ascontiguousarray(np.atleast_1d(np.asarray(a, dtype=np.float64))) for a in (xi, H, eta, rho, T, K)]
    n = len(arrs[0])
    Zc = np.ascontiguousarray(Zc, dtype=np.float64)
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    Mc, two, N = Zc.shape
    M = Z.shape[0]
    price, stat, alpha, Q = (np.empty(n) for _ in range(4))
    cnt = np.empty(n, dtype=np.int64)
    rc = lib().rbgo_price_rt_cv(n, *[a.ctypes.data_as(_dp) for a in arrs], N, Mc, Zc.ctypes.data_as(_dp), M,
                                Z.ctypes.data_as(_dp), float(Qmax), nthreads, price.ctypes.data_as(_dp),
                                stat.ctypes.data_as(_dp), alpha.ctypes.data_as(_dp), Q.ctypes.data_as(_dp),
                                cnt.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc:
        raise MemoryError("oracle allocation failed")
    return price, stat, alpha, Q, cnt


def ml_ref_available() -> bool:
    return os.path.exists(ML_REF_SO)


def ml_ref_price_rt_cv(xi, H, eta, rho, T, K, N, M, Mc, seed):
    """ComputeIVRTVarRed of the compiled reference (ML_console_ST) with a
    Mc-path pilot: (price, stat, iv) per tuple, and the normals it drew,
    pilot [Mc, 2, N] and main [M, 2, N]."""
    R = C.CDLL(ML_REF_SO)
    R.mlglue_price_rt_varred.argtypes = [_dp] * 6 + [C.c_long, C.c_int, C.c_long, C.c_long, _u64p, C.c_int,
                                                     _dp, _dp, _dp]
    R.mlglue_normals.argtypes = [_u64p, C.c_int, C.c_long, _dp]
    arrs = [np.ascontiguousarray(np.atleast_1d(np.asarray(a, dtype=np.float64))) for a in (xi, H, eta, rho, T, K)]
    n = len(arrs[0])
    price, stat, iv = np.empty(n), np.empty(n), np.empty(n)
    sd = (C.c_uint64 * len(seed))(*[int(x) for x in seed])
    R.mlglue_price_rt_varred(*[a.ctypes.data_as(_dp) for a in arrs], n, N, M, Mc, sd, len(seed),
                             price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp), iv.ctypes.data_as(_dp))
    Zall = np.empty((Mc + M, 2, N))
    R.mlglue_normals(sd, len(seed), (Mc + M) * 2 * N, Zall.ctypes.data_as(_dp))
    return price, stat, iv, Zall[:Mc], Zall[Mc:]


def ref():
    """The reference library compiled from its own sources (oracle/_ref)."""
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError(f"{REF_SO} not built (make -C oracle ref)")
        R = C.CDLL(REF_SO)
        R.computeIVRT_tensor_quadrature.argtypes = [C.c_double, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int,
                                                    C.c_int, C.c_long, _dp, C.c_int, _dp]
        full = [C.c_double, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_long, _u64p, C.c_int,
                C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]
        R.computeIVRT_tensor.argtypes = full
        R.computeIV_tensor.argtypes = full
        R.refglue_st_normals.argtypes = [_u64p, C.c_int, C.c_long, _dp]
        _ref = R
    return _ref


def ref_st_normals(seed, M: int, N: int, nstreams: int) -> np.ndarray:
    """The normals the reference's single-threaded pricer draws for `seed`,
    shaped [M, nstreams, N] (mt19937_64 + std::normal_distribution)."""
    out = np.empty((M, nstreams, N))
    sd = (C.c_uint64 * len(seed))(*[int(x) for x in seed])
    ref().refglue_st_normals(sd, len(seed), M * nstreams * N, out.ctypes.data_as(_dp))
    return out


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


# ----------------------------------------------------------------- generator
def philox(ctr, key) -> np.ndarray:
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().rbgo_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def fold_seed(seed) -> int:
    s = (C.c_uint64 * max(1, len(seed)))(*[int(x) for x in seed])
    return int(lib().rbgo_fold_seed(s, len(seed)))


def normals_f64(seed: int, M: int, N: int, nstreams: int = 2, path0: int = 0) -> np.ndarray:
    """FP64 Philox normals, layout [M, nstreams, N] (quadrature layout)."""
    Z = np.empty((M, nstreams, N), dtype=np.float64)
    lib().rbgo_normals_f64(C.c_uint64(seed), path0, M, N, nstreams, Z.ctypes.data_as(_dp))
    return Z


# ------------------------------------------------------------------- pricing
def gamma(H: float, N: int) -> np.ndarray:
    g = np.empty(N)
    lib().rbgo_gamma(H, N, g.ctypes.data_as(_dp))
    return g


def bs_call(S0, K, tau, sigma) -> float:
    return lib().rbgo_bs_call(S0, K, tau, sigma)


def iv_call(price, K, T) -> float:
    return lib().rbgo_iv_call(price, K, T)


def payoffs_rt(xi, H, eta, rho, T, K, Z, nthreads: int = 0) -> np.ndarray:
    """Per-sample RT payoffs [M, P*O] from normals Z [M, 2, N]."""
    Hs, Hp = _d(H); es, ep = _d(eta); rs, rp = _d(rho); Ts, Tp = _d(T); Ks, Kp = _d(K)
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    M, two, N = Z.shape
    assert two == 2
    out = np.empty((M, len(Hs) * len(Ts)))
    rc = lib().rbgo_payoffs_rt(xi, Hp, ep, rp, len(Hs), Tp, Kp, len(Ts), N, M, Z.ctypes.data_as(_dp),
                               nthreads, out.ctypes.data_as(_dp))
    if rc:
        raise MemoryError("oracle allocation failed")
    return out


def payoffs_mc(xi, H, eta, rho, T, K, Z, nthreads: int = 0) -> np.ndarray:
    """Per-sample plain-MC payoffs [M, P*O] from normals Z [M, 3, N]."""
    Hs, Hp = _d(H); es, ep = _d(eta); rs, rp = _d(rho); Ts, Tp = _d(T); Ks, Kp = _d(K)
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    M, three, N = Z.shape
    assert three == 3
    out = np.empty((M, len(Hs) * len(Ts)))
    rc = lib().rbgo_payoffs_mc(xi, Hp, ep, rp, len(Hs), Tp, Kp, len(Ts), N, M, Z.ctypes.data_as(_dp),
                               nthreads, out.ctypes.data_as(_dp))
    if rc:
        raise MemoryError("oracle allocation failed")
    return out


def reduce(payoff: np.ndarray):
    """Reference mean / standard error of a payoff matrix [M, out]."""
    payoff = np.ascontiguousarray(payoff, dtype=np.float64)
    M, out = payoff.shape
    price = np.empty(out); stat = np.empty(out)
    lib().rbgo_reduce(payoff.ctypes.data_as(_dp), M, out, price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp))
    return price, stat


def price_rt_philox(xi, H, eta, rho, T, K, N, M, seed: int, nthreads: int = 0):
    """RT prices on the project's FP64 Philox stream (blocks of paths)."""
    Hs, Hp = _d(H); es, ep = _d(eta); rs, rp = _d(rho); Ts, Tp = _d(T); Ks, Kp = _d(K)
    out = len(Hs) * len(Ts)
    price = np.empty(out); stat = np.empty(out); s1 = np.empty(out); s2 = np.empty(out)
    rc = lib().rbgo_price_rt_philox(xi, Hp, ep, rp, len(Hs), Tp, Kp, len(Ts), N, M, C.c_uint64(seed), nthreads,
                                    price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                                    s1.ctypes.data_as(_dp), s2.ctypes.data_as(_dp))
    if rc:
        raise MemoryError("oracle allocation failed")
    return price, stat


def max_threads() -> int:
    return int(lib().rbgo_max_threads())


# ------------------------------------------------------- the reference itself
def ref_payoffs_rt(xi, H, eta, rho, T, K, Z) -> np.ndarray:
    """computeIVRT_tensor_quadrature of the compiled reference, num_threads = 1
    (the multi-threaded RT drivers share W1perp between threads)."""
    Hs, Hp = _d(H); es, ep = _d(eta); rs, rp = _d(rho); Ts, Tp = _d(T); Ks, Kp = _d(K)
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    M, two, N = Z.shape
    out = np.empty((M, len(Hs) * len(Ts)))
    ref().computeIVRT_tensor_quadrature(xi, Hp, ep, rp, len(Hs), Tp, Kp, len(Ts), N, M,
                                        Z.ctypes.data_as(_dp), 1, out.ctypes.data_as(_dp))
    return out


def ref_compute(fn: str, xi, H, eta, rho, T, K, N, M, seed, num_threads=1):
    """computeIVRT_tensor / computeIV_tensor of the compiled reference."""
    Hs, Hp = _d(H); es, ep = _d(eta); rs, rp = _d(rho); Ts, Tp = _d(T); Ks, Kp = _d(K)
    out = len(Hs) * len(Ts)
    arrs = [np.empty(out) for _ in range(8)]
    sd = (C.c_uint64 * len(seed))(*[int(x) for x in seed])
    getattr(ref(), fn)(xi, Hp, ep, rp, len(Hs), Tp, Kp, len(Ts), N, M, sd, len(seed), num_threads,
                       *[a.ctypes.data_as(_dp) for a in arrs], out)
    names = ["price", "iv", "stat", "H", "eta", "rho", "T", "K"]
    return dict(zip(names, arrs))


# ----------------------------------------------------------- Sobol' QMC
# rBergomi/qmc.cpp, rBergomi/sobol.cpp (i8_sobol), rBergomi/aux.h (breakZ,
# hierarchical2increments).  V: direction integers [dims][62] uint64, point
# s coordinate d = (XOR of V[d][k] over the set bits k of s ^ (s >> 1)) 2^-62.
SOBOL_BITS = 62


def sobol_directions_from_points(points):
    """Direction integers from a generator's points at indices 2^(k+1) - 1
    (whose Gray code is 2^k): points[k][d] * 2^62 = V[d][k], exact for k <= 52."""
    P = np.asarray(points, np.float64)
    q = P * 2.0 ** 62
    if not np.all(q == np.floor(q)):
        raise ValueError("points are not multiples of 2^-62")
    V = np.zeros((P.shape[1], SOBOL_BITS), np.uint64)
    V[:, :P.shape[0]] = q.T.astype(np.uint64)
    return V


def inv_normal(p):
    L = lib()
    return np.array([L.rbgo_inv_normal(float(x)) for x in np.ravel(p)]).reshape(np.shape(p))


def sobol_point(V, s, dims=None):
    V = np.ascontiguousarray(V, np.uint64)
    dims = V.shape[0] if dims is None else dims
    x = np.empty(dims)
    lib().rbgo_sobol_point(V.ctypes.data_as(_u64p), dims, int(s), x.ctypes.data_as(_dp))
    return x


def hier(Z):
    Z = np.ascontiguousarray(Z, np.float64)
    out = np.empty_like(Z)
    if lib().rbgo_hier(Z.ctypes.data_as(_dp), len(Z), out.ctypes.data_as(_dp)):
        raise ValueError("length must be a power of two")
    return out


def sobol_normals(V, N, M, path0=0, bridge=False):
    """[M, 2, N] normals: path m takes point path0 + m + 1; W1 = even
    coordinates, W1perp = odd ones; bridge: hierarchical2increments per stream."""
    V = np.ascontiguousarray(V, np.uint64)
    Z = np.empty((M, 2, N))
    if lib().rbgo_sobol_normals(V.ctypes.data_as(_u64p), V.shape[0], N, path0, M, int(bridge), Z.ctypes.data_as(_dp)):
        raise ValueError("bad Sobol' sizes")
    return Z


def qmc_ref_available() -> bool:
    return os.path.exists(QMC_REF_SO)


_qmc = None


def _qmc_ref():
    global _qmc
    if _qmc is None:
        if not qmc_ref_available():
            raise FileNotFoundError(f"{QMC_REF_SO} not built (make -C oracle ref)")
        R = C.CDLL(QMC_REF_SO)
        lp = C.POINTER(C.c_longlong)
        R.qmcglue_sobol_walk.argtypes = [C.c_int, C.c_longlong, lp, C.c_int, _dp]
        R.qmcglue_normal_sample.argtypes = [C.c_int, C.c_longlong, _dp]
        R.qmcglue_hier.argtypes = [_dp, C.c_int, _dp]
        _qmc = R
    return _qmc


def qmc_ref_points(dims, seeds):
    """The reference's i8_sobol points at the given ascending indices (one sequential walk)."""
    seeds = np.ascontiguousarray(seeds, np.int64)
    out = np.empty((len(seeds), dims))
    _qmc_ref().qmcglue_sobol_walk(dims, int(seeds[-1]), seeds.ctypes.data_as(C.POINTER(C.c_longlong)), len(seeds),
                                  out.ctypes.data_as(_dp))
    return out


def qmc_ref_normal_sample(dims, i):
    """The reference's normalQMC_sample(Z, dims, i) (quantile from the Boost stand-in)."""
    z = np.empty(dims)
    _qmc_ref().qmcglue_normal_sample(dims, int(i), z.ctypes.data_as(_dp))
    return z


def qmc_ref_hier(Z):
    Z = np.ascontiguousarray(Z, np.float64)
    out = np.empty_like(Z)
    _qmc_ref().qmcglue_hier(Z.ctypes.data_as(_dp), len(Z), out.ctypes.data_as(_dp))
    return out
