"""rbergomi_gb300 -- GB300-native rough Bergomi Romano-Touzi pricer.

A ctypes binding of ``librbergomi_gb300.so`` (C ABI in
``include/rbergomi_gb300.h``).  The functions mirror the reference's
interface (rBergLib/cinterface.h, rBergLib/interface.h): the same argument
meaning, ParamTot output layout and result fields (``price``, ``iv``,
``stat`` and the ``*_tot`` parameter echoes).

There is no CPU fallback: importing works without a GPU, but every pricing
call runs the CUDA kernels and fails loudly if the library or the GPU is
missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librbergomi_gb300.so")

FP64, MIXED = 0, 1
CONV_AUTO, CONV_GEMM, CONV_FFT, CONV_DIRECT = 0, 1, 2, 3
NORMALS_F64, NORMALS_F32 = 0, 1
SPLIT_BF16X3, SPLIT_F16X3, SPLIT_TF32X2 = 0, 1, 2

_dp = C.POINTER(C.c_double)
_u64p = C.POINTER(C.c_uint64)


class RbgParams(C.Structure):
    _fields_ = [("xi", C.c_double), ("H", _dp), ("eta", _dp), ("rho", _dp), ("par_size", C.c_int),
                ("T", _dp), ("K", _dp), ("op_size", C.c_int), ("N", C.c_int), ("M", C.c_int64)]


class RbgUnordered(C.Structure):
    _fields_ = [("xi", C.c_double), ("H", _dp), ("eta", _dp), ("rho", _dp), ("T", _dp), ("K", _dp),
                ("size", C.c_long), ("N", C.c_int), ("M", C.c_int64)]


class RbgCvParams(C.Structure):
    _fields_ = [("xi", _dp), ("H", _dp), ("eta", _dp), ("rho", _dp), ("T", _dp), ("K", _dp), ("size", C.c_long),
                ("N", C.c_int), ("M", C.c_int64), ("M_control", C.c_int64), ("Q_max", C.c_double)]


class RbgOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("conv", C.c_int), ("normals", C.c_int), ("split", C.c_int),
                ("compute_iv", C.c_int), ("seed", C.c_uint64), ("path_offset", C.c_int64),
                ("stream", C.c_void_p)]


class RbgError(RuntimeError):
    pass


_lib = None

EXPORTS = [
    "computeIVRT_tensor", "computeIVRT_tensor_quadrature", "rbg_default_options", "rbg_price_rt",
    "rbg_price_rt_sums", "rbg_payoffs_rt", "rbg_generate_normals", "rbg_implied_vol", "rbg_last_error",
    "rbg_launch_count", "rbg_synchronize", "rbg_release", "rbg_plan_info", "rbg_profile_enable",
    "rbg_profile_reset", "rbg_profile_read", "rbg_last_transfer_bytes", "rbg_debug_mixed_paths",
    "rbg_debug_mixed_profile", "rbg_server_default_config", "rbg_server_create", "rbg_server_submit",
    "rbg_server_poll", "rbg_server_wait", "rbg_server_get_stats", "rbg_server_destroy", "rbg_server_last_error",
    "rbg_price_rt_unordered", "computeIV_tensor", "rbg_price_mc", "rbg_payoffs_mc", "rbg_generate_normals_streams",
    "rbg_plan_info_mc", "rbg_plan_info_unordered", "rbg_price_rt_cv", "rbg_price_rt_cv_normals",
    "rbg_price_rt_sobol", "rbg_sobol_normals", "rbg_debug_wait_timeout", "rbg_merge_sums",
    "rbg_server_wait_timed",
]

STAGE_NORMALS, STAGE_PATH_FP64, STAGE_MIXED, STAGE_PAYOFF, STAGE_REDUCE = 0, 1, 2, 3, 4


def lib():
    """The loaded shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RbgError(f"{LIB_PATH} is missing; build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        full = [C.c_double, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_long, _u64p, C.c_int,
                C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.computeIVRT_tensor.argtypes = full
        L.computeIVRT_tensor.restype = None
        L.computeIV_tensor.argtypes = full
        L.computeIV_tensor.restype = None
        L.computeIVRT_tensor_quadrature.argtypes = [C.c_double, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int,
                                                    C.c_int, C.c_long, _dp, C.c_int, _dp]
        L.computeIVRT_tensor_quadrature.restype = None
        P, O = C.POINTER(RbgParams), C.POINTER(RbgOptions)
        L.rbg_default_options.argtypes = [O]
        L.rbg_price_rt.argtypes = [P, O, _dp, _dp, _dp]
        L.rbg_price_rt.restype = C.c_int
        L.rbg_price_rt_sums.argtypes = [P, O, _dp, _dp]
        L.rbg_price_rt_sums.restype = C.c_int
        L.rbg_merge_sums.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int64, _dp, _dp]
        L.rbg_merge_sums.restype = C.c_int
        L.rbg_payoffs_rt.argtypes = [P, O, C.c_void_p, C.c_void_p, C.c_int]
        L.rbg_payoffs_rt.restype = C.c_int
        L.rbg_price_mc.argtypes = [P, O, _dp, _dp, _dp]
        L.rbg_price_mc.restype = C.c_int
        L.rbg_payoffs_mc.argtypes = [P, O, C.c_void_p, C.c_void_p, C.c_int]
        L.rbg_payoffs_mc.restype = C.c_int
        L.rbg_generate_normals_streams.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int, _dp]
        L.rbg_price_rt_sobol.argtypes = [P, O, _u64p, C.c_int, C.c_int, _dp, _dp, _dp]
        L.rbg_sobol_normals.argtypes = [_u64p, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int, C.c_int, _dp]
        L.rbg_generate_normals_streams.restype = C.c_int
        L.rbg_generate_normals.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int, C.c_int, _dp]
        L.rbg_generate_normals.restype = C.c_int
        L.rbg_implied_vol.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        L.rbg_implied_vol.restype = C.c_int
        L.rbg_last_error.restype = C.c_char_p
        L.rbg_launch_count.restype = C.c_uint64
        L.rbg_synchronize.restype = C.c_int
        L.rbg_release.restype = C.c_int
        L.rbg_plan_info.argtypes = [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]
        L.rbg_plan_info.restype = C.c_int
        L.rbg_profile_enable.argtypes = [C.c_int]
        L.rbg_profile_enable.restype = None
        L.rbg_profile_reset.restype = None
        L.rbg_profile_read.argtypes = [C.c_int, _dp, C.POINTER(C.c_uint64)]
        L.rbg_profile_read.restype = C.c_int
        L.rbg_last_transfer_bytes.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.rbg_last_transfer_bytes.restype = None
        _fp = C.POINTER(C.c_float)
        L.rbg_debug_mixed_paths.argtypes = [P, O, _fp, _fp, _fp]
        L.rbg_debug_mixed_paths.restype = C.c_int
        L.rbg_debug_mixed_profile.argtypes = [P, O, C.POINTER(C.c_uint64), C.c_int]
        L.rbg_debug_mixed_profile.restype = C.c_int
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RbgError(f"rbg status {rc}: {lib().rbg_last_error().decode()}")


def _arr(x) -> np.ndarray:
    return np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=np.float64)))


class _Params:
    """Keeps the numpy arrays alive behind an RbgParams struct."""

    def __init__(self, xi, H, eta, rho, T, K, N, M):
        self.H, self.eta, self.rho = _arr(H), _arr(eta), _arr(rho)
        self.T, self.K = _arr(T), _arr(K)
        if not (len(self.H) == len(self.eta) == len(self.rho)):
            raise ValueError("H, eta, rho must have the same length (par_size)")
        if len(self.T) != len(self.K):
            raise ValueError("T and K must have the same length (op_size)")
        self.s = RbgParams(float(xi), self.H.ctypes.data_as(_dp), self.eta.ctypes.data_as(_dp),
                           self.rho.ctypes.data_as(_dp), len(self.H), self.T.ctypes.data_as(_dp),
                           self.K.ctypes.data_as(_dp), len(self.T), int(N), int(M))
        self.out = len(self.H) * len(self.T)


def options(precision=FP64, conv=CONV_AUTO, normals=NORMALS_F64, split=SPLIT_BF16X3, compute_iv=True, seed=0,
            path_offset=0, stream=None) -> RbgOptions:
    o = RbgOptions()
    lib().rbg_default_options(C.byref(o))
    o.precision, o.conv, o.normals, o.split = precision, conv, normals, split
    o.compute_iv = 1 if compute_iv else 0
    o.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    o.path_offset = int(path_offset)
    o.stream = stream
    return o


@dataclass
class ResultSimple:
    """Same fields as the reference's ResultSimple (rBergLib/interface.h:23-36)."""
    price: np.ndarray
    iv: np.ndarray
    H: np.ndarray
    rho: np.ndarray
    eta: np.ndarray
    T: np.ndarray
    K: np.ndarray
    xi: float
    stat: np.ndarray
    N: int
    M: int
    numThreads: int


def computeIV_tensor(xi, H, eta, rho, T, K, N, M, seed, num_threads=1) -> ResultSimple:
    """Drop-in plain Monte Carlo pricing (rBergLib/cinterface.h:63-66) through
    the C ABI.  As in the reference (cinterface.cpp:45) the library writes rho
    into eta_tot and eta into rho_tot; the fields here are read back as the
    C arrays hold them."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    seed = np.ascontiguousarray(np.atleast_1d(np.asarray(seed, dtype=np.uint64)))
    outs = [np.empty(p.out) for _ in range(8)]
    lib().computeIV_tensor(float(xi), p.s.H, p.s.eta, p.s.rho, p.s.par_size, p.s.T, p.s.K, p.s.op_size, int(N),
                           int(M), seed.ctypes.data_as(_u64p), len(seed), int(num_threads),
                           *[o.ctypes.data_as(_dp) for o in outs], p.out)
    price, iv, stat, Ht, et, rt, Tt, Kt = outs
    return ResultSimple(price, iv, Ht, rt, et, Tt, Kt, float(xi), stat, int(N), int(M), int(num_threads))


def computeIVRT_tensor(xi, H, eta, rho, T, K, N, M, seed, num_threads=1) -> ResultSimple:
    """Drop-in RT pricing (rBergLib/cinterface.h:68-71) through the C ABI."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    seed = np.ascontiguousarray(np.atleast_1d(np.asarray(seed, dtype=np.uint64)))
    outs = [np.empty(p.out) for _ in range(8)]
    lib().computeIVRT_tensor(float(xi), p.s.H, p.s.eta, p.s.rho, p.s.par_size, p.s.T, p.s.K, p.s.op_size, int(N),
                             int(M), seed.ctypes.data_as(_u64p), len(seed), int(num_threads),
                             *[o.ctypes.data_as(_dp) for o in outs], p.out)
    price, iv, stat, Ht, et, rt, Tt, Kt = outs
    return ResultSimple(price, iv, Ht, rt, et, Tt, Kt, float(xi), stat, int(N), int(M), int(num_threads))


def computeIVRT_tensor_quadrature(xi, H, eta, rho, T, K, Z, num_threads=1) -> np.ndarray:
    """Drop-in per-sample RT payoffs (rBergLib/cinterface.h:73-75).

    Z: normals [M, 2, N] (or flat 2*N*M).  Returns payoff [M, par_size*op_size]."""
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    M, two, N = Z.shape
    if two != 2:
        raise ValueError("Z must be [M, 2, N]")
    p = _Params(xi, H, eta, rho, T, K, N, M)
    pay = np.empty((M, p.out))
    lib().computeIVRT_tensor_quadrature(float(xi), p.s.H, p.s.eta, p.s.rho, p.s.par_size, p.s.T, p.s.K,
                                        p.s.op_size, int(N), int(M), Z.ctypes.data_as(_dp), int(num_threads),
                                        pay.ctypes.data_as(_dp))
    return pay


def price_rt(xi, H, eta, rho, T, K, N, M, **opts):
    """Extended API: returns (price, stat, iv) arrays."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    o = options(**opts)
    price, stat, iv = np.empty(p.out), np.empty(p.out), np.empty(p.out)
    _check(lib().rbg_price_rt(C.byref(p.s), C.byref(o), price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                              iv.ctypes.data_as(_dp)))
    return price, stat, iv


class RtPricer:
    """price_rt with its arguments marshalled once, for repeated calls on
    one grid (a calibration or risk loop, a benchmark): each call passes the
    same C structures and output arrays and changes only the seed, the path
    offset or the stream.  With the library's plan cache (a call repeating
    the previous call's inputs reuses its plan and device tables), a repeated
    call costs the C call and the kernels.  The returned arrays are reused by
    the next call: copy them to keep them."""

    def __init__(self, xi, H, eta, rho, T, K, N, M, **opts):
        self._p = _Params(xi, H, eta, rho, T, K, N, M)
        self._o = options(**opts)
        out = self._p.out
        self.price, self.stat, self.iv = np.empty(out), np.empty(out), np.empty(out)
        self._ptrs = (self.price.ctypes.data_as(_dp), self.stat.ctypes.data_as(_dp), self.iv.ctypes.data_as(_dp))
        self._fn = lib().rbg_price_rt

    def __call__(self, seed=None, path_offset=None, stream=None):
        o = self._o
        if seed is not None:
            o.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        if path_offset is not None:
            o.path_offset = int(path_offset)
        if stream is not None:
            o.stream = stream
        _check(self._fn(C.byref(self._p.s), C.byref(o), *self._ptrs))
        return self.price, self.stat, self.iv


def price_rt_unordered(xi, H, eta, rho, T, K, N, M, **opts):
    """Unordered parameter list (the reference's ComputeIVRTMTunstructured,
    rBergomi/rBergomiMT.cpp:837-938): output i prices (H[i], eta[i], rho[i],
    T[i], K[i]).  Returns (price, stat, iv) arrays."""
    arrs = [_arr(x) for x in (H, eta, rho, T, K)]
    n = len(arrs[0])
    if any(len(x) != n for x in arrs):
        raise ValueError("H, eta, rho, T, K must have the same length")
    u = RbgUnordered(float(xi), *[x.ctypes.data_as(_dp) for x in arrs], n, int(N), int(M))
    o = options(**opts)
    price, stat, iv = np.empty(n), np.empty(n), np.empty(n)
    _check(lib().rbg_price_rt_unordered(C.byref(u), C.byref(o), price.ctypes.data_as(_dp),
                                        stat.ctypes.data_as(_dp), iv.ctypes.data_as(_dp)))
    return price, stat, iv


def _cv_params(xi, H, eta, rho, T, K, N, M, M_control, Q_max):
    arrs = [_arr(x) for x in (H, eta, rho, T, K)]
    n = len(arrs[0])
    xis = np.full(n, float(xi)) if np.ndim(xi) == 0 else _arr(xi)
    if any(len(x) != n for x in arrs + [xis]):
        raise ValueError("xi, H, eta, rho, T, K must have the same length")
    p = RbgCvParams(xis.ctypes.data_as(_dp), *[x.ctypes.data_as(_dp) for x in arrs], n, int(N), int(M),
                    int(M_control), float(Q_max))
    return p, n, (xis, arrs)


def price_rt_cv(xi, H, eta, rho, T, K, N, M, M_control=10000, Q_max=10000.0, **opts):
    """Romano-Touzi with the McCrickerd-Pakkanen control variate and
    antithetic paths (ML_console_ST's ComputeIVRTVarRed), one tuple per
    output, xi per tuple (scalar or array), FP64: (price, stat, iv)."""
    p, n, keep = _cv_params(xi, H, eta, rho, T, K, N, M, M_control, Q_max)
    o = options(**opts)
    price, stat, iv = np.empty(n), np.empty(n), np.empty(n)
    _check(lib().rbg_price_rt_cv(C.byref(p), C.byref(o), price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                                 iv.ctypes.data_as(_dp)))
    return price, stat, iv


def price_rt_cv_normals(xi, H, eta, rho, T, K, Zc, Z, Q_max=10000.0):
    """The control-variate estimator on caller normals: pilot Zc [Mc, 2, N],
    main Z [M, 2, N]."""
    Zc = np.ascontiguousarray(Zc, dtype=np.float64)
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    Mc, two, N = Zc.shape
    p, n, keep = _cv_params(xi, H, eta, rho, T, K, N, Z.shape[0], Mc, Q_max)
    price, stat, iv = np.empty(n), np.empty(n), np.empty(n)
    _check(lib().rbg_price_rt_cv_normals(C.byref(p), Zc.ctypes.data_as(_dp), Z.ctypes.data_as(_dp),
                                         price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                                         iv.ctypes.data_as(_dp)))
    return price, stat, iv


def price_rt_sums(xi, H, eta, rho, T, K, N, M, **opts):
    """Extended API: raw (sum x, sum x^2) per output over this call's paths."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    o = options(**opts)
    s1, s2 = np.empty(p.out), np.empty(p.out)
    _check(lib().rbg_price_rt_sums(C.byref(p.s), C.byref(o), s1.ctypes.data_as(_dp), s2.ctypes.data_as(_dp)))
    return s1, s2


def merge_sums(s1, s2, M):
    """(price, stat) of path shards through rbg_merge_sums: s1, s2 are
    [n_shards, out] (or [out] after an all-reduce) arrays of price_rt_sums
    outputs, M the total path count.  Host-only."""
    s1 = np.ascontiguousarray(np.atleast_2d(np.asarray(s1, dtype=np.float64)))
    s2 = np.ascontiguousarray(np.atleast_2d(np.asarray(s2, dtype=np.float64)))
    if s1.shape != s2.shape:
        raise ValueError("sum and sum2 must have the same shape")
    n_shards, n = s1.shape
    price, stat = np.empty(n), np.empty(n)
    _check(lib().rbg_merge_sums(n_shards, n, s1.ctypes.data_as(_dp), s2.ctypes.data_as(_dp), int(M),
                                price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp)))
    return price, stat


def payoffs_rt(xi, H, eta, rho, T, K, Z, device_ptrs=False, M=None, N=None, **opts):
    """Per-path FP64 payoffs.  Z is a host [M, 2, N] array, or (device_ptrs=True)
    a device address with M, N given; then payoff is returned as None and the
    caller passes ``out`` via opts['out_ptr']."""
    out_ptr = opts.pop("out_ptr", None)
    o = options(**opts)
    if device_ptrs:
        p = _Params(xi, H, eta, rho, T, K, N, M)
        _check(lib().rbg_payoffs_rt(C.byref(p.s), C.byref(o), C.c_void_p(int(Z)), C.c_void_p(int(out_ptr)), 1))
        return None
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    M, two, N = Z.shape
    p = _Params(xi, H, eta, rho, T, K, N, M)
    pay = np.empty((M, p.out))
    _check(lib().rbg_payoffs_rt(C.byref(p.s), C.byref(o), Z.ctypes.data, pay.ctypes.data, 0))
    return pay


def generate_normals(seed, M, N, precision=FP64, path_offset=0, streams=2) -> np.ndarray:
    """The normals the pricer draws: [M, streams, N] float64 (FP32 values
    widened exactly when precision=MIXED); streams=3 adds plain MC's Wperp."""
    Z = np.empty((M, streams, N))
    _check(lib().rbg_generate_normals_streams(int(seed) & 0xFFFFFFFFFFFFFFFF, int(path_offset), int(M), int(N),
                                              int(precision), int(streams), Z.ctypes.data_as(_dp)))
    return Z


SOBOL_BITS = 62


def _sobol_table(directions):
    V = np.asarray(directions)
    if V.ndim != 2 or V.shape[1] > SOBOL_BITS:
        raise ValueError("Sobol' directions must be [dims, <= 62] integers")
    T = np.zeros((V.shape[0], SOBOL_BITS), np.uint64)
    T[:, :V.shape[1]] = V.astype(np.uint64)
    return T


def sobol_directions_from_points(points) -> np.ndarray:
    """Direction table [dims, 62] from a Sobol' generator's points at indices
    2^(k+1) - 1, k = 0, 1, ... (rows of `points`): those points have Gray code
    2^k, so point * 2^62 is column k (exact for k <= 52)."""
    P = np.asarray(points, np.float64)
    q = P * 2.0 ** 62
    if P.ndim != 2 or P.shape[0] > 52 or not np.all(q == np.floor(q)):
        raise ValueError("expected points at indices 2^(k+1) - 1 on the 2^-62 grid, k < 52")
    V = np.zeros((P.shape[1], SOBOL_BITS), np.uint64)
    V[:, :P.shape[0]] = q.T.astype(np.uint64)
    return V


def sobol_normals(directions, N, M, path_offset=0, bridge=False, precision=FP64) -> np.ndarray:
    """Sobol' quasi-Monte Carlo normals [M, 2, N] (rBergomi/qmc.cpp
    normalQMC_sample + breakZ): path m takes point path_offset + m + 1.
    directions: [dims, 62] direction integers (coordinate d of point s is the
    XOR of directions[d, k] over the set bits k of s ^ (s >> 1), times 2^-62).
    bridge: Brownian-bridge map of each stream (rBergomi/aux.h
    hierarchical2increments; N a power of two).  precision=MIXED: the mixed
    form's FP32 normals (with the bridge in FP32), widened to double."""
    V = _sobol_table(directions)
    Z = np.empty((M, 2, N))
    _check(lib().rbg_sobol_normals(V.ctypes.data_as(C.POINTER(C.c_uint64)), V.shape[0], int(N), int(M),
                                   int(path_offset), int(bool(bridge)), int(precision), Z.ctypes.data_as(_dp)))
    return Z


def price_rt_sobol(xi, H, eta, rho, T, K, N, M, directions, bridge=False, **opts):
    """RT prices over Sobol' normals (the reference's ComputeIVRTMT_sobol,
    rBergomi/rBergomiMT.cpp:610-715): (price, stat, iv).  FP64 form by
    default; precision=MIXED runs the same points through the tensor-core
    form, with or without the Brownian bridge, on either backend."""
    V = _sobol_table(directions)
    p = _Params(xi, H, eta, rho, T, K, N, M)
    opts.setdefault("precision", FP64)
    o = options(**opts)
    price, stat, iv = np.empty(p.out), np.empty(p.out), np.empty(p.out)
    _check(lib().rbg_price_rt_sobol(C.byref(p.s), C.byref(o), V.ctypes.data_as(C.POINTER(C.c_uint64)), V.shape[0],
                                    int(bool(bridge)), price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                                    iv.ctypes.data_as(_dp)))
    return price, stat, iv


def price_mc(xi, H, eta, rho, T, K, N, M, **opts):
    """Plain Monte Carlo (the estimator behind computeIV_tensor): (price, stat, iv)."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    o = options(**opts)
    price, stat, iv = np.empty(p.out), np.empty(p.out), np.empty(p.out)
    _check(lib().rbg_price_mc(C.byref(p.s), C.byref(o), price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                              iv.ctypes.data_as(_dp)))
    return price, stat, iv


def payoffs_mc(xi, H, eta, rho, T, K, Z, **opts):
    """Plain MC per-path FP64 payoffs for host normals Z [M, 3, N]."""
    o = options(**opts)
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    M, three, N = Z.shape
    if three != 3:
        raise ValueError("Z must be [M, 3, N]")
    p = _Params(xi, H, eta, rho, T, K, N, M)
    pay = np.empty((M, p.out))
    _check(lib().rbg_payoffs_mc(C.byref(p.s), C.byref(o), Z.ctypes.data, pay.ctypes.data, 0))
    return pay


def implied_vol(price, K, T) -> np.ndarray:
    price, K, T = _arr(price), _arr(K), _arr(T)
    iv = np.empty(len(price))
    _check(lib().rbg_implied_vol(len(price), price.ctypes.data_as(_dp), K.ctypes.data_as(_dp),
                                 T.ctypes.data_as(_dp), iv.ctypes.data_as(_dp)))
    return iv


def plan_info(xi, H, eta, rho, T, K, N, M=1):
    """Host-only: (n_volterra_passes, n_variance_groups, group_of_output)."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    nv, ng, no = C.c_int(), C.c_int(), C.c_int()
    groups = (C.c_int * p.out)()
    _check(lib().rbg_plan_info(C.byref(p.s), C.byref(nv), C.byref(ng), C.byref(no), groups))
    return nv.value, ng.value, np.array(list(groups), dtype=np.int64)


def plan_info_mc(xi, H, eta, rho, T, K, N, M=1):
    """Host-only plain-MC plan: (n_passes, n_groups, group_of_output, rho_of_output)."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    nv, ng = C.c_int(), C.c_int()
    groups = (C.c_int * p.out)()
    rhos = np.empty(p.out)
    _check(lib().rbg_plan_info_mc(C.byref(p.s), C.byref(nv), C.byref(ng), groups, rhos.ctypes.data_as(_dp)))
    return nv.value, ng.value, np.array(list(groups), dtype=np.int64), rhos


def plan_info_unordered(xi, H, eta, rho, T, K, N, M=1):
    """Host-only unordered plan: (n_passes, n_groups, group_of_output)."""
    arrs = [_arr(x) for x in (H, eta, rho, T, K)]
    n = len(arrs[0])
    u = RbgUnordered(float(xi), *[x.ctypes.data_as(_dp) for x in arrs], n, int(N), int(M))
    nv, ng = C.c_int(), C.c_int()
    groups = (C.c_int * n)()
    _check(lib().rbg_plan_info_unordered(C.byref(u), C.byref(nv), C.byref(ng), groups))
    return nv.value, ng.value, np.array(list(groups), dtype=np.int64)


def launch_count() -> int:
    return int(lib().rbg_launch_count())


def synchronize() -> None:
    _check(lib().rbg_synchronize())


def release() -> None:
    _check(lib().rbg_release())


def profile_enable(on=True) -> None:
    lib().rbg_profile_enable(1 if on else 0)


def profile_reset() -> None:
    lib().rbg_profile_reset()


def profile_read(stage: int):
    """(total milliseconds, kernel launches) recorded for a stage."""
    ms, n = C.c_double(), C.c_uint64()
    _check(lib().rbg_profile_read(int(stage), C.byref(ms), C.byref(n)))
    return ms.value, int(n.value)


def last_transfer_bytes():
    """(host->device, device->host) bytes of this thread's last pricing call."""
    a, b = C.c_uint64(), C.c_uint64()
    lib().rbg_last_transfer_bytes(C.byref(a), C.byref(b))
    return int(a.value), int(b.value)


def debug_mixed_paths(xi, H, eta, rho, T, K, N, M, **opts):
    """Diagnostic run of the mixed path kernel: (normals [M, 2, Np],
    X [M, Np], ivb [n_groups, M, 2]) as float32, Np = N rounded up to 32."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    o = options(precision=MIXED, **opts)
    _, ng, _ = plan_info(xi, H, eta, rho, T, K, N, M)
    Np = (int(N) + 31) // 32 * 32
    w = np.empty((M, 2, Np), np.float32)
    x = np.empty((M, Np), np.float32)
    iv = np.empty((ng, M, 2), np.float32)
    fp = C.POINTER(C.c_float)
    _check(lib().rbg_debug_mixed_paths(C.byref(p.s), C.byref(o), w.ctypes.data_as(fp), x.ctypes.data_as(fp),
                                       iv.ctypes.data_as(fp)))
    return w, x, iv


PROFILE_SITES = {1: "producer wait (free stage)", 2: "epilogue wait (MMA results)", 3: "MMA wait (strip load)",
                 4: "MMA wait (TMEM free)", 5: "MMA wait (A tile)", 7: "epilogue wait (producer tile)",
                 8: "epilogue wait (next producer tile)", 9: "MMA wait (cached-tile slot free)",
                 10: "MMA wait (cached tile)", 11: "MMA wait (A tile stored)", 12: "MMA wait (stores complete)",
                 16: "producer busy", 17: "epilogue busy", 18: "MMA busy", 20: "epilogue fused payoffs"}


def debug_mixed_profile(xi, H, eta, rho, T, K, N, M, **opts):
    """Cycle counters of one diagnostic mixed-kernel run (see the header)."""
    p = _Params(xi, H, eta, rho, T, K, N, M)
    o = options(precision=MIXED, **opts)
    c = (C.c_uint64 * 32)()
    _check(lib().rbg_debug_mixed_profile(C.byref(p.s), C.byref(o), c, 32))
    return {PROFILE_SITES.get(i, str(i)): int(c[i]) for i in range(32) if c[i]}


# ------------------------------------------------------------ serving loop
class RbgServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("high_priority_slots", C.c_int), ("hbm_budget", C.c_uint64),
                ("max_batch_paths", C.c_int64), ("small_request_path_steps", C.c_double),
                ("table_cache_entries", C.c_int), ("use_graphs", C.c_int), ("device", C.c_int),
                ("batch_slots", C.c_int), ("max_batch_jobs", C.c_int), ("batch_path_steps", C.c_double),
                ("batch_wait_us", C.c_double)]


class RbgServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("completed", "failed", "pending", "in_flight", "hbm_in_use",
                                          "table_cache_hits", "table_cache_misses", "graph_launches",
                                          "graph_instantiations", "graph_updates", "max_launch_us", "pin_growths",
                                          "batches", "batched_requests", "max_alloc_us", "max_tables_us",
                                          "max_upload_us", "max_graph_us")]


def _server_lib():
    L = lib()
    if not getattr(L, "_server_ready", False):
        SP = C.c_void_p
        L.rbg_server_default_config.argtypes = [C.POINTER(RbgServerConfig)]
        L.rbg_server_create.argtypes = [C.POINTER(RbgServerConfig), C.POINTER(SP)]
        L.rbg_server_create.restype = C.c_int
        L.rbg_server_submit.argtypes = [SP, C.POINTER(RbgParams), C.POINTER(RbgOptions), C.POINTER(C.c_uint64)]
        L.rbg_server_submit.restype = C.c_int
        L.rbg_server_poll.argtypes = [SP, C.c_uint64, C.POINTER(C.c_int)]
        L.rbg_server_poll.restype = C.c_int
        L.rbg_server_wait.argtypes = [SP, C.c_uint64, _dp, _dp, _dp, _dp]
        L.rbg_server_wait.restype = C.c_int
        L.rbg_server_wait_timed.argtypes = [SP, C.c_uint64, _dp, _dp, _dp, _dp]
        L.rbg_server_wait_timed.restype = C.c_int
        L.rbg_server_get_stats.argtypes = [SP, C.POINTER(RbgServerStats)]
        L.rbg_server_get_stats.restype = C.c_int
        L.rbg_server_destroy.argtypes = [SP]
        L.rbg_server_destroy.restype = C.c_int
        L.rbg_server_last_error.restype = C.c_char_p
        L._server_ready = True
    return L


class Server:
    """Continuously batched pricing loop (rbg_server_* in the C ABI).

    submit() copies the request and returns a ticket at once; wait(ticket)
    blocks until its results are on the host and returns (price, stat, iv,
    latency_ms), latency measured by the server from submit to completion."""

    def __init__(self, **cfg):
        L = _server_lib()
        c = RbgServerConfig()
        L.rbg_server_default_config(C.byref(c))
        for k, v in cfg.items():
            setattr(c, k, v)
        self._h = C.c_void_p()
        rc = L.rbg_server_create(C.byref(c), C.byref(self._h))
        if rc:
            raise RbgError(f"server create: {L.rbg_server_last_error().decode()}")
        self._nout = {}

    def submit(self, xi, H, eta, rho, T, K, N, M, **opts) -> int:
        p = _Params(xi, H, eta, rho, T, K, N, M)
        o = options(precision=MIXED, **opts)
        t = C.c_uint64()
        rc = _server_lib().rbg_server_submit(self._h, C.byref(p.s), C.byref(o), C.byref(t))
        if rc:
            raise RbgError(f"submit status {rc}: {_server_lib().rbg_server_last_error().decode()}")
        self._nout[t.value] = p.out
        return t.value

    def wait(self, ticket):
        n = self._nout.pop(ticket)
        price, stat, iv, lat = np.empty(n), np.empty(n), np.empty(n), C.c_double()
        rc = _server_lib().rbg_server_wait(self._h, ticket, price.ctypes.data_as(_dp), stat.ctypes.data_as(_dp),
                                           iv.ctypes.data_as(_dp), C.byref(lat))
        if rc:
            raise RbgError(f"request status {rc}: {_server_lib().rbg_server_last_error().decode()}")
        return price, stat, iv, lat.value

    def wait_timed(self, ticket):
        """wait() with the latency split: (price, stat, iv, (queue_ms,
        service_ms, total_ms)), queue = submit to admission onto a slot."""
        n = self._nout.pop(ticket)
        price, stat, iv, t = np.empty(n), np.empty(n), np.empty(n), np.empty(3)
        rc = _server_lib().rbg_server_wait_timed(self._h, ticket, price.ctypes.data_as(_dp),
                                                 stat.ctypes.data_as(_dp), iv.ctypes.data_as(_dp),
                                                 t.ctypes.data_as(_dp))
        if rc:
            raise RbgError(f"request status {rc}: {_server_lib().rbg_server_last_error().decode()}")
        return price, stat, iv, (float(t[0]), float(t[1]), float(t[2]))

    def stats(self) -> dict:
        s = RbgServerStats()
        _server_lib().rbg_server_get_stats(self._h, C.byref(s))
        return {n: int(getattr(s, n)) for n, _ in RbgServerStats._fields_}

    def close(self):
        if self._h:
            _server_lib().rbg_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
