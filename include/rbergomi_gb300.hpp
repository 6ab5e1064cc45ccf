/*
 * rbergomi_gb300.hpp -- the reference library's C++ interface over the C ABI.
 *
 * Replaces rBergLib/interface.h:23-62 (ResultSimple, ParSimple and the four
 * ComputeIV[RT]_{single,multi}Thread drivers) and the IV_call of
 * rBergLib/BlackScholes.h:16, so a C++ caller written against interface.h
 * (testRBergLib/tests.cpp:14-70, the console mains) relinks against
 * librbergomi_gb300.so with this header in place of interface.h.
 *
 * Semantics (implemented in rbergomi_gb300/csrc/rbg_cxx.cpp):
 *   - H, eta, rho are aligned (par_size each), T and K aligned (op_size
 *     each); output i <-> (H, eta, rho)[i / op_size], (T, K)[i % op_size]
 *     (rBergLib/ParamTot.h:28-33).  S0 = 1, r = 0.
 *   - ComputeIV_* price with the plain Monte Carlo estimator (the reference's
 *     ComputeIV / ComputeIVMT), ComputeIVRT_* with the Romano-Touzi one
 *     (ComputeIVRT / ComputeIVRTMT).  price, iv and stat are always filled.
 *   - The result's H, rho, eta, T, K vectors echo the parameters per output,
 *     as Result2ResultSimple does (rBergLib/interface.cpp:36-49); they are
 *     not swapped.  numThreads is 1 for the single-threaded drivers.
 *   - The seed words fold into one Philox key as in computeIVRT_tensor.  One
 *     GPU does the work: numThreads is validated (>= 1) and otherwise
 *     ignored, so single- and multi-threaded calls with the same seed give
 *     the same prices (the reference's depend on the thread count).
 *   - Precision: FP64 unless the environment sets RBG_PRECISION=mixed.
 *   - Failures throw: std::invalid_argument for bad arguments (sizes,
 *     numThreads < 1), std::runtime_error with the library's message for a
 *     CUDA failure.  The reference has no error path here.
 */
#ifndef RBERGOMI_GB300_HPP
#define RBERGOMI_GB300_HPP

#include <cstddef>
#include <cstdint>
#include <vector>

#include "rbergomi_gb300.h"

/* rBergLib/RBergomi.h:46 */
typedef std::vector<double> Vector;

/* rBergLib/interface.h:23-36: field order kept (aggregate initialisation). */
struct ResultSimple {
    Vector price; /* one price per (H, eta, rho) x (T, K) combination */
    Vector iv;    /* implied vols, always filled */
    Vector H;     /* the same size as price: H[i] is used for price[i], ... */
    Vector rho;
    Vector eta;
    Vector T;
    Vector K;
    double xi;
    Vector stat; /* Monte Carlo standard errors */
    int N;
    long M;
    int numThreads;
};

/* rBergLib/interface.h:39-49: a C-style array of H values. */
struct ParSimple {
    double* H;
    size_t n_H;
    ParSimple();
    ParSimple(double* h, size_t n_h);
    ParSimple(const ParSimple& other);
    ParSimple& operator=(const ParSimple& other);
    ~ParSimple();
    Vector getH() const;
};

ResultSimple ComputeIV_singleThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                    std::vector<uint64_t> seed);

ResultSimple ComputeIV_multiThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                   int numThreads, std::vector<uint64_t> seed);

ResultSimple ComputeIVRT_singleThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                      std::vector<uint64_t> seed);

ResultSimple ComputeIVRT_multiThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                     int numThreads, std::vector<uint64_t> seed);

/* rBergLib/BlackScholes.h:16: Black-Scholes implied vol of a call price
 * (S0, K, tau, rate r), by the library's FP64 inversion on the GPU
 * (rbg_implied_vol after the homogeneity map to S0 = 1, r = 0).  NaN where
 * no volatility reproduces the price. */
double IV_call(double price, double S0, double K, double tau, double r = 0.0);

#endif /* RBERGOMI_GB300_HPP */
