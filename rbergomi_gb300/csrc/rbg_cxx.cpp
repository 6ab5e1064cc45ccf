// rbg_cxx.cpp -- the reference's C++ interface (rBergLib/interface.h:23-62,
// BlackScholes.h:16) as thin wrappers over the rbg_* C ABI.  Declared in
// include/rbergomi_gb300.hpp.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>

#include "rbergomi_gb300.hpp"
#include "rbg_internal.hpp"

namespace {

// The drop-in layer's precision switch: FP64 unless RBG_PRECISION=mixed.
int env_precision()
{
    const char* prec = std::getenv("RBG_PRECISION");
    return (prec && std::strcmp(prec, "mixed") == 0) ? RBG_MIXED : RBG_FP64;
}

void throw_on(int rc, const char* what)
{
    if (rc == RBG_OK) return;
    const std::string msg = std::string(what) + ": " + rbg_last_error();
    if (rc == RBG_ERR_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

// One driver for all four entry points (interface.cpp:11-34): ParamTot
// layout, price / iv / stat, and the echoed parameters of Result2ResultSimple
// (interface.cpp:36-49).
ResultSimple compute(bool rt, double xi, const Vector& H, const Vector& eta, const Vector& rho, const Vector& T,
                     const Vector& K, int N, long M, int numThreads, const std::vector<uint64_t>& seed)
{
    if (numThreads < 1) throw std::invalid_argument("numThreads has to be a positive integer");
    if (H.size() != eta.size() || H.size() != rho.size())
        throw std::invalid_argument("H, eta and rho must have the same length");
    if (T.size() != K.size()) throw std::invalid_argument("T and K must have the same length");
    const size_t par = H.size(), op = T.size(), out = par * op;
    ResultSimple r{Vector(out, 0.0), Vector(out, 0.0), Vector(out), Vector(out), Vector(out), Vector(out),
                   Vector(out), xi, Vector(out, 0.0), N, M, numThreads};
    for (size_t i = 0; i < out; ++i) {
        r.H[i] = H[i / op];
        r.rho[i] = rho[i / op];
        r.eta[i] = eta[i / op];
        r.T[i] = T[i % op];
        r.K[i] = K[i % op];
    }
    if (out == 0) return r;  // an empty grid: the reference's loops run zero times
    rbg_params p{xi, H.data(), eta.data(), rho.data(), (int)par, T.data(), K.data(), (int)op, N, (int64_t)M};
    rbg_options o;
    rbg_default_options(&o);
    o.precision = env_precision();
    o.seed = rbg::fold_seed(seed.data(), (int)seed.size());
    const int rc = rt ? rbg_price_rt(&p, &o, r.price.data(), r.stat.data(), r.iv.data())
                      : rbg_price_mc(&p, &o, r.price.data(), r.stat.data(), r.iv.data());
    throw_on(rc, rt ? "ComputeIVRT" : "ComputeIV");
    return r;
}

}  // namespace

ParSimple::ParSimple() : H(nullptr), n_H(0) {}

ParSimple::ParSimple(double* h, size_t n_h) : H(n_h ? new double[n_h] : nullptr), n_H(n_h)
{
    if (n_h) std::copy(h, h + n_h, H);
}

ParSimple::ParSimple(const ParSimple& other) : ParSimple(other.H, other.n_H) {}

ParSimple& ParSimple::operator=(const ParSimple& other)
{
    if (this != &other) {
        double* h = other.n_H ? new double[other.n_H] : nullptr;
        if (other.n_H) std::copy(other.H, other.H + other.n_H, h);
        delete[] H;
        H = h;
        n_H = other.n_H;
    }
    return *this;
}

ParSimple::~ParSimple() { delete[] H; }

Vector ParSimple::getH() const { return n_H ? Vector(H, H + n_H) : Vector(); }

ResultSimple ComputeIV_singleThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                    std::vector<uint64_t> seed)
{
    return compute(false, xi, H, eta, rho, T, K, N, M, 1, seed);
}

ResultSimple ComputeIV_multiThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                   int numThreads, std::vector<uint64_t> seed)
{
    return compute(false, xi, H, eta, rho, T, K, N, M, numThreads, seed);
}

ResultSimple ComputeIVRT_singleThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                      std::vector<uint64_t> seed)
{
    return compute(true, xi, H, eta, rho, T, K, N, M, 1, seed);
}

ResultSimple ComputeIVRT_multiThread(double xi, Vector H, Vector eta, Vector rho, Vector T, Vector K, int N, long M,
                                     int numThreads, std::vector<uint64_t> seed)
{
    return compute(true, xi, H, eta, rho, T, K, N, M, numThreads, seed);
}

// Call prices are homogeneous: C(S0, K, tau, sigma, r) = S0 C(1, K e^{-r tau} / S0,
// tau, sigma, 0), so the S0 = 1, r = 0 inversion serves every (S0, r).
double IV_call(double price, double S0, double K, double tau, double r)
{
    if (!(S0 > 0.0)) return std::numeric_limits<double>::quiet_NaN();
    const double p = price / S0, k = K * std::exp(-r * tau) / S0;
    double iv = 0.0;
    throw_on(rbg_implied_vol(1, &p, &k, &tau, &iv), "IV_call");
    return iv;
}
