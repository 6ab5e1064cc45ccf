// ml_glue.cpp -- TEST INFRASTRUCTURE, linked only into oracle/_ref/libml_ref.so.
//
// Drives the reference's Romano-Touzi control-variate estimator,
// RBergomi::ComputeIVRTVarRed (ML_console_ST/RBergomi.cpp:218-306, pilot
// estimateControlVariate :493-540, payoff updatePayoffControlVariate
// :478-491), compiled unmodified from ML_console_ST.  The class fixes its
// pilot size at 10,000 paths in the constructor (:34); the glue reaches the
// private member to make small golden cases possible.
//
// mlglue_normals reproduces the Gaussian stream the class draws
// (RBergomi::setGen / genGaussian, ML_console_ST/RBergomi.cpp:308-317):
// std::seed_seq over the seed words, generate() back into them,
// mt19937_64.seed(seed[0]), std::normal_distribution<double>(0, 1) drawn in
// order -- pilot paths first (W1 then W1perp per path), then the main paths.
#include <fftw3.h>

#include <algorithm>
#include <boost/math/tools/roots.hpp>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <sstream>
#include <fstream>
#include <iostream>
#include <iterator>
#include <numeric>
#include <random>
#include <string>
#include <vector>

// every standard header the class pulls in is already included above, so
// only the class's own declarations see the access change
#define private public
#include "RBergomi.h"
#undef private

extern "C" int mlglue_price_rt_varred(const double* xi, const double* H, const double* eta, const double* rho,
                                      const double* T, const double* K, long n, int N, long M, long Mcontrol,
                                      const uint64_t* seed, int seed_size, double* price, double* stat, double* iv)
{
    Vector x(xi, xi + n), h(H, H + n), e(eta, eta + n), r(rho, rho + n), t(T, T + n), k(K, K + n);
    std::vector<uint64_t> s(seed, seed + seed_size);
    RBergomi rb(x, h, e, r, t, k, N, M, s);
    rb.Mcontrol = Mcontrol;
    Result res = rb.ComputeIVRTVarRed();
    for (long i = 0; i < n; ++i) {
        price[i] = res.price[i];
        stat[i] = res.stat[i];
        iv[i] = res.iv[i];
    }
    return 0;
}

extern "C" void mlglue_normals(const uint64_t* seed, int seed_size, long count, double* out)
{
    std::vector<uint64_t> s(seed, seed + seed_size);
    std::seed_seq seeder(s.begin(), s.end());
    seeder.generate(s.begin(), s.end());
    std::mt19937_64 gen;
    gen.seed(s[0]);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (long i = 0; i < count; ++i) out[i] = dist(gen);
}
