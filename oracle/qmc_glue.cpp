// qmc_glue.cpp -- TEST INFRASTRUCTURE, linked only into oracle/_ref/libqmc_ref.so
// with the reference's own rBergomi/sobol.cpp and rBergomi/qmc.cpp.
//
// Exposes, over a C ABI for ctypes:
//   qmcglue_sobol          i8_sobol's point `seed` in dimension `dim`;
//   qmcglue_normal_sample  normalQMC_sample (rBergomi/qmc.cpp:29-38): the point's
//                          coordinates through the normal quantile (here the
//                          from-scratch Boost stand-in in oracle/shims/);
//   qmcglue_hier           hierarchical2increments (rBergomi/aux.h:106-125).
// i8_sobol keeps its sequence state in statics and does not reset it when the
// dimension changes, so every query first asks for point 0, which restarts
// the state for the requested dimension.
#include <algorithm>
#include <vector>

#include "qmc.h"

static void restart(int dim)
{
    std::vector<double> scratch(dim);
    long long zero = 0;
    i8_sobol(dim, &zero, scratch.data());
}

extern "C" void qmcglue_sobol(int dim, long long seed, double* quasi)
{
    restart(dim);
    i8_sobol(dim, &seed, quasi);
}

extern "C" void qmcglue_normal_sample(int dim, long long i, double* out)
{
    restart(dim);
    Vector z(dim);
    normalQMC_sample(z, dim, i);
    std::copy(z.begin(), z.end(), out);
}

extern "C" void qmcglue_hier(const double* Z, int n, double* dW)
{
    Vector z(Z, Z + n), w(n);
    hierarchical2increments(z, w);
    std::copy(w.begin(), w.end(), dW);
}

// Points 1, 2, ..., last in one sequential walk (each i8_sobol call then
// costs one XOR per coordinate); the points whose index is listed in `want`
// (ascending) are copied out, dim values each.
extern "C" void qmcglue_sobol_walk(int dim, long long last, const long long* want, int nwant, double* out)
{
    restart(dim);
    std::vector<double> x(dim);
    int w = 0;
    for (long long s = 1; s <= last && w < nwant; ++s) {
        long long seed = s;
        i8_sobol(dim, &seed, x.data());
        if (s == want[w]) std::copy(x.begin(), x.end(), out + (size_t)dim * w++);
    }
}
