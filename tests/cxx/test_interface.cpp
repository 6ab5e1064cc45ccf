// A C++ caller of the reference's interface.h API, relinked against
// librbergomi_gb300.so: the pricing checks of the reference's own unit test
// (testRBergLib/tests.cpp:14-70, "Test the single and multi-threaded pricing
// routines"), the same parameters, reference prices and tolerances, with a
// small REQUIRE in place of the Catch framework.  One implied-vol check is
// taken against the compiled reference's own output instead of trueVol (see
// below: the reference misses it too).  Prints every result as
//   <driver> <i> <price> <stat> <iv> <H> <eta> <rho> <T> <K>
// for the Python test to compare with the C-ABI calls, and exits nonzero if
// any check fails.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "rbergomi_gb300.hpp"

static int g_failed = 0;

#define REQUIRE(cond)                                                             \
    do {                                                                          \
        if (!(cond)) {                                                            \
            std::fprintf(stderr, "%s:%d: REQUIRE(%s) failed\n", __FILE__, __LINE__, #cond); \
            ++g_failed;                                                           \
        }                                                                         \
    } while (0)

static void print(const char* name, const ResultSimple& r)
{
    for (size_t i = 0; i < r.price.size(); ++i)
        std::printf("%s %zu %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", name, i, r.price[i], r.stat[i], r.iv[i],
                    r.H[i], r.eta[i], r.rho[i], r.T[i], r.K[i]);
}

int main()
{
    const double xi = 0.07;
    const Vector H{0.07, 0.1};
    Vector eta{2.2, 2.4};
    Vector rho{-0.9, -0.85};
    Vector T{0.5, 1.0};
    Vector K{0.8, 1.0};
    Vector truePrice{0.2149403, 0.08461882, 0.2157838, 0.07758564};
    long steps = 256;
    long M = 10 * static_cast<long>(std::pow(static_cast<double>(steps), 2.0));
    std::vector<uint64_t> seed{123, 452, 567, 248, 9436, 675, 194, 6702};
    const int numThreads = 8;
    const double epsilon = 0.005;

    Vector trueVol(truePrice.size());
    trueVol[0] = IV_call(truePrice[0], 1.0, K[0], T[0]);
    trueVol[1] = IV_call(truePrice[1], 1.0, K[1], T[1]);
    trueVol[2] = IV_call(truePrice[2], 1.0, K[0], T[0]);
    trueVol[3] = IV_call(truePrice[3], 1.0, K[1], T[1]);

    const struct {
        const char* name;
        ResultSimple (*single)(double, Vector, Vector, Vector, Vector, Vector, int, long, std::vector<uint64_t>);
        ResultSimple (*multi)(double, Vector, Vector, Vector, Vector, Vector, int, long, int, std::vector<uint64_t>);
    } drivers[] = {{"IV", ComputeIV_singleThread, ComputeIV_multiThread},
                   {"IVRT", ComputeIVRT_singleThread, ComputeIVRT_multiThread}};
    for (const auto& d : drivers) {
        const ResultSimple single = d.single(xi, H, eta, rho, T, K, (int)steps, M, seed);
        const ResultSimple multi = d.multi(xi, H, eta, rho, T, K, (int)steps, M, numThreads, seed);
        for (const ResultSimple* res : {&single, &multi}) {
            REQUIRE(res->price.size() == 4 && res->iv.size() == 4 && res->stat.size() == 4);
            for (int i = 0; i < 4; ++i) {
                REQUIRE(std::fabs(res->price[i] - truePrice[i]) < epsilon + res->stat[i]);
                // the reference's own build misses its implied-vol check at i = 0 (T = 0.5, K = 0.8:
                // iv 0.31006 against trueVol 0.30471 on these seeds, its price 5 standard errors from
                // truePrice where vega is small), as this estimator does; there the implied vol is
                // checked against the compiled reference's value with the same tolerance
                if (i == 0)
                    REQUIRE(std::fabs(res->iv[i] - 0.31005859) < epsilon);
                else
                    REQUIRE(std::fabs(res->iv[i] - trueVol[i]) < epsilon);
                // and the pricer's implied vol is the inversion of its own price
                REQUIRE(std::fabs(res->iv[i] - IV_call(res->price[i], 1.0, res->K[i], res->T[i])) < 1e-10);
            }
            REQUIRE(res->xi == xi && res->N == (int)steps && res->M == M);
        }
        REQUIRE(single.numThreads == 1 && multi.numThreads == numThreads);
        // one GPU does the work: the thread count does not change the draw
        for (int i = 0; i < 4; ++i) REQUIRE(single.price[i] == multi.price[i]);
        print(d.name, single);
    }

    // argument errors throw instead of exiting
    bool threw = false;
    try {
        ComputeIVRT_multiThread(xi, H, eta, rho, T, K, (int)steps, 1024, 0, seed);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    REQUIRE(threw);

    ParSimple par(const_cast<double*>(H.data()), H.size());
    ParSimple copy = par;
    REQUIRE(copy.getH() == H);

    if (g_failed) std::fprintf(stderr, "%d check(s) failed\n", g_failed);
    return g_failed ? 1 : 0;
}
