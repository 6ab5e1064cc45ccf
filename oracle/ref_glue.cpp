// ref_glue.cpp -- TEST INFRASTRUCTURE, linked only into oracle/_ref/.
//
// Reproduces the Gaussian stream the reference's single-threaded class draws,
// so the drop-in calls computeIVRT_tensor / computeIV_tensor with
// num_threads == 1 can be replayed on identical normals:
//   RBergomiST::setGen (rBergLib/RBergomi.cpp:234-242): std::seed_seq over the
//     caller's seed words, generate() back into the same words, then
//     mt19937_64.seed(seed[0]);
//   RBergomiST::genGaussian (RBergomi.cpp:244-247): std::normal_distribution
//     <double>(0, 1) drawn sequentially; per sample W1[0..N) then W1perp[0..N)
//     (ComputePriceRT, RBergomi.cpp:180-181) or W1, W1perp, Wperp
//     (ComputePrice, RBergomi.cpp:99-101).
#include <cstdint>
#include <random>
#include <vector>

extern "C" void refglue_st_normals(const uint64_t* seed, int seed_size, long count, double* out)
{
    std::vector<uint64_t> s(seed, seed + seed_size);
    std::seed_seq seeder(s.begin(), s.end());
    seeder.generate(s.begin(), s.end());
    std::mt19937_64 gen;
    gen.seed(s[0]);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (long i = 0; i < count; ++i) out[i] = dist(gen);
}
