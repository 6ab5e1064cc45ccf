// rbg_device.cuh -- device helpers shared by the FP64 and mixed kernels:
// Philox4x32-10 (Salmon et al., SC'11), Box-Muller transforms, the
// conditional Black-Scholes call, compensated sums.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rbg {

// Philox4x32-10: ten rounds of two 32x32->64 multiplies and a Feistel-like
// permutation, Weyl key schedule between rounds.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Counter layout of the project's normal stream: steps 4g..4g+3 of stream s
// (0 = W1, 1 = W1perp, 2 = Wperp) of global path p.
__device__ __forceinline__ uint4 philox_group(uint64_t seed, uint64_t p, uint32_t g, uint32_t s)
{
    return philox4x32_10(make_uint4(g, (uint32_t)p, (uint32_t)(p >> 32), s),
                         make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

// FP64 Box-Muller on uniforms (x + 1/2) 2^-32.
__device__ __forceinline__ void box_muller_f64(uint32_t a, uint32_t b, double& z0, double& z1)
{
    const double u0 = ((double)a + 0.5) * 2.3283064365386963e-10;
    const double u1 = ((double)b + 0.5) * 2.3283064365386963e-10;
    const double r = sqrt(-2.0 * log(u0));
    double s, c;
    sincospi(2.0 * u1, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// FP32 Box-Muller on the same uniforms (mixed form).
__device__ __forceinline__ void box_muller_f32(uint32_t a, uint32_t b, float& z0, float& z1)
{
    const float u0 = fmaf((float)a, 2.3283064e-10f, 1.1641532e-10f);
    const float u1 = fmaf((float)b, 2.3283064e-10f, 1.1641532e-10f);
    const float r = sqrtf(-2.0f * logf(u0));
    float s, c;
    sincospif(2.0f * u1, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// Normal CDF and BS call, rBergLib/BlackScholes.cpp:11-21 with tau = 1, r = 0
// (the RT payoff always calls BS_call_price(spot, K, 1.0, vol)).
__device__ __forceinline__ double phi_cdf(double x) { return 0.5 * erfc(-x * 0.70710678118654752440); }

__device__ __forceinline__ double bs_call_tau1(double S0, double K, double sigma)
{
    const double d1 = (log(S0 / K) + 0.5 * sigma * sigma) / sigma;
    const double d2 = d1 - sigma;
    return phi_cdf(d1) * S0 - phi_cdf(d2) * K;
}

// RT conditional payoff, rBergLib/rBergomiMT.cpp:598-602.
__device__ __forceinline__ double rt_payoff(double Ivdt, double IsvdW, double rho, double K)
{
    const double vol = sqrt((1.0 - rho * rho) * Ivdt);
    const double spot = exp(-0.5 * rho * rho * Ivdt + rho * IsvdW);
    return bs_call_tau1(spot, K, vol);
}

// Neumaier compensated accumulation.
__device__ __forceinline__ void neumaier_add(double& s, double& c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

}  // namespace rbg
