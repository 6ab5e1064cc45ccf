// rbg_device.cuh -- device helpers shared by the FP64 and mixed kernels:
// Philox4x32-10 (Salmon et al., SC'11), Box-Muller transforms, the
// conditional Black-Scholes call, compensated sums.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rbg {

// Philox4x32-10: ten rounds of two 32x32->64 multiplies and a Feistel-like
// permutation, Weyl key schedule between rounds.  The round keys depend only
// on the seed, so callers that draw many blocks precompute them once.
struct PhiloxKeys {
    uint32_t a[10], b[10];
};

__device__ __forceinline__ PhiloxKeys philox_keys(uint64_t seed)
{
    PhiloxKeys k;
    uint32_t x = (uint32_t)seed, y = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        k.a[r] = x;
        k.b[r] = y;
        x += 0x9E3779B9u;
        y += 0xBB67AE85u;
    }
    return k;
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, const PhiloxKeys& k)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k.a[r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k.b[r],
                       (uint32_t)p0);
    }
    return c;
}

// Counter layout of the project's normal stream: steps 4g..4g+3 of stream s
// (0 = W1, 1 = W1perp, 2 = Wperp) of global path p.
__device__ __forceinline__ uint4 philox_group(const PhiloxKeys& k, uint64_t p, uint32_t g, uint32_t s)
{
    return philox4x32_10(make_uint4(g, (uint32_t)p, (uint32_t)(p >> 32), s), k);
}

__device__ __forceinline__ uint4 philox_group(uint64_t seed, uint64_t p, uint32_t g, uint32_t s)
{
    return philox_group(philox_keys(seed), p, g, s);
}

// Hardware approximations (PTX .approx instructions on the MUFU pipe).
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_approx(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sqrt_approx(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void sincos_approx(float x, float& s, float& c)
{
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(x));
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(x));
}

// Standard normal quantile of u in (0, 1/2] in FP32 (the mixed form's Sobol'
// normals).  The form of M. Giles, "Approximating the erfinv function" (GPU
// Computing Gems, Jade Edition, 2011): Phi^-1(u) = sqrt(2) x P(w) with
// x = 2u - 1 and w = -ln(1 - x^2) = -ln(4u(1 - u)); P is a degree-8
// polynomial in w - 2.5 for w < 5 and in sqrt(w) - 3 above.  The coefficients
// were fitted for this library (weighted least squares on the relative error
// against double-precision erfinv, w in [0, 5) and [5, 22.5], i.e. u down to
// 2^-32): relative error <= 6e-7 of the exact quantile of the FP32 input.
__device__ __forceinline__ float normal_quantile_lower_f32(float u)
{
    const float x = fmaf(2.f, u, -1.f);
    const float w = -0.693147181f * lg2_approx(4.f * u * (1.f - u));
    float p;
    if (w < 5.f) {
        const float t = w - 2.5f;
        const float c[9] = {2.853470238e-8f, 3.437269397e-7f, -3.528858501e-6f, -4.396779949e-6f, 2.186021901e-4f, -1.253707519e-3f, -4.177707740e-3f, 2.466407261e-1f, 1.501409422e+0f};
        p = c[0];
#pragma unroll
        for (int i = 1; i < 9; ++i) p = fmaf(p, t, c[i]);
    } else {
        const float s = sqrt_approx(w) - 3.f;
        const float c[9] = {-8.581864353e-6f, -1.442782343e-4f, 1.150858774e-3f, -3.388356747e-3f, 5.807593624e-3f, -7.720514824e-3f, 9.428526195e-3f, 1.001682603e+0f, 2.832977331e+0f};
        p = c[0];
#pragma unroll
        for (int i = 1; i < 9; ++i) p = fmaf(p, s, c[i]);
    }
    return 1.41421356f * x * p;
}

// Sobol' normal in FP32 from the top 32 bits q of a coordinate (x = q 2^-32):
// the quantile of the lower tail u = min(x, 1 - x), so points near 1 keep
// their relative precision; sign restored after.  For x >= 1/2 the tail
// 1 - x = (~q + 1) 2^-32 is formed as float(~q) 2^-32 + 2^-32 in one FMA:
// exact below 2^-8, within one float ulp of the correctly rounded tail above.
// (~q, not 0 - q: the subtraction form is the integer absolute-value idiom,
// which the compiler turns into a signed abs that reads q = 2^31 as -2^31.)
// Both ~q (x >= 1/2) and q (x < 1/2) lie below 2^31.
__device__ __forceinline__ float sobol_normal_f32(unsigned int q)
{
    const unsigned int up = (unsigned int)((int)q >> 31);  // all ones for x >= 1/2
    const float f = __uint2float_rn(q ^ up);
    const float z = normal_quantile_lower_f32(fmaf(f, 0x1p-32f, __uint_as_float(up & 0x2f800000u)));
    return __uint_as_float(__float_as_uint(z) ^ (up & 0x80000000u));
}

// FP32 Box-Muller on uniforms (x + 1/2) 2^-32 (mixed form), on the MUFU pipe:
// r = sqrt(-2 ln 2 log2 u0); the angle is taken as t = 2 pi u1 - pi, which
// lies in (-pi, pi) where sin/cos.approx are accurate, and
// cos(2 pi u1) = -cos t, sin(2 pi u1) = -sin t.
__device__ __forceinline__ void box_muller_f32(uint32_t a, uint32_t b, float& z0, float& z1)
{
    const float u0 = fmaf((float)a, 2.3283064e-10f, 1.1641532e-10f);
    const float u1 = fmaf((float)b, 2.3283064e-10f, 1.1641532e-10f);
    const float nr = -sqrt_approx(-1.3862944f * lg2_approx(u0));
    const float th = fmaf(6.2831853f, u1, -3.14159265f);
    float s, c;
    sincos_approx(th, s, c);
    z0 = nr * c;
    z1 = nr * s;
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

// Plain Monte Carlo payoff (rBergLib/rBergomiMT.cpp:134-136 updateZ, :129-132
// scaleZ, :111-116 updateS, aux.h:31-34 posPart): with Z = rho W1 + sqrt(1 - rho^2) Wperp,
// log S = sum sqrt(v) sdt Z - dt/2 sum v = rho IsvdW + sqrt(1 - rho^2) IsvdWp
// - Ivdt / 2, the same sum regrouped by normal stream.
__device__ __forceinline__ double mc_payoff(double Ivdt, double IsvdW, double IsvdWp, double rho, double K)
{
    const double S = exp(rho * IsvdW + sqrt(1.0 - rho * rho) * IsvdWp - 0.5 * Ivdt);
    const double d = S - K;
    return d > 0.0 ? d : 0.0;
}

// Neumaier compensated accumulation.
__device__ __forceinline__ void neumaier_add(double& s, double& c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Complementary error function for z >= 0 by the Chebyshev fit of
// Press, Teukolsky, Vetterling & Flannery, "Numerical Recipes" (2nd ed.,
// section 6.2, function erfcc): erfc(z) = t exp(-z^2 + P(t)),
// t = 1 / (1 + z/2), fractional error below 1.2e-7 for every z >= 0 -- so the
// tails keep their relative accuracy.  One reciprocal and one ex2 on MUFU.
__device__ __forceinline__ float erfc_cheb(float z)
{
    const float t = rcp_approx(fmaf(0.5f, z, 1.0f));
    float p = 0.17087277f;
    p = fmaf(p, t, -0.82215223f);
    p = fmaf(p, t, 1.48851587f);
    p = fmaf(p, t, -1.13520398f);
    p = fmaf(p, t, 0.27886807f);
    p = fmaf(p, t, -0.18628806f);
    p = fmaf(p, t, 0.09678418f);
    p = fmaf(p, t, 0.37409196f);
    p = fmaf(p, t, 1.00002368f);
    p = fmaf(p, t, -1.26551223f);
    return t * ex2_approx(1.4426950408889634f * fmaf(-z, z, p));
}

// Standard normal CDF with relative accuracy in the lower tail.
__device__ __forceinline__ float phi_f32(float x)
{
    const float z = -0.70710678118654752f * x;
    const float e = 0.5f * erfc_cheb(fabsf(z));
    return z >= 0.0f ? e : 1.0f - e;
}

// Kahan compensated accumulation in FP32: s holds the sum, c the running
// error (subtract c to recover the compensated value).
__device__ __forceinline__ void kahan_add_f32(float& s, float& c, float x)
{
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

}  // namespace rbg
