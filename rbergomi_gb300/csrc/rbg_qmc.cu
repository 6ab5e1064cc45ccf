// rbg_qmc.cu -- Sobol' quasi-Monte Carlo normals (FP64 form; FP32 for the mixed form).
//
// Restates
//   rBergomi/rBergomiMT.cpp:669-670 (ComputePriceRTMT_sobol): path m takes
//     Sobol' point m + 1 in dimension 2N, then breakZ (rBergomi/aux.h:186-191):
//     W1 = coordinates 0, 2, 4, ..., W1perp = coordinates 1, 3, 5, ...;
//   rBergomi/qmc.cpp:29-38 (normalQMC_sample): the normal quantile of every
//     coordinate (here CUDA's FP64 normcdfinv);
//   rBergomi/sobol.cpp i8_sobol: points in Antonov-Saleev (Gray-code) order,
//     point s = (XOR of the direction integers v[d][k] over the set bits k of
//     s ^ (s >> 1)) * 2^-62;
//   rBergomi/aux.h:106-125 (hierarchical2increments): the Brownian-bridge
//     (Haar) map of each N = 2^m stream, when the caller asks for it.
// The reference walks the sequence point by point under a lock; here each
// (path, coordinate pair) is computed on its own from its Gray code, so
// batches and path offsets need no state.  The direction integers are the
// caller's ([dims][62], uploaded transposed to [62][2N]).
#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>

#include "rbg_device.cuh"
#include "rbg_internal.hpp"

namespace rbg {

// the 62-bit integers of coordinates 2j and 2j + 1 of point s; Vt is [kSobolBits][2N]
__device__ __forceinline__ void sobol_pair_q(const unsigned long long* __restrict__ Vt, int N, unsigned long long s,
                                             int j, unsigned long long& q0, unsigned long long& q1)
{
    unsigned long long g = s ^ (s >> 1);
    q0 = q1 = 0;
    const ulonglong2* col = reinterpret_cast<const ulonglong2*>(Vt) + j;  // 16-byte aligned: 2N columns per row
    while (g) {
        const int k = __ffsll((long long)g) - 1;
        const ulonglong2 v = __ldg(col + (size_t)k * N);
        q0 ^= v.x;
        q1 ^= v.y;
        g &= g - 1;
    }
}

__device__ __forceinline__ void sobol_pair(const unsigned long long* __restrict__ Vt, int N, unsigned long long s,
                                           int j, double& x0, double& x1)
{
    unsigned long long q0, q1;
    sobol_pair_q(Vt, N, s, j, q0, q1);
    x0 = __ull2double_rn(q0) * 0x1p-62;
    x1 = __ull2double_rn(q1) * 0x1p-62;
}

// Z[b][0][j], Z[b][1][j] for paths b < B (point s0 + b).  F32: the mixed
// form's normals (top 32 bits, FP32 quantile), widened exactly to double.
template <bool F32>
__global__ void k_sobol_normals(const unsigned long long* __restrict__ Vt, int N, unsigned long long s0, int64_t B,
                                double* __restrict__ Z)
{
    const int64_t total = B * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / N;
        const int j = (int)(idx - b * N);
        unsigned long long q0, q1;
        sobol_pair_q(Vt, N, s0 + (unsigned long long)b, j, q0, q1);
        double* z = Z + (size_t)b * 2 * N;
        if (F32) {
            z[j] = (double)sobol_normal_f32((unsigned int)(q0 >> 30));
            z[N + j] = (double)sobol_normal_f32((unsigned int)(q1 >> 30));
        } else {
            z[j] = normcdfinv(__ull2double_rn(q0) * 0x1p-62);
            z[N + j] = normcdfinv(__ull2double_rn(q1) * 0x1p-62);
        }
    }
}

// The same, then each stream through the hierarchical map; one block per
// path, the path's 2N normals staged in shared memory.  The sum runs in the
// reference's order, dW[i] = c0 Z[0] + sum_n (c_n w) Z[index].  FP64 (the FP64
// form): every product and sum rounded separately (no contraction into FMA).
// F32 (the mixed form): the FP32 quantile of each coordinate's top 32 bits and
// the same sum in FP32, widened exactly to double -- GB300's FP64 pipe made the
// FP64 map the whole cost of the mixed form's bridged pricing.
template <bool F32>
__global__ void k_sobol_bridge(const unsigned long long* __restrict__ Vt, int N, unsigned long long s0, int64_t B,
                               const __grid_constant__ SobolBridge br, double* __restrict__ Z)
{
    using T = typename std::conditional<F32, float, double>::type;
    extern __shared__ double zs_raw[];  // [2][N] of T
    T* zs = reinterpret_cast<T*>(zs_raw);
    for (int64_t b = blockIdx.x; b < B; b += gridDim.x) {
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            unsigned long long q0, q1;
            sobol_pair_q(Vt, N, s0 + (unsigned long long)b, j, q0, q1);
            if (F32) {
                zs[j] = (T)sobol_normal_f32((unsigned int)(q0 >> 30));
                zs[N + j] = (T)sobol_normal_f32((unsigned int)(q1 >> 30));
            } else {
                zs[j] = (T)normcdfinv(__ull2double_rn(q0) * 0x1p-62);
                zs[N + j] = (T)normcdfinv(__ull2double_rn(q1) * 0x1p-62);
            }
        }
        __syncthreads();
        double* z = Z + (size_t)b * 2 * N;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
#pragma unroll
            for (int st = 0; st < 2; ++st) {
                const T* y = zs + st * N;
                T w;
                if (F32) {
                    w = (T)br.c[0] * y[0];
                    for (int n = 1; n <= br.m; ++n) {
                        const int i2nm = i >> (br.m - n);  // floor(i 2^(n - m))
                        const int iota = (i2nm + 1) & 1;
                        const int index = (1 << (n - 1)) + ((i2nm + iota + 1) >> 1) - 1;
                        const T cn = (T)br.c[n];
                        w = fmaf(iota ? cn : -cn, y[index], w);
                    }
                } else {
                    w = __dmul_rn(br.c[0], y[0]);
                    for (int n = 1; n <= br.m; ++n) {
                        const int i2nm = i >> (br.m - n);
                        const int iota = (i2nm + 1) & 1;
                        const int index = (1 << (n - 1)) + ((i2nm + iota + 1) >> 1) - 1;
                        w = __dadd_rn(w, __dmul_rn(iota ? br.c[n] : -br.c[n], y[index]));
                    }
                }
                z[st * N + i] = (double)w;
            }
        }
        __syncthreads();
    }
}

int launch_sobol_normals(const unsigned long long* Vt, int N, uint64_t s0, int64_t B, const SobolBridge* br,
                         double* Z, void* stream, int f32)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st = (cudaStream_t)stream;
    if (!br) {
        const int64_t total = B * N;
        int64_t blocks = (total + 255) / 256;
        if (blocks > (int64_t)sms * 64) blocks = (int64_t)sms * 64;
        if (f32)
            k_sobol_normals<true><<<(unsigned)blocks, 256, 0, st>>>(Vt, N, (unsigned long long)s0, B, Z);
        else
            k_sobol_normals<false><<<(unsigned)blocks, 256, 0, st>>>(Vt, N, (unsigned long long)s0, B, Z);
    } else {
        const size_t smem = (f32 ? sizeof(float) : sizeof(double)) * 2 * (size_t)N;
        auto kern = f32 ? k_sobol_bridge<true> : k_sobol_bridge<false>;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return -1;
        const int threads = N >= 256 ? 256 : ((N + 31) / 32) * 32;
        const int64_t blocks = B < (int64_t)sms * 8 ? B : (int64_t)sms * 8;
        kern<<<(unsigned)blocks, threads, smem, st>>>(Vt, N, (unsigned long long)s0, B, *br, Z);
    }
    count_launch();
    return 0;
}

}  // namespace rbg
