// rbg_fft.cu -- the long-horizon Volterra backend of the mixed form: a
// hand-written batched FFT convolution (no cuFFT) fused with Philox
// generation and the variance-path epilogue.
//
// The hybrid-scheme sum Y2[j] = sum_{k<j} W1[k] Gamma[j-k], j < N
// (rBergLib/rBergomiMT.cpp:83-109, where the reference runs three FFTW DFTs of
// length 2N-1 per path) is the first N terms of a circular convolution of
// length L = 2^ceil(log2 2N) of the zero-padded sequences.  Two paths share
// one complex transform: z = W1_a + i W1_b, and because Gamma is real,
// IFFT(FFT(z) * G^) = (W1_a * Gamma) + i (W1_b * Gamma).  G^ = FFT(Gamma)/L
// is computed once per (H, N) on the host in FP64 and stored as FP32.
//
// Transform: radix-4 Stockham auto-sort stages (a radix-2 first stage when
// log2 L is odd) between two shared-memory buffers, twiddles from an FP32
// table of exp(-2 pi i t / L) built on the host in FP64.  One CTA of 512
// threads owns a pair of paths at a time and loops over pairs.
//
// The epilogue is the GEMM kernel's: X = Y2 + a1 W1 + a2 W1perp,
// sqrt(v_{j+1}) = 2^(alpha/2 X_j - beta_j/2), per-group sums of v and
// sqrt(v) W1 reduced across the block in FP32, written as float2 per
// (variance group, path).
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "rbg_device.cuh"
#include "rbg_mixed.hpp"

namespace rbg {

constexpr int kFftThreads = 512;
constexpr int kFftWarps = kFftThreads / 32;

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// One Stockham pass of radix R over L points, src -> dst, span Ns.
template <int R, bool INV>
__device__ __forceinline__ void stockham_pass(const float2* __restrict__ src, float2* __restrict__ dst, int L,
                                              int lns, const float2* __restrict__ tw, int logL)
{
    const int nb = L / R;
    const int Ns = 1 << lns;
    const int lr = (R == 2) ? 1 : 2;
    const int lstep = logL - lns - lr;  // log2(L / (Ns R))
    for (int j = threadIdx.x; j < nb; j += kFftThreads) {
        const int k = j & (Ns - 1);
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[j + r * nb];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 t = __ldg(tw + ((k * r) << lstep));
                if (INV) t.y = -t.y;
                v[r] = cmul(v[r], t);
            }
        }
        const int d = ((j >> lns) << (lns + lr)) + k;
        if (R == 2) {
            dst[d] = cadd(v[0], v[1]);
            dst[d + Ns] = csub(v[0], v[1]);
        } else {
            const float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
            const float2 c = cadd(v[1], v[3]), e = csub(v[1], v[3]);
            // forward: multiply e by -i; inverse: by +i
            const float2 ie = INV ? make_float2(-e.y, e.x) : make_float2(e.y, -e.x);
            dst[d] = cadd(a, c);
            dst[d + Ns] = cadd(b, ie);
            dst[d + 2 * Ns] = csub(a, c);
            dst[d + 3 * Ns] = csub(b, ie);
        }
    }
}

// Full transform; returns the buffer holding the result.
template <bool INV>
__device__ float2* fft_L(float2* a, float2* b, int L, int logL, const float2* __restrict__ tw)
{
    int lns = 0;
    if (logL & 1) {
        stockham_pass<2, INV>(a, b, L, lns, tw, logL);
        __syncthreads();
        float2* t = a; a = b; b = t;
        lns = 1;
    }
    for (; lns < logL; lns += 2) {
        stockham_pass<4, INV>(a, b, L, lns, tw, logL);
        __syncthreads();
        float2* t = a; a = b; b = t;
    }
    return a;
}

struct FftSmem {
    int buf0, buf1, w, red, total;
};

__host__ __device__ inline FftSmem fft_smem(int L, int Np, int n_g)
{
    FftSmem S;
    S.buf0 = 0;
    S.buf1 = L * 8;
    S.w = 2 * L * 8;                               // [2 paths][W1 | W1perp][Np + 1]
    S.red = S.w + 2 * 2 * (Np + 4) * 4;
    S.total = S.red + kFftWarps * n_g * 4 * 4 + 64;
    return S;
}

__global__ void __launch_bounds__(kFftThreads) k_mixed_fft(const __grid_constant__ MixedArgs a)
{
    extern __shared__ __align__(16) unsigned char smf[];
    const int L = a.L, N = a.N, Np = a.Np;
    const FftSmem S = fft_smem(L, Np, a.n_g);
    float2* b0 = (float2*)(smf + S.buf0);
    float2* b1 = (float2*)(smf + S.buf1);
    float* ws = (float*)(smf + S.w);  // path q, stream s: ws + (2q + s) * (Np + 4)
    float* red = (float*)(smf + S.red);
    const int W = Np + 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const PhiloxKeys keys = philox_keys(a.seed);
    const int64_t npairs = (a.B + 1) / 2;
    const int ngrp = (N + 3) >> 2;

    for (int64_t pr = blockIdx.x; pr < npairs; pr += gridDim.x) {
        // 1. normals of both paths, both streams (Np + 1 entries: W1[N] pairs with the last column)
        for (int q = threadIdx.x; q < 4 * ngrp; q += kFftThreads) {
            const int g = q % ngrp, s = (q / ngrp) & 1, pth = q / (2 * ngrp);
            const int64_t m = 2 * pr + pth;
            float z[4] = {0.f, 0.f, 0.f, 0.f};
            if (m < a.B) {
                const uint4 x = philox_group(keys, (uint64_t)(a.path0 + m), (uint32_t)g, (uint32_t)s);
                box_muller_f32(x.x, x.y, z[0], z[1]);
                box_muller_f32(x.z, x.w, z[2], z[3]);
            }
            float* o = ws + (2 * pth + s) * W + 4 * g;
#pragma unroll
            for (int e = 0; e < 4; ++e) o[e] = (4 * g + e < N) ? z[e] : 0.f;
        }
        __syncthreads();
        // 2. z = W1_a + i W1_b, zero-padded to L
        for (int n = threadIdx.x; n < L; n += kFftThreads)
            b0[n] = (n < N) ? make_float2(ws[n], ws[2 * W + n]) : make_float2(0.f, 0.f);
        if (threadIdx.x < 4) {
            // padding entries [N, Np + 4) of the normal rows read as zeros below
            for (int n = N; n < W; ++n) ws[threadIdx.x * W + n] = 0.f;
        }
        __syncthreads();
        // 3. forward FFT, spectrum product (includes 1/L), inverse FFT
        float2* f = fft_L<false>(b0, b1, L, a.logL, a.tw);
        for (int n = threadIdx.x; n < L; n += kFftThreads) f[n] = cmul(f[n], __ldg(a.spec + n));
        __syncthreads();
        float2* g2 = (f == b0) ? b1 : b0;
        float2* y = fft_L<true>(f, g2, L, a.logL, a.tw);
        // 4. epilogue: thread-strided columns for both paths
        const float* w1a = ws;
        const float* w1pa = ws + W;
        const float* w1b = ws + 2 * W;
        const float* w1pb = ws + 3 * W;
        for (int g = 0; g < a.n_g; ++g) {
            const float ah = a.alpha[g];
            const float* bt = a.beta + (size_t)g * Np;
            const int lim = a.nsteps[g] - 1;
            float sva = 0.f, swa = 0.f, svb = 0.f, swb = 0.f;
            for (int j = threadIdx.x; j < lim; j += kFftThreads) {
                const float2 yj = y[j];
                const float bj = __ldg(bt + j);
                const float xa = yj.x + a.a1 * w1a[j] + a.a2 * w1pa[j];
                const float xb = yj.y + a.a1 * w1b[j] + a.a2 * w1pb[j];
                const float sua = ex2_approx(fmaf(ah, xa, -bj));
                const float sub = ex2_approx(fmaf(ah, xb, -bj));
                sva = fmaf(sua, sua, sva);
                swa = fmaf(sua, w1a[j + 1], swa);
                svb = fmaf(sub, sub, svb);
                swb = fmaf(sub, w1b[j + 1], swb);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sva += __shfl_xor_sync(0xffffffffu, sva, o);
                swa += __shfl_xor_sync(0xffffffffu, swa, o);
                svb += __shfl_xor_sync(0xffffffffu, svb, o);
                swb += __shfl_xor_sync(0xffffffffu, swb, o);
            }
            if (lane == 0) {
                float* r = red + (warp * a.n_g + g) * 4;
                r[0] = sva; r[1] = swa; r[2] = svb; r[3] = swb;
            }
        }
        if (a.dbg_x) {
            for (int j = threadIdx.x; j < Np; j += kFftThreads) {
                const float2 yj = y[j];
                const int64_t ma = 2 * pr, mb = 2 * pr + 1;
                if (ma < a.B) a.dbg_x[ma * Np + j] = (j < N) ? yj.x + a.a1 * w1a[j] + a.a2 * w1pa[j] : 0.f;
                if (mb < a.B) a.dbg_x[mb * Np + j] = (j < N) ? yj.y + a.a1 * w1b[j] + a.a2 * w1pb[j] : 0.f;
            }
        }
        if (a.dbg_w) {
            for (int j = threadIdx.x; j < Np; j += kFftThreads)
                for (int pth = 0; pth < 2; ++pth) {
                    const int64_t m = 2 * pr + pth;
                    if (m < a.B) {
                        a.dbg_w[(m * 2 + 0) * Np + j] = ws[(2 * pth) * W + j];
                        a.dbg_w[(m * 2 + 1) * Np + j] = ws[(2 * pth + 1) * W + j];
                    }
                }
        }
        __syncthreads();
        if (threadIdx.x < 2 * a.n_g) {
            const int g = threadIdx.x >> 1, pth = threadIdx.x & 1;
            float sv = 0.f, sw = 0.f;
            for (int k = 0; k < kFftWarps; ++k) {
                const float* r = red + (k * a.n_g + g) * 4 + 2 * pth;
                sv += r[0];
                sw += r[1];
            }
            const int64_t m = 2 * pr + pth;
            if (m < a.B) {
                const float w10 = ws[(2 * pth) * W];
                const float Ivdt = a.dt[g] * (a.xi + sv);
                const float IsvdW = a.sdt[g] * fmaf(a.sqrt_xi, w10, sw);
                a.ivb[(size_t)(a.g0 + g) * a.B + m] = make_float2(Ivdt, IsvdW);
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------- host
namespace {

void fft_host(std::vector<std::complex<double>>& x, bool inverse)
{
    const int n = (int)x.size();
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    const double pi = 3.14159265358979323846;
    for (int len = 2; len <= n; len <<= 1) {
        const double ang = 2 * pi / len * (inverse ? 1 : -1);
        for (int s = 0; s < n; s += len)
            for (int k = 0; k < len / 2; ++k) {
                const std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
                const std::complex<double> u = x[s + k], v = x[s + k + len / 2] * w;
                x[s + k] = u + v;
                x[s + k + len / 2] = u - v;
            }
    }
}

}  // namespace

int fft_log2_len(int N)
{
    int logL = 1;
    while ((1 << logL) < 2 * N) ++logL;
    return logL;
}

size_t fft_smem_bytes(int N, int n_g)
{
    const int L = 1 << fft_log2_len(N);
    const int Np = (N + 31) / 32 * 32;
    return (size_t)fft_smem(L, Np, n_g).total;
}

// spectrum G^ = FFT(Gamma zero-padded to L) / L, FP32; twiddles exp(-2 pi i t / L)
void fft_tables(const double* gamma, int N, int logL, float* spec, float* tw)
{
    const int L = 1 << logL;
    std::vector<std::complex<double>> x(L, 0.0);
    for (int n = 0; n < N; ++n) x[n] = gamma[n];
    fft_host(x, false);
    for (int k = 0; k < L; ++k) {
        spec[2 * k] = (float)(x[k].real() / L);
        spec[2 * k + 1] = (float)(x[k].imag() / L);
    }
    const double pi = 3.14159265358979323846;
    for (int t = 0; t < L; ++t) {
        tw[2 * t] = (float)std::cos(-2 * pi * t / L);
        tw[2 * t + 1] = (float)std::sin(-2 * pi * t / L);
    }
}

cudaError_t launch_mixed_fft(const MixedArgs& A, int sms, cudaStream_t st)
{
    const int smem = fft_smem(A.L, A.Np, A.n_g).total;
    cudaError_t e = cudaFuncSetAttribute(k_mixed_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed_fft, kFftThreads, smem);
    if (per_sm < 1) per_sm = 1;
    const int64_t npairs = (A.B + 1) / 2;
    const int grid = (int)std::min<int64_t>(npairs, (int64_t)sms * per_sm);
    k_mixed_fft<<<grid, kFftThreads, smem, st>>>(A);
    return cudaGetLastError();
}

}  // namespace rbg
