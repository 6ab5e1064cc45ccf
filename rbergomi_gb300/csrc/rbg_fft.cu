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
// Transform: Stockham auto-sort passes held in registers, in place in one
// shared-memory buffer: every thread loads its butterflies' inputs, the
// block synchronises, then every thread writes its outputs.  Radix 16 (a
// 4 x 4 decomposition with constant inner twiddles) for four bits of log2 L
// at a time, one radix-2/4/8 pass first for the remainder, so L = 4096 takes
// three passes per transform.  Pass twiddles come from an FP32 table of
// exp(-2 pi i t / L) built on the host in FP64.  The buffer inserts one
// padding element per 16, which keeps the strided writes of the first
// passes off a single bank.  One CTA owns a pair of paths at a time and
// loops over pairs; several CTAs share an SM.
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

// Threads per CTA: one radix-16 butterfly each (L / 16), between one warp and
// 256 threads; L = 8192 runs two butterflies per thread.
__host__ __device__ constexpr int fft_threads(int logL)
{
    return logL >= 12 ? 256 : (logL >= 10 ? (1 << logL) / 16 : 32);
}
// CTAs per SM the launch bounds promise: at most 128 registers a thread below
// L = 8192 (which runs one CTA per SM at up to 255).
__host__ __device__ constexpr int fft_min_blocks(int logL) { return logL >= 13 ? 1 : 65536 / (fft_threads(logL) * 128); }

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) { return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x); }

// padded shared-memory index: one spare element after every 16
__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }

template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b)
{
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3)
{
    const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = mul_mi<INV>(csub(a1, a3));
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

// exp(-+ 2 pi i m / 16) for the inner twiddles of the 4 x 4 radix-16 DFT
template <bool INV>
__device__ __forceinline__ float2 w16(int m)
{
    constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
    float2 w;
    switch (m) {
        case 1: w = make_float2(c1, s1); break;
        case 2: w = make_float2(h, h); break;
        case 3: w = make_float2(s1, c1); break;
        case 6: w = make_float2(-h, h); break;
        case 9: w = make_float2(-c1, -s1); break;
        default: w = make_float2(1.f, 0.f); break;
    }
    if (!INV) w.y = -w.y;
    return w;
}

// In-register DFT of radix R in {2, 4, 8, 16}; v[q'] holds input n = q' and,
// on return, output k at position perm(k): R <= 4 natural order, R = 8, 16
// transposed (k = k1 + A k2 sits at v[4 k1 + k2] with A = R / 4).
template <int R, bool INV>
__device__ __forceinline__ void dft_r(float2 (&v)[R])
{
    if (R == 2) {
        dft2<INV>(v[0], v[1]);
    } else if (R == 4) {
        dft4<INV>(v[0], v[1], v[2], v[3]);
    } else if (R == 8) {
        // n = 4 n1 + n2 (n1 < 2, n2 < 4); k = k1 + 2 k2
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) dft2<INV>(v[n2], v[4 + n2]);
        // twiddle W8^(n2 k1) on (n2, k1 = 1): v[4 + n2]
        constexpr float h = 0.70710678118654752f;
        v[5] = cmul(v[5], make_float2(h, INV ? h : -h));
        v[6] = mul_mi<INV>(v[6]);
        v[7] = cmul(v[7], make_float2(-h, INV ? h : -h));
        dft4<INV>(v[0], v[1], v[2], v[3]);
        dft4<INV>(v[4], v[5], v[6], v[7]);
    } else {
        // n = 4 n1 + n2; k = k1 + 4 k2
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) dft4<INV>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
#pragma unroll
        for (int k1 = 1; k1 < 4; ++k1)
#pragma unroll
            for (int n2 = 1; n2 < 4; ++n2) {
                const int m = n2 * k1;
                if (m == 4) v[4 * k1 + n2] = mul_mi<INV>(v[4 * k1 + n2]);
                else v[4 * k1 + n2] = cmul(v[4 * k1 + n2], w16<INV>(m));
            }
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    }
}

template <int R>
__device__ __forceinline__ int out_slot(int k)
{
    return (R <= 4) ? k : 4 * (k % (R / 4)) + k / (R / 4);
}

// Where the first forward pass reads its input: the transform buffer, or the
// generated normals directly, z[n] = W1_a[n] + i W1_b[n] for n < N and zero
// above (SRC_WS), or the same sequence with every element doubled, which is
// what a radix-2 first pass makes of a zero upper half (SRC_WS_DUP).
enum { SRC_BUF = 0, SRC_WS = 1, SRC_WS_DUP = 2 };

struct FftIn {
    const float* w1a;  // W1 of the pair's first path
    const float* w1b;  // W1 of the second path
    int N;
};

__device__ __forceinline__ float2 ws_z(const FftIn& in, int n)
{
    return n < in.N ? make_float2(in.w1a[n], in.w1b[n]) : make_float2(0.f, 0.f);
}

// One in-place Stockham pass of radix R over L = 2^LOGL points, span 2^LNS.
// ZHI: the upper half of the input is zero (the first forward pass: the
// zero-padded sequence has N <= L / 2 entries), so those loads are skipped.
// SPEC: multiply every output by the spectrum (the last forward pass).
// HALF: store only outputs below L / 2 (the last inverse pass: the Volterra
// sum needs N <= L / 2 of them).
template <int R, int LOGL, int LNS, bool INV, int T, bool ZHI = false, int SRC = SRC_BUF, bool SPEC = false,
          bool HALF = false>
__device__ __forceinline__ void fft_pass(float2* __restrict__ buf, const float2* __restrict__ tw, const FftIn& in,
                                         const float2* __restrict__ spec)
{
    constexpr int L = 1 << LOGL, NB = L / R, NS = 1 << LNS;
    constexpr int LR = (R == 2) ? 1 : (R == 4) ? 2 : (R == 8) ? 3 : 4;
    constexpr int LSTEP = LOGL - LNS - LR;
    constexpr int BPT = (NB + T - 1) / T;  // butterflies per thread
    // only the data stays live across the barrier; twiddles are read after it
    float2 v[BPT][R];
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
        const int j = threadIdx.x + b * T;
        if (NB % T == 0 || j < NB) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int n = j + r * NB;
                if (ZHI && r >= R / 2) v[b][r] = make_float2(0.f, 0.f);
                else if (SRC == SRC_WS) v[b][r] = ws_z(in, n);
                else if (SRC == SRC_WS_DUP) v[b][r] = ws_z(in, n >> 1);
                else v[b][r] = buf[pidx(n)];
            }
        }
    }
    if (SRC == SRC_BUF) __syncthreads();  // reading the normals leaves the buffer free to write
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
        const int j = threadIdx.x + b * T;
        if (NB % T == 0 || j < NB) {
            const int k = j & (NS - 1);
            if (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    if (ZHI && r >= R / 2) continue;
                    float2 t = __ldg(tw + ((k * r) << LSTEP));
                    if (INV) t.y = -t.y;
                    v[b][r] = cmul(v[b][r], t);
                }
            }
            dft_r<R, INV>(v[b]);
            const int d = ((j >> LNS) << (LNS + LR)) + k;
#pragma unroll
            for (int q = 0; q < (HALF ? R / 2 : R); ++q) {
                float2 y = v[b][out_slot<R>(q)];
                if (SPEC) y = cmul(y, __ldg(spec + d + q * NS));
                buf[pidx(d + q * NS)] = y;
            }
        }
    }
    __syncthreads();
}

// Radix-16 passes from span 2^LNS up to L; FIRST marks the transform's first
// pass (SRC and ZHI apply), the last pass gets SPEC (forward) or HALF (inverse).
template <int LOGL, int LNS, bool INV, int T, bool ZHI, int SRC>
__device__ __forceinline__ void fft_r16(float2* buf, const float2* tw, const FftIn& in, const float2* spec)
{
    if constexpr (LNS < LOGL) {
        constexpr bool LAST = LNS + 4 == LOGL;
        fft_pass<16, LOGL, LNS, INV, T, ZHI, SRC, LAST && !INV, LAST && INV>(buf, tw, in, spec);
        fft_r16<LOGL, LNS + 4, INV, T, false, SRC_BUF>(buf, tw, in, spec);
    }
}

// Forward transform of the pair's normals times the spectrum, or inverse
// transform of the buffer.  L >= 16.  For odd log2 L the radix-2 first pass
// of the forward transform is the SRC_WS_DUP read.  The input descriptor is
// passed by value and the Philox round keys come from parameter space: with
// both, the kernel needs no local memory at L = 4096 and 8192 (it spilled
// 84 B at L = 4096 before).  Compiling the transforms as functions of their
// own also removes the spill but measured 13 % slower at L = 4096: the
// scheduler can no longer overlap a pass's twiddle loads with other work.
template <int LOGL, bool INV, int T>
__device__ __forceinline__ void fft_inplace(float2* buf, const float2* tw, const FftIn in, const float2* spec)
{
    constexpr int REM = LOGL % 4;
    if constexpr (INV) {
        if constexpr (REM == 1) fft_pass<2, LOGL, 0, true, T>(buf, tw, in, spec);
        if constexpr (REM == 2) fft_pass<4, LOGL, 0, true, T>(buf, tw, in, spec);
        if constexpr (REM == 3) fft_pass<8, LOGL, 0, true, T>(buf, tw, in, spec);
        fft_r16<LOGL, REM, true, T, false, SRC_BUF>(buf, tw, in, spec);
    } else {
        if constexpr (REM == 1) {
            fft_r16<LOGL, 1, false, T, false, SRC_WS_DUP>(buf, tw, in, spec);
        } else if constexpr (REM == 0) {
            fft_r16<LOGL, 0, false, T, true, SRC_WS>(buf, tw, in, spec);
        } else {
            if constexpr (REM == 2) fft_pass<4, LOGL, 0, false, T, true, SRC_WS>(buf, tw, in, spec);
            if constexpr (REM == 3) fft_pass<8, LOGL, 0, false, T, true, SRC_WS>(buf, tw, in, spec);
            fft_r16<LOGL, REM, false, T, false, SRC_BUF>(buf, tw, in, spec);
        }
    }
}

struct FftSmem {
    int buf, w, red, total;
};

// ns normal streams per path: 2 (RT) or 3 (plain Monte Carlo adds Wperp)
__host__ __device__ inline FftSmem fft_smem(int L, int Np, int n_g, int ns = 2)
{
    int logL = 0;
    while ((1 << logL) < L) ++logL;
    const int warps = fft_threads(logL) / 32;
    FftSmem S;
    S.buf = 0;
    S.w = ((L + L / 16) * 8 + 15) & ~15;           // padded transform buffer; the normals start 16-byte aligned
    S.red = S.w + 2 * ns * (Np + 4) * 4;           // [2 paths][W1 | W1perp (| Wperp)][Np + 4]
    S.total = S.red + warps * n_g * 2 * ns * 4 + 64;
    return S;
}

// MC: plain Monte Carlo, a third normal stream (Wperp) and IsvdWp per path.
template <int LOGL, bool MC>
__global__ void __launch_bounds__(fft_threads(LOGL), fft_min_blocks(LOGL)) k_mixed_fft(const __grid_constant__ MixedArgs a)
{
    constexpr int T = fft_threads(LOGL), L = 1 << LOGL, WARPS = T / 32, NS = MC ? 3 : 2;
    extern __shared__ __align__(16) unsigned char smf[];
    const int N = a.N, Np = a.Np;
    const FftSmem S = fft_smem(L, Np, a.n_g, NS);
    float2* buf = (float2*)(smf + S.buf);
    float* ws = (float*)(smf + S.w);  // path q, stream s: ws + (NS q + s) * (Np + 4)
    float* red = (float*)(smf + S.red);
    const int W = Np + 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const PhiloxKeys& keys = *reinterpret_cast<const PhiloxKeys*>(a.pk);  // parameter space, no registers
    const int64_t npairs = (a.B + 1) / 2;
    const int ngrp = (N + 3) >> 2;

    for (int64_t pr = blockIdx.x; pr < npairs; pr += gridDim.x) {
        // 1. normals of both paths, both streams (Np + 1 entries: W1[N] pairs with the last column)
        // q = (pth NS + s) ngrp + g runs over the block with stride T; (g, s, pth)
        // are carried along instead of divided out
        int g = threadIdx.x, s = 0, pth = 0;
        while (g >= ngrp) {
            g -= ngrp;
            if (++s == NS) { s = 0; ++pth; }
        }
        while (pth < 2) {
            const int64_t m = 2 * pr + pth;
            float z[4] = {0.f, 0.f, 0.f, 0.f};
            if (m < a.B && a.ext) {
                // the caller's FP64 normals, quadrature layout [B][NS][N]
                const double* zz = a.ext + ((size_t)m * NS + s) * N + 4 * g;
#pragma unroll
                for (int e = 0; e < 4; ++e) z[e] = (4 * g + e < N) ? (float)zz[e] : 0.f;
            } else if (m < a.B) {
                const uint4 x = philox_group(keys, (uint64_t)(a.path0 + m), (uint32_t)g, (uint32_t)s);
                box_muller_f32(x.x, x.y, z[0], z[1]);
                box_muller_f32(x.z, x.w, z[2], z[3]);
            }
            // one 16-byte store (W and the row bases are multiples of 4 floats): four
            // scalar stores 16 bytes apart would each be 4-way bank conflicted
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (4 * g + e >= N) z[e] = 0.f;
            *(float4*)(ws + (NS * pth + s) * W + 4 * g) = make_float4(z[0], z[1], z[2], z[3]);
            g += T;
            while (g >= ngrp) {
                g -= ngrp;
                if (++s == NS) { s = 0; ++pth; }
            }
        }
        for (int n = N + threadIdx.x; n < W; n += T)  // tails of the rows read as zeros
#pragma unroll
            for (int r = 0; r < 2 * NS; ++r) ws[r * W + n] = 0.f;
        __syncthreads();
        // 2-3. forward FFT of z = W1_a + i W1_b (zero-padded to L) times the
        // spectrum (which includes 1/L), then the inverse FFT
        const FftIn in{ws, ws + NS * W, N};
        fft_inplace<LOGL, false, T>(buf, a.tw, in, a.spec);
        fft_inplace<LOGL, true, T>(buf, a.tw, in, a.spec);
        // 4. epilogue: thread-strided columns for both paths
        const float* w1a = ws;
        const float* w1pa = ws + W;
        const float* w1b = ws + NS * W;
        const float* w1pb = ws + (NS + 1) * W;
        const float* wqa = ws + 2 * W;         // plain Monte Carlo only
        const float* wqb = ws + (NS + 2) * W;
        for (int g = 0; g < a.n_g; ++g) {
            const float ah = a.alpha[g];
            const float* bt = a.beta + (size_t)g * Np;
            const int lim = a.nsteps[g] - 1;
            float sva = 0.f, swa = 0.f, svb = 0.f, swb = 0.f, sqa = 0.f, sqb = 0.f;
            for (int j = threadIdx.x; j < lim; j += T) {
                const float2 yj = buf[pidx(j)];
                const float bj = __ldg(bt + j);
                const float xa = yj.x + a.a1 * w1a[j] + a.a2 * w1pa[j];
                const float xb = yj.y + a.a1 * w1b[j] + a.a2 * w1pb[j];
                const float sua = ex2_approx(fmaf(ah, xa, -bj));
                const float sub = ex2_approx(fmaf(ah, xb, -bj));
                sva = fmaf(sua, sua, sva);
                swa = fmaf(sua, w1a[j + 1], swa);
                svb = fmaf(sub, sub, svb);
                swb = fmaf(sub, w1b[j + 1], swb);
                if (MC) {
                    sqa = fmaf(sua, wqa[j + 1], sqa);
                    sqb = fmaf(sub, wqb[j + 1], sqb);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sva += __shfl_xor_sync(0xffffffffu, sva, o);
                swa += __shfl_xor_sync(0xffffffffu, swa, o);
                svb += __shfl_xor_sync(0xffffffffu, svb, o);
                swb += __shfl_xor_sync(0xffffffffu, swb, o);
                if (MC) {
                    sqa += __shfl_xor_sync(0xffffffffu, sqa, o);
                    sqb += __shfl_xor_sync(0xffffffffu, sqb, o);
                }
            }
            if (lane == 0) {
                float* r = red + (warp * a.n_g + g) * 2 * NS;
                r[0] = sva; r[1] = swa; r[2] = svb; r[3] = swb;
                if (MC) { r[4] = sqa; r[5] = sqb; }
            }
        }
        if (a.dbg_x) {
            for (int j = threadIdx.x; j < Np; j += T) {
                const float2 yj = (j < N) ? buf[pidx(j)] : make_float2(0.f, 0.f);
                const int64_t ma = 2 * pr, mb = 2 * pr + 1;
                if (ma < a.B) a.dbg_x[ma * Np + j] = (j < N) ? yj.x + a.a1 * w1a[j] + a.a2 * w1pa[j] : 0.f;
                if (mb < a.B) a.dbg_x[mb * Np + j] = (j < N) ? yj.y + a.a1 * w1b[j] + a.a2 * w1pb[j] : 0.f;
            }
        }
        if (a.dbg_w) {
            for (int j = threadIdx.x; j < Np; j += T)
                for (int pth = 0; pth < 2; ++pth) {
                    const int64_t m = 2 * pr + pth;
                    if (m < a.B) {
                        a.dbg_w[(m * 2 + 0) * Np + j] = ws[(NS * pth) * W + j];
                        a.dbg_w[(m * 2 + 1) * Np + j] = ws[(NS * pth + 1) * W + j];
                    }
                }
        }
        __syncthreads();
        if (threadIdx.x < 2 * a.n_g) {
            const int g = threadIdx.x >> 1, pth = threadIdx.x & 1;
            float sv = 0.f, sw = 0.f, sq = 0.f;
            for (int k = 0; k < WARPS; ++k) {
                const float* r = red + (k * a.n_g + g) * 2 * NS;
                sv += r[2 * pth];
                sw += r[2 * pth + 1];
                if (MC) sq += r[4 + pth];
            }
            const int64_t m = 2 * pr + pth;
            if (m < a.B) {
                const float w10 = ws[(NS * pth) * W];
                const float Ivdt = a.dt[g] * (a.xi + sv);
                const float IsvdW = a.sdt[g] * fmaf(a.sqrt_xi, w10, sw);
                a.ivb[(size_t)(a.g0 + g) * a.B + m] = make_float2(Ivdt, IsvdW);
                if (MC) a.ivq[(size_t)(a.g0 + g) * a.B + m] = a.sdt[g] * fmaf(a.sqrt_xi, ws[(NS * pth + 2) * W], sq);
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

// L = 2^ceil(log2 2N), at least 16 so that every transform has a radix-16 pass
int fft_log2_len(int N)
{
    int logL = 4;
    while ((1 << logL) < 2 * N) ++logL;
    return logL;
}

size_t fft_smem_bytes(int N, int n_g, int ns)
{
    const int L = 1 << fft_log2_len(N);
    const int Np = (N + 31) / 32 * 32;
    return (size_t)fft_smem(L, Np, n_g, ns).total;
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

// The FP64 form's FFT convolution: spec[v] = FFT(Gamma_v zero-padded to L,
// Gamma_v[0] = 0, as the direct sum over k < j leaves it out) / L and the
// twiddles exp(-2 pi i q / L), complex doubles (re, im)
void fp64_fft_tables(const double* gamma, int n_vol, int N, int logL, double* spec, double* tw)
{
    const int L = 1 << logL;
    for (int v = 0; v < n_vol; ++v) {
        std::vector<std::complex<double>> x(L, 0.0);
        for (int n = 1; n < N; ++n) x[n] = gamma[(size_t)v * N + n];
        fft_host(x, false);
        for (int k = 0; k < L; ++k) {
            spec[((size_t)v * L + k) * 2] = x[k].real() / L;
            spec[((size_t)v * L + k) * 2 + 1] = x[k].imag() / L;
        }
    }
    const double pi = 3.14159265358979323846;
    for (int q = 0; q < L; ++q) {
        tw[2 * q] = std::cos(-2 * pi * q / L);
        tw[2 * q + 1] = std::sin(-2 * pi * q / L);
    }
}

template <int LOGL, bool MC>
static cudaError_t launch_fft_lm(const MixedArgs& A, int sms, cudaStream_t st)
{
    const int smem = fft_smem(1 << LOGL, A.Np, A.n_g, MC ? 3 : 2).total;
    cudaError_t e = cudaFuncSetAttribute(k_mixed_fft<LOGL, MC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed_fft<LOGL, MC>, fft_threads(LOGL), smem);
    if (per_sm < 1) per_sm = 1;
    const int64_t npairs = (A.B + 1) / 2;
    const int grid = (int)std::min<int64_t>(npairs, (int64_t)sms * per_sm);
    k_mixed_fft<LOGL, MC><<<grid, fft_threads(LOGL), smem, st>>>(A);
    return cudaGetLastError();
}

template <int LOGL>
static cudaError_t launch_fft_l(const MixedArgs& A, int sms, cudaStream_t st)
{
    return A.ivq ? launch_fft_lm<LOGL, true>(A, sms, st) : launch_fft_lm<LOGL, false>(A, sms, st);
}

cudaError_t launch_mixed_fft(const MixedArgs& A, int sms, cudaStream_t st)
{
    switch (A.logL) {
        case 4: return launch_fft_l<4>(A, sms, st);
        case 5: return launch_fft_l<5>(A, sms, st);
        case 6: return launch_fft_l<6>(A, sms, st);
        case 7: return launch_fft_l<7>(A, sms, st);
        case 8: return launch_fft_l<8>(A, sms, st);
        case 9: return launch_fft_l<9>(A, sms, st);
        case 10: return launch_fft_l<10>(A, sms, st);
        case 11: return launch_fft_l<11>(A, sms, st);
        case 12: return launch_fft_l<12>(A, sms, st);
        case 13: return launch_fft_l<13>(A, sms, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace rbg
