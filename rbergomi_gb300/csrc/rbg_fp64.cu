// rbg_fp64.cu -- the plain FP64 form of the RT pricer on the GPU.
//
// Kernels (one pass over a batch of paths):
//   k_normals      Philox4x32-10 -> FP64 normals, quadrature layout [B][2][N]
//   k_path_fp64    per path: Volterra sum Y2 = (W1 * Gamma)[0..N) as a direct
//                  causal FP64 sum, X = Y2 + a1 W1 + a2 W1perp, then for every
//                  variance group v, Ivdt = dt sum v, IsvdW = sum sqrt(v) sdt W1
//                  (rBergLib/rBergomiMT.cpp:73-109, 163-167, 427-436)
//   k_path_fp64_fft  the same pass with Y2 as an FP64 FFT convolution, two
//                  paths per complex transform (from 200 steps; the direct
//                  sum's N^2 / 2 DFMA per path outgrow it there)
//   k_payoff_sums  conditional BS per (path, output) and compensated per-chunk
//                  sums of x and x^2 (rBergomiMT.cpp:598-602, 404-409)
//   k_accumulate   fixed-order Neumaier merge of chunk sums (deterministic)
//   k_finalize     price, stat (reference formula), implied vol
//   k_payoff_store per-path payoffs for the quadrature entry point
// GB300's FP64 pipe (~2 DFMA/clk/SM) bounds every kernel here except the
// normal writer; this form exists for 1e-12 parity, not speed.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "rbg_device.cuh"
#include "rbg_internal.hpp"

namespace rbg {

// ------------------------------------------------------------------ normals
// FP64 Box-Muller by table-driven logarithm and sine/cosine (P. T. P. Tang's
// table method, ACM TOMS 15 (1989) and 16 (1990)): the same normals as
// sqrt(-2 ln u0) (cos, sin)(2 pi u1) on uniforms (x + 1/2) 2^-32 to a few
// 1e-16, with about 40 FP64 operations per pair instead of the library log
// and sincospi's 60-odd -- this kernel is bound by GB300's FP64 pipe.
//   ln u0: u0 = q 2^-33 with q = 2a + 1 odd; q = 2^e m, m in [1, 2), and
//     ln m = ln c_k + log1p((m - c_k) / c_k) at the nearest of 128 centres
//     c_k = 1 + (k + 1/2) / 128 (|t| <= 2^-8, Mercator series to t^7).  The top
//     interval, u0 >= 1 - 2^-8, takes log1p(u0 - 1) with u0 - 1 exact, so
//     sqrt(-2 ln u0) keeps its relative accuracy as u0 -> 1.
//   2 pi u1 = pi p 2^-32 with p = 2b + 1: the nearest table angle pi k / 128
//     plus |d| <= pi / 256, whose sine and cosine are Taylor series to d^7.
// The tables come from CUDA's own sincospi, division and log, once per device.
__device__ double2 g_bm_trig[256];  // (cos, sin)(pi k / 128)
__device__ double2 g_bm_logt[128];  // (1 / c_k, ln c_k)

__global__ void k_bm_tables()
{
    const int k = threadIdx.x;
    double sn, cs;
    sincospi(k / 128.0, &sn, &cs);
    g_bm_trig[k] = make_double2(cs, sn);
    if (k < 128) {
        const double c = 1.0 + (k + 0.5) / 128.0;
        g_bm_logt[k] = make_double2(1.0 / c, log(c));
    }
}

// log1p(t) for |t| <= 2^-8: t - t^2/2 + ... + t^7/7 (truncation below 2^-66)
__device__ __forceinline__ double log1p_small(double t)
{
    double p = 1.0 / 7;
    p = fma(p, t, -1.0 / 6);
    p = fma(p, t, 1.0 / 5);
    p = fma(p, t, -1.0 / 4);
    p = fma(p, t, 1.0 / 3);
    p = fma(p, t, -1.0 / 2);
    p = fma(p, t, 1.0);
    return p * t;
}

__device__ __forceinline__ void box_muller_f64_tab(uint32_t a, uint32_t b, double& z0, double& z1)
{
    // ln 2 split so that (e - 33) ln2_hi is exact for |e - 33| <= 33 (the fdlibm constants)
    constexpr double kLn2Hi = 6.93147180369123816490e-01, kLn2Lo = 1.90821492927058770002e-10;
    const uint64_t q = 2ull * a + 1ull;  // u0 = q 2^-33, q < 2^33
    double lnu;
    if (q >= 0x1FE000000ull) {
        lnu = log1p_small((double)(int64_t)(q - (1ull << 33)) * 0x1p-33);
    } else {
        const uint64_t bits = (uint64_t)__double_as_longlong((double)q);
        const int e = (int)(bits >> 52) - 1023;
        const int k = (int)(bits >> 45) & 127;
        const double m = __longlong_as_double((long long)((bits & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull));
        const double2 lc = g_bm_logt[k];
        const double t = (m - (1.0 + (k + 0.5) * 0.0078125)) * lc.x;
        const double ef = (double)(e - 33);
        lnu = fma(ef, kLn2Hi, lc.y + fma(ef, kLn2Lo, log1p_small(t)));
    }
    const double r = sqrt(-2.0 * lnu);
    const uint64_t p = 2ull * b + 1ull;  // 2 pi u1 = pi p 2^-32
    const uint64_t kk = (p + (1ull << 24)) >> 25;
    const double d = (double)(int64_t)(p - (kk << 25)) * (3.14159265358979323846 * 0x1p-32);
    const double d2 = d * d;
    const double sd = d * fma(fma(fma(-1.0 / 5040, d2, 1.0 / 120), d2, -1.0 / 6), d2, 1.0);
    const double cd = fma(fma(fma(-1.0 / 720, d2, 1.0 / 24), d2, -0.5), d2, 1.0);
    const double2 cs = g_bm_trig[kk & 255];
    z0 = r * fma(cs.x, cd, -cs.y * sd);
    z1 = r * fma(cs.y, cd, cs.x * sd);
}

// Z[m][s][j], s < ns: W1, W1perp and (plain MC) Wperp on Philox streams 0, 1, 2.
template <int F32>
__global__ void k_normals(uint64_t seed, int64_t path0, int64_t B, int N, int ns, double* __restrict__ Z)
{
    const int ng = (N + 3) >> 2;
    const int64_t total = B * ns * ng;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(t % ng);
        const int64_t r = t / ng;
        const int s = (int)(r % ns);
        const int64_t m = r / ns;
        const uint4 x = philox_group(seed, (uint64_t)(path0 + m), (uint32_t)g, (uint32_t)s);
        double z[4];
        if (F32) {
            float f0, f1, f2, f3;
            box_muller_f32(x.x, x.y, f0, f1);
            box_muller_f32(x.z, x.w, f2, f3);
            z[0] = f0; z[1] = f1; z[2] = f2; z[3] = f3;
        } else {
            box_muller_f64_tab(x.x, x.y, z[0], z[1]);
            box_muller_f64_tab(x.z, x.w, z[2], z[3]);
        }
        double* o = Z + (m * ns + s) * (int64_t)N + 4 * g;
        const int left = N - 4 * g;
        if (left >= 4) {
            o[0] = z[0]; o[1] = z[1]; o[2] = z[2]; o[3] = z[3];
        } else {
            for (int q = 0; q < left; ++q) o[q] = z[q];
        }
    }
}

void launch_normals(uint64_t seed, int64_t path0, int64_t B, int N, int f32, double* Z, void* stream, int ns)
{
    if (!f32) {
        // the Box-Muller tables, once per device (the stream is synchronised so that
        // launches on other streams find them written)
        static std::mutex mu;
        static bool ready[64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(mu);
        if (dev >= 0 && dev < 64 && !ready[dev]) {
            k_bm_tables<<<1, 256, 0, (cudaStream_t)stream>>>();
            count_launch();
            if (cudaStreamSynchronize((cudaStream_t)stream) == cudaSuccess) ready[dev] = true;
        }
    }
    const int64_t total = B * ns * ((N + 3) / 4);
    const int threads = 256;
    int64_t blocks = (total + threads - 1) / threads;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    if (f32) k_normals<1><<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(seed, path0, B, N, ns, Z);
    else k_normals<0><<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(seed, path0, B, N, ns, Z);
    count_launch();
}

// --------------------------------------------------------------- path pass
// One warp per path.  Shared memory: Gamma of the current pass (N doubles),
// then per warp W1 (N) and X (N).  NS = 3 (plain MC) also sums
// IsvdWp = sum sqrt(v) sdt Wperp into ivp.
// ANTI (control-variate form): also the antithetic path -W1, -W1perp.  The
// Volterra sum is linear, so its X is exactly -X; ivn[g][B] gets its
// (Ivdt, IsvdW).
template <int NS, bool ANTI>
__global__ void k_path_fp64(Fp64Tables t, const double* __restrict__ Z, int64_t B, double2* __restrict__ ivb,
                            double* __restrict__ ivp, double2* __restrict__ ivn)
{
    extern __shared__ double sm[];
    const int N = t.N;
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* G = sm;
    double* W1s = sm + N + (size_t)w * 2 * N;
    double* X = W1s + N;
    const int64_t m = (int64_t)blockIdx.x * warps + w;
    const bool active = m < B;
    const double* W1 = Z + m * NS * (int64_t)N;
    const double* W1p = W1 + N;
    const double* Wperp = W1 + 2 * N;  // NS = 3 only
    if (active)
        for (int j = lane; j < N; j += 32) W1s[j] = W1[j];

    for (int v = 0; v < t.n_vol; ++v) {
        __syncthreads();
        for (int j = threadIdx.x; j < N; j += blockDim.x) G[j] = t.gamma[(size_t)v * N + j];
        __syncthreads();
        if (!active) continue;
        const VolDev vol = t.vols[v];
        // Y2[j] = sum_{k<j} W1[k] Gamma[j-k]   (Gamma[0] = 0)
        for (int j = lane; j < N; j += 32) {
            double acc = 0.0;
            for (int k = 0; k < j; ++k) acc = fma(W1s[k], G[j - k], acc);
            X[j] = acc + (vol.a1 * W1s[j] + vol.a2 * W1p[j]);
        }
        __syncwarp();
        for (int g = vol.vg_begin; g < vol.vg_end; ++g) {
            const VGDev vg = t.vgs[g];
            const double* comp = t.comp + (size_t)g * N;
            double sv = 0.0, sw = 0.0, sp = 0.0, nv = 0.0, nw = 0.0;
            // sqrt(v_j) = sqrt(xi) exp(a_j / 2) and v_j = sqrt(v_j)^2: one exp, no sqrt per step
            const double sxi = sqrt(vg.xi);
            for (int j = lane; j < vg.nsteps; j += 32) {
                const double su = (j == 0) ? sxi : sxi * exp(0.5 * (vg.eta * (vg.scale * X[j - 1]) - comp[j - 1]));
                const double vj = (j == 0) ? vg.xi : su * su;
                sv += vj;
                const double sq = su * vg.sdt;
                sw += sq * W1s[j];
                if (NS == 3) sp += sq * Wperp[j];
                if (ANTI) {
                    const double sa = (j == 0) ? sxi : sxi * exp(0.5 * (vg.eta * (vg.scale * -X[j - 1]) - comp[j - 1]));
                    nv += (j == 0) ? vg.xi : sa * sa;
                    nw += sa * vg.sdt * -W1s[j];
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sv += __shfl_xor_sync(0xffffffffu, sv, o);
                sw += __shfl_xor_sync(0xffffffffu, sw, o);
                if (NS == 3) sp += __shfl_xor_sync(0xffffffffu, sp, o);
                if (ANTI) {
                    nv += __shfl_xor_sync(0xffffffffu, nv, o);
                    nw += __shfl_xor_sync(0xffffffffu, nw, o);
                }
            }
            if (lane == 0) {
                ivb[(size_t)g * B + m] = make_double2(vg.dt * sv, sw);
                if (NS == 3) ivp[(size_t)g * B + m] = sp;
                if (ANTI) ivn[(size_t)g * B + m] = make_double2(vg.dt * nv, nw);
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------ path pass, FFT
// The same pass with the Volterra sum as an FP64 FFT convolution: O(N log N)
// FP64 operations per path instead of N^2 / 2, so from a few hundred steps it
// does the FP64 pipe a fraction of the work.  The reference convolves the
// same way (fftOMP over FFTW, rBergLib/rBergomiMT.cpp:83-109); the results
// differ from the direct sum by roundoff.
//
// One CTA of 256 threads per pair of paths (a, b): z = W1_a + i W1_b,
// zero-padded to L = 2^logL >= 2N - 1, so the circular convolution with the
// real Gamma holds both linear ones, y = conv(z, Gamma) = Y2_a + i Y2_b.
// y = IFFT(FFT(z) FFT(Gamma)) = conj(FFT(conj(FFT(z) spec))) with
// spec = FFT(Gamma) / L, so one forward Stockham transform serves both
// directions.  FFT(z) is kept for every distinct H (pass v).
//
// Stockham autosort, radix 4 (one radix-2 pass first when logL is odd), in
// place: each thread loads its butterflies' inputs, the block synchronises,
// then each thread writes its outputs (the formulation of Govindaraju et al.,
// "High performance discrete Fourier transforms on graphics processors",
// SC'08: pass (R, Ns) reads x[j + r L / R], twiddles by exp(-2 pi i r (j mod
// Ns) / (Ns R)) and writes x[(j - j mod Ns) R + j mod Ns + r Ns]).
constexpr int kFftThreads = 256;
constexpr int kFp64FftMinLogL = 8;  // shorter transforms run at L = 256 (any L >= 2N - 1 holds the sums)

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// MAXB: butterflies per thread, L / R / 256 rounded up
template <int R, int MAXB>
__device__ __forceinline__ void stockham_pass(double2* x, int L, int Ns, const double2* __restrict__ tw)
{
    const int nb = L / R;
    const int tstep = L / (Ns * R);
    double2 v[MAXB][R];
#pragma unroll
    for (int b = 0; b < MAXB; ++b) {
        const int j = threadIdx.x + b * kFftThreads;
        if (j < nb) {
            const int k = j & (Ns - 1);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double2 a = x[j + r * nb];
                v[b][r] = (r == 0 || k == 0) ? a : cmul(a, __ldg(tw + r * k * tstep));
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < MAXB; ++b) {
        const int j = threadIdx.x + b * kFftThreads;
        if (j < nb) {
            const int k = j & (Ns - 1);
            const int d = (j - k) * R + k;
            if (R == 2) {
                const double2 a = v[b][0], c = v[b][1];
                x[d] = make_double2(a.x + c.x, a.y + c.y);
                x[d + Ns] = make_double2(a.x - c.x, a.y - c.y);
            } else {
                // X0 = a + b + c + e, X1 = a - i b - c + i e, X2 = a - b + c - e, X3 = a + i b - c - i e
                const double2 a = v[b][0], bb = v[b][1], c = v[b][2], e = v[b][3];
                const double2 s0 = make_double2(a.x + c.x, a.y + c.y), d0 = make_double2(a.x - c.x, a.y - c.y);
                const double2 s1 = make_double2(bb.x + e.x, bb.y + e.y), d1 = make_double2(bb.x - e.x, bb.y - e.y);
                x[d] = make_double2(s0.x + s1.x, s0.y + s1.y);
                x[d + Ns] = make_double2(d0.x + d1.y, d0.y - d1.x);       // d0 - i d1
                x[d + 2 * Ns] = make_double2(s0.x - s1.x, s0.y - s1.y);
                x[d + 3 * Ns] = make_double2(d0.x - d1.y, d0.y + d1.x);   // d0 + i d1
            }
        }
    }
    __syncthreads();
}

// forward DFT of x (L = 2^LOGL) in natural order
template <int LOGL>
__device__ __forceinline__ void fft_forward(double2* x, const double2* __restrict__ tw)
{
    constexpr int L = 1 << LOGL;
    constexpr int B2 = (L / 2 + kFftThreads - 1) / kFftThreads, B4 = (L / 4 + kFftThreads - 1) / kFftThreads;
    int Ns = 1;
    if (LOGL & 1) {
        stockham_pass<2, B2>(x, L, Ns, tw);
        Ns = 2;
    }
#pragma unroll 1
    for (; Ns < L; Ns *= 4) stockham_pass<4, B4>(x, L, Ns, tw);
}

// block sum over the 128 threads of one path half (threads 0..127 or 128..255)
__device__ __forceinline__ double half_sum(double s, double* red, int slot)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red[slot * 8 + w] = s;
    __syncthreads();
    const int w0 = (threadIdx.x >> 7) * 4;
    const double r = (red[slot * 8 + w0] + red[slot * 8 + w0 + 1]) + (red[slot * 8 + w0 + 2] + red[slot * 8 + w0 + 3]);
    return r;
}

template <int LOGL, int NS, bool ANTI>
__global__ void __launch_bounds__(kFftThreads) k_path_fp64_fft(Fp64Tables t, const double* __restrict__ Z, int64_t B,
                                                              double2* __restrict__ ivb, double* __restrict__ ivp,
                                                              double2* __restrict__ ivn)
{
    extern __shared__ double2 fsm[];
    constexpr int L = 1 << LOGL;
    const int N = t.N;
    double2* zf = fsm;      // FFT(z), kept across passes v
    double2* y = fsm + L;   // work buffer
    double* red = (double*)(fsm + 2 * L);  // [5 sums][8 warps]
    const int64_t ma = 2 * (int64_t)blockIdx.x, mb = ma + 1;
    const bool has_b = mb < B;
    const double* Wa = Z + ma * NS * (int64_t)N;
    const double* Wb = Z + mb * NS * (int64_t)N;
    for (int k = threadIdx.x; k < L; k += kFftThreads)
        zf[k] = k < N ? make_double2(Wa[k], has_b ? Wb[k] : 0.0) : make_double2(0.0, 0.0);
    __syncthreads();
    fft_forward<LOGL>(zf, t.tw);
    // this thread's path and steps in the variance loops
    const int half = threadIdx.x >> 7, jt = threadIdx.x & 127;
    const int64_t m = half ? mb : ma;
    const bool active = half ? has_b : true;
    const double* W1 = Z + m * NS * (int64_t)N;  // valid only when active
    for (int v = 0; v < t.n_vol; ++v) {
        const double2* sp = t.spec + (size_t)v * L;
        for (int k = threadIdx.x; k < L; k += kFftThreads) {
            const double2 u = cmul(zf[k], __ldg(sp + k));
            y[k] = make_double2(u.x, -u.y);
        }
        __syncthreads();
        fft_forward<LOGL>(y, t.tw);
        // X = Y2 + a1 W1 + a2 W1perp: Y2_a = Re y = Re FFT(w), Y2_b = Im y = -Im FFT(w)
        const VolDev vol = t.vols[v];
        for (int j = threadIdx.x; j < N; j += kFftThreads) {
            const double2 q = y[j];
            const double xa = q.x + (vol.a1 * Wa[j] + vol.a2 * Wa[N + j]);
            const double xb = has_b ? -q.y + (vol.a1 * Wb[j] + vol.a2 * Wb[N + j]) : 0.0;
            y[j] = make_double2(xa, xb);
        }
        __syncthreads();
        for (int g = vol.vg_begin; g < vol.vg_end; ++g) {
            const VGDev vg = t.vgs[g];
            const double* comp = t.comp + (size_t)g * N;
            double sv = 0.0, sw = 0.0, sp2 = 0.0, nv = 0.0, nw = 0.0;
            if (active) {
                const double sxi = sqrt(vg.xi);
                for (int j = jt; j < vg.nsteps; j += 128) {
                    const double xp = (j == 0) ? 0.0 : (half ? y[j - 1].y : y[j - 1].x);
                    const double su = (j == 0) ? sxi : sxi * exp(0.5 * (vg.eta * (vg.scale * xp) - comp[j - 1]));
                    const double vj = (j == 0) ? vg.xi : su * su;
                    sv += vj;
                    const double sq = su * vg.sdt;
                    sw += sq * W1[j];
                    if (NS == 3) sp2 += sq * W1[2 * N + j];
                    if (ANTI) {
                        const double sa = (j == 0) ? sxi : sxi * exp(0.5 * (vg.eta * (vg.scale * -xp) - comp[j - 1]));
                        nv += (j == 0) ? vg.xi : sa * sa;
                        nw += sa * vg.sdt * -W1[j];
                    }
                }
            }
            sv = half_sum(sv, red, 0);
            sw = half_sum(sw, red, 1);
            if (NS == 3) sp2 = half_sum(sp2, red, 2);
            if (ANTI) {
                nv = half_sum(nv, red, 3);
                nw = half_sum(nw, red, 4);
            }
            if (jt == 0 && active) {
                ivb[(size_t)g * B + m] = make_double2(vg.dt * sv, sw);
                if (NS == 3) ivp[(size_t)g * B + m] = sp2;
                if (ANTI) ivn[(size_t)g * B + m] = make_double2(vg.dt * nv, nw);
            }
            __syncthreads();  // red is reused by the next group
        }
    }
}

size_t path_fp64_fft_smem(int logL) { return (size_t)2 * (16u << logL) + 5 * 8 * sizeof(double); }

int fp64_fft_log2_len(int N)
{
    int logL = kFp64FftMinLogL;
    while ((1 << logL) < 2 * N - 1) ++logL;
    return (N >= 2 && logL <= kFp64FftMaxLogL) ? logL : 0;
}

template <int LOGL>
static void launch_fp64_fft(const Fp64Tables& t, const double* Z, int64_t B, double* ivb, cudaStream_t st,
                            double* ivp, double* ivn)
{
    const size_t smem = path_fp64_fft_smem(LOGL);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_path_fp64_fft<LOGL, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_path_fp64_fft<LOGL, 3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_path_fp64_fft<LOGL, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    const unsigned pairs = (unsigned)((B + 1) / 2);
    if (ivn)
        k_path_fp64_fft<LOGL, 2, true><<<pairs, kFftThreads, smem, st>>>(t, Z, B, (double2*)ivb, nullptr,
                                                                         (double2*)ivn);
    else if (ivp)
        k_path_fp64_fft<LOGL, 3, false><<<pairs, kFftThreads, smem, st>>>(t, Z, B, (double2*)ivb, ivp, nullptr);
    else
        k_path_fp64_fft<LOGL, 2, false><<<pairs, kFftThreads, smem, st>>>(t, Z, B, (double2*)ivb, nullptr, nullptr);
}

int path_fp64_warps(int N)
{
    const size_t budget = 200 * 1024;
    size_t per = 16 * (size_t)N;
    size_t w = (budget - 8 * (size_t)N) / per;
    if (w > 8) w = 8;
    if (w < 1) w = 1;
    return (int)w;
}

size_t path_fp64_smem(int N, int warps) { return 8 * (size_t)N + (size_t)warps * 16 * N; }

void launch_path_fp64(const Fp64Tables& t, const double* Z, int64_t B, double* ivb, void* stream, double* ivp,
                      double* ivn)
{
    const int warps = path_fp64_warps(t.N);
    const size_t smem = path_fp64_smem(t.N, warps);
    static size_t configured = 0;
    if (smem > configured) {
        cudaFuncSetAttribute(k_path_fp64<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_path_fp64<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_path_fp64<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (t.logL > 0) {
        switch (t.logL) {
        case 8: launch_fp64_fft<8>(t, Z, B, ivb, st, ivp, ivn); break;
        case 9: launch_fp64_fft<9>(t, Z, B, ivb, st, ivp, ivn); break;
        case 10: launch_fp64_fft<10>(t, Z, B, ivb, st, ivp, ivn); break;
        case 11: launch_fp64_fft<11>(t, Z, B, ivb, st, ivp, ivn); break;
        default: launch_fp64_fft<12>(t, Z, B, ivb, st, ivp, ivn); break;
        }
        count_launch();
        return;
    }
    const int64_t blocks = (B + warps - 1) / warps;
    if (ivn)
        k_path_fp64<2, true><<<(unsigned)blocks, warps * 32, smem, st>>>(t, Z, B, (double2*)ivb, nullptr,
                                                                         (double2*)ivn);
    else if (ivp)
        k_path_fp64<3, false><<<(unsigned)blocks, warps * 32, smem, st>>>(t, Z, B, (double2*)ivb, ivp, nullptr);
    else
        k_path_fp64<2, false><<<(unsigned)blocks, warps * 32, smem, st>>>(t, Z, B, (double2*)ivb, nullptr, nullptr);
    count_launch();
}

// ------------------------------------------------------------ payoff sums
constexpr int kOPB = 8;  // outputs per block

// grid (nchunks, ceil(n_out / kOPB)), 256 threads; chunk c covers paths
// [c G 256, (c+1) G 256) of the batch; part[(c * n_out + i) * 4 + {0,1,2,3}] =
// (sum, comp, sum2, comp2).
// MC = 1: plain Monte Carlo payoff from (Ivdt, IsvdW) and ivp = IsvdWp.
template <int MC>
__global__ void __launch_bounds__(256) k_payoff_sums(Fp64Tables t, const double2* __restrict__ ivb, int64_t B,
                                                     int64_t stride, int G, double* __restrict__ part,
                                                     const double* __restrict__ ivp)
{
    __shared__ double red[8][kOPB][2];
    const int c = blockIdx.x;
    const int o0 = blockIdx.y * kOPB;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double S = 0, CS = 0, S2 = 0, CS2 = 0;  // meaningful in threads q < kOPB
    OutDev od[kOPB];
#pragma unroll
    for (int q = 0; q < kOPB; ++q) {
        const int i = o0 + q;
        od[q] = (i < t.n_out) ? t.outs[i] : OutDev{0.0, 1.0, -1, 0};
    }
    for (int sub = 0; sub < G; ++sub) {
        const int64_t m = ((int64_t)c * G + sub) * 256 + threadIdx.x;
#pragma unroll
        for (int q = 0; q < kOPB; ++q) {
            double x = 0.0;
            if (m < B && od[q].vg >= 0) {
                const size_t at = (size_t)od[q].vg * stride + m;
                const double2 iv = ivb[at];
                x = MC ? mc_payoff(iv.x, iv.y, ivp[at], od[q].rho, od[q].K) : rt_payoff(iv.x, iv.y, od[q].rho, od[q].K);
            }
            double x2 = x * x;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(0xffffffffu, x, o);
                x2 += __shfl_xor_sync(0xffffffffu, x2, o);
            }
            if (lane == 0) { red[w][q][0] = x; red[w][q][1] = x2; }
        }
        __syncthreads();
        if (threadIdx.x < kOPB) {
            const int q = threadIdx.x;
            double a = 0, a2 = 0;
            for (int k = 0; k < 8; ++k) { a += red[k][q][0]; a2 += red[k][q][1]; }
            neumaier_add(S, CS, a);
            neumaier_add(S2, CS2, a2);
        }
        __syncthreads();
    }
    if (threadIdx.x < kOPB && o0 + (int)threadIdx.x < t.n_out) {
        double* p = part + ((size_t)c * t.n_out + o0 + threadIdx.x) * 4;
        p[0] = S; p[1] = CS; p[2] = S2; p[3] = CS2;
    }
}

void launch_payoff_sums(const Fp64Tables& t, const double* ivb, int64_t B, int64_t stride, int G, double* part,
                        int nchunks, void* stream, const double* ivp)
{
    dim3 grid(nchunks, (t.n_out + kOPB - 1) / kOPB);
    if (ivp)
        k_payoff_sums<1><<<grid, 256, 0, (cudaStream_t)stream>>>(t, (const double2*)ivb, B, stride, G, part, ivp);
    else
        k_payoff_sums<0><<<grid, 256, 0, (cudaStream_t)stream>>>(t, (const double2*)ivb, B, stride, G, part, ivp);
    count_launch();
}

// acc[i * 4 + {0..3}] += the batch's chunk sums.  One block per output:
// strided Neumaier sums per thread, then a fixed-shape tree, so the result
// does not depend on scheduling.
// Output i of a fixed-order merge of chunk sums into acc (fresh: acc holds
// zeros, read as such -- the job-table launches skip the clearing memset).
// Shared by the per-request and job-table kernels.
__device__ __forceinline__ void accumulate_block(const double* __restrict__ part, int nchunks, int n_out,
                                                 double* __restrict__ acc, int i, bool fresh, double (*sh)[256])
{
    double S = 0, C = 0, S2 = 0, C2 = 0;
    for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
        const double* p = part + ((size_t)c * n_out + i) * 4;
        neumaier_add(S, C, p[0]);
        neumaier_add(S, C, p[1]);
        neumaier_add(S2, C2, p[2]);
        neumaier_add(S2, C2, p[3]);
    }
    sh[0][threadIdx.x] = S; sh[1][threadIdx.x] = C; sh[2][threadIdx.x] = S2; sh[3][threadIdx.x] = C2;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            const int j = threadIdx.x + h;
            double a = sh[0][threadIdx.x], ac = sh[1][threadIdx.x];
            neumaier_add(a, ac, sh[0][j]);
            neumaier_add(a, ac, sh[1][j]);
            double b = sh[2][threadIdx.x], bc = sh[3][threadIdx.x];
            neumaier_add(b, bc, sh[2][j]);
            neumaier_add(b, bc, sh[3][j]);
            sh[0][threadIdx.x] = a; sh[1][threadIdx.x] = ac; sh[2][threadIdx.x] = b; sh[3][threadIdx.x] = bc;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double a = 0, ac = 0, b = 0, bc = 0;
        if (!fresh) { a = acc[i * 4 + 0]; ac = acc[i * 4 + 1]; b = acc[i * 4 + 2]; bc = acc[i * 4 + 3]; }
        neumaier_add(a, ac, sh[0][0]);
        neumaier_add(a, ac, sh[1][0]);
        neumaier_add(b, bc, sh[2][0]);
        neumaier_add(b, bc, sh[3][0]);
        acc[i * 4 + 0] = a; acc[i * 4 + 1] = ac; acc[i * 4 + 2] = b; acc[i * 4 + 3] = bc;
    }
}

__global__ void __launch_bounds__(256) k_accumulate(const double* __restrict__ part, int nchunks, int n_out,
                                                    double* __restrict__ acc)
{
    __shared__ double sh[4][256];
    accumulate_block(part, nchunks, n_out, acc, blockIdx.x, false, sh);
}

// Job-table form: block b merges output b - jobs[k].block0 of job k.
__global__ void __launch_bounds__(256) k_accumulate_jobs(const AccJob* __restrict__ jobs, int n_jobs)
{
    __shared__ double sh[4][256];
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].block0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const AccJob& J = jobs[lo];
    accumulate_block(J.part, J.nchunks, J.n_out, J.acc, (int)((int64_t)blockIdx.x - J.block0), true, sh);
}

void launch_accumulate_jobs(const AccJob* jobs, int n_jobs, int64_t blocks, void* stream)
{
    k_accumulate_jobs<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(jobs, n_jobs);
    count_launch();
}

void launch_accumulate(const double* part, int nchunks, int n_out, double* acc, void* stream)
{
    k_accumulate<<<n_out, 256, 0, (cudaStream_t)stream>>>(part, nchunks, n_out, acc);
    count_launch();
}

// ------------------------------------------------------------- IV (FP64)
__device__ double bs_gen(double K, double T, double s, int put)
{
    const double sq = sqrt(T);
    const double d1 = (log(1.0 / K) + 0.5 * s * s * T) / (s * sq);
    const double d2 = d1 - s * sq;
    return put ? (-phi_cdf(-d1) + phi_cdf(-d2) * K) : (phi_cdf(d1) - phi_cdf(d2) * K);
}

// The out-of-the-money Black-Scholes price in FP32 (S0 = 1, r = 0): the
// bracketing rounds of implied_vol_warp.  lnK1 = ln(1 / K), sqT = sqrt(T).
__device__ __forceinline__ float bs_gen_f32(float lnK1, float sqT, float K, float s, int put)
{
    const float ssq = s * sqT;
    const float d1 = fmaf(0.5f, ssq, lnK1 * rcp_approx(ssq));
    const float d2 = d1 - ssq;
    return put ? fmaf(K, phi_f32(-d2), -phi_f32(-d1)) : fmaf(-K, phi_f32(d2), phi_f32(d1));
}

// Implied vol by a warp: inverts on the out-of-the-money side (put-call
// parity for K < 1, as rBergLib/BlackScholes.cpp:38-41 does).  The 32 lanes
// price 32 volatilities at once:
//   1. a geometric grid 1e-3 * 2^(l/2) brackets the root within a factor
//      sqrt(2), in FP32; where the FP32 grid brackets nothing, the same grid in
//      FP64 decides (no bracket there: no volatility fits, NaN);
//   2. three 33-section rounds in FP32 narrow the bracket ~36,000-fold (FP32
//      resolves it no further);
//   3. one FP64 step checks the narrowed bracket (lanes 0 and 1 price its
//      ends, widened by 1e-6) while lane 2 prices its middle; if the check
//      fails -- FP32 cannot resolve the price, e.g. far in a wing -- the FP64
//      grid and FP64 33-section rounds (to 1e-6) take over;
//   4. from the checked bracket's middle one Halley step on the log price
//      (cubic: from a 1e-5 bracket the error left is 1e-15 near the money,
//      below ~1e-12 in the wings), then safeguarded Newton on the
//      log price where a step is still larger than that.
// The search is a chain of serial FP64 evaluations on GB300's slow FP64 pipe,
// so fewer of them is what makes it fast: two on the common path.  All lanes
// return the same value; NaN when no volatility fits.
__device__ double implied_vol_warp(double price, double K, double T)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int put = 1.0 > K;
    const double target = put ? price - 1.0 + K : price;
    const double upper = put ? K : 1.0;
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    if (!(target > 0.0) || !(target < upper) || !(T > 0.0)) return nan;
    const float lnK1 = (float)log(1.0 / K), sqT32 = (float)sqrt(T), K32 = (float)K, t32 = (float)target;
    double lo = 0.0, hi = 0.0;
    bool narrowed = false;
    double s = 0.0, p0 = 0.0;
    {
        // FP32 grid and rounds, then the FP64 check
        const unsigned b32 = __ballot_sync(FULL, bs_gen_f32(lnK1, sqT32, K32, 1e-3f * exp2f(0.5f * lane), put) >= t32);
        if (b32 != 0u) {
            const int f = __ffs(b32) - 1;
            const double glo = (f > 0) ? 1e-3 * exp2(0.5 * (f - 1)) : 0.0, ghi = 1e-3 * exp2(0.5 * f);
            float lo32 = (float)glo, hi32 = (float)ghi;
#pragma unroll 1
            for (int it = 0; it < 3; ++it) {
                const float sl = fmaf(hi32 - lo32, (float)(lane + 1) * (1.0f / 33.0f), lo32);
                const unsigned bb = __ballot_sync(FULL, bs_gen_f32(lnK1, sqT32, K32, sl, put) >= t32);
                const int ff = bb ? __ffs(bb) - 1 : 32;
                const float nlo = __shfl_sync(FULL, sl, ff > 0 ? ff - 1 : 0);
                const float nhi = __shfl_sync(FULL, sl, ff < 32 ? ff : 31);
                if (ff > 0) lo32 = nlo;
                if (ff < 32) hi32 = nhi;
            }
            const double lo2 = fmax(glo, (double)lo32 * (1.0 - 1e-6)), hi2 = fmin(ghi, (double)hi32 * (1.0 + 1e-6));
            const double sv = lane == 0 ? lo2 : (lane == 1 ? hi2 : 0.5 * (lo2 + hi2));
            const double pv = (sv > 0.0) ? bs_gen(K, T, sv, put) : 0.0;  // zero volatility: the OTM price is 0
            const double plo = __shfl_sync(FULL, pv, 0), phi_ = __shfl_sync(FULL, pv, 1);
            const double pmid = __shfl_sync(FULL, pv, 2);
            if (lo2 < hi2 && plo < target && phi_ >= target) {
                narrowed = true;
                lo = lo2;
                hi = hi2;
                s = 0.5 * (lo2 + hi2);
                p0 = pmid;
            }
        }
    }
    if (!narrowed) {
        // FP64 grid, then FP64 33-section rounds (one evaluation per lane)
        // until the bracket is within 1e-6 relative
        const double sig = 1e-3 * exp2(0.5 * lane);
        unsigned b = __ballot_sync(FULL, bs_gen(K, T, sig, put) >= target);
        if (b == 0u) return nan;
        int f = __ffs(b) - 1;
        lo = (f > 0) ? 1e-3 * exp2(0.5 * (f - 1)) : 0.0;
        hi = 1e-3 * exp2(0.5 * f);
        for (int it = 0; it < 14 && hi - lo > 1e-6 * hi; ++it) {
            const double sl = lo + (hi - lo) * (double)(lane + 1) / 33.0;
            b = __ballot_sync(FULL, bs_gen(K, T, sl, put) >= target);
            f = b ? __ffs(b) - 1 : 32;
            const double nlo = __shfl_sync(FULL, sl, f > 0 ? f - 1 : 0);
            const double nhi = __shfl_sync(FULL, sl, f < 32 ? f : 31);
            if (f > 0) lo = nlo;
            if (f < 32) hi = nhi;
        }
        s = 0.5 * (lo + hi);
    }
    const double lt = log(target), sqT = sqrt(T);
    if (narrowed && p0 > 0.0) {
        // Halley on g(s) = log p(s) - log target: g' = vega / p and
        // g'' = (vomma p - vega^2) / p^2 with vomma = vega d1 d2 / s
        const double d1 = (log(1.0 / K) + 0.5 * s * s * T) / (s * sqT);
        const double d2 = d1 - s * sqT;
        const double vega = exp(-0.5 * d1 * d1) * 0.39894228040143267794 * sqT;
        const double g = log(p0) - lt, g1 = vega / p0, g2 = (vega * d1 * d2 / s) / p0 - g1 * g1;
        const double nt = s - 2.0 * g * g1 / (2.0 * g1 * g1 - g * g2);
        if (nt > lo && nt < hi) {
            if (fabs(nt - s) <= 1e-5 * s) return nt;  // cubic: the error left is below ~1e-12 relative
            s = nt;
        }
        if (p0 > target) hi = 0.5 * (lo + hi);
        else lo = 0.5 * (lo + hi);
        if (!(s > lo && s < hi)) s = 0.5 * (lo + hi);
    }
    // safeguarded Newton on the log price (every lane computes the same
    // iterate).  A Newton step below 1e-14 relative ends the search: the
    // convergence is quadratic, so the iterate it gives is at roundoff.  A
    // step that leaves the bracket, or a vanishing price, falls back to
    // bisection; 40 halvings take a 1e-6 bracket below 1e-15 on their own.
    for (int it = 0; it < 40; ++it) {
        const double p = bs_gen(K, T, s, put);
        if (p == target) break;
        if (p > target) hi = s;
        else lo = s;
        double sn = 0.5 * (lo + hi);
        if (p > 0.0) {
            const double d1 = (log(1.0 / K) + 0.5 * s * s * T) / (s * sqT);
            const double vega = exp(-0.5 * d1 * d1) * 0.39894228040143267794 * sqT;
            const double nt = s - (log(p) - lt) * p / vega;
            if (fabs(nt - s) <= 1e-14 * s) {
                s = nt;
                break;
            }
            if (nt > lo && nt < hi) sn = nt;
        }
        s = sn;
        if (hi - lo <= 1e-15 * hi) break;
    }
    return s;
}

// res: [0,n) price, [n,2n) stat, [2n,3n) iv, [3n,4n) sum, [4n,5n) sum2.
// One warp per output.
// Output i (one warp) of the price / stat / implied vol; shared by the
// per-request and job-table kernels.
__device__ __forceinline__ void finalize_warp(const double* __restrict__ acc, int n_out, int64_t M,
                                              const OutDev* __restrict__ outs, const double* __restrict__ Tv,
                                              int compute_iv, double* __restrict__ res, int i)
{
    const double S = acc[i * 4 + 0] + acc[i * 4 + 1];
    const double S2 = acc[i * 4 + 2] + acc[i * 4 + 3];
    // rBergLib/rBergomiMT.cpp:404-409
    const double price = S * (1.0 / (double)M);
    const double var = 1.0 * (S2 * (1.0 / (double)M)) + -1.0 * (price * price);
    const double stat = sqrt(var) * (1.0 / sqrt((double)M));
    const double iv = compute_iv ? implied_vol_warp(price, outs[i].K, Tv[i]) : 0.0;
    if ((threadIdx.x & 31) == 0) {
        res[i] = price;
        res[n_out + i] = stat;
        res[2 * n_out + i] = iv;
        res[3 * n_out + i] = S;
        res[4 * n_out + i] = S2;
    }
}

__global__ void k_finalize(const double* __restrict__ acc, int n_out, int64_t M, const OutDev* __restrict__ outs,
                           const double* __restrict__ Tv, int compute_iv, double* __restrict__ res)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n_out) return;  // whole warps leave together
    finalize_warp(acc, n_out, M, outs, Tv, compute_iv, res, i);
}

// Job-table form: one warp (block) per output, block b finalizes output
// b - jobs[k].block0 of job k.
__global__ void k_finalize_jobs(const FinJob* __restrict__ jobs, int n_jobs)
{
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].block0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const FinJob& J = jobs[lo];
    finalize_warp(J.acc, J.n_out, J.M, J.outs, J.Tv, J.compute_iv, J.res, (int)((int64_t)blockIdx.x - J.block0));
}

void launch_finalize_jobs(const FinJob* jobs, int n_jobs, int64_t blocks, void* stream)
{
    k_finalize_jobs<<<(unsigned)blocks, 32, 0, (cudaStream_t)stream>>>(jobs, n_jobs);
    count_launch();
}

void reduce_preload()
{
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, k_accumulate);
    cudaFuncGetAttributes(&fa, k_accumulate_jobs);
    cudaFuncGetAttributes(&fa, k_finalize);
    cudaFuncGetAttributes(&fa, k_finalize_jobs);
    cudaGetLastError();
}

void launch_finalize(const double* acc, int n_out, int64_t M, const OutDev* outs, const double* Tvals,
                     int compute_iv, double* res, void* stream)
{
    // one output (one warp) per block: the implied-vol search is FP64-bound,
    // and GB300's FP64 pipe is per SM, so the outputs spread over the SMs
    const int threads = 32;
    const int blocks = (int)(((int64_t)n_out * 32 + threads - 1) / threads);
    k_finalize<<<blocks, threads, 0, (cudaStream_t)stream>>>(acc, n_out, M, outs, Tvals, compute_iv, res);
    count_launch();
}

__global__ void k_implied_vol(int n, const double* price, const double* K, const double* T, double* iv)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    const double v = implied_vol_warp(price[i], K[i], T[i]);
    if ((threadIdx.x & 31) == 0) iv[i] = v;
}

void launch_implied_vol(int n, const double* price, const double* K, const double* T, double* iv, void* stream)
{
    k_implied_vol<<<n, 32, 0, (cudaStream_t)stream>>>(n, price, K, T, iv);  // one warp (output) per block
    count_launch();
}

// ------------------------------------------------------------ quadrature
template <int MC>
__global__ void k_payoff_store(Fp64Tables t, const double2* __restrict__ ivb, int64_t B, int64_t stride,
                               double* __restrict__ payoff, const double* __restrict__ ivp)
{
    const int64_t total = B * t.n_out;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = idx / t.n_out;
        const int i = (int)(idx - m * t.n_out);
        const OutDev od = t.outs[i];
        const size_t at = (size_t)od.vg * stride + m;
        const double2 iv = ivb[at];
        payoff[idx] = MC ? mc_payoff(iv.x, iv.y, ivp[at], od.rho, od.K) : rt_payoff(iv.x, iv.y, od.rho, od.K);
    }
}

void launch_payoff_store(const Fp64Tables& t, const double* ivb, int64_t B, int64_t stride, double* payoff,
                         void* stream, const double* ivp)
{
    const int64_t total = B * t.n_out;
    int64_t blocks = (total + 255) / 256;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    if (ivp)
        k_payoff_store<1><<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(t, (const double2*)ivb, B, stride,
                                                                             payoff, ivp);
    else
        k_payoff_store<0><<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(t, (const double2*)ivb, B, stride,
                                                                             payoff, ivp);
    count_launch();
}

// ------------------------------------------------------- control variate
// The Romano-Touzi estimator with the control variate of McCrickerd and
// Pakkanen and antithetic paths, as ML_console_ST/RBergomi.cpp implements it
// (estimateControlVariate :493-540, ComputePriceRTVarRed :218-289,
// updatePayoffControlVariate :478-491).
//   X = BS(S, K, 1, sqrt((1 - rho^2) Ivdt)),  S = exp(-rho^2 Ivdt / 2 + rho IsvdW)
//   Y = BS(S, K, 1, sqrt(rho^2 (Q - Ivdt)))   (Qmax in place of Q where Q <= Ivdt)

// Fixed-shape block sum (256 threads): the same order on every run.
__device__ double block_sum_256(double x, double* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < 8; ++k) t += red[k];
    return t;
}

// One block of 256 threads per output: Q = max_m 2 Ivdt_m; X_m, Y_m on the
// pilot paths (stored in xy); means; centred covariance sums (two passes, as
// aux.h:206-220 computes them); alpha = -cov(X, Y) / cov(Y, Y).
__global__ void __launch_bounds__(256) k_cv_pilot(Fp64Tables t, const double2* __restrict__ ivb, int64_t Mc,
                                                  double* __restrict__ xy, double* __restrict__ alpha,
                                                  double* __restrict__ Qout)
{
    __shared__ double red[8];
    const int i = blockIdx.x;
    const OutDev od = t.outs[i];
    const double2* iv = ivb + (size_t)od.vg * Mc;
    double* X = xy + (size_t)i * 2 * Mc;
    double* Y = X + Mc;
    double q = 0.0;
    for (int64_t m = threadIdx.x; m < Mc; m += 256) q = fmax(q, 2 * iv[m].x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) q = fmax(q, __shfl_xor_sync(0xffffffffu, q, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = q;
    __syncthreads();
    q = 0.0;
    for (int k = 0; k < 8; ++k) q = fmax(q, red[k]);
    const double r = od.rho;
    double sx = 0.0, sy = 0.0;
    for (int64_t m = threadIdx.x; m < Mc; m += 256) {
        const double a = iv[m].x, b = iv[m].y;
        const double spot = exp(-0.5 * r * r * a + r * b);
        X[m] = bs_call_tau1(spot, od.K, sqrt((1.0 - r * r) * a));
        Y[m] = bs_call_tau1(spot, od.K, sqrt(r * r * (q - a)));
        sx += X[m];
        sy += Y[m];
    }
    const double mx = block_sum_256(sx, red) / (double)Mc;
    const double my = block_sum_256(sy, red) / (double)Mc;
    double cxy = 0.0, cyy = 0.0;
    for (int64_t m = threadIdx.x; m < Mc; m += 256) {
        const double dy = Y[m] - my;
        cxy += (X[m] - mx) * dy;
        cyy += dy * dy;
    }
    cxy = block_sum_256(cxy, red);
    cyy = block_sum_256(cyy, red);
    if (threadIdx.x == 0) {
        alpha[i] = -(cxy / (double)(Mc - 1)) / (cyy / (double)(Mc - 1));
        Qout[i] = q;
    }
}

void launch_cv_pilot(const Fp64Tables& t, const double* ivb, int64_t Mc, double* xy, double* alpha, double* Q,
                     void* stream)
{
    k_cv_pilot<<<t.n_out, 256, 0, (cudaStream_t)stream>>>(t, (const double2*)ivb, Mc, xy, alpha, Q);
    count_launch();
}

__device__ __forceinline__ double cv_half(double2 iv, double rho, double K, double alpha, double Q, double Qmax,
                                          unsigned& exc)
{
    const double spot = exp(-0.5 * rho * rho * iv.x + rho * iv.y);
    const double x = bs_call_tau1(spot, K, sqrt((1.0 - rho * rho) * iv.x));
    const bool inside = Q > iv.x;
    if (!inside) ++exc;
    const double y = bs_call_tau1(spot, K, inside ? sqrt(rho * rho * (Q - iv.x)) : sqrt(rho * rho * (Qmax - iv.x)));
    return x + alpha * y;
}

// grid (nchunks, ceil(n_out / kOPB)), as k_payoff_sums: per path the
// antithetic mean 0.5 (f(W) + f(-W)).
__global__ void __launch_bounds__(256) k_payoff_sums_cv(Fp64Tables t, const double2* __restrict__ ivb,
                                                        const double2* __restrict__ ivn, int64_t B,
                                                        const double* __restrict__ alpha,
                                                        const double* __restrict__ Q, double Qmax, int G,
                                                        double* __restrict__ part,
                                                        unsigned long long* __restrict__ count)
{
    __shared__ double red[8][kOPB][2];
    const int c = blockIdx.x;
    const int o0 = blockIdx.y * kOPB;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double S = 0, CS = 0, S2 = 0, CS2 = 0;
    OutDev od[kOPB];
    double al[kOPB], qq[kOPB];
    unsigned exc[kOPB];
#pragma unroll
    for (int q = 0; q < kOPB; ++q) {
        const int i = o0 + q;
        od[q] = (i < t.n_out) ? t.outs[i] : OutDev{0.0, 1.0, -1, 0};
        al[q] = (i < t.n_out) ? alpha[i] : 0.0;
        qq[q] = (i < t.n_out) ? Q[i] : 0.0;
        exc[q] = 0;
    }
    for (int sub = 0; sub < G; ++sub) {
        const int64_t m = ((int64_t)c * G + sub) * 256 + threadIdx.x;
#pragma unroll
        for (int q = 0; q < kOPB; ++q) {
            double x = 0.0;
            if (m < B && od[q].vg >= 0) {
                const size_t at = (size_t)od[q].vg * B + m;
                x = 0.5 * cv_half(ivb[at], od[q].rho, od[q].K, al[q], qq[q], Qmax, exc[q]);
                x += 0.5 * cv_half(ivn[at], od[q].rho, od[q].K, al[q], qq[q], Qmax, exc[q]);
            }
            double x2 = x * x;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(0xffffffffu, x, o);
                x2 += __shfl_xor_sync(0xffffffffu, x2, o);
            }
            if (lane == 0) { red[w][q][0] = x; red[w][q][1] = x2; }
        }
        __syncthreads();
        if (threadIdx.x < kOPB) {
            const int q = threadIdx.x;
            double a = 0, a2 = 0;
            for (int k = 0; k < 8; ++k) { a += red[k][q][0]; a2 += red[k][q][1]; }
            neumaier_add(S, CS, a);
            neumaier_add(S2, CS2, a2);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < kOPB; ++q) {
        unsigned e = exc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
        if (lane == 0 && e && o0 + q < t.n_out) atomicAdd(count + o0 + q, (unsigned long long)e);
    }
    if (threadIdx.x < kOPB && o0 + (int)threadIdx.x < t.n_out) {
        double* p = part + ((size_t)c * t.n_out + o0 + threadIdx.x) * 4;
        p[0] = S; p[1] = CS; p[2] = S2; p[3] = CS2;
    }
}

void launch_payoff_sums_cv(const Fp64Tables& t, const double* ivb, const double* ivn, int64_t B, const double* alpha,
                           const double* Q, double Qmax, int G, double* part, unsigned long long* count, int nchunks,
                           void* stream)
{
    dim3 grid(nchunks, (t.n_out + kOPB - 1) / kOPB);
    k_payoff_sums_cv<<<grid, 256, 0, (cudaStream_t)stream>>>(t, (const double2*)ivb, (const double2*)ivn, B, alpha,
                                                             Q, Qmax, G, part, count);
    count_launch();
}

// price = mean - alpha ((1 - p) BS(1, K, 1, sqrt(rho^2 Q)) + p BS(1, K, 1, sqrt(rho^2 Qmax))),
// p = exceptions / M; stat from the unadjusted payoffs (RBergomi.cpp:266-284).
__global__ void k_finalize_cv(const double* __restrict__ acc, int n_out, int64_t M, const OutDev* __restrict__ outs,
                              const double* __restrict__ Tv, const double* __restrict__ alpha,
                              const double* __restrict__ Q, const unsigned long long* __restrict__ count,
                              double Qmax, int compute_iv, double* __restrict__ res)
{
    const int i = blockIdx.x;
    if (i >= n_out) return;
    const double S = acc[i * 4 + 0] + acc[i * 4 + 1];
    const double S2 = acc[i * 4 + 2] + acc[i * 4 + 3];
    const double mean = S * (1.0 / (double)M);
    const double var = 1.0 * (S2 * (1.0 / (double)M)) + -1.0 * (mean * mean);
    const double stat = sqrt(var) * (1.0 / sqrt((double)M));
    const double p = (double)count[i] / (double)M, r = outs[i].rho, K = outs[i].K;
    const double adj = (1.0 - p) * bs_call_tau1(1.0, K, sqrt(r * r * Q[i])) + p * bs_call_tau1(1.0, K, sqrt(r * r * Qmax));
    const double price = mean - alpha[i] * adj;
    const double iv = compute_iv ? implied_vol_warp(price, K, Tv[i]) : 0.0;
    if ((threadIdx.x & 31) == 0) {
        res[i] = price;
        res[n_out + i] = stat;
        res[2 * n_out + i] = iv;
        res[3 * n_out + i] = S;
        res[4 * n_out + i] = S2;
    }
}

void launch_finalize_cv(const double* acc, int n_out, int64_t M, const OutDev* outs, const double* Tvals,
                        const double* alpha, const double* Q, const unsigned long long* count, double Qmax,
                        int compute_iv, double* res, void* stream)
{
    k_finalize_cv<<<n_out, 32, 0, (cudaStream_t)stream>>>(acc, n_out, M, outs, Tvals, alpha, Q, count, Qmax,
                                                          compute_iv, res);
    count_launch();
}

}  // namespace rbg
