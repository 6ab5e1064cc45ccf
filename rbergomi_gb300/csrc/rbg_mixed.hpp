// rbg_mixed.hpp -- the mixed-precision form: tcgen05 Toeplitz-GEMM path
// kernel fused with Philox generation and the variance-path epilogue, plus
// the FP32 payoff / FP64 reduction kernel.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "rbg_internal.hpp"

namespace rbg {

constexpr int kMixedMaxGroups = 16;  // variance groups handled by one launch
constexpr int kMixedMaxFused = 64;   // outputs whose payoffs one launch can price in its epilogue

// Kernel arguments (passed by value as a __grid_constant__).
struct MixedArgs {
    const unsigned char* strip;  // [hi | lo]: Np rows x 64 B (SW64, one pass) or Np + 16 rows x 32 B (SW32)
    const float* beta;           // [n_g][Np] (log2 compensator - log2 xi) / 2
    float2* ivb;                 // [n_vg_total][B] (Ivdt, IsvdW)
    float* ivq;                  // plain Monte Carlo: [n_vg_total][B] IsvdWp = sum sqrt(v) sdt Wperp
    unsigned int* err;           // 0, or the id of the wait that expired
    float* dbg_w;                // optional [B][2][Np] normals the producers drew
    float* dbg_x;                // optional [B][Np] X = Y2 + a1 W1 + a2 W1perp
    const float4* otab;          // fused outputs: (rho, K, log K, local group), n_o entries
    const int* oidx;             // fused outputs: global output index
    double* part;                // fused outputs: [CTA][n_out_total][S, C, S2, C2] partial sums
    unsigned long long* prof;    // diagnostic runs only: wait cycles per site, busy cycles per role
    const float2* spec;          // FFT backend: FFT(Gamma)/L, L points
    const float2* tw;            // FFT backend: exp(-2 pi i t / L), L points
    const unsigned int* sob;     // Sobol' normals (GEMM backend, RT): [32][2N] bits 30..61 of the direction integers
    const double* ext;           // caller normals for this launch's paths, [B][ns][N] FP64 (quadrature layout)
    uint64_t seed;
    int64_t path0, B;
    int N, Np, nc, n_g, g0, tmem_cols, stages;
    int n0;                // GEMM backend, Np > 512: chunks of the first TMEM pass (0: one pass)
    int n_o, n_out_total;  // fused outputs of this launch; all outputs of the job
    int L, logL;  // FFT backend transform length
    float a1, a2, xi, sqrt_xi;
    float alpha[kMixedMaxGroups];  // eta * scale * log2(e) / 2
    float dt[kMixedMaxGroups], sdt[kMixedMaxGroups];
    int nsteps[kMixedMaxGroups];
    // Appended last on purpose: a field inserted before the per-group arrays
    // moves them in the kernel's parameter space, which measured 4% slower on
    // the headline kernel (5.54 -> 5.78 ms at N = 512, 2^22 paths).
    int np;  // GEMM backend: TMEM passes per tile (1 .. 8)
    // Job-table launches (the serving loop's shared launches): this launch's
    // tiles belong to n_jobs requests; job j's arguments are jobs[j] (device
    // memory, pointers filled) and its tiles are [job_tile0[j], job_tile0[j + 1])
    // of the launch.  Unused (null / 0) in ordinary launches.
    const MixedArgs* jobs;
    const int64_t* job_tile0;
    int n_jobs;
    // Philox4x32-10 round keys of `seed` in the PhiloxKeys layout (pk[r] = lo +
    // r 0x9E3779B9, pk[10 + r] = hi + r 0xBB67AE85), set with it by
    // mixed_set_seed.  The FFT kernel reads them from parameter space, where
    // each round's key is an operand of its XOR instead of one of 20 registers
    // held across the whole kernel.
    uint32_t pk[20];
    // Pass mode 3 (GEMM backend, 512 < Np <= 1024, 16-bit splits, RT, Philox):
    // per-CTA global cache of the A tiles later passes read back, ncache
    // chunks of 16 KB per CTA (CTA b's at acache + b * ncache * 16 KB).
    unsigned char* acache;
    int ncache;
};

// Sets a.seed and its Philox round keys a.pk.
inline void mixed_set_seed(MixedArgs& a, uint64_t seed)
{
    a.seed = seed;
    uint32_t x = (uint32_t)seed, y = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        a.pk[r] = x;
        a.pk[10 + r] = y;
        x += 0x9E3779B9u;
        y += 0xBB67AE85u;
    }
}

struct MixedLaunch {
    MixedArgs args;  // device pointers filled at launch time
    size_t off_strip = 0, off_beta = 0, off_spec = 0, off_otab = 0, off_oidx = 0;
    int stages_pm1 = 0;  // pass mode 3 jobs: pipeline stages of the two-pass kernel that takes other normal sources
};

struct MixedJob {
    int64_t batch = 0;           // paths per launch
    size_t workspace_bytes = 0;  // error word + strips + beta tables
    size_t off_err = 0;
    int N = 0, n_vol = 0, n_vg = 0, split = 0, sms = 0;
    int backend = RBG_CONV_GEMM;  // RBG_CONV_GEMM or RBG_CONV_FFT
    bool fused = false;           // payoffs priced inside the path kernel (GEMM backend, <= 64 per launch)
    bool mc = false;              // plain Monte Carlo: third normal stream Wperp and IsvdWp per (group, path)
    const unsigned int* sob = nullptr;  // Sobol' table on the device (set by the caller): QMC normals, not Philox
    size_t off_tw = 0;
    // GEMM kernel pass mode: 0 one TMEM pass, 1 two, 2 up to eight, 3 two
    // 256-column buffers with the A-tile cache at off_acache (workspace bytes
    // past the uploaded image)
    int pmode = 0;
    size_t off_acache = 0;
    std::vector<MixedLaunch> launches;   // one per (Volterra pass, <= 16 groups)
    std::vector<const void*> table_dev;  // optional device copies of each launch's strip / spectrum
    std::vector<unsigned char> host_ws;  // image uploaded by mixed_upload
};

// mc: the plain Monte Carlo estimator (a third normal stream; both backends, every pass mode).
// tile_cache: pass mode 3 may be chosen (its A-tile cache, sms x up to 16 x
// 16 KB of device memory, is part of workspace_bytes).
int mixed_prepare(const Plan& plan, const rbg_options& o, int64_t M, MixedJob& job, std::string& err,
                  int64_t max_batch = 0, bool mc = false, bool tile_cache = true);
// Byte range of launch i's strip (GEMM) or spectrum (FFT) inside host_ws, and
// of the shared FFT twiddle table (empty for the GEMM backend).
void mixed_table_range(const MixedJob& job, int i, size_t* off, size_t* bytes);
void mixed_twiddle_range(const MixedJob& job, size_t* off, size_t* bytes);
int mixed_upload(const MixedJob& job, void* ws, cudaStream_t st, std::string& err);
// Launches the path kernel(s) for paths [path0, path0 + B).  Unfused jobs
// write (Ivdt, IsvdW) to ivb; fused jobs add their payoff sums to `part`
// (rows = mixed_part_rows(job, B), zeroed by the caller) and write ivb only
// when it is non-null.
// Plain Monte Carlo jobs also write IsvdWp per (group, path) to ivq.
// ext: the caller's normals for paths [0, B) of this launch ([B][ns][N] FP64
// on the device) instead of the Philox stream.
int mixed_launch(const MixedJob& job, void* ws, uint64_t seed, int64_t path0, int64_t B, void* ivb,
                 cudaStream_t st, std::string& err, float* dbg_w = nullptr, float* dbg_x = nullptr,
                 double* part = nullptr, unsigned long long* prof = nullptr, float* ivq = nullptr,
                 const double* ext = nullptr);
int mixed_part_rows(const MixedJob& job, int64_t B);
int mixed_check(const MixedJob& job, void* ws, cudaStream_t st, std::string& err);
// Loads the path and payoff kernels a serving loop may launch (modules load lazily).
void mixed_preload();
// one warp waits on an mbarrier nothing arrives on, with the pipeline's bounded
// wait and a 20 ms limit; *err receives `site` on expiry
int launch_wait_probe(unsigned int* err, unsigned int site, cudaStream_t st);
// FFT backend (rbg_fft.cu)
int fft_log2_len(int N);
size_t fft_smem_bytes(int N, int n_g, int ns = 2);
void fft_tables(const double* gamma, int N, int logL, float* spec, float* tw);
cudaError_t launch_mixed_fft(const MixedArgs& A, int sms, cudaStream_t st);

// ivq non-null: plain Monte Carlo payoffs max(S_T - K, 0) from (Ivdt, IsvdW, IsvdWp)
// per-path FP32 payoffs, payoff[m * n_out + i] as double (mixed quadrature)
void launch_payoff_store_f32(const OutDev* outs, int n_out, const void* ivb, const float* ivq, int64_t B,
                             double* payoff, cudaStream_t st);
void launch_payoff_sums_f32(const OutDev* outs, int n_out, const void* ivb, int64_t B, int G, double* part,
                            int nchunks, cudaStream_t st, const float* ivq = nullptr);
void launch_payoff_sums_f32_jobs(const PayoffJob* jobs, int n_jobs, int64_t blocks, cudaStream_t st);

// ---- job-table launches of the path kernel (the serving loop's shared launches)
// A request whose prepared job is one launch of one TMEM pass (N <= 512) of the
// RT estimator on Philox normals, payoffs in the separate kernels.
bool mixed_job_batchable(const MixedJob& job);
// One job of a shared launch: its prepared job, its workspace image on the
// device, its paths and its (Ivdt, IsvdW) buffer.
struct MixedJobRef {
    const MixedJob* job;
    const void* ws;
    uint64_t seed;
    int64_t path0, B;
    void* ivb;
};
// Device bytes of the job table of n jobs.
size_t mixed_jobs_table_bytes(int n);
// Fills the job table for `jobs` (all of one split) into host_table (grown to
// mixed_jobs_table_bytes) for the device address `table`, and the launch's own
// arguments into *launch_args; returns the CTA count.  The caller copies the
// table to the device before the launch.
int mixed_jobs_prepare(const std::vector<MixedJobRef>& jobs, void* table, unsigned int* err, int sms,
                       std::vector<unsigned char>& host_table, MixedArgs* launch_args, std::string& errmsg);
// Launches the path kernel over every job's tiles (grid: mixed_jobs_prepare's CTA count).
int mixed_launch_jobs(const MixedArgs& launch_args, int split, int grid, cudaStream_t st, std::string& errmsg);

// Control-variate payoff sums from two path-kernel runs with xi = 0 in their
// final sums, the second with the variance exponent's coefficient negated
// (the antithetic paths): per chunk (S, C, S2, C2) of 0.5 (f(W) + f(-W)), the
// Q_max exceptions counted per output.  alpha, Q: the pilot's, per output.
void launch_payoff_sums_cv_f32(const OutDev* outs, const VGDev* vgs, int n_out, const void* ivb, const void* ivn,
                               int64_t B, int G, uint64_t seed, int64_t path0, const double* alpha, const double* Q,
                               double Qmax, double* part, unsigned long long* count, int nchunks, cudaStream_t st);

}  // namespace rbg
