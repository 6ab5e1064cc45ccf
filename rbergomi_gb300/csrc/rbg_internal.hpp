// rbg_internal.hpp -- types shared by the host planner, the launchers and the
// kernels of librbergomi_gb300.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <vector_types.h>

#include "rbergomi_gb300.h"

namespace rbg {

// One Volterra pass: a distinct H at which the reference's HTrigger fired.
// X_j = Y2_j + a1 W1_j + a2 W1perp_j with Y2 = (W1 * Gamma_H)[0..N) is shared
// by every variance group of this pass (rBergLib/rBergomiMT.cpp:83-109).
struct VolGroup {
    double H;
    double c;       // sqrt(2H) * N^-H          (rBergomiMT.cpp:107-108)
    double a1, a2;  // rhoH / s2H, sqrt(1 - rhoH^2) / s2H  (rBergomiMT.cpp:87-89)
    int vg_begin, vg_end;  // its variance groups, contiguous after sorting
};

// One variance path: the state after the reference's H/T/eta trigger chain
// (rBergomiMT.cpp:493-507).  WS_j = scale * X_j with scale = c * T_s^H_s;
// v_0 = xi, v_j = xi exp(eta WS_{j-1} - comp[j-1]) with
// comp[j] = 0.5 eta eta (j dt)^{2 H_v} (rBergomiMT.cpp:73-80).
struct VGroup {
    int vol;
    double Hs, Ts;  // H and T at the last H-or-T trigger (scaleWtilde)
    double Hv, eta; // H and eta at the last H-or-T-or-eta trigger (updateV)
    double scale, dt, sdt;
    double xi;  // forward variance (per tuple in the control-variate form, else the plan's)
    int nsteps;
};

struct OutMap {
    int vg;
    double rho, K, T;
};

struct Plan {
    double xi = 0;
    int N = 0;
    // compensator index: v_i = xi exp(eta WS_{i-1} - eta^2/2 ((i - 1 + comp_shift) dt)^{2H});
    // 0 for rBergLib (rBergomiMT.cpp:73-80), 1 for ML_console_ST (RBergomi.cpp:365-372)
    int comp_shift = 0;
    std::vector<VolGroup> vols;
    std::vector<VGroup> vgs;
    std::vector<OutMap> outs;
    std::vector<double> gamma;  // [n_vol][N] (rBergomiMT.cpp:143-149)
    std::vector<double> comp;   // [n_vg][N], comp[N-1] unused
};

// Builds the plan with the reference's ParamTot trigger semantics
// (rBergLib/ParamTot.h:28-43, eps 1e-10 at ParamTot.cpp:27).  Volterra passes
// are deduplicated by exact H value, variance groups by exact tuple.
// Returns false and sets err on invalid input.
// plain_mc: outputs carry the rho of the last H/T/eta/rho trigger, the
// state the reference's plain Monte Carlo driver prices S with.
bool build_plan(const rbg_params& p, Plan& plan, std::string& err, bool plain_mc = false);
// The unordered form: one output per tuple, every tuple's chain recomputed
// as the reference's updatePayoffUnordered does (equal tuples share state).
// xi_per: optional per-tuple forward variances (groups then split by xi);
// comp_shift as in Plan.
bool build_plan_unordered(const rbg_unordered& u, Plan& plan, std::string& err, const double* xi_per = nullptr,
                          int comp_shift = 0);

// ---- device-side views -------------------------------------------------
struct VolDev {
    double a1, a2;
    int vg_begin, vg_end;
};
struct VGDev {
    double scale, eta, dt, sdt, xi;
    int nsteps, vol;
};
struct OutDev {
    double rho, K;
    int vg, pad;
};

// ---- launchers (rbg_fp64.cu) -------------------------------------------
struct Fp64Tables {
    const VolDev* vols;
    const VGDev* vgs;
    const OutDev* outs;
    const double* gamma;
    const double* comp;
    int n_vol, n_vg, n_out, N;
    double xi;
    // FFT convolution (logL > 0): per pass v the spectrum FFT(Gamma_v, zero-
    // padded to L = 2^logL, Gamma_v[0] = 0) / L, and exp(-2 pi i q / L)
    const double2* spec;
    const double2* tw;
    int logL;
};

// FP64 Volterra sum by FFT from this many steps (the direct sum below);
// transforms up to 2^kFp64FftMaxLogL points
constexpr int kFp64FftMinN = 200;
constexpr int kFp64FftMaxLogL = 12;
// log2 L of the FP64 form's FFT for N steps (L >= 2N - 1), 0 when it cannot run
int fp64_fft_log2_len(int N);
// host tables of the FP64 FFT: spec [n_vol][L], tw [L] (complex doubles)
void fp64_fft_tables(const double* gamma, int n_vol, int N, int logL, double* spec, double* tw);

// ns normal streams per path: 2 (W1, W1perp) for RT, 3 (+ Wperp) for plain MC
void launch_normals(uint64_t seed, int64_t path0, int64_t B, int N, int f32, double* Z, void* stream, int ns = 2);

// Sobol' quasi-Monte Carlo normals (rbg_qmc.cu).  Direction integers per
// coordinate: kSobolBits columns; coordinate d of point s is (XOR of
// V[d][k] over the set bits k of s ^ (s >> 1)) * 2^-62.
constexpr int kSobolBits = 62;
constexpr int kMaxBridgeLevels = 13;  // Brownian bridge: N = 2^m, m <= 13
struct SobolBridge {
    double c[kMaxBridgeLevels + 1];  // c[0] = 2^(-m/2), c[n] = 2^((n - m - 1)/2)
    int m;
};
// Z [B][2][N] for points s0 .. s0 + B - 1; Vt = [kSobolBits][2N] on the
// device; br = nullptr: no bridge; f32: the mixed form's FP32 normals (FP32
// quantile, and the bridge in FP32), widened to double.  Returns nonzero when the bridge's shared
// memory cannot be granted.
int launch_sobol_normals(const unsigned long long* Vt, int N, uint64_t s0, int64_t B, const SobolBridge* br,
                         double* Z, void* stream, int f32 = 0);
int path_fp64_warps(int N);
size_t path_fp64_smem(int N, int warps);
// ivp non-null: Z has three streams per path (plain MC) and ivp[g][B] gets IsvdWp
void launch_path_fp64(const Fp64Tables& t, const double* Z, int64_t B, double* ivb, void* stream,
                      double* ivp = nullptr, double* ivn = nullptr);
// control-variate form (ML_console_ST): pilot statistics per output -- Q = max
// 2 Ivdt over the pilot, alpha = -cov(X, Y) / var(Y) -- from the pilot's
// (Ivdt, IsvdW) [group][Mc]; xy scratch holds 2 Mc doubles per output
void launch_cv_pilot(const Fp64Tables& t, const double* ivb, int64_t Mc, double* xy, double* alpha, double* Q,
                     void* stream);
// per chunk (S, C, S2, C2) of the antithetic control-variate payoffs, and the
// Qmax-exception count per output (atomically added, integer)
void launch_payoff_sums_cv(const Fp64Tables& t, const double* ivb, const double* ivn, int64_t B, const double* alpha,
                           const double* Q, double Qmax, int G, double* part, unsigned long long* count, int nchunks,
                           void* stream);
void launch_finalize_cv(const double* acc, int n_out, int64_t M, const OutDev* outs, const double* Tvals,
                        const double* alpha, const double* Q, const unsigned long long* count, double Qmax,
                        int compute_iv, double* res, void* stream);
void launch_payoff_sums(const Fp64Tables& t, const double* ivb, int64_t B, int64_t ivb_stride, int G,
                        double* part, int nchunks, void* stream, const double* ivp = nullptr);
void launch_accumulate(const double* part, int nchunks, int n_out, double* acc, void* stream);
void launch_finalize(const double* acc, int n_out, int64_t M, const OutDev* outs, const double* Tvals,
                     int compute_iv, double* res, void* stream);
void launch_payoff_store(const Fp64Tables& t, const double* ivb, int64_t B, int64_t ivb_stride, double* payoff,
                         void* stream, const double* ivp = nullptr);
void launch_implied_vol(int n, const double* price, const double* K, const double* T, double* iv, void* stream);

// ---- job-table forms of the payoff, merge and finalize kernels ----------
// (the serving loop's shared launches: one launch serves many requests; each
// job's arithmetic is the per-request kernels' own, block for block)
// Block b of a launch belongs to the last job whose block0 <= b.
struct PayoffJob {      // FP32 RT payoff sums, nchunks x ceil(n_out / 8) blocks
    const OutDev* outs;
    const float2* ivb;  // [group][B] (Ivdt, IsvdW)
    double* part;       // [chunk][n_out][4]
    int64_t B, block0;
    int n_out, G, nchunks, pad;
};
struct AccJob {  // fixed-order merge of the chunk sums into acc (written, not added to), n_out blocks
    const double* part;
    double* acc;
    int64_t block0;
    int nchunks, n_out;
};
struct FinJob {  // price, stat, implied vol, n_out blocks of one warp
    const double* acc;
    const OutDev* outs;
    const double* Tv;
    double* res;
    int64_t M, block0;
    int n_out, compute_iv;
};
void launch_accumulate_jobs(const AccJob* jobs, int n_jobs, int64_t blocks, void* stream);
void launch_finalize_jobs(const FinJob* jobs, int n_jobs, int64_t blocks, void* stream);
// Loads the merge and finalize kernels (modules load lazily, on first use).
void reduce_preload();

// Kernel-launch counter shared by all launchers.
void count_launch(int n = 1);

// The drop-in layer's seed folding: seed[0] for one word, splitmix64
// chaining of the words otherwise, 0 for none (one 64-bit Philox key).
uint64_t fold_seed(const uint64_t* seed, int seed_size);

// SMs of the current device (cached per device ordinal; 1 if unknown).
int device_sms();

// Payoff-reduction chunking of a batch of B paths: chunks of 256 G paths,
// one 256-thread block each, every thread summing G paths in FP32 (stride
// 256).  G is the smallest that keeps the chunk count at about four per SM.
// Results depend on G, so every entry point that must reproduce another's
// sums takes G from this one rule and the same B.
inline int payoff_paths_per_thread(int64_t B, int sms)
{
    const int64_t target = 4 * (int64_t)(sms > 0 ? sms : 1);
    const int64_t g = (B + 256 * target - 1) / (256 * target);
    return (int)(g > 1 ? g : 1);
}

}  // namespace rbg
