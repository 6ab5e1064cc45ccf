/*
 * rbergomi_gb300.h -- C ABI of the GB300 rough Bergomi Romano-Touzi pricer.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the exact signatures, argument meaning, output
 *    layout and error exits of the reference library's C interface
 *    (rBergLib/cinterface.h:62-76).  A caller linked against librBergLib can
 *    relink against librbergomi_gb300.so unchanged.
 *
 * 2. An extended, status-returning API (rbg_*) that exposes precision mode,
 *    convolution backend, Philox seed, path offset and CUDA stream, and never
 *    exits the process.
 *
 * Conventions shared by both layers
 *   - ParamTot layout: output index i <-> (H, eta, rho)[i / op_size] and
 *     (T, K)[i % op_size] (rBergLib/ParamTot.h:28-33).  H, eta, rho are aligned
 *     arrays of length par_size (not a tensor product); T, K have length op_size.
 *   - S0 = 1, r = 0, constant forward variance xi.
 *   - Normals come from a counter-based Philox4x32-10 stream: key = the 64-bit
 *     seed, counter = (step group g, path lo32, path hi32, stream), four normals
 *     per call for steps 4g..4g+3 of stream 0 (W1) or 1 (W1perp).  Results do
 *     not depend on batching, thread count or device.
 */
#ifndef RBERGOMI_GB300_H
#define RBERGOMI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Drop-in layer                                                            */
/* ------------------------------------------------------------------------ */

/* Plain Monte Carlo prices, implied vols and MC standard errors over the
 * ParamTot grid.  Replaces computeIV_tensor, rBergLib/cinterface.h:63-66
 * (cinterface.cpp:10-46; estimator rBergomiMT.cpp:174-289): a third normal
 * stream Wperp per path, S_T = exp(sum sqrt(v) sqrt(dt) Z - dt/2 sum v) with
 * Z = rho W1 + sqrt(1 - rho^2) Wperp, payoff max(S_T - K, 0); S is
 * recomputed on the reference's rho trigger (eps 1e-10).  Same size checks,
 * exit codes and seed folding as computeIVRT_tensor.  FP64 unless the
 * environment sets RBG_PRECISION=mixed.  Like the reference
 * (cinterface.cpp:45), eta_tot receives the rho values and rho_tot the eta
 * values. */
void computeIV_tensor(double xi, double* H, double* eta, double* rho, int par_size, double* T, double* K,
                      int op_size, int N, long M, uint64_t* seed, int seed_size, int num_threads, double* price,
                      double* iv, double* stat, double* H_tot, double* eta_tot, double* rho_tot, double* T_tot,
                      double* K_tot, int out_size);

/* Romano-Touzi prices, implied vols and MC standard errors over the ParamTot
 * grid.  Replaces computeIVRT_tensor, rBergLib/cinterface.h:68-71
 * (cinterface.cpp:49-85).  out_size must equal par_size * op_size, else the
 * process exits with status 17 after a message on stderr; num_threads < 1
 * exits with status 21 (cinterface.cpp:54-59, 76-81).  num_threads is
 * otherwise ignored: one GPU does the work.  The seed words are folded into
 * one 64-bit Philox key (seed[0] when seed_size == 1, splitmix64 chaining
 * otherwise).  Precision: FP64 unless the environment sets
 * RBG_PRECISION=mixed.  Any CUDA failure prints to stderr and exits with
 * status 70. */
void computeIVRT_tensor(double xi, double* H, double* eta, double* rho, int par_size, double* T, double* K,
                        int op_size, int N, long M, uint64_t* seed, int seed_size, int num_threads, double* price,
                        double* iv, double* stat, double* H_tot, double* eta_tot, double* rho_tot, double* T_tot,
                        double* K_tot, int out_size);

/* RT payoffs for caller-supplied normals.  Replaces
 * computeIVRT_tensor_quadrature, rBergLib/cinterface.h:73-75
 * (cinterface.cpp:102-131).  Z holds 2*N*M doubles: sample m uses
 * Z[2mN, 2mN+N) as W1 and Z[(2m+1)N, (2m+2)N) as W1perp.  payoff receives
 * M * par_size * op_size doubles, payoff[m*out_size + i].  FP64 unless the
 * environment sets RBG_PRECISION=mixed (then the mixed form's FP32 payoffs
 * per path, widened to double). */
void computeIVRT_tensor_quadrature(double xi, double* H, double* eta, double* rho, int par_size, double* T,
                                   double* K, int op_size, int N, long M, double* Z, int num_threads,
                                   double* payoff);

/* ------------------------------------------------------------------------ */
/* Extended layer                                                           */
/* ------------------------------------------------------------------------ */

enum rbg_status {
    RBG_OK = 0,
    RBG_ERR_ARG = 1,      /* bad argument (sizes, null pointers, ranges) */
    RBG_ERR_CUDA = 2,     /* a CUDA runtime call or kernel failed */
    RBG_ERR_NOMEM = 3,    /* device allocation failed or over budget */
    RBG_ERR_UNSUPPORTED = 4, /* option combination not available */
    RBG_ERR_TIMEOUT = 5   /* a bounded device-side wait expired */
};

enum rbg_precision { RBG_FP64 = 0, RBG_MIXED = 1 };

/* Volterra convolution backend.  In mixed mode AUTO picks the tcgen05
 * Toeplitz GEMM for N <= 4096 (one TMEM pass up to 512 steps, one more per
 * further 512; measured faster than the batched FFT convolution at every N
 * up to 4096); FFT selects the batched FFT convolution (N <= 4096).  The
 * FP64 form has two: the direct causal sum (DIRECT) and an FP64 FFT
 * convolution (FFT, 2 <= N <= 2048); AUTO takes the FFT from 200 steps to
 * 2048.  GEMM is mixed-mode only. */
enum rbg_conv { RBG_CONV_AUTO = 0, RBG_CONV_GEMM = 1, RBG_CONV_FFT = 2, RBG_CONV_DIRECT = 3 };

/* Normal transform used by the FP64 form: its own FP64 Box-Muller (default),
 * or the FP32 Box-Muller values of the mixed form widened to FP64, so an FP64
 * run sees exactly the normals a mixed run with the same seed sees. */
enum rbg_normals { RBG_NORMALS_F64 = 0, RBG_NORMALS_F32 = 1 };

/* Split used by the mixed-form tensor-core convolution: BF16x3 and FP16x3
 * split both operands into 16-bit hi + lo and sum three products (lo x lo
 * dropped); TF32X2 rounds the normals to TF32 (kind::tf32, round to nearest)
 * and splits the kernel table Gamma into TF32 hi + lo: two products, one
 * compensation term. */
enum rbg_split { RBG_SPLIT_BF16X3 = 0, RBG_SPLIT_F16X3 = 1, RBG_SPLIT_TF32X2 = 2 };

typedef struct rbg_params {
    double xi;
    const double* H;
    const double* eta;
    const double* rho;
    int par_size;
    const double* T;
    const double* K;
    int op_size;
    int N;     /* time steps per path (dt = T / N for every maturity) */
    int64_t M; /* paths */
} rbg_params;

typedef struct rbg_options {
    int precision;       /* enum rbg_precision */
    int conv;            /* enum rbg_conv */
    int normals;         /* enum rbg_normals (FP64 form only) */
    int split;           /* enum rbg_split (mixed form only) */
    int compute_iv;      /* nonzero: fill iv[] (FP64 inversion on the GPU) */
    uint64_t seed;       /* Philox key */
    int64_t path_offset; /* global index of the first path (replicas/shards) */
    void* stream;        /* cudaStream_t to run on; NULL = the library's stream */
} rbg_options;

/* Fills opts with defaults: FP64, AUTO, F64 normals, BF16x3, iv on, seed 0. */
void rbg_default_options(rbg_options* opts);

/* Prices on the Philox stream.  price, stat, iv: host arrays of
 * par_size*op_size doubles (iv may be NULL).  Returns enum rbg_status. */
int rbg_price_rt(const rbg_params* p, const rbg_options* o, double* price, double* stat, double* iv);

/* Unordered parameter list: output i prices the tuple (H[i], eta[i],
 * rho[i], T[i], K[i]); every array has `size` entries.  Replaces the
 * reference's ParamTotUnordered + ComputeIVRTMTunstructured
 * (rBergomi/ParamTot.h:57-75, rBergomi/rBergomiMT.cpp:837-938), the form
 * calibration-style traffic sends. */
typedef struct rbg_unordered {
    double xi;
    const double* H;
    const double* eta;
    const double* rho;
    const double* T;
    const double* K;
    long size;
    int N;
    int64_t M;
} rbg_unordered;

/* Prices an unordered list on the Philox stream; price, stat, iv as for
 * rbg_price_rt with `size` entries.  Tuples are not required to be sorted:
 * equal H share one Volterra pass and equal (H, T, eta) one variance path. */
int rbg_price_rt_unordered(const rbg_unordered* u, const rbg_options* o, double* price, double* stat, double* iv);

/* Romano-Touzi prices with the control variate of McCrickerd and Pakkanen
 * and antithetic paths, as ML_console_ST's RBergomi::ComputeIVRTVarRed does
 * it (ML_console_ST/RBergomi.cpp:218-306, 478-540), over an unordered list
 * with one xi per tuple and that code's (i dt)^{2H} compensator:
 *   pilot: M_control paths give Q_i = max 2 Ivdt and alpha_i = -cov(X, Y) /
 *   var(Y), X the RT payoff, Y = BS(S, K, 1, sqrt(rho^2 (Q - Ivdt)));
 *   main: M paths, each the mean of X + alpha Y at W and at -W (Q_max where
 *   Q <= Ivdt), then price -= alpha E[Y] in closed form.
 * Pilot normals come from Philox paths 2^62 + path_offset + m, main normals
 * from paths path_offset + m.  o->precision RBG_FP64: every stage in FP64.
 * RBG_MIXED: the pilot in FP64 on FP32 normals, the main paths through the
 * tensor-core path kernel (twice: W, and -W by the negated variance
 * exponent) and FP32 payoffs with FP64 sums; the FP64 form with
 * o->normals = RBG_NORMALS_F32 draws the same normals.  The caller-normals
 * entry below is FP64 only. */
typedef struct rbg_cv_params {
    const double* xi;
    const double* H;
    const double* eta;
    const double* rho;
    const double* T;
    const double* K;
    long size;
    int N;
    int64_t M;          /* main paths (each also priced antithetically) */
    int64_t M_control;  /* pilot paths (the reference uses 10000) */
    double Q_max;       /* the reference uses 10000 */
} rbg_cv_params;

int rbg_price_rt_cv(const rbg_cv_params* p, const rbg_options* o, double* price, double* stat, double* iv);
/* Same on caller normals (host pointers): Zc holds 2*N*M_control doubles for
 * the pilot, Z 2*N*M for the main paths, W1 then W1perp per path. */
int rbg_price_rt_cv_normals(const rbg_cv_params* p, const double* Zc, const double* Z, double* price, double* stat,
                            double* iv);

/* Same, with the raw sums instead of finished moments: sum[i] = sum_m x,
 * sum2[i] = sum_m x^2 over this call's paths (for merging shards/replicas). */
int rbg_price_rt_sums(const rbg_params* p, const rbg_options* o, double* sum, double* sum2);

/* Merges path shards (or replicas on disjoint path ranges): sum and sum2 are
 * [n_shards][n] arrays of rbg_price_rt_sums outputs (n_shards = 1 after the
 * caller's own all-reduce), M the total path count over all shards.  Adds
 * the shards in index order with Neumaier compensation, then applies the
 * reference's moment formula (rBergLib/rBergomiMT.cpp:404-409):
 * price = S / M, stat = sqrt(S2 / M - price^2) / sqrt(M).  Host-only; no GPU
 * needed.  Implied vols of the merged prices: rbg_implied_vol. */
int rbg_merge_sums(int n_shards, int n, const double* sum, const double* sum2, int64_t M, double* price,
                   double* stat);

/* Per-path payoffs for caller-supplied normals (quadrature layout).  Z and
 * payoff are host pointers unless device_ptrs != 0, in which case both are
 * device pointers on the current device.  o->precision RBG_MIXED runs the
 * caller's normals (read as FP32) through the tensor-core path kernel and
 * writes each path's FP32 payoff as double; NULL o or RBG_FP64: FP64. */
int rbg_payoffs_rt(const rbg_params* p, const rbg_options* o, const double* Z, double* payoff, int device_ptrs);

/* Plain Monte Carlo on the Philox stream (streams W1, W1perp, Wperp): the
 * estimator of computeIV_tensor with status codes.  FP64, or the mixed form
 * (tcgen05 GEMM for N <= 4096, or the batched FFT by option). */
int rbg_price_mc(const rbg_params* p, const rbg_options* o, double* price, double* stat, double* iv);

/* Plain Monte Carlo per-path payoffs for caller-supplied normals: Z holds
 * 3*N*M doubles, sample m uses Z[3mN + sN, 3mN + sN + N) for s = 0 (W1),
 * 1 (W1perp), 2 (Wperp); payoff[m*out + i].  Precision as rbg_payoffs_rt. */
int rbg_payoffs_mc(const rbg_params* p, const rbg_options* o, const double* Z, double* payoff, int device_ptrs);

/* Writes the normals the pricer would draw for paths
 * [path_offset, path_offset + M), N steps, streams W1 and W1perp, in the
 * quadrature layout (M * 2 * N doubles, host pointer).  precision selects the
 * FP64 or the FP32 transform (the latter widened exactly to double). */
int rbg_generate_normals(uint64_t seed, int64_t path_offset, int64_t M, int N, int precision, double* Z);
/* Same with 2 (RT) or 3 (plain MC: + Wperp) streams per path, M*streams*N doubles. */
int rbg_generate_normals_streams(uint64_t seed, int64_t path_offset, int64_t M, int N, int precision, int streams,
                                 double* Z);

/* ---- Sobol' quasi-Monte Carlo (rBergomi/rBergomiMT.cpp:610-715,
 * ComputePriceRTMT_sobol / ComputeIVRTMT_sobol, and their single-threaded
 * twins :717-805; rBergomi/qmc.cpp:25-38 normalQMC_sample).
 *
 * Path m (global index path_offset + m) takes Sobol' point m + 1 + path_offset
 * in dimension 2N; W1 = coordinates 0, 2, 4, ..., W1perp = 1, 3, 5, ...
 * (rBergomi/aux.h:186-191 breakZ), each through the FP64 normal quantile.
 * The caller supplies the direction integers, dims x 62 uint64 row-major:
 * coordinate d of point s is (XOR of directions[d*62 + k] over the set bits k
 * of s ^ (s >> 1)) * 2^-62, which is the point rBergomi/sobol.cpp i8_sobol
 * returns for seed s when given its own table (the integers v[d][k] after
 * its column scaling).  dims >= 2N; point indices stay below 2^62.  The
 * library ships no table.
 * bridge != 0 maps each stream through the Brownian-bridge ("hierarchical")
 * construction of rBergomi/aux.h:106-125 (N a power of two, N <= 8192).
 * The reference has no C export for these; this is the replacement for
 * linking its C++ functions. */

/* RT prices over Sobol' normals; the seed is unused, o->path_offset shifts
 * the point range.  stat is the reference's Monte Carlo formula applied to
 * the QMC sample.  o->precision == RBG_FP64: the FP64 form (normcdfinv),
 * bridge allowed.  RBG_MIXED: the tensor-core form on the same points, any
 * backend and N the mixed form takes.  Without the bridge its normals are the
 * FP32 quantile of each coordinate's top 32 bits: drawn by the GEMM kernel's
 * producer for N <= 1024 and point indices below 2^32, otherwise materialized
 * per batch on the device.  With the bridge those FP32 normals go through
 * the bridge in FP32 (materialized). */
int rbg_price_rt_sobol(const rbg_params* p, const rbg_options* o, const uint64_t* directions, int dims, int bridge,
                       double* price, double* stat, double* iv);
/* Failure-detection check (no counterpart in the reference): one warp waits,
 * with the pricing kernels' bounded-wait helper and a 20 ms limit, on an
 * mbarrier nothing arrives on.  Returns RBG_ERR_TIMEOUT with the expiring
 * wait's site in *site (as a stalled pipeline reports), leaving the context
 * usable. */
int rbg_debug_wait_timeout(unsigned int* site);

/* The Sobol' normals those prices use: M*2*N doubles in the quadrature
 * layout, host pointer.  precision RBG_FP64: normcdfinv of the 62-bit point;
 * RBG_MIXED: the mixed form's FP32 normals (top 32 bits of the point, FP32
 * quantile; with the bridge, the bridge in FP32), widened exactly to double. */
int rbg_sobol_normals(const uint64_t* directions, int dims, int N, int64_t M, int64_t path_offset, int bridge,
                      int precision, double* Z);

/* Implied vols of call prices (S0 = 1, r = 0) on the GPU; NaN where no
 * volatility reproduces the price. */
int rbg_implied_vol(int n, const double* price, const double* K, const double* T, double* iv);

/* Message for the last failing rbg_* call on this thread. */
const char* rbg_last_error(void);

/* Number of kernels this library has launched in this process. */
uint64_t rbg_launch_count(void);

/* Waits for the library's own stream on the current device (work a caller
 * queued on its own streams is the caller's to wait for). */
int rbg_synchronize(void);

/* Waits for the current device, then releases the cached device buffers and
 * tables of every context (one per caller stream) on it. */
int rbg_release(void);

/* Host-only introspection of the ParamTot plan (no GPU needed): the number
 * of distinct Volterra passes (H values), variance groups ((H, T, eta)
 * after the reference's trigger chain) and outputs; vgroup_of_output
 * (length par_size*op_size, may be NULL) receives each output's group. */
int rbg_plan_info(const rbg_params* p, int* n_vol, int* n_vgroups, int* n_out, int* vgroup_of_output);
/* Host-only plan of the plain Monte Carlo estimator: as rbg_plan_info, plus
 * the rho each output's S_T is computed with (the rho of the last
 * H/T/eta/rho trigger, eps 1e-10). */
int rbg_plan_info_mc(const rbg_params* p, int* n_vol, int* n_vgroups, int* vgroup_of_output, double* rho_of_output);
/* Host-only plan of an unordered list: Volterra passes and variance groups. */
int rbg_plan_info_unordered(const rbg_unordered* u, int* n_vol, int* n_vgroups, int* vgroup_of_output);

/* Stage timing: when enabled, CUDA events bracket each stage on the stream
 * that launches it (stage 0 normals, 1 FP64 path pass, 2 mixed tcgen05 path
 * kernel, 3 payoff sums, 4 chunk merge); rbg_profile_read returns the summed
 * milliseconds and kernel launches since the last reset. */
void rbg_profile_enable(int on);
void rbg_profile_reset(void);
int rbg_profile_read(int stage, double* total_ms, uint64_t* launches);

/* Host<->device bytes copied by this thread's last rbg_price_rt* call. */
void rbg_last_transfer_bytes(uint64_t* h2d, uint64_t* d2h);

/* Diagnostic run of the mixed-form path kernel on at most 2^20 paths with
 * the same arguments as rbg_price_rt: copies out the FP32 normals it drew
 * (normals: M * 2 * Np floats, Np = N rounded up to 32, [path][W1|W1perp][step]),
 * its X = Y2 + a1 W1 + a2 W1perp per step (x: M * Np) and its (Ivdt, IsvdW)
 * per variance group and path (ivb: 2 * n_vgroups * M, [group][path][2]).
 * Any output pointer may be NULL. */
int rbg_debug_mixed_paths(const rbg_params* p, const rbg_options* o, float* normals, float* x, float* ivb);

/* Diagnostic run of the mixed-form path kernel(s) over M paths (one batch)
 * with per-role cycle counters: cycles[site] = cycles lane 0 of each warp
 * spent waiting at a pipeline barrier (1 producer/empty, 2 epilogue/MMA
 * results, 3 strip load, 4 MMA/TMEM free, 5 MMA/A tile, 7 and 8 epilogue/
 * producer tiles), cycles[16..18] = busy cycles of producer, epilogue and
 * MMA warps, cycles[20] = epilogue cycles in the fused payoffs.  n >= 32. */
int rbg_debug_mixed_profile(const rbg_params* p, const rbg_options* o, uint64_t* cycles, int n);

/* ------------------------------------------------------------------------ */
/* Serving loop (no counterpart in the reference: its callers fan out over   */
/* console processes, rBergomiR/rbergomi_console.R:88-160)                  */
/* ------------------------------------------------------------------------ */

/* A persistent, continuously batched pricing loop.  Submitted requests are
 * admitted onto device slots (each with its own CUDA stream) as soon as a
 * slot and enough of the HBM budget are free, first fit in arrival order;
 * the footprint charged is M * N * 4 bytes plus the request's tables.  Small
 * requests (M*N*n_H <= small_request_path_steps) use high-priority streams;
 * large ones are cut into launches of at most max_batch_paths paths so they
 * yield the GPU between launches.  Volterra tables are cached on the device
 * per (backend, H, N, split).  With use_graphs, the device work of each
 * shared launch, and of each request of one launch, runs as a CUDA graph,
 * one executable per batch slot or launch shape, updated in place.  All
 * requests run the mixed form; results do not depend on what else is in
 * flight, nor on whether they ran alone or in a shared launch
 * (counter-based normals, per-request sums, the same per-path arithmetic). */
typedef struct rbg_server rbg_server;

typedef struct rbg_server_config {
    int slots;                       /* concurrent requests on the device (1..64) */
    int high_priority_slots;         /* of which on high-priority streams */
    uint64_t hbm_budget;             /* admission budget in bytes */
    int64_t max_batch_paths;         /* paths per kernel launch */
    double small_request_path_steps; /* threshold for the high-priority slots */
    int table_cache_entries;         /* device-resident Volterra tables kept */
    int use_graphs;                  /* launch each request as a CUDA graph */
    int device;                      /* CUDA device, -1 = current */
    /* Shared launches: requests one one-pass launch can price (N <= 512, at
     * most max_batch_paths paths, one distinct H) are gathered, all that are
     * pending when a batch slot frees up, into one job-table launch of the
     * path, payoff, merge and finalize kernels, replayed as one CUDA graph per
     * batch slot.  0 batch slots: every request alone on its own slot. */
    int batch_slots;                 /* shared launches in flight at once */
    int max_batch_jobs;              /* requests per shared launch (1..64) */
    double batch_path_steps;         /* path-steps per shared launch (a request larger than this still runs, alone) */
    double batch_wait_us;            /* a batch slot waits up to this long after the oldest pending request's
                                        submit for more requests (fewer than max_batch_jobs pending); 0: none */
} rbg_server_config;

typedef struct rbg_server_stats {
    uint64_t completed, failed, pending, in_flight, hbm_in_use;
    uint64_t table_cache_hits, table_cache_misses, graph_launches;
    uint64_t graph_instantiations, graph_updates; /* executable graphs built / updated in place */
    uint64_t max_launch_us;                       /* longest admission-to-launched time on the scheduler */
    uint64_t pin_growths;                         /* pinned result buffers regrown (a device-wide wait each) */
    uint64_t batches, batched_requests;           /* shared launches, and the requests they priced */
    /* longest scheduler-thread time of one launch in each phase (us): device
     * buffers, Volterra tables, uploads, graph capture + instantiate/update + launch */
    uint64_t max_alloc_us, max_tables_us, max_upload_us, max_graph_us;
} rbg_server_stats;

void rbg_server_default_config(rbg_server_config* cfg);
int rbg_server_create(const rbg_server_config* cfg, rbg_server** out);
/* Copies the request (parameters and options; precision is forced to mixed)
 * and returns a ticket at once. */
int rbg_server_submit(rbg_server* s, const rbg_params* p, const rbg_options* o, uint64_t* ticket);
/* done = 1 once the request's results are on the host. */
int rbg_server_poll(rbg_server* s, uint64_t ticket, int* done);
/* Blocks until the request is done, copies its prices, standard errors and
 * implied vols (any may be NULL) and the latency from submit to completion,
 * and forgets the ticket.  Returns the request's status. */
int rbg_server_wait(rbg_server* s, uint64_t ticket, double* price, double* stat, double* iv, double* latency_ms);
/* rbg_server_wait with the latency split: times[0] = submit to admission
 * (queueing), times[1] = admission to results on the host (service),
 * times[2] = their sum, all in ms (times may be NULL). */
int rbg_server_wait_timed(rbg_server* s, uint64_t ticket, double* price, double* stat, double* iv, double* times);
int rbg_server_get_stats(rbg_server* s, rbg_server_stats* st);
/* Finishes the queued work and frees the server. */
int rbg_server_destroy(rbg_server* s);
const char* rbg_server_last_error(void);

/* Allocation-free pricing.  No counterpart in the reference (it has no GPU).
 * For callers that cannot call cudaMalloc -- a host that reserved all device
 * memory for its own pool at start-up, or a latency-critical loop that cannot
 * take cudaMalloc's device-wide synchronisation.  Same arguments, kernels and
 * results as rbg_price_rt, mixed precision only (RBG_ERR_UNSUPPORTED
 * otherwise), but every scratch buffer lives in one 16 MiB file-scope device
 * array (rbg_static_scratch_bytes()) that each GPU loading the library holds
 * until exit; no device memory is allocated or freed.  Limits: at most 4096
 * outputs, and the job's tables must fit the array (RBG_ERR_ARG with a
 * message from rbg_static_last_error() otherwise); M is unbounded (paths are
 * processed in batches that fit, cut at the same payoff-chunk boundaries as
 * rbg_price_rt's, so prices agree to FP64 roundoff).  One exception: for
 * 512 < N <= 1024 with the 16-bit splits, rbg_price_rt's path kernel keeps
 * A tiles in a per-CTA device cache (tens of MB) that the array cannot hold,
 * so this entry runs the two-pass kernel that draws them again: the same
 * products in another FP32 accumulation order, prices equal to within about
 * 1e-6 relative.  A NULL o->stream runs
 * on the calling thread's per-thread default stream.  Every call
 * synchronises its stream before returning (it reads the results back), so
 * it cannot be recorded under stream capture.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); the address is
 * kept for the life of the process, so cudaDeviceReset between calls is not
 * supported.  All
 * calls share the array and see the previous call's contents; each call
 * clears what must start at zero.  Calls that overlap on the GPU race on the
 * array: serialise them.  A call that fails after queuing work waits for
 * that work before returning. */
int rbg_price_rt_static(const rbg_params* p, const rbg_options* o, double* price, double* stat, double* iv);
size_t rbg_static_scratch_bytes(void);
const char* rbg_static_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* RBERGOMI_GB300_H */
