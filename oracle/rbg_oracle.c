/*
 * rbg_oracle.c -- CPU oracle for the rough Bergomi Romano-Touzi pricer.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference rBergLib arithmetic, used by tests/, by the smoke check and by the
 * CPU-baseline leg of bench.py as the checker.  The product library
 * (rbergomi_gb300/) never links, loads or calls it.
 *
 * Parity pins (see tests/test_oracle_cpu.py):
 *   - the 200 per-path payoffs of the reference dump rBergomi/testing/debug8.txt~
 *     (deterministic inputs W1 = W1perp = cos(i*m)), reproduced to the dump's
 *     6 printed digits;
 *   - the reference library itself, compiled from its own sources against
 *     from-scratch FFTW/Boost shims (the `ref` target of oracle/Makefile), on seeded normals;
 *     the outputs of that build are frozen in tests/golden/.
 *
 * Every function cites the reference file:line it restates.  The one deliberate
 * difference: the Volterra convolution is a direct causal sum (k ascending)
 * instead of the reference's FFTW product of three length-(2N-1) DFTs; both are
 * the same linear convolution, differing only in roundoff (~1e-15 relative).
 *
 * The Philox4x32-10 normal generator below is NOT from the reference (which
 * uses std::mt19937_64 + std::normal_distribution); it restates the counter
 * layout of this project's GPU generator (Salmon et al., "Parallel random
 * numbers: as easy as 1, 2, 3", SC'11) so tests can regenerate its stream.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_SQRT1_2
#define M_SQRT1_2 0.70710678118654752440
#endif

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al. SC'11) and the project's normal layout.      */
/* ------------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void rbgo_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Seed folding used by the drop-in ABI: one 64-bit Philox key from the
 * caller's seed array (splitmix64 finaliser between words). */
static uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

uint64_t rbgo_fold_seed(const uint64_t* seed, int seed_size)
{
    if (seed_size <= 0 || !seed) return 0;
    uint64_t h = seed[0];
    for (int i = 1; i < seed_size; ++i) h = splitmix64(h + seed[i]);
    return h;
}

/* FP64 normals of stream s (0 = W1, 1 = W1perp, 2 = Wperp) for paths
 * [path0, path0+M), N steps each.  Layout: Z[((m * nstreams) + s) * N + j],
 * i.e. per path W1[0..N) then W1perp[0..N) (then Wperp), which is the
 * reference quadrature layout (rBergLib/cinterface.cpp:116-119).
 * Counter (g, path_lo, path_hi, s) for steps 4g..4g+3; key = seed. */
void rbgo_normals_f64(uint64_t seed, int64_t path0, int64_t M, int N, int nstreams, double* Z)
{
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const double two32i = 2.3283064365386963e-10; /* 2^-32 */
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < M; ++m) {
        uint64_t p = (uint64_t)(path0 + m);
        for (int s = 0; s < nstreams; ++s) {
            double* z = Z + ((size_t)m * nstreams + s) * (size_t)N;
            for (int g = 0; 4 * g < N; ++g) {
                uint32_t ctr[4] = {(uint32_t)g, (uint32_t)p, (uint32_t)(p >> 32), (uint32_t)s};
                uint32_t x[4];
                rbgo_philox4x32_10(ctr, key, x);
                double u0 = ((double)x[0] + 0.5) * two32i, u1 = ((double)x[1] + 0.5) * two32i;
                double u2 = ((double)x[2] + 0.5) * two32i, u3 = ((double)x[3] + 0.5) * two32i;
                double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
                double v[4] = {r0 * cos(2.0 * M_PI * u1), r0 * sin(2.0 * M_PI * u1),
                               r1 * cos(2.0 * M_PI * u3), r1 * sin(2.0 * M_PI * u3)};
                for (int q = 0; q < 4 && 4 * g + q < N; ++q) z[4 * g + q] = v[q];
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Black-Scholes pieces: rBergLib/BlackScholes.cpp:11-21.                    */
/* ------------------------------------------------------------------------ */
static double Phi(double x) { return 0.5 * erfc(-x * M_SQRT1_2); } /* BlackScholes.cpp:11-14 */

double rbgo_bs_call(double S0, double K, double tau, double sigma) /* BlackScholes.cpp:16-21, r = 0 */
{
    double d1 = (log(S0 / K) + (0.5 * sigma * sigma) * tau) / (sigma * sqrt(tau));
    double d2 = d1 - sigma * sqrt(tau);
    return Phi(d1) * S0 - Phi(d2) * K;
}

static double bs_put(double S0, double K, double tau, double sigma) /* BlackScholes.cpp:24-28, r = 0 */
{
    double d1 = (log(S0 / K) + (0.5 * sigma * sigma) * tau) / (sigma * sqrt(tau));
    double d2 = d1 - sigma * sqrt(tau);
    return -Phi(-d1) * S0 + Phi(-d2) * K;
}

/* Implied volatility of a call (S0 = 1, r = 0).  The reference inverts with
 * Boost's bracket_and_solve_root to 2^-10 relative (BlackScholes.cpp:36-63,
 * put-call parity for ITM at :38-41).  This is the project's FP64 inversion
 * (same root, to ~1e-14): out-of-the-money side by put-call parity, bracket by
 * doubling, then Newton steps on log(price) -- nearly linear in the deep wings
 * where Newton on the price itself crawls -- safeguarded by bisection.  NaN
 * when no root exists. */
double rbgo_iv_call(double price, double K, double T)
{
    const double S0 = 1.0;
    int use_put = S0 > K;
    double target = use_put ? price - S0 + K : price;
    double lower_bound = 0.0, upper_bound = use_put ? K : S0;
    if (!(target > lower_bound) || !(target < upper_bound) || !(T > 0.0)) return NAN;
    double lo = 0.0, hi = 0.5;
    for (int it = 0; it < 60; ++it) {
        double p = use_put ? bs_put(S0, K, T, hi) : rbgo_bs_call(S0, K, T, hi);
        if (p >= target) break;
        lo = hi;
        hi *= 2.0;
    }
    double ltarget = log(target);
    double s = 0.5 * (lo + hi);
    for (int it = 0; it < 200; ++it) {
        double p = use_put ? bs_put(S0, K, T, s) : rbgo_bs_call(S0, K, T, s);
        if (p > target) hi = s; else lo = s;
        double sn;
        if (p > 0.0) {
            double d1 = (log(S0 / K) + 0.5 * s * s * T) / (s * sqrt(T));
            double vega = S0 * exp(-0.5 * d1 * d1) * 0.39894228040143267794 * sqrt(T);
            sn = s - (log(p) - ltarget) * p / vega;
        } else {
            sn = 0.5 * (lo + hi);
        }
        if (!(sn > lo && sn < hi)) sn = 0.5 * (lo + hi);
        if (fabs(sn - s) <= 1e-15 * s || hi - lo <= 1e-15 * hi) { s = sn; break; }
        s = sn;
    }
    return s;
}

/* ------------------------------------------------------------------------ */
/* Path kernels: rBergLib/rBergomiMT.cpp.                                   */
/* ------------------------------------------------------------------------ */

/* getGamma, rBergLib/rBergomiMT.cpp:143-149 (b* kernel of the hybrid scheme). */
void rbgo_gamma(double H, int N, double* G)
{
    double alpha = H - 0.5;
    G[0] = 0.0;
    for (int i = 1; i < N; ++i)
        G[i] = (pow(i + 1.0, alpha + 1.0) - pow(i, alpha + 1.0)) / (alpha + 1.0);
}

/* updateWtilde, rBergLib/rBergomiMT.cpp:83-109.  Y2 = (W1 * Gamma)[0..N) as a
 * direct causal sum in axpy order (for every Y2[j] the terms are added with k
 * ascending), then Wtilde = c*Y2 + c*W1hat with c = sqrt(2H) N^-H. */
static void wtilde(double* Wt, const double* W1, const double* W1perp, const double* G,
                   double H, int N, double* Y2)
{
    double s2H = sqrt(2.0 * H);
    double rhoH = s2H / (H + 0.5);
    double a1 = rhoH / s2H, a2 = sqrt(1.0 - rhoH * rhoH) / s2H;
    for (int j = 0; j < N; ++j) Y2[j] = 0.0;
    for (int k = 0; k < N; ++k) {
        double w = W1[k];
        const double* g = G - k;
        for (int j = k + 1; j < N; ++j) Y2[j] += w * g[j];
    }
    double c = sqrt(2.0 * H) * pow(1.0 / N, H);
    for (int j = 0; j < N; ++j) {
        double w1hat = a1 * W1[j] + a2 * W1perp[j];
        Wt[j] = c * Y2[j] + c * w1hat;
    }
}

/* updateV, rBergLib/rBergomiMT.cpp:73-80 -- note the ((i-1) dt)^{2H}
 * compensator of the reference. */
static void update_v(double* v, const double* WS, double xi, double H, double eta, double dt, int N)
{
    v[0] = xi;
    for (int i = 1; i < N; ++i)
        v[i] = xi * exp(eta * WS[i - 1] - 0.5 * eta * eta * pow((i - 1) * dt, 2 * H));
}

/* ParamTot index map and triggers, rBergLib/ParamTot.h:28-43 (eps 1e-10,
 * rBergLib/ParamTot.cpp:27). */
typedef struct {
    const double *H, *eta, *rho, *T, *K;
    long P, O;
} partot;
#define PT_EPS 0.0000000001
static double pH(const partot* p, long I) { return p->H[I / p->O]; }
static double pEta(const partot* p, long I) { return p->eta[I / p->O]; }
static double pRho(const partot* p, long I) { return p->rho[I / p->O]; }
static double pT(const partot* p, long I) { return p->T[I % p->O]; }
static double pK(const partot* p, long I) { return p->K[I % p->O]; }
static int trigH(const partot* p, long I) { return I == 0 || fabs(pH(p, I) - pH(p, I - 1)) > PT_EPS; }
static int trigEta(const partot* p, long I) { return I == 0 || fabs(pEta(p, I) - pEta(p, I - 1)) > PT_EPS; }
static int trigRho(const partot* p, long I) { return I == 0 || fabs(pRho(p, I) - pRho(p, I - 1)) > PT_EPS; }
static int trigT(const partot* p, long I) { return I == 0 || fabs(pT(p, I) - pT(p, I - 1)) > PT_EPS; }

/* RT payoffs for every sample and ParamTot index: ComputePayoffRTsamples_ST,
 * rBergLib/rBergomiMT.cpp:528-610 (same trigger chain, same arithmetic),
 * parallel over samples with private buffers.  Z in the quadrature layout
 * (rBergLib/cinterface.cpp:116-119); payoff[m*out + i] (cinterface.cpp:127-130). */
int rbgo_payoffs_rt(double xi, const double* H, const double* eta, const double* rho, int P,
                    const double* T, const double* K, int O, int N, int64_t M, const double* Z,
                    int nthreads, double* payoff)
{
    partot pt = {H, eta, rho, T, K, P, O};
    long out = (long)P * O;
    double* G = (double*)malloc(sizeof(double) * (size_t)N * (size_t)P);
    if (!G) return -1;
    for (int q = 0; q < P; ++q) rbgo_gamma(H[q], N, G + (size_t)q * N);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int fail = 0;
#pragma omp parallel
    {
        double* buf = (double*)malloc(sizeof(double) * (size_t)N * 4);
        if (!buf) {
#pragma omp atomic write
            fail = 1;
        } else {
            double *Wt = buf, *WS = buf + N, *v = buf + 2 * N, *Y2 = buf + 3 * N;
#pragma omp for schedule(static)
            for (int64_t m = 0; m < M; ++m) {
                const double* W1 = Z + (size_t)(2 * m) * N;
                const double* W1perp = Z + (size_t)(2 * m + 1) * N;
                double dt = 0.0, sdt = 0.0;
                for (long i = 0; i < out; ++i) {
                    int update = trigH(&pt, i);
                    if (update) {
                        const double* g = NULL;
                        for (int q = 0; q < P; ++q)
                            if (H[q] == pH(&pt, i)) { g = G + (size_t)q * N; break; }
                        wtilde(Wt, W1, W1perp, g, pH(&pt, i), N, Y2);
                    }
                    update = update || trigT(&pt, i);
                    if (update) { /* scaleWtilde, rBergomiMT.cpp:163-167 */
                        for (int j = 0; j < N; ++j) WS[j] = pow(pT(&pt, i), pH(&pt, i)) * Wt[j];
                        dt = pT(&pt, i) / N;
                        sdt = sqrt(dt);
                    }
                    update = update || trigEta(&pt, i);
                    if (update) update_v(v, WS, xi, pH(&pt, i), pEta(&pt, i), dt, N);
                    /* intVdt / intRootVdW, rBergomiMT.cpp:427-436 */
                    double acc = 0.0;
                    for (int j = 0; j < N; ++j) acc += v[j];
                    double Ivdt = dt * acc;
                    double IsvdW = 0.0;
                    for (int j = 0; j < N; ++j) IsvdW += sqrt(v[j]) * sdt * W1[j];
                    /* conditional BS price, rBergomiMT.cpp:598-602 */
                    double r = pRho(&pt, i);
                    double vol = sqrt((1.0 - r * r) * Ivdt);
                    double spot = exp(-0.5 * r * r * Ivdt + r * IsvdW);
                    payoff[(size_t)m * out + i] = rbgo_bs_call(spot, pK(&pt, i), 1.0, vol);
                }
            }
            free(buf);
        }
    }
    free(G);
    return fail ? -1 : 0;
}

/* Plain Monte Carlo payoffs max(S-K,0): ComputePriceMT's per-sample body,
 * rBergLib/rBergomiMT.cpp:231-267 (rho trigger -> Z = rho W1 + sqrt(1-rho^2)
 * Wperp, S = exp(sum sqrt(v) sdt Z - v dt / 2)).  Z holds three streams per
 * path: W1, W1perp, Wperp. */
int rbgo_payoffs_mc(double xi, const double* H, const double* eta, const double* rho, int P,
                    const double* T, const double* K, int O, int N, int64_t M, const double* Z,
                    int nthreads, double* payoff)
{
    partot pt = {H, eta, rho, T, K, P, O};
    long out = (long)P * O;
    double* G = (double*)malloc(sizeof(double) * (size_t)N * (size_t)P);
    if (!G) return -1;
    for (int q = 0; q < P; ++q) rbgo_gamma(H[q], N, G + (size_t)q * N);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int fail = 0;
#pragma omp parallel
    {
        double* buf = (double*)malloc(sizeof(double) * (size_t)N * 4);
        if (!buf) {
#pragma omp atomic write
            fail = 1;
        } else {
            double *Wt = buf, *WS = buf + N, *v = buf + 2 * N, *Y2 = buf + 3 * N;
#pragma omp for schedule(static)
            for (int64_t m = 0; m < M; ++m) {
                const double* W1 = Z + (size_t)(3 * m) * N;
                const double* W1perp = Z + (size_t)(3 * m + 1) * N;
                const double* Wperp = Z + (size_t)(3 * m + 2) * N;
                double dt = 0.0, sdt = 0.0, S = 0.0;
                for (long i = 0; i < out; ++i) {
                    int update = trigH(&pt, i);
                    if (update) {
                        const double* g = NULL;
                        for (int q = 0; q < P; ++q)
                            if (H[q] == pH(&pt, i)) { g = G + (size_t)q * N; break; }
                        wtilde(Wt, W1, W1perp, g, pH(&pt, i), N, Y2);
                    }
                    update = update || trigT(&pt, i);
                    if (update) {
                        for (int j = 0; j < N; ++j) WS[j] = pow(pT(&pt, i), pH(&pt, i)) * Wt[j];
                        dt = pT(&pt, i) / N;
                        sdt = sqrt(dt);
                    }
                    update = update || trigEta(&pt, i);
                    if (update) update_v(v, WS, xi, pH(&pt, i), pEta(&pt, i), dt, N);
                    update = update || trigRho(&pt, i);
                    if (update) { /* updateZ, scaleZ, updateS: rBergomiMT.cpp:111-136 */
                        double r = pRho(&pt, i), rc = sqrt(1.0 - r * r);
                        double X = 0.0;
                        for (int j = 0; j < N; ++j) {
                            double zs = sdt * (r * W1[j] + rc * Wperp[j]);
                            X += sqrt(v[j]) * zs - 0.5 * v[j] * dt;
                        }
                        S = exp(X);
                    }
                    double d = S - pK(&pt, i);
                    payoff[(size_t)m * out + i] = d > 0 ? d : 0; /* posPart, rBergLib/aux.h:31-34 */
                }
            }
            free(buf);
        }
    }
    free(G);
    return fail ? -1 : 0;
}

/* Monte Carlo mean and standard error with the reference's formula,
 * rBergLib/rBergomiMT.cpp:404-409: price = sum/M, var = sum2/M - price^2,
 * stat = sqrt(var)/sqrt(M).  payoff[m*out + i]. */
void rbgo_reduce(const double* payoff, int64_t M, long out, double* price, double* stat)
{
    for (long i = 0; i < out; ++i) {
        double s = 0.0, s2 = 0.0;
        for (int64_t m = 0; m < M; ++m) {
            double x = payoff[(size_t)m * out + i];
            s += x;
            s2 += x * x;
        }
        double p = s * (1.0 / (double)M);
        double e2 = s2 * (1.0 / (double)M);
        double var = 1.0 * e2 + -1.0 * (p * p);
        price[i] = p;
        stat[i] = sqrt(var) * (1.0 / sqrt((double)M));
    }
}

/* Whole RT pricing on the project's Philox normals, processed in path blocks
 * so host memory stays bounded (CPU baseline and statistical checks). */
int rbgo_price_rt_philox(double xi, const double* H, const double* eta, const double* rho, int P,
                         const double* T, const double* K, int O, int N, int64_t M, uint64_t seed,
                         int nthreads, double* price, double* stat, double* sum, double* sum2)
{
    long out = (long)P * O;
    const int64_t B = 8192;
    double* Z = (double*)malloc(sizeof(double) * (size_t)B * 2 * N);
    double* pay = (double*)malloc(sizeof(double) * (size_t)B * out);
    if (!Z || !pay) { free(Z); free(pay); return -1; }
    for (long i = 0; i < out; ++i) { sum[i] = 0.0; sum2[i] = 0.0; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int64_t m0 = 0; m0 < M; m0 += B) {
        int64_t nb = (M - m0 < B) ? M - m0 : B;
        rbgo_normals_f64(seed, m0, nb, N, 2, Z);
        if (rbgo_payoffs_rt(xi, H, eta, rho, P, T, K, O, N, nb, Z, nthreads, pay)) {
            free(Z); free(pay); return -1;
        }
        for (int64_t m = 0; m < nb; ++m)
            for (long i = 0; i < out; ++i) {
                double x = pay[(size_t)m * out + i];
                sum[i] += x;
                sum2[i] += x * x;
            }
    }
    for (long i = 0; i < out; ++i) {
        double p = sum[i] * (1.0 / (double)M);
        double var = sum2[i] * (1.0 / (double)M) - p * p;
        price[i] = p;
        stat[i] = sqrt(var) * (1.0 / sqrt((double)M));
    }
    free(Z);
    free(pay);
    return 0;
}

int rbgo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * Romano-Touzi estimator with the control variate of McCrickerd & Pakkanen
 * and antithetic paths, as ML_console_ST implements it for an unordered
 * parameter list (xi, H, eta, rho, T, K per tuple):
 *   computeIvdtIsvdW         ML_console_ST/RBergomi.cpp:464-476, with updateV's
 *                            (i dt)^{2H} compensator (:365-372; rBergLib uses i-1)
 *   estimateControlVariate   :493-540 -- pilot paths: Q_i = max_m 2 Ivdt_im,
 *                            X = BS(S, K, 1, sqrt((1-rho^2) Ivdt)),
 *                            Y = BS(S, K, 1, sqrt(rho^2 (Q - Ivdt))),
 *                            alpha_i = -cov(X, Y) / cov(Y, Y) (aux.h:206-220)
 *   ComputePriceRTVarRed     :218-289 -- per main path the mean of the payoff
 *                            X + alpha Y at W and at -W; Y takes Qmax where
 *                            Q <= Ivdt (counted, over both halves, and
 *                            divided by M); price -= alpha ((1 - p) BS(1, K, 1,
 *                            sqrt(rho^2 Q)) + p BS(1, K, 1, sqrt(rho^2 Qmax)))
 * Normals: Zc [Mc][2][N] pilot, Z [M][2][N] main.  Outputs per tuple: the
 * adjusted price, stat (of the unadjusted payoffs, as the reference), alpha,
 * Q and the exception count.
 * ------------------------------------------------------------------------- */
static void ivdt_isvdw_ml(double xi, double H, double eta, double T, int N, const double* W1,
                          const double* W1perp, const double* G, double sgn, double* buf, double* Ivdt,
                          double* IsvdW)
{
    double *w1 = buf, *w1p = buf + N, *Wt = buf + 2 * N, *Y2 = buf + 3 * N, *v = buf + 4 * N;
    for (int j = 0; j < N; ++j) { w1[j] = sgn * W1[j]; w1p[j] = sgn * W1perp[j]; }
    wtilde(Wt, w1, w1p, G, H, N, Y2);
    const double dt = T / N, sdt = sqrt(dt), tH = pow(T, H);
    v[0] = xi;
    for (int i = 1; i < N; ++i)
        v[i] = xi * exp(eta * (tH * Wt[i - 1]) - 0.5 * eta * eta * pow(i * dt, 2 * H));
    double a = 0.0, b = 0.0;
    for (int j = 0; j < N; ++j) a += v[j];
    for (int j = 0; j < N; ++j) b += sqrt(v[j]) * sdt * w1[j];
    *Ivdt = dt * a;
    *IsvdW = b;
}

static double rt_spot(double rho, double Ivdt, double IsvdW)
{
    return exp(-0.5 * rho * rho * Ivdt + rho * IsvdW);
}

int rbgo_price_rt_cv(long n, const double* xi, const double* H, const double* eta, const double* rho,
                     const double* T, const double* K, int N, int64_t Mc, const double* Zc, int64_t M,
                     const double* Z, double Qmax, int nthreads, double* price, double* stat, double* alpha,
                     double* Q, int64_t* count)
{
    double* G = (double*)malloc(sizeof(double) * (size_t)N * (size_t)n);
    double* piv = (double*)malloc(sizeof(double) * 2 * (size_t)n * (size_t)Mc);
    if (!G || !piv) { free(G); free(piv); return -1; }
    for (long i = 0; i < n; ++i) rbgo_gamma(H[i], N, G + (size_t)i * N);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int fail = 0;
    /* pilot integrals */
#pragma omp parallel
    {
        double* buf = (double*)malloc(sizeof(double) * 5 * (size_t)N);
        if (!buf) {
#pragma omp atomic write
            fail = 1;
        } else {
#pragma omp for schedule(static)
            for (int64_t m = 0; m < Mc; ++m)
                for (long i = 0; i < n; ++i) {
                    const double* z = Zc + (size_t)m * 2 * N;
                    ivdt_isvdw_ml(xi[i], H[i], eta[i], T[i], N, z, z + N, G + (size_t)i * N, 1.0, buf,
                                  &piv[((size_t)i * Mc + m) * 2], &piv[((size_t)i * Mc + m) * 2 + 1]);
                }
            free(buf);
        }
    }
    if (fail) { free(G); free(piv); return -1; }
    for (long i = 0; i < n; ++i) {
        const double* pv = piv + (size_t)i * Mc * 2;
        double q = 0.0;
        for (int64_t m = 0; m < Mc; ++m) q = fmax(q, 2 * pv[2 * m]);
        Q[i] = q;
        double r = rho[i], mx = 0.0, my = 0.0;
        double* X = (double*)malloc(sizeof(double) * 2 * (size_t)Mc);
        if (!X) { free(G); free(piv); return -1; }
        double* Y = X + Mc;
        for (int64_t m = 0; m < Mc; ++m) {
            const double iv = pv[2 * m], iw = pv[2 * m + 1], s = rt_spot(r, iv, iw);
            X[m] = rbgo_bs_call(s, K[i], 1.0, sqrt((1.0 - r * r) * iv));
            Y[m] = rbgo_bs_call(s, K[i], 1.0, sqrt(r * r * (q - iv)));
            mx += X[m];
            my += Y[m];
        }
        mx /= (double)Mc;
        my /= (double)Mc;
        double cxy = 0.0, cyy = 0.0;
        for (int64_t m = 0; m < Mc; ++m) {
            cxy += (X[m] - mx) * (Y[m] - my);
            cyy += (Y[m] - my) * (Y[m] - my);
        }
        alpha[i] = -(cxy / (double)(Mc - 1)) / (cyy / (double)(Mc - 1));
        free(X);
    }
    free(piv);
    /* main paths, antithetic pairs */
    double* s1 = (double*)calloc((size_t)n, sizeof(double));
    double* s2 = (double*)calloc((size_t)n, sizeof(double));
    int64_t* cnt = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    if (!s1 || !s2 || !cnt) { free(G); free(s1); free(s2); free(cnt); return -1; }
#pragma omp parallel
    {
        double* buf = (double*)malloc(sizeof(double) * 5 * (size_t)N);
        double* l1 = (double*)calloc((size_t)n, sizeof(double));
        double* l2 = (double*)calloc((size_t)n, sizeof(double));
        int64_t* lc = (int64_t*)calloc((size_t)n, sizeof(int64_t));
        if (!buf || !l1 || !l2 || !lc) {
#pragma omp atomic write
            fail = 1;
        } else {
#pragma omp for schedule(static)
            for (int64_t m = 0; m < M; ++m) {
                const double* z = Z + (size_t)m * 2 * N;
                for (long i = 0; i < n; ++i) {
                    double pay = 0.0;
                    for (int h = 0; h < 2; ++h) {
                        double iv, iw;
                        ivdt_isvdw_ml(xi[i], H[i], eta[i], T[i], N, z, z + N, G + (size_t)i * N, h ? -1.0 : 1.0, buf,
                                      &iv, &iw);
                        const double r = rho[i], s = rt_spot(r, iv, iw);
                        const double x = rbgo_bs_call(s, K[i], 1.0, sqrt((1.0 - r * r) * iv));
                        const double vy = Q[i] > iv ? sqrt(r * r * (Q[i] - iv)) : sqrt(r * r * (Qmax - iv));
                        if (Q[i] <= iv) lc[i]++;
                        pay += 0.5 * (x + alpha[i] * rbgo_bs_call(s, K[i], 1.0, vy));
                    }
                    l1[i] += pay;
                    l2[i] += pay * pay;
                }
            }
#pragma omp critical
            for (long i = 0; i < n; ++i) { s1[i] += l1[i]; s2[i] += l2[i]; cnt[i] += lc[i]; }
        }
        free(buf); free(l1); free(l2); free(lc);
    }
    if (!fail) {
        for (long i = 0; i < n; ++i) {
            const double p = s1[i] * (1.0 / (double)M);
            const double var = 1.0 * (s2[i] * (1.0 / (double)M)) + -1.0 * (p * p);
            stat[i] = sqrt(var) * (1.0 / sqrt((double)M));
            const double pex = (double)cnt[i] / (double)M, r = rho[i];
            const double adj = (1.0 - pex) * rbgo_bs_call(1.0, K[i], 1.0, sqrt(r * r * Q[i])) +
                               pex * rbgo_bs_call(1.0, K[i], 1.0, sqrt(r * r * Qmax));
            price[i] = p - alpha[i] * adj;
            count[i] = cnt[i];
        }
    }
    free(G); free(s1); free(s2); free(cnt);
    return fail ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* Sobol' quasi-Monte Carlo normals.                                         */
/*   rBergomi/rBergomiMT.cpp:669-670 (ComputePriceRTMT_sobol): path m takes  */
/*     Sobol' point m+1 in dimension 2N, then breakZ;                        */
/*   rBergomi/qmc.cpp:21-38 (normalQMC_sample): i8_sobol, then the normal    */
/*     quantile of every coordinate (qmc.h:36-46);                           */
/*   rBergomi/sobol.cpp i8_sobol: Antonov-Saleev (Gray-code) order, point s  */
/*     = XOR of the scaled direction integers v[d][k] over the set bits k of */
/*     gray(s) = s ^ (s >> 1), times 2^-62;                                  */
/*   rBergomi/aux.h:186-191 (breakZ): W1 = even coordinates, W1perp = odd;   */
/*   rBergomi/aux.h:106-125 (hierarchical2increments): the Brownian-bridge   */
/*     (Haar) map of one N = 2^m vector, used per stream when asked.         */
/* The direction integers are the caller's: V[d * 62 + k].                   */
/* ------------------------------------------------------------------------ */
#define SOBOL_BITS 62

/* Normal quantile: Hastings' start (Abramowitz & Stegun 26.2.23), then three
 * Halley steps on Phi(x) = q in the lower tail.  Same steps as the oracle's
 * Boost stand-in (oracle/shims/boost/math/distributions/normal.hpp). */
double rbgo_inv_normal(double p)
{
    if (!(p > 0.0)) return p == 0.0 ? -INFINITY : NAN;
    if (!(p < 1.0)) return p == 1.0 ? INFINITY : NAN;
    const int upper = p > 0.5;
    const double q = upper ? 1.0 - p : p;
    const double t = sqrt(-2.0 * log(q));
    double x = -(t - (2.515517 + t * (0.802853 + t * 0.010328)) / (1.0 + t * (1.432788 + t * (0.189269 + t * 0.001308))));
    for (int i = 0; i < 3; ++i) {
        const double e = 0.5 * erfc(-x * 0.70710678118654752440) - q;
        const double u = e * 2.50662827463100050242 * exp(0.5 * x * x);
        x = x - u / (1.0 + 0.5 * x * u);
    }
    return upper ? -x : x;
}

/* Coordinates [0, dims) of Sobol' point s (rBergomi/sobol.cpp i8_sobol). */
void rbgo_sobol_point(const uint64_t* V, int dims, uint64_t s, double* x)
{
    const uint64_t g = s ^ (s >> 1);
    for (int d = 0; d < dims; ++d) {
        uint64_t q = 0;
        for (int k = 0; k < SOBOL_BITS; ++k)
            if ((g >> k) & 1u) q ^= V[(size_t)d * SOBOL_BITS + k];
        x[d] = (double)q * 2.168404344971008868e-19; /* 2^-62 */
    }
}

/* rBergomi/aux.h:106-125.  n must be 2^m; returns -1 otherwise. */
int rbgo_hier(const double* Z, int n, double* dW)
{
    int m = 0;
    while ((1 << m) < n) ++m;
    if ((1 << m) != n) return -1;
    for (int i = 0; i < n; ++i) {
        double w = exp2(-0.5 * m) * Z[0];
        for (int k = 1; k <= m; ++k) {
            const int i2nm = i >> (m - k); /* floor(i 2^(k-m)) */
            const int iota = (i2nm + 1) % 2;
            const int weight = 2 * iota - 1;
            const int index = (1 << (k - 1)) + (i2nm + iota + 1) / 2 - 1;
            w += exp2(0.5 * (k - m - 1)) * weight * Z[index];
        }
        dW[i] = w;
    }
    return 0;
}

/* Z[(m * 2 + s) * N + j] for paths [path0, path0 + M): point path0 + m + 1,
 * W1 (s = 0) = coordinates 0, 2, 4, ..., W1perp (s = 1) = 1, 3, 5, ...;
 * bridge: each stream through rbgo_hier.  Returns -1 on bad sizes. */
int rbgo_sobol_normals(const uint64_t* V, int dims, int N, int64_t path0, int64_t M, int bridge, double* Z)
{
    if (dims < 2 * N) return -1;
    if (bridge && (N & (N - 1))) return -1;
    int bad = 0;
#pragma omp parallel
    {
        double* x = (double*)malloc(sizeof(double) * 2 * (size_t)N);
        double* t = (double*)malloc(sizeof(double) * (size_t)N);
#pragma omp for schedule(static)
        for (int64_t m = 0; m < M; ++m) {
            rbgo_sobol_point(V, 2 * N, (uint64_t)(path0 + m + 1), x);
            double* z = Z + (size_t)m * 2 * N;
            for (int j = 0; j < N; ++j) {
                z[j] = rbgo_inv_normal(x[2 * j]);
                z[N + j] = rbgo_inv_normal(x[2 * j + 1]);
            }
            if (bridge) {
                for (int s = 0; s < 2; ++s) {
                    if (rbgo_hier(z + s * N, N, t)) bad = 1;
                    memcpy(z + s * N, t, sizeof(double) * N);
                }
            }
        }
        free(x);
        free(t);
    }
    return bad ? -1 : 0;
}
