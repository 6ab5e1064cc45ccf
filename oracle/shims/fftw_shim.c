/*
 * fftw_shim.c -- Bluestein DFT behind the FFTW-API shim (shims/fftw3.h).
 * TEST INFRASTRUCTURE for building the reference in oracle/_ref/.
 *
 * Arbitrary n:  X[k] = c[k] * sum_j (x[j] c[j]) * conj(c[k-j]),
 * c[m] = exp(sign * i*pi * m^2 / n), the convolution done with power-of-two
 * radix-2 FFTs of length L >= 2n-1.  Each plan owns its scratch, so distinct
 * plans may execute concurrently (the reference runs one plan per OpenMP
 * thread).
 */
#include "fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct rbg_fftw_plan_s {
    int n, sign, L;
    double (*in)[2];
    double (*out)[2];
    double* chirp;  /* 2n: c[m] for m in [0,n) */
    double* filt;   /* 2L: FFT of conj(c) placed circularly */
    double* work;   /* 2L */
    double* tw;     /* 2*(L/2) twiddles exp(-2 pi i t / L) */
};

static void fft_pow2(double* a, int L, const double* tw, int inverse)
{
    /* iterative radix-2, bit reversal first */
    for (int i = 1, j = 0; i < L; ++i) {
        int bit = L >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = a[2 * i], ti = a[2 * i + 1];
            a[2 * i] = a[2 * j]; a[2 * i + 1] = a[2 * j + 1];
            a[2 * j] = tr; a[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= L; len <<= 1) {
        int half = len >> 1, step = L / len;
        for (int s = 0; s < L; s += len) {
            for (int k = 0; k < half; ++k) {
                double wr = tw[2 * k * step], wi = tw[2 * k * step + 1];
                if (inverse) wi = -wi;
                double* u = a + 2 * (s + k);
                double* v = a + 2 * (s + k + half);
                double xr = v[0] * wr - v[1] * wi;
                double xi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - xr; v[1] = u[1] - xi;
                u[0] += xr; u[1] += xi;
            }
        }
    }
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags)
{
    (void)flags;
    struct rbg_fftw_plan_s* p = (struct rbg_fftw_plan_s*)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->n = n; p->sign = sign; p->in = in; p->out = out;
    int L = 1;
    while (L < 2 * n - 1) L <<= 1;
    if (L < 2) L = 2;
    p->L = L;
    p->chirp = (double*)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    p->filt = (double*)calloc(2 * (size_t)L, sizeof(double));
    p->work = (double*)malloc(sizeof(double) * 2 * (size_t)L);
    p->tw = (double*)malloc(sizeof(double) * (size_t)L);
    const double pi = 3.14159265358979323846;
    for (int t = 0; t < L / 2; ++t) {
        p->tw[2 * t] = cos(-2.0 * pi * t / L);
        p->tw[2 * t + 1] = sin(-2.0 * pi * t / L);
    }
    for (int m = 0; m < n; ++m) {
        /* m^2 mod 2n keeps the angle argument small and exact */
        long long q = ((long long)m * m) % (2LL * n);
        double ang = sign * pi * (double)q / n;
        p->chirp[2 * m] = cos(ang);
        p->chirp[2 * m + 1] = sin(ang);
    }
    for (int m = 0; m < n; ++m) {
        double cr = p->chirp[2 * m], ci = -p->chirp[2 * m + 1]; /* conj(c[m]) */
        p->filt[2 * m] = cr; p->filt[2 * m + 1] = ci;
        if (m > 0) { p->filt[2 * (L - m)] = cr; p->filt[2 * (L - m) + 1] = ci; }
    }
    fft_pow2(p->filt, L, p->tw, 0);
    return p;
}

void fftw_execute(const fftw_plan p)
{
    int n = p->n, L = p->L;
    double* w = p->work;
    memset(w, 0, sizeof(double) * 2 * (size_t)L);
    for (int j = 0; j < n; ++j) {
        double xr = p->in[j][0], xi = p->in[j][1];
        double cr = p->chirp[2 * j], ci = p->chirp[2 * j + 1];
        w[2 * j] = xr * cr - xi * ci;
        w[2 * j + 1] = xr * ci + xi * cr;
    }
    fft_pow2(w, L, p->tw, 0);
    for (int t = 0; t < L; ++t) {
        double ar = w[2 * t], ai = w[2 * t + 1];
        double br = p->filt[2 * t], bi = p->filt[2 * t + 1];
        w[2 * t] = ar * br - ai * bi;
        w[2 * t + 1] = ar * bi + ai * br;
    }
    fft_pow2(w, L, p->tw, 1);
    double inv = 1.0 / L;
    for (int k = 0; k < n; ++k) {
        double yr = w[2 * k] * inv, yi = w[2 * k + 1] * inv;
        double cr = p->chirp[2 * k], ci = p->chirp[2 * k + 1];
        p->out[k][0] = yr * cr - yi * ci;
        p->out[k][1] = yr * ci + yi * cr;
    }
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    free(p->chirp); free(p->filt); free(p->work); free(p->tw);
    free(p);
}
