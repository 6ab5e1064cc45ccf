/*
 * fftw3.h -- minimal, from-scratch stand-in for the FFTW3 API subset the
 * reference rBergLib sources call (fftw_complex, fftw_plan_dft_1d,
 * fftw_execute, FFTW_FORWARD/BACKWARD, FFTW_ESTIMATE).  TEST INFRASTRUCTURE:
 * it exists only so oracle/Makefile (target `ref`) can compile the unmodified reference
 * sources into oracle/_ref/ on a machine without FFTW.
 *
 * Semantics follow FFTW's documented unnormalised complex DFT of arbitrary
 * length n:  out[k] = sum_j in[j] * exp(sign * 2*pi*i * j*k / n).
 * The implementation (fftw_shim.c) is Bluestein's chirp-z algorithm around a
 * radix-2 FFT, so lengths like 2N-1 = 199 are exact DFTs, not padded ones.
 */
#ifndef RBG_FFTW3_SHIM_H
#define RBG_FFTW3_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct rbg_fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif

#endif
