/*
 * oracle_fft.h -- double-precision mixed-radix FFT used by the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file belongs to the oracle: it is the
 * checker for the GPU path and is never linked into the product library.
 *
 * The reference (FLCT 1.01, source/flct.c and source/warp.c) does all its
 * transforms through FFTW 3 (flct.c:27, warp.c:27; FFTW version unpinned,
 * README.md:104-113).  FFTW is not available here, so this is a
 * project-written restatement of the published Cooley-Tukey mixed-radix
 * algorithm with the same conventions FFTW documents:
 *   - unnormalised transforms, out[k] = sum_j in[j] * exp(sign*2*pi*i*j*k/n),
 *     sign = -1 (forward) or +1 (backward);
 *   - row-major 2-D arrays;
 *   - real-to-complex output of an n0 x n1 real array is the n0 x (n1/2+1)
 *     non-redundant half; complex-to-real consumes that half and treats it as
 *     Hermitian (the imaginary parts of the self-conjugate last-axis entries
 *     are ignored).
 * Complex arrays are interleaved (re, im) doubles.
 */
#ifndef ORACLE_FFT_H
#define ORACLE_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct offt_plan1d offt_plan1d;

/* Plan a length-n complex transform (any n >= 1). NULL on allocation failure. */
offt_plan1d *offt_plan1d_create(int n);
void offt_plan1d_destroy(offt_plan1d *p);
int offt_plan1d_len(const offt_plan1d *p);

/* out = DFT_sign(in), unnormalised.  in has stride istride (in complex
 * elements), out is contiguous.  in and out must not overlap. */
void offt_exec1d(const offt_plan1d *p, const double *in, int istride,
                 double *out, int sign);

/* 2-D helpers (row-major, n0 slow, n1 fast).  They allocate their own
 * scratch; return 0 on success, nonzero on allocation failure. */
int offt_c2c_2d(int n0, int n1, const double *in, double *out, int sign);
int offt_r2c_2d(int n0, int n1, const double *in, double *out);
int offt_c2r_2d(int n0, int n1, const double *in, double *out);

/* Reusable 2-D context: plans and scratch for one (n0, n1) pair, so that the
 * per-window transforms of the velocity loop do not allocate. */
typedef struct offt_ctx2d offt_ctx2d;
offt_ctx2d *offt_ctx2d_create(int n0, int n1);
void offt_ctx2d_destroy(offt_ctx2d *c);
void offt_ctx2d_c2c(offt_ctx2d *c, const double *in, double *out, int sign);
void offt_ctx2d_r2c(offt_ctx2d *c, const double *in, double *out);
void offt_ctx2d_c2r(offt_ctx2d *c, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
