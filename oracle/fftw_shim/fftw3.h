/*
 * fftw3.h -- project-written stand-in for the subset of the FFTW 3 C API that
 * FLCT 1.01 calls (source/flct.c:1380-1419, 1435-1436, 1481, 1494-1505;
 * source/warp.c:772-783, 806, 855, 866-875, 899-909, 934, 1000-1008).
 *
 * TEST INFRASTRUCTURE ONLY.  It exists so the unmodified reference sources
 * can be compiled in place as an oracle (FFTW itself is not installed and
 * cannot be fetched).  The names, types and flag values must match FFTW's
 * public API for the reference to compile unchanged; the transforms behind
 * them are the project's own double-precision FFT (oracle_fft.c).
 */
#ifndef ORACLE_FFTW_SHIM_H
#define ORACLE_FFTW_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct oshim_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
