/*
 * fftw_shim.c -- FFTW-API subset on top of the oracle FFT (see fftw3.h).
 * TEST INFRASTRUCTURE ONLY: linked only into oracle/_ref builds of the
 * unmodified reference sources.
 */
#include "fftw3.h"
#include "../oracle_fft.h"

#include <stdlib.h>

enum { OSHIM_R2C, OSHIM_C2R, OSHIM_C2C };

struct oshim_plan_s {
    int kind, n0, n1, sign;
    void *in, *out;
    offt_ctx2d *ctx;
};

void *fftw_malloc(size_t n) { return malloc(n ? n : 1); }
void fftw_free(void *p) { free(p); }

static fftw_plan mk(int kind, int n0, int n1, void *in, void *out, int sign)
{
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->kind = kind;
    p->n0 = n0;
    p->n1 = n1;
    p->in = in;
    p->out = out;
    p->sign = sign;
    p->ctx = offt_ctx2d_create(n0, n1);
    if (!p->ctx) { free(p); return NULL; }
    return p;
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags)
{
    (void)flags;
    return mk(OSHIM_R2C, n0, n1, in, out, FFTW_FORWARD);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags)
{
    (void)flags;
    return mk(OSHIM_C2R, n0, n1, in, out, FFTW_BACKWARD);
}

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags)
{
    (void)flags;
    return mk(OSHIM_C2C, n0, n1, in, out, sign);
}

void fftw_execute(const fftw_plan p)
{
    if (!p) return;
    switch (p->kind) {
    case OSHIM_R2C:
        offt_ctx2d_r2c(p->ctx, (const double *)p->in, (double *)p->out);
        break;
    case OSHIM_C2R:
        offt_ctx2d_c2r(p->ctx, (const double *)p->in, (double *)p->out);
        break;
    default:
        offt_ctx2d_c2c(p->ctx, (const double *)p->in, (double *)p->out, p->sign);
        break;
    }
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    offt_ctx2d_destroy(p->ctx);
    free(p);
}
