/*
 * oracle_fft.c -- double-precision mixed-radix FFT for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle_fft.h).  Recursive decimation-in-time
 * Cooley-Tukey: n = r * m, the r interleaved length-m sub-sequences are
 * transformed recursively, then combined with twiddles W_n^{q k} and r-point
 * butterflies.  Radix 4, 2 and 3 have dedicated butterflies; any other
 * prime factor uses a direct r-point DFT, so every length is supported.
 */
#include "oracle_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OFFT_MAXFAC 64

struct offt_plan1d {
    int n;
    int nfac;
    int fac[OFFT_MAXFAC];
    int maxr;     /* largest radix (scratch size for generic butterflies) */
    double *tw;   /* tw[2j], tw[2j+1] = cos, sin of 2*pi*j/n */
};

static int factorise(int n, int *fac)
{
    int nf = 0;
    while (n % 4 == 0 && n > 4) { fac[nf++] = 4; n /= 4; }
    while (n % 2 == 0) { fac[nf++] = 2; n /= 2; }
    for (int p = 3; n > 1; p += 2) {
        while (n % p == 0) { fac[nf++] = p; n /= p; }
        if (p * p > n && n > 1) { fac[nf++] = n; n = 1; }
    }
    return nf;
}

offt_plan1d *offt_plan1d_create(int n)
{
    if (n < 1) return NULL;
    offt_plan1d *p = (offt_plan1d *)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->n = n;
    p->nfac = (n == 1) ? 0 : factorise(n, p->fac);
    p->maxr = 1;
    for (int i = 0; i < p->nfac; i++)
        if (p->fac[i] > p->maxr) p->maxr = p->fac[i];
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!p->tw) { free(p); return NULL; }
    for (int j = 0; j < n; j++) {
        double a = 2.0 * M_PI * (double)j / (double)n;
        p->tw[2 * j] = cos(a);
        p->tw[2 * j + 1] = sin(a);
    }
    return p;
}

void offt_plan1d_destroy(offt_plan1d *p)
{
    if (!p) return;
    free(p->tw);
    free(p);
}

int offt_plan1d_len(const offt_plan1d *p) { return p->n; }

/* W_N^{e} for sign: exp(sign * 2 pi i e / N) */
static inline void twid(const offt_plan1d *p, long e, int sign, double *c, double *s)
{
    long j = e % p->n;
    *c = p->tw[2 * j];
    *s = sign * p->tw[2 * j + 1];
}

static void rec(const offt_plan1d *p, const double *in, long istride,
                double *out, int n, int fi, int sign)
{
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    const int r = p->fac[fi];
    const int m = n / r;
    for (int q = 0; q < r; q++)
        rec(p, in + 2 * q * istride, istride * r, out + 2 * q * m, m, fi + 1, sign);

    const long tstep = p->n / n; /* W_n^{x} = W_N^{x * tstep} */
    double tre[16], tim[16];
    double *gre = tre, *gim = tim;
    double *heap = NULL;
    if (r > 16) {
        heap = (double *)malloc(sizeof(double) * 2 * (size_t)r);
        gre = heap;
        gim = heap + r;
    }
    for (int k = 0; k < m; k++) {
        /* twiddled inputs t[q] = out[q*m+k] * W_n^{q k} */
        for (int q = 0; q < r; q++) {
            double xr = out[2 * (q * m + k)], xi = out[2 * (q * m + k) + 1];
            if (q == 0 || k == 0) {
                gre[q] = xr;
                gim[q] = xi;
            } else {
                double c, s;
                twid(p, (long)q * k * tstep, sign, &c, &s);
                gre[q] = xr * c - xi * s;
                gim[q] = xr * s + xi * c;
            }
        }
        if (r == 2) {
            double ar = gre[0], ai = gim[0], br = gre[1], bi = gim[1];
            out[2 * k] = ar + br;            out[2 * k + 1] = ai + bi;
            out[2 * (k + m)] = ar - br;      out[2 * (k + m) + 1] = ai - bi;
        } else if (r == 4) {
            double ar = gre[0], ai = gim[0], br = gre[1], bi = gim[1];
            double cr = gre[2], ci = gim[2], dr = gre[3], di = gim[3];
            double s0r = ar + cr, s0i = ai + ci, s1r = ar - cr, s1i = ai - ci;
            double s2r = br + dr, s2i = bi + di, s3r = br - dr, s3i = bi - di;
            /* multiply s3 by sign*i: (x + i y) * (sign i) = -sign*y + i sign*x */
            double rr = -sign * s3i, ri = sign * s3r;
            out[2 * k] = s0r + s2r;              out[2 * k + 1] = s0i + s2i;
            out[2 * (k + m)] = s1r + rr;         out[2 * (k + m) + 1] = s1i + ri;
            out[2 * (k + 2 * m)] = s0r - s2r;    out[2 * (k + 2 * m) + 1] = s0i - s2i;
            out[2 * (k + 3 * m)] = s1r - rr;     out[2 * (k + 3 * m) + 1] = s1i - ri;
        } else if (r == 3) {
            const double c1 = -0.5, s1 = sign * 0.86602540378443864676;
            double ar = gre[0], ai = gim[0];
            double pr = gre[1] + gre[2], pi = gim[1] + gim[2];
            double mr = gre[1] - gre[2], mi = gim[1] - gim[2];
            double tr = ar + c1 * pr, ti = ai + c1 * pi;
            out[2 * k] = ar + pr;                out[2 * k + 1] = ai + pi;
            out[2 * (k + m)] = tr - s1 * mi;     out[2 * (k + m) + 1] = ti + s1 * mr;
            out[2 * (k + 2 * m)] = tr + s1 * mi; out[2 * (k + 2 * m) + 1] = ti - s1 * mr;
        } else {
            /* direct r-point DFT: X[s] = sum_q g[q] W_r^{q s} */
            const long rstep = p->n / r;
            for (int s = 0; s < r; s++) {
                double accr = 0.0, acci = 0.0;
                for (int q = 0; q < r; q++) {
                    double c, sn;
                    twid(p, (long)((q * s) % r) * rstep, sign, &c, &sn);
                    accr += gre[q] * c - gim[q] * sn;
                    acci += gre[q] * sn + gim[q] * c;
                }
                out[2 * (k + s * m)] = accr;
                out[2 * (k + s * m) + 1] = acci;
            }
        }
    }
    free(heap);
}

void offt_exec1d(const offt_plan1d *p, const double *in, int istride,
                 double *out, int sign)
{
    rec(p, in, istride, out, p->n, 0, sign);
}

/* ---------------------------------------------------------------- 2-D ---- */

struct offt_ctx2d {
    int n0, n1;
    offt_plan1d *p0, *p1;
    double *row;   /* 2*n1 doubles */
    double *col;   /* 2*n0 doubles */
    double *col2;  /* 2*n0 doubles */
    double *tmp;   /* 2*n0*n1 doubles */
};

offt_ctx2d *offt_ctx2d_create(int n0, int n1)
{
    offt_ctx2d *c = (offt_ctx2d *)calloc(1, sizeof(*c));
    if (!c) return NULL;
    c->n0 = n0;
    c->n1 = n1;
    c->p0 = offt_plan1d_create(n0);
    c->p1 = offt_plan1d_create(n1);
    c->row = (double *)malloc(sizeof(double) * 4 * (size_t)n1);
    c->col = (double *)malloc(sizeof(double) * 2 * (size_t)n0);
    c->col2 = (double *)malloc(sizeof(double) * 2 * (size_t)n0);
    c->tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * n1);
    if (!c->p0 || !c->p1 || !c->row || !c->col || !c->col2 || !c->tmp) {
        offt_ctx2d_destroy(c);
        return NULL;
    }
    return c;
}

void offt_ctx2d_destroy(offt_ctx2d *c)
{
    if (!c) return;
    offt_plan1d_destroy(c->p0);
    offt_plan1d_destroy(c->p1);
    free(c->row);
    free(c->col);
    free(c->col2);
    free(c->tmp);
    free(c);
}

/* transform every column j < ncols of a row-major n0 x ld complex array */
static void cols(offt_ctx2d *c, double *a, int ld, int ncols, int sign)
{
    for (int j = 0; j < ncols; j++) {
        offt_exec1d(c->p0, a + 2 * j, ld, c->col, sign);
        for (int i = 0; i < c->n0; i++) {
            a[2 * ((long)i * ld + j)] = c->col[2 * i];
            a[2 * ((long)i * ld + j) + 1] = c->col[2 * i + 1];
        }
    }
}

void offt_ctx2d_c2c(offt_ctx2d *c, const double *in, double *out, int sign)
{
    const int n0 = c->n0, n1 = c->n1;
    /* rows go through scratch so that in == out (in-place) also works */
    for (int i = 0; i < n0; i++) {
        memcpy(c->row, in + 2 * (long)i * n1, sizeof(double) * 2 * n1);
        offt_exec1d(c->p1, c->row, 1, out + 2 * (long)i * n1, sign);
    }
    cols(c, out, n1, n1, sign);
}

void offt_ctx2d_r2c(offt_ctx2d *c, const double *in, double *out)
{
    const int n0 = c->n0, n1 = c->n1, nh = n1 / 2 + 1;
    double *cin = c->row, *cout = c->row + 2 * n1;
    for (int i = 0; i < n0; i++) {
        for (int j = 0; j < n1; j++) {
            cin[2 * j] = in[(long)i * n1 + j];
            cin[2 * j + 1] = 0.0;
        }
        offt_exec1d(c->p1, cin, 1, cout, -1);
        memcpy(out + 2 * (long)i * nh, cout, sizeof(double) * 2 * nh);
    }
    cols(c, out, nh, nh, -1);
}

void offt_ctx2d_c2r(offt_ctx2d *c, const double *in, double *out)
{
    const int n0 = c->n0, n1 = c->n1, nh = n1 / 2 + 1;
    double *half = c->tmp;
    memcpy(half, in, sizeof(double) * 2 * (size_t)n0 * nh);
    cols(c, half, nh, nh, +1);
    double *full = c->row, *res = c->row + 2 * n1;
    for (int i = 0; i < n0; i++) {
        const double *h = half + 2 * (long)i * nh;
        for (int k = 0; k < nh; k++) {
            full[2 * k] = h[2 * k];
            full[2 * k + 1] = h[2 * k + 1];
        }
        /* self-conjugate entries are real in a Hermitian spectrum */
        full[1] = 0.0;
        if (n1 % 2 == 0) full[2 * (n1 / 2) + 1] = 0.0;
        for (int k = nh; k < n1; k++) {
            full[2 * k] = h[2 * (n1 - k)];
            full[2 * k + 1] = -h[2 * (n1 - k) + 1];
        }
        offt_exec1d(c->p1, full, 1, res, +1);
        for (int j = 0; j < n1; j++) out[(long)i * n1 + j] = res[2 * j];
    }
}

int offt_c2c_2d(int n0, int n1, const double *in, double *out, int sign)
{
    offt_ctx2d *c = offt_ctx2d_create(n0, n1);
    if (!c) return 1;
    offt_ctx2d_c2c(c, in, out, sign);
    offt_ctx2d_destroy(c);
    return 0;
}

int offt_r2c_2d(int n0, int n1, const double *in, double *out)
{
    offt_ctx2d *c = offt_ctx2d_create(n0, n1);
    if (!c) return 1;
    offt_ctx2d_r2c(c, in, out);
    offt_ctx2d_destroy(c);
    return 0;
}

int offt_c2r_2d(int n0, int n1, const double *in, double *out)
{
    offt_ctx2d *c = offt_ctx2d_create(n0, n1);
    if (!c) return 1;
    offt_ctx2d_c2r(c, in, out);
    offt_ctx2d_destroy(c);
    return 0;
}
