/*
 * flct_oracle.c -- CPU restatement of the FLCT 1.01 hot path in double
 * precision.  TEST INFRASTRUCTURE ONLY (see flct_oracle.h): the checker the
 * GPU kernels are compared with, never part of the product.
 *
 * Citations are to the reference project's source/flct.c and source/warp.c.
 * The arithmetic of every step is kept in the reference's order of
 * operations so that, compiled without FMA contraction, the restatement
 * rounds like the reference compiled against the same FFT.
 */
#include "flct_oracle.h"
#include "oracle_fft.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define XMISS (-999999.)        /* flct.c:279 */
#define TOL (1e-2)              /* flct.c:278 */
#define WARP_PI 3.1415926535898 /* warp.c:768, 895 (truncated pi) */

/* ------------------------------------------------------------ helpers ---- */

/* Wavenumbers in FFT storage order; the Nyquist entry of an even length is
 * +n/2 (flct.c:1651-1692, warp.c:316-360). */
static void make_freq(double *k, int n)
{
    int half = n / 2 - 1, next, i;
    for (i = 0; i <= half; i++) k[i] = (double)i;
    next = half + 1;
    if ((n / 2) * 2 != n) {
        k[next++] = (double)(n / 2);
        k[next++] = -(double)(n / 2);
    } else {
        k[next++] = (double)(n / 2);
    }
    for (i = next; i < n; i++) k[i] = -(double)(half - (i - next));
}

/* First strict maximum, as a sequential scan (flct.c:2142-2161). */
static int first_max(const double *a, long len)
{
    double best = a[0];
    int loc = 0;
    for (long i = 1; i < len; i++)
        if (a[i] > best) {
            best = a[i];
            loc = (int)i;
        }
    return loc;
}

/* Box start along one axis: centred on i, pinned inside [0, n) (flct.c:773-788). */
static int box_start(int i, int n, int nsize)
{
    int lo0 = (0 > (i - (nsize - 1))) ? 0 : i - (nsize - 1);
    int hi0 = ((n - 1) < (i + nsize)) ? n - 1 : i + nsize;
    return (hi0 == n - 1) ? n - 1 - (2 * nsize - 1) : lo0;
}

/* ----------------------------------------------------- peak and fit ---- */

void oflct_peak_fit(const double *cc, int n0, int n1, int *ixmax, int *iymax,
                    double *subx, double *suby)
{
    /* flct.c:1515-1553 */
    int ind = first_max(cc, (long)n0 * n1);
    int have = (cc[ind] == 0.) ? 0 : 1;
    int ix = have ? ind / n1 : n0 / 2;
    int iy = have ? ind % n1 : n1 / 2;
    double sx = 0., sy = 0.;
    if (ix > 0 && ix < n0 - 1 && iy > 0 && iy < n1 - 1 && have) {
#define CC(a, b) cc[(long)(a) * n1 + (b)]
        double fx = 0.5 * (CC(ix + 1, iy) - CC(ix - 1, iy));
        double fy = 0.5 * (CC(ix, iy + 1) - CC(ix, iy - 1));
        double fxx = (CC(ix + 1, iy) + CC(ix - 1, iy) - 2. * (CC(ix, iy)));
        double fyy = (CC(ix, iy + 1) + CC(ix, iy - 1) - 2. * (CC(ix, iy)));
        double fxy = 0.25 * (CC(ix + 1, iy + 1) + CC(ix - 1, iy - 1) -
                             CC(ix + 1, iy - 1) - CC(ix - 1, iy + 1));
#undef CC
        sx = (fyy * fx - fy * fxy) / (fxy * fxy - fxx * fyy);
        sy = (fxx * fy - fx * fxy) / (fxy * fxy - fxx * fyy);
    }
    *ixmax = ix;
    *iymax = iy;
    *subx = sx;
    *suby = sy;
}

/* ------------------------------------------------------- cross_cor ---- */

typedef struct {
    int n0, n1, nh;
    offt_ctx2d *fft;
    double *ca, *cb, *cc; /* n0*nh complex */
    double *real;         /* n0*n1 */
    double *shifted;      /* n0*n1 */
    double *filt;         /* n0*n1 or NULL */
    double *interp;       /* 21*21 (hires) */
} xc_ctx;

static void xc_free(xc_ctx *x)
{
    if (!x) return;
    offt_ctx2d_destroy(x->fft);
    free(x->ca);
    free(x->cb);
    free(x->cc);
    free(x->real);
    free(x->shifted);
    free(x->filt);
    free(x->interp);
    free(x);
}

static xc_ctx *xc_new(int n0, int n1, int filter, double kr)
{
    xc_ctx *x = (xc_ctx *)calloc(1, sizeof(*x));
    if (!x) return NULL;
    x->n0 = n0;
    x->n1 = n1;
    x->nh = n1 / 2 + 1;
    size_t nc = (size_t)n0 * x->nh * 2, nr = (size_t)n0 * n1;
    x->fft = offt_ctx2d_create(n0, n1);
    x->ca = (double *)malloc(sizeof(double) * nc);
    x->cb = (double *)malloc(sizeof(double) * nc);
    x->cc = (double *)malloc(sizeof(double) * nc);
    x->real = (double *)malloc(sizeof(double) * nr);
    x->shifted = (double *)malloc(sizeof(double) * nr);
    x->interp = (double *)malloc(sizeof(double) * 21 * 21);
    if (!x->fft || !x->ca || !x->cb || !x->cc || !x->real || !x->shifted ||
        !x->interp) {
        xc_free(x);
        return NULL;
    }
    if (filter) {
        /* gaussfilt (flct.c:1694-1715) on make_freq wavenumbers */
        double *kx = (double *)malloc(sizeof(double) * n0);
        double *ky = (double *)malloc(sizeof(double) * n1);
        x->filt = (double *)malloc(sizeof(double) * nr);
        if (!kx || !ky || !x->filt) {
            free(kx);
            free(ky);
            xc_free(x);
            return NULL;
        }
        make_freq(kx, n0);
        make_freq(ky, n1);
        double kxroll = kr * kx[n0 / 2], kyroll = kr * ky[n1 / 2];
        double smx = 1. / kxroll, smy = 1. / kyroll;
        for (int i = 0; i < n0; i++) {
            double ax = kx[i] * smx;
            for (int j = 0; j < n1; j++) {
                double ay = ky[j] * smy;
                x->filt[(long)i * n1 + j] = exp(-(ax * ax + ay * ay));
            }
        }
        free(kx);
        free(ky);
    }
    return x;
}

static void xc_run(xc_ctx *x, const double *g1, const double *g2, int hires,
                   double *shiftx, double *shifty, double *absout)
{
    const int n0 = x->n0, n1 = x->n1, nh = x->nh;
    const long nr = (long)n0 * n1, nc = (long)n0 * nh;

    /* forward transforms of both sub-images (flct.c:1421-1436) */
    offt_ctx2d_r2c(x->fft, g1, x->ca);
    offt_ctx2d_r2c(x->fft, g2, x->cb);

    double normfac = (1. / ((double)n0 * n1)); /* flct.c:1440-1441 */
    normfac *= normfac;

    if (x->filt) { /* flct.c:1445-1457 */
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < nh; j++) {
                double f = x->filt[(long)i * n1 + j];
                long k = 2 * ((long)i * nh + j);
                x->ca[k] = x->ca[k] * f;
                x->ca[k + 1] = x->ca[k + 1] * f;
                x->cb[k] = x->cb[k] * f;
                x->cb[k + 1] = x->cb[k + 1] * f;
            }
    }
    /* conj(A) * B * normfac (flct.c:1461-1477) */
    for (long k = 0; k < nc; k++) {
        double ar = x->ca[2 * k], ai = x->ca[2 * k + 1];
        double br = x->cb[2 * k], bi = x->cb[2 * k + 1];
        x->cc[2 * k] = (ar * br + ai * bi) * normfac;
        x->cc[2 * k + 1] = (ar * bi - ai * br) * normfac;
    }
    offt_ctx2d_c2r(x->fft, x->cc, x->real); /* flct.c:1481 */

    /* |c|, then circular shift by (n0/2, n1/2) (flct.c:1485-1488, 2111-2140) */
    for (int i = 0; i < n0; i++) {
        int ii = (i + n0 / 2) % n0;
        for (int j = 0; j < n1; j++) {
            int jj = (j + n1 / 2) % n1;
            x->shifted[(long)ii * n1 + jj] = fabs(x->real[(long)i * n1 + j]);
        }
    }
    if (absout) memcpy(absout, x->shifted, sizeof(double) * nr);

    int ix, iy;
    double sx, sy, outx, outy;
    oflct_peak_fit(x->shifted, n0, n1, &ix, &iy, &sx, &sy);
    if (hires) {
        /* -h: 21x21 cubic-convolution zoom at 0.1 px, then the same fit on
         * the zoomed |c| (flct.c:1345-1368, 1564-1635) */
        const int ni = 21, per = 10;
        double range = (double)(ni - 1) / per;
        double xw[21], yw[21];
        for (int i = 0; i < ni; i++)
            xw[i] = ((((double)i) * range) / ((double)(ni - 1))) - 0.5 * range + (double)ix;
        for (int j = 0; j < ni; j++)
            yw[j] = ((((double)j) * range) / ((double)(ni - 1))) - 0.5 * range + (double)iy;
        oflct_interpcc2d(x->shifted, 0., n0, n1, xw, ni, yw, ni, x->interp);
        int m = first_max(x->interp, ni * ni);
        int ixx = m / ni, iyy = m % ni;
        double ssx = 0., ssy = 0.;
        if (ixx > 0 && ixx < ni - 1 && iyy > 0 && iyy < ni - 1) {
#define PA(a, b) x->interp[(a) * ni + (b)]
            double fx = 0.5 * (PA(ixx + 1, iyy) - PA(ixx - 1, iyy));
            double fy = 0.5 * (PA(ixx, iyy + 1) - PA(ixx, iyy - 1));
            double fxx = (PA(ixx + 1, iyy) + PA(ixx - 1, iyy) - 2. * (PA(ixx, iyy)));
            double fyy = (PA(ixx, iyy + 1) + PA(ixx, iyy - 1) - 2. * (PA(ixx, iyy)));
            double fxy = 0.25 * (PA(ixx + 1, iyy + 1) + PA(ixx - 1, iyy - 1) -
                                 PA(ixx + 1, iyy - 1) - PA(ixx - 1, iyy + 1));
#undef PA
            ssx = ((fyy * fx - fy * fxy) / (fxy * fxy - fxx * fyy)) * range / ((double)(ni - 1));
            ssy = ((fxx * fy - fx * fxy) / (fxy * fxy - fxx * fyy)) * range / ((double)(ni - 1));
        }
        outx = xw[ixx] + ssx;
        outy = yw[iyy] + ssy;
    } else {
        outx = (double)ix + sx;
        outy = (double)iy + sy;
    }
    *shiftx = outx - (double)(n0 / 2); /* flct.c:1639-1640 */
    *shifty = outy - (double)(n1 / 2);
}

int oflct_cross_cor(const double *g1, const double *g2, int n0, int n1,
                    int filter, double kr, int hires, double *shiftx,
                    double *shifty, double *absccor)
{
    if (!g1 || !g2 || !shiftx || !shifty || n0 < 1 || n1 < 1) return OFLCT_ERR_ARG;
    xc_ctx *x = xc_new(n0, n1, filter, kr);
    if (!x) return OFLCT_ERR_ALLOC;
    xc_run(x, g1, g2, hires, shiftx, shifty, absccor);
    xc_free(x);
    return OFLCT_OK;
}

typedef struct {
    const double *g1, *g2;
    int n, nwin, filter;
    double kr;
    double *sx, *sy;
    int next;
    pthread_mutex_t mu;
    int err;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *b = (batch_job *)arg;
    xc_ctx *x = xc_new(b->n, b->n, b->filter, b->kr);
    if (!x) {
        pthread_mutex_lock(&b->mu);
        b->err = OFLCT_ERR_ALLOC;
        pthread_mutex_unlock(&b->mu);
        return NULL;
    }
    const long w2 = (long)b->n * b->n;
    for (;;) {
        pthread_mutex_lock(&b->mu);
        int w = b->next;
        b->next += 64;
        pthread_mutex_unlock(&b->mu);
        if (w >= b->nwin) break;
        int e = (w + 64 < b->nwin) ? w + 64 : b->nwin;
        for (; w < e; w++)
            xc_run(x, b->g1 + w * w2, b->g2 + w * w2, 0, b->sx + w, b->sy + w, NULL);
    }
    xc_free(x);
    return NULL;
}

int oflct_cross_cor_batch(const double *g1, const double *g2, int n, int nwin,
                          int filter, double kr, double *shiftx,
                          double *shifty, int nthreads)
{
    if (!g1 || !g2 || !shiftx || !shifty || n < 1 || nwin < 0) return OFLCT_ERR_ARG;
    batch_job b = {g1, g2, n, nwin, filter, kr, shiftx, shifty, 0,
                   PTHREAD_MUTEX_INITIALIZER, 0};
    if (nthreads < 1) nthreads = 1;
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &b);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    return b.err;
}

/* --------------------------------------------------- parameter setup ---- */

int oflct_derive(const oflct_params *p, const double *f1, const double *f2,
                 int nx, int ny, oflct_derived *d)
{
    if (!p || !f1 || !f2 || !d || nx < 1 || ny < 1) return OFLCT_ERR_ARG;
    memset(d, 0, sizeof(*d));
    int skip = p->skip, pp = p->poffset, qq = p->qoffset;
    /* -s checks at parse time (flct.c:433-452); skip == 0 means no -s */
    if (skip < 0) return OFLCT_ERR_SKIP_NONPOSITIVE;
    if (skip > 0 && (abs(pp) >= skip || abs(qq) >= skip)) return OFLCT_ERR_SKIP_OFFSET;
    /* negative offsets wrap (flct.c:535-538) */
    if (pp < 0) pp = skip - abs(pp);
    if (qq < 0) qq = skip - abs(qq);
    /* transposed storage: q runs along the C slow axis (flct.c:736-745) */
    d->xoffset = qq;
    d->yoffset = pp;
    /* flct.c:559-563 */
    if (skip >= nx || skip >= ny) return OFLCT_ERR_SKIP_TOO_BIG;
    d->global_mode = (p->sigma > 0.) ? 0 : 1;
    if (!d->global_mode) {
        /* sliding box (flct.c:567-580) */
        int nt = (int)((int)p->sigma * sqrt(log(1. / TOL)));
        int ndmin = (nx < ny) ? (((nx / 3) / 2)) * 2 : (((ny / 3) / 2)) * 2;
        d->nsize = ((nt / 2) * 2 < ndmin) ? (nt / 2) * 2 : ndmin;
        if (d->nsize <= 0) return OFLCT_ERR_BOX_SIZE;
    }
    d->thresh_abs_value = p->thresh;
    if (!d->global_mode && p->thresh > 0. && p->thresh < 1. && !p->thresh_abs) {
        /* relative threshold: scale by max(|f1|,|f2|) (flct.c:594-629) */
        long n = (long)nx * ny;
        double *t = (double *)malloc(sizeof(double) * n);
        if (!t) return OFLCT_ERR_ALLOC;
        for (long i = 0; i < n; i++) t[i] = fabs(f1[i]);
        double m1 = t[first_max(t, n)];
        for (long i = 0; i < n; i++) t[i] = fabs(f2[i]);
        double m2 = t[first_max(t, n)];
        free(t);
        double fmax = (m1 > m2) ? m1 : m2;
        d->thresh_abs_value = p->thresh * fmax;
    }
    return OFLCT_OK;
}

/* ---------------------------------------------------- velocity loop ---- */

typedef struct {
    const oflct_params *p;
    const oflct_derived *d;
    const double *f1, *f2;
    int nx, ny;
    double *vx, *vy, *vm;
    const double *gtab; /* (2n+1)^2 Gaussian table indexed by offsets */
    int next_row;
    pthread_mutex_t mu;
    int err;
} vel_job;

/* Does pixel (i, j) need a correlation window?  (flct.c:721-755; the init
 * windows forced at the first and last pixel do not change any output and
 * are not recomputed here.) */
static int pixel_state(const vel_job *v, int i, int j, int *below, int *grid)
{
    double fabsbar = 0.5 * (fabs(v->f1[(long)i * v->ny + j] + v->f2[(long)i * v->ny + j]));
    *below = (fabsbar < v->d->thresh_abs_value);
    if (v->p->skip > 0) {
        *grid = !((i - v->d->xoffset) % v->p->skip) && !((j - v->d->yoffset) % v->p->skip);
    } else {
        *grid = 1;
    }
    return !*below && *grid;
}

static void *vel_worker(void *arg)
{
    vel_job *v = (vel_job *)arg;
    const int nx = v->nx, ny = v->ny, ns = v->d->nsize, n = 2 * ns;
    const long gw = 2 * n + 1;
    xc_ctx *x = xc_new(n, n, v->p->filter, v->p->kr);
    double *g1 = (double *)malloc(sizeof(double) * n * n);
    double *g2 = (double *)malloc(sizeof(double) * n * n);
    if (!x || !g1 || !g2) {
        pthread_mutex_lock(&v->mu);
        v->err = OFLCT_ERR_ALLOC;
        pthread_mutex_unlock(&v->mu);
        xc_free(x);
        free(g1);
        free(g2);
        return NULL;
    }
    const double deltinv = 1. / v->p->deltat; /* flct.c:343 */
    for (;;) {
        pthread_mutex_lock(&v->mu);
        int i = v->next_row++;
        pthread_mutex_unlock(&v->mu);
        if (i >= nx) break;
        for (int j = 0; j < ny; j++) {
            int below, grid;
            long o = (long)i * ny + j;
            if (!pixel_state(v, i, j, &below, &grid)) {
                /* flct.c:918-930 */
                v->vx[o] = XMISS;
                v->vy[o] = XMISS;
                v->vm[o] = 0.;
                continue;
            }
            int imin = box_start(i, nx, ns), jmin = box_start(j, ny, ns);
            /* FP64 local means, summed in row-major order (flct.c:815-827) */
            double s1 = 0., s2 = 0.;
            for (int ii = 0; ii < n; ii++)
                for (int jj = 0; jj < n; jj++) {
                    s1 = s1 + v->f1[(long)(ii + imin) * ny + (jj + jmin)];
                    s2 = s2 + v->f2[(long)(ii + imin) * ny + (jj + jmin)];
                }
            s1 = s1 / ((double)n * n);
            s2 = s2 / ((double)n * n);
            /* Gaussian centred on (i, j), not on the box (flct.c:852-870) */
            for (int ii = 0; ii < n; ii++)
                for (int jj = 0; jj < n; jj++) {
                    double w = v->gtab[(ii + imin - i + n) * gw + (jj + jmin - j + n)];
                    long src = (long)(ii + imin) * ny + (jj + jmin);
                    g1[ii * n + jj] = w * (v->f1[src] - s1);
                    g2[ii * n + jj] = w * (v->f2[src] - s2);
                }
            double shx, shy;
            xc_run(x, g1, g2, v->p->hires, &shx, &shy, NULL);
            /* transposed storage swaps the velocity components (flct.c:901-905) */
            v->vx[o] = shy * deltinv * v->p->deltas;
            v->vy[o] = shx * deltinv * v->p->deltas;
            v->vm[o] = 1.;
        }
    }
    xc_free(x);
    free(g1);
    free(g2);
    return NULL;
}

int oflct_extract_window(const oflct_params *p, const double *f1,
                         const double *f2, int nx, int ny, int i, int j,
                         double *g1, double *g2, int *nout)
{
    oflct_derived d;
    int e = oflct_derive(p, f1, f2, nx, ny, &d);
    if (e) return e;
    if (d.global_mode || i < 0 || j < 0 || i >= nx || j >= ny) return OFLCT_ERR_ARG;
    const int ns = d.nsize, n = 2 * ns;
    const double sigminv = 1. / p->sigma;
    int imin = box_start(i, nx, ns), jmin = box_start(j, ny, ns);
    double s1 = 0., s2 = 0.;
    for (int ii = 0; ii < n; ii++)
        for (int jj = 0; jj < n; jj++) {
            s1 = s1 + f1[(long)(ii + imin) * ny + (jj + jmin)];
            s2 = s2 + f2[(long)(ii + imin) * ny + (jj + jmin)];
        }
    s1 = s1 / ((double)n * n);
    s2 = s2 / ((double)n * n);
    for (int ii = 0; ii < n; ii++) {
        double argx = sigminv * (double)(ii + imin - i);
        for (int jj = 0; jj < n; jj++) {
            double argy = sigminv * (double)(jj + jmin - j);
            double w = exp(-argx * argx - argy * argy);
            long src = (long)(ii + imin) * ny + (jj + jmin);
            g1[ii * n + jj] = w * (f1[src] - s1);
            g2[ii * n + jj] = w * (f2[src] - s2);
        }
    }
    if (nout) *nout = n;
    return OFLCT_OK;
}

static int global_shift(const oflct_params *p, const double *f1, const double *f2,
                        int nx, int ny, double *vx, double *vy, double *vm)
{
    /* sigma <= 0: one correlation of the whole mean-subtracted frames, no
     * Gaussian, threshold ignored (flct.c:581-586, 666-675, 802-808, 920) */
    long n = (long)nx * ny;
    double *g1 = (double *)malloc(sizeof(double) * n);
    double *g2 = (double *)malloc(sizeof(double) * n);
    if (!g1 || !g2) {
        free(g1);
        free(g2);
        return OFLCT_ERR_ALLOC;
    }
    double s1 = 0., s2 = 0.;
    for (int ii = 0; ii < nx; ii++)
        for (int jj = 0; jj < ny; jj++) {
            s1 = s1 + f1[(long)ii * ny + jj];
            s2 = s2 + f2[(long)ii * ny + jj];
        }
    s1 = s1 / ((double)nx * ny);
    s2 = s2 / ((double)nx * ny);
    for (long k = 0; k < n; k++) {
        g1[k] = 1. * (f1[k] - s1);
        g2[k] = 1. * (f2[k] - s2);
    }
    double shx, shy;
    int e = oflct_cross_cor(g1, g2, nx, ny, p->filter, p->kr, p->hires, &shx, &shy, NULL);
    free(g1);
    free(g2);
    if (e) return e;
    double deltinv = 1. / p->deltat;
    vx[0] = shy * deltinv * p->deltas;
    vy[0] = shx * deltinv * p->deltas;
    vm[0] = 1.;
    return OFLCT_OK;
}

/* Skip-grid interpolation and the final xmiss reset (flct.c:958-1133). */
static int skip_post(const oflct_params *p, const oflct_derived *d, int nx, int ny,
                     double *vx, double *vy, double *vm)
{
    const int skip = p->skip, xo = d->xoffset, yo = d->yoffset;
    if (skip > 0 && p->interpolate) {
        int icnt = 0, jcnt = 0;
        for (int i = 0; i < nx; i++) icnt += !((i - xo) % skip);
        for (int j = 0; j < ny; j++) jcnt += !((j - yo) % skip);
        /* interpcc2d reads three grid points per axis; smaller grids make the
         * reference read outside its arrays, so they are rejected here. */
        if (icnt < 3 || jcnt < 3) return OFLCT_ERR_GRID_TOO_SMALL;
        double *gx = (double *)malloc(sizeof(double) * icnt * jcnt);
        double *gy = (double *)malloc(sizeof(double) * icnt * jcnt);
        double *xw = (double *)malloc(sizeof(double) * nx);
        double *yw = (double *)malloc(sizeof(double) * ny);
        double *ix = (double *)malloc(sizeof(double) * (long)nx * ny);
        double *iy = (double *)malloc(sizeof(double) * (long)nx * ny);
        if (!gx || !gy || !xw || !yw || !ix || !iy) {
            free(gx); free(gy); free(xw); free(yw); free(ix); free(iy);
            return OFLCT_ERR_ALLOC;
        }
        int ic = -1;
        for (int i = 0; i < nx; i++) {
            int gi = !((i - xo) % skip);
            if (gi) ic++;
            int jc = -1;
            for (int j = 0; j < ny; j++) {
                int gj = !((j - yo) % skip);
                if (gj) jc++;
                if (gi && gj) {
                    gx[ic * jcnt + jc] = vx[(long)i * ny + j];
                    gy[ic * jcnt + jc] = vy[(long)i * ny + j];
                }
            }
        }
        for (int i = 0; i < nx; i++) xw[i] = ((double)(i - xo)) / (double)(skip);
        for (int j = 0; j < ny; j++) yw[j] = ((double)(j - yo)) / (double)(skip);
        oflct_interpcc2d(gx, XMISS, icnt, jcnt, xw, nx, yw, ny, ix);
        oflct_interpcc2d(gy, XMISS, icnt, jcnt, xw, nx, yw, ny, iy);
        for (int i = 0; i < nx; i++) {
            int gi = !((i - xo) % skip);
            for (int j = 0; j < ny; j++) {
                int gj = !((j - yo) % skip);
                if (!(gi && gj)) {
                    long o = (long)i * ny + j;
                    vx[o] = ix[o];
                    vy[o] = iy[o];
                    vm[o] = 0.5;
                }
            }
        }
        free(gx); free(gy); free(xw); free(yw); free(ix); free(iy);
    }
    for (long o = 0; o < (long)nx * ny; o++) {
        if (vx[o] == XMISS) vm[o] = 0.;
        if (vx[o] == XMISS) vx[o] = 0.;
        if (vy[o] == XMISS) vy[o] = 0.;
    }
    return OFLCT_OK;
}

int oflct_velocity(const oflct_params *p, const double *f1, const double *f2,
                   int nx, int ny, double *vx, double *vy, double *vm,
                   int nthreads)
{
    if (!p || !f1 || !f2 || !vx || !vy || !vm) return OFLCT_ERR_ARG;
    oflct_derived d;
    int e = oflct_derive(p, f1, f2, nx, ny, &d);
    if (e) return e;
    if (d.global_mode) {
        if (p->skip > 0 && p->interpolate) return OFLCT_ERR_GRID_TOO_SMALL;
        return global_shift(p, f1, f2, nx, ny, vx, vy, vm);
    }
    if (p->skip > 0 && p->interpolate) {
        int icnt = 0, jcnt = 0;
        for (int i = 0; i < nx; i++) icnt += !((i - d.xoffset) % p->skip);
        for (int j = 0; j < ny; j++) jcnt += !((j - d.yoffset) % p->skip);
        if (icnt < 3 || jcnt < 3) return OFLCT_ERR_GRID_TOO_SMALL;
    }
    /* Gaussian weights by offset from the window centre, same formula as the
     * 2nx x 2ny master table (flct.c:652-665) */
    const int n = 2 * d.nsize;
    const long gw = 2 * n + 1;
    double *gtab = (double *)malloc(sizeof(double) * gw * gw);
    if (!gtab) return OFLCT_ERR_ALLOC;
    const double sigminv = 1. / p->sigma;
    for (long a = 0; a < gw; a++) {
        double argx = sigminv * (double)(a - n);
        for (long b = 0; b < gw; b++) {
            double argy = sigminv * (double)(b - n);
            gtab[a * gw + b] = exp(-argx * argx - argy * argy);
        }
    }
    vel_job v;
    memset(&v, 0, sizeof(v));
    v.p = p;
    v.d = &d;
    v.f1 = f1;
    v.f2 = f2;
    v.nx = nx;
    v.ny = ny;
    v.vx = vx;
    v.vy = vy;
    v.vm = vm;
    v.gtab = gtab;
    pthread_mutex_init(&v.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, vel_worker, &v);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&v.mu);
    free(gtab);
    if (v.err) return v.err;
    return skip_post(p, &d, nx, ny, vx, vy, vm);
}

/* ----------------------------------------------------- interpcc2d ---- */

/* Keys cubic-convolution kernel, a = -0.5 (flct.c:2398-2419) */
static inline double keys(double t)
{
    return (t >= (double)1.0)
               ? (((((double)(-0.5)) * t + ((double)2.5)) * t) - (double)4.) * t + (double)2.
               : (((double)(1.5)) * t - ((double)(2.5))) * t * t + (double)1.;
}

int oflct_interpcc2d(const double *f, double xmiss, int nx, int ny,
                     const double *xwant, int nxi, const double *ywant,
                     int nyi, double *out)
{
    if (!f || !xwant || !ywant || !out || nx < 3 || ny < 3) return OFLCT_ERR_ARG;
    const long w = ny + 2;
    double *c = (double *)malloc(sizeof(double) * (long)(nx + 2) * w);
    if (!c) return OFLCT_ERR_ALLOC;
#define F(a, b) f[(long)(a) * ny + (b)]
#define C(a, b) c[(long)(a) * w + (b)]
    /* interior, then the one-cell border extrapolated as 3 f0 - 3 f1 + f2
     * (flct.c:2257-2336) */
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) C(i + 1, j + 1) = F(i, j);
    for (int j = 0; j < ny; j++) {
        C(0, j + 1) = F(2, j) - 3. * (F(1, j)) + 3. * (F(0, j));
        C(nx + 1, j + 1) = F(nx - 3, j) - 3. * (F(nx - 2, j)) + 3. * (F(nx - 1, j));
    }
    for (int i = 0; i < nx; i++) {
        C(i + 1, 0) = F(i, 2) - 3. * (F(i, 1)) + 3. * (F(i, 0));
        C(i + 1, ny + 1) = F(i, ny - 3) - 3. * (F(i, ny - 2)) + 3. * (F(i, ny - 1));
    }
    /* corners, each from its own border column or row (flct.c:2318-2336) */
    C(0, 0) = 3. * (C(1, 0)) - 3. * (C(2, 0)) + C(3, 0);
    C(nx + 1, 0) = 3. * (C(nx, 0)) - 3. * (C(nx - 1, 0)) + C(nx - 2, 0);
    C(0, ny + 1) = 3. * (C(0, ny)) - 3. * (C(0, ny - 1)) + C(0, ny - 2);
    C(nx + 1, ny + 1) = 3. * (C(nx, ny + 1)) - 3. * (C(nx - 1, ny + 1)) + C(nx - 2, ny + 1);
#undef F
    for (int i = 0; i < nxi; i++) {
        double xi = xwant[i];
        int it = ((int)xi > 0) ? (int)xi : 0;
        int i0 = (it < (nx - 2)) ? it : nx - 2;
        for (int j = 0; j < nyi; j++) {
            double yj = ywant[j];
            double *o = out + (long)i * nyi + j;
            if ((yj < 0.) || (yj > (double)(ny - 1)) || ((xi < 0) || (xi > (double)(nx - 1)))) {
                *o = xmiss;
                continue;
            }
            int jt = ((int)yj > 0) ? (int)yj : 0;
            int j0 = (jt < (ny - 2)) ? jt : ny - 2;
            double acc = (double)0.;
            int bad = 0;
            for (int a = -1; a < 3; a++) {
                double rx = keys(fabs(xi - (double)(i0 + a)));
                for (int b = -1; b < 3; b++) {
                    double ry = keys(fabs(yj - (double)(j0 + b)));
                    double cv = C(i0 + 1 + a, j0 + 1 + b);
                    acc = acc + cv * rx * ry;
                    if (cv == xmiss) bad = 1;
                }
            }
            *o = bad ? xmiss : acc;
        }
    }
#undef C
    free(c);
    return OFLCT_OK;
}

/* ------------------------------------------------------------ warp ---- */

int oflct_shift_frac2d(const double *arr, double delx, double dely,
                       double *out, int nx, int ny, int transp)
{
    /* warp.c:757-881 */
    long n = (long)nx * ny;
    double *a = (double *)malloc(sizeof(double) * 2 * n);
    double *b = (double *)malloc(sizeof(double) * 2 * n);
    double *kx = (double *)malloc(sizeof(double) * nx);
    double *ky = (double *)malloc(sizeof(double) * ny);
    double *crx = (double *)malloc(sizeof(double) * nx), *cix = (double *)malloc(sizeof(double) * nx);
    double *cry = (double *)malloc(sizeof(double) * ny), *ciy = (double *)malloc(sizeof(double) * ny);
    offt_ctx2d *ctx = offt_ctx2d_create(nx, ny);
    int err = OFLCT_OK;
    if (!a || !b || !kx || !ky || !crx || !cix || !cry || !ciy || !ctx) {
        err = OFLCT_ERR_ALLOC;
        goto done;
    }
    make_freq(kx, nx);
    make_freq(ky, ny);
    double normfac = (1. / ((double)nx * ny));
    for (long i = 0; i < n; i++) {
        a[2 * i] = arr[i];
        a[2 * i + 1] = (double)0.;
    }
    offt_ctx2d_c2c(ctx, a, b, -1);
    double dxarg, dyarg;
    if (transp) {
        dxarg = -dely / ((double)nx);
        dyarg = -delx / ((double)ny);
    } else {
        dxarg = -delx / ((double)nx);
        dyarg = -dely / ((double)ny);
    }
    for (int i = 0; i < nx; i++) {
        crx[i] = cos(2. * WARP_PI * kx[i] * dxarg);
        cix[i] = sin(2. * WARP_PI * kx[i] * dxarg);
    }
    for (int j = 0; j < ny; j++) {
        cry[j] = cos(2. * WARP_PI * ky[j] * dyarg);
        ciy[j] = sin(2. * WARP_PI * ky[j] * dyarg);
    }
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            double er = crx[i] * cry[j] - cix[i] * ciy[j];
            double ei = crx[i] * ciy[j] + cix[i] * cry[j];
            long k = 2 * ((long)i * ny + j);
            double xr = b[k], xi = b[k + 1];
            b[k] = (xr * er - xi * ei);
            b[k + 1] = (xr * ei + xi * er);
        }
    offt_ctx2d_c2c(ctx, b, a, +1);
    for (long i = 0; i < n; i++) out[i] = (double)(a[2 * i]) * normfac;
done:
    free(a); free(b); free(kx); free(ky); free(crx); free(cix); free(cry); free(ciy);
    offt_ctx2d_destroy(ctx);
    return err;
}

typedef struct {
    const double *spec, *delx, *dely, *kx, *ky;
    double *out;
    int nx, ny, transp, next;
    pthread_mutex_t mu;
} warp_job;

static void *warp_worker(void *arg)
{
    warp_job *w = (warp_job *)arg;
    const int nx = w->nx, ny = w->ny;
    double *ckx = (double *)malloc(sizeof(double) * nx), *skx = (double *)malloc(sizeof(double) * nx);
    double *cky = (double *)malloc(sizeof(double) * ny), *sky = (double *)malloc(sizeof(double) * ny);
    const double normfac = (1. / ((double)nx * ny));
    const double nxinv = 1. / ((double)nx), nyinv = 1. / ((double)ny);
    for (;;) {
        pthread_mutex_lock(&w->mu);
        int i = w->next++;
        pthread_mutex_unlock(&w->mu);
        if (i >= nx) break;
        for (int j = 0; j < ny; j++) {
            /* warp.c:946-996 */
            double sx, sy;
            if (w->transp) {
                sx = w->dely[(long)i * ny + j];
                sy = w->delx[(long)i * ny + j];
            } else {
                sx = w->delx[(long)i * ny + j];
                sy = w->dely[(long)i * ny + j];
            }
            double xarg = 2. * WARP_PI * (((double)i) - sx) * nxinv;
            double yarg = 2. * WARP_PI * (((double)j) - sy) * nyinv;
            for (int a = 0; a < nx; a++) {
                ckx[a] = cos(w->kx[a] * xarg);
                skx[a] = sin(w->kx[a] * xarg);
            }
            for (int b = 0; b < ny; b++) {
                cky[b] = cos(w->ky[b] * yarg);
                sky[b] = sin(w->ky[b] * yarg);
            }
            double tot = (double)0.;
            for (int a = 0; a < nx; a++)
                for (int b = 0; b < ny; b++) {
                    double er = ckx[a] * cky[b] - skx[a] * sky[b];
                    double ei = ckx[a] * sky[b] + skx[a] * cky[b];
                    const double *s = w->spec + 2 * ((long)a * ny + b);
                    tot += (s[0] * er - s[1] * ei);
                }
            w->out[(long)i * ny + j] = (double)tot * normfac;
        }
    }
    free(ckx); free(skx); free(cky); free(sky);
    return NULL;
}

int oflct_warp_frac2d(const double *arr, const double *delx,
                      const double *dely, double *out, int nx, int ny,
                      int transp, int nthreads)
{
    /* warp.c:883-1011: one forward FFT, then a direct spectral sum per pixel */
    long n = (long)nx * ny;
    double *a = (double *)malloc(sizeof(double) * 2 * n);
    double *spec = (double *)malloc(sizeof(double) * 2 * n);
    double *kx = (double *)malloc(sizeof(double) * nx);
    double *ky = (double *)malloc(sizeof(double) * ny);
    if (!a || !spec || !kx || !ky) {
        free(a); free(spec); free(kx); free(ky);
        return OFLCT_ERR_ALLOC;
    }
    make_freq(kx, nx);
    make_freq(ky, ny);
    for (long i = 0; i < n; i++) {
        a[2 * i] = (double)arr[i];
        a[2 * i + 1] = (double)0.;
    }
    if (offt_c2c_2d(nx, ny, a, spec, -1)) {
        free(a); free(spec); free(kx); free(ky);
        return OFLCT_ERR_ALLOC;
    }
    warp_job w = {spec, delx, dely, kx, ky, out, nx, ny, transp, 0,
                  PTHREAD_MUTEX_INITIALIZER};
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, warp_worker, &w);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(a); free(spec); free(kx); free(ky);
    return OFLCT_OK;
}
