/*
 * flct_oracle.h -- CPU restatement of the FLCT 1.01 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path:
 * tests/, the smoke check and bench.py's CPU-baseline leg may call it; the
 * product library (pyflct_gb300) never links or calls it.
 *
 * Everything is double precision, single-window-at-a-time, exactly the
 * algorithm of source/flct.c and source/warp.c (each function cites the
 * lines it follows).  Windows are independent, so oflct_velocity may spread
 * them over several host threads; results do not depend on the thread count.
 */
#ifndef FLCT_ORACLE_H
#define FLCT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (numerically identical to the product's flct_status) */
#define OFLCT_OK 0
#define OFLCT_ERR_ARG 1
#define OFLCT_ERR_SKIP_NONPOSITIVE 2
#define OFLCT_ERR_SKIP_OFFSET 3
#define OFLCT_ERR_SKIP_TOO_BIG 4
#define OFLCT_ERR_BOX_SIZE 5
#define OFLCT_ERR_GRID_TOO_SMALL 6
#define OFLCT_ERR_ALLOC 9
#define OFLCT_ERR_WARP_DIMS 11

/* The parsed state of the flct command line (flct.c:370-487). */
typedef struct {
    double deltat;     /* time between images */
    double deltas;     /* pixel length unit */
    double sigma;      /* Gaussian width; <= 0 selects the global-shift mode */
    double thresh;     /* -t value with any trailing 'a' removed */
    int thresh_abs;    /* 1 if the -t string had an 'a' */
    int skip;          /* -s N; 0 when -s absent */
    int poffset;       /* p (may be negative, as typed) */
    int qoffset;       /* q (may be negative, as typed) */
    int interpolate;   /* 'i' in the -s string */
    int filter;        /* 1 if -k given */
    double kr;         /* -k value */
    int hires;         /* 1 if -h given */
} oflct_params;

/* Derived quantities (flct.c:535-538, 559-629). */
typedef struct {
    int nsize;          /* half box; box side is 2*nsize */
    double thresh_abs_value;  /* threshold in image units */
    int xoffset, yoffset;     /* grid offsets along C slow / fast axis */
    int global_mode;          /* sigma <= 0 */
} oflct_derived;

int oflct_derive(const oflct_params *p, const double *f1, const double *f2,
                 int nx, int ny, oflct_derived *d);

/* Full velocity computation.  f1, f2, vx, vy, vm are C-order [nx][ny]
 * arrays (nx slow).  In the global-shift mode (sigma <= 0) vx, vy, vm hold
 * a single value each.  nthreads <= 0 uses one thread. */
int oflct_velocity(const oflct_params *p, const double *f1, const double *f2,
                   int nx, int ny, double *vx, double *vy, double *vm,
                   int nthreads);

/* The two windowed, mean-subtracted sub-images the velocity loop builds for
 * pixel (i, j) (flct.c:773-870); g1, g2 receive n x n doubles, n = 2 nsize.
 * Returns the box side in *n. */
int oflct_extract_window(const oflct_params *p, const double *f1,
                         const double *f2, int nx, int ny, int i, int j,
                         double *g1, double *g2, int *n);

/* One window: the cross_cor unit (flct.c:1325-1649) for n0 x n1 windows
 * g1, g2.  hires is 1 for the -h refinement.  If absccor is non-NULL it
 * receives |c| after the half-size circular shift (n0*n1 doubles). */
int oflct_cross_cor(const double *g1, const double *g2, int n0, int n1,
                    int filter, double kr, int hires, double *shiftx,
                    double *shifty, double *absccor);

/* Same, for nwin windows stored back to back (each n x n); threads >= 1. */
int oflct_cross_cor_batch(const double *g1, const double *g2, int n, int nwin,
                          int filter, double kr, double *shiftx,
                          double *shifty, int nthreads);

/* 3x3 Taylor peak fit (flct.c:1536-1553) on a row-major n0 x n1 |c| that is
 * already half-shifted, around the first strict maximum.  Outputs the peak
 * indices and sub-pixel offsets exactly as cross_cor computes them. */
void oflct_peak_fit(const double *absccor, int n0, int n1, int *ixmax,
                    int *iymax, double *subx, double *suby);

/* Cubic-convolution interpolation (flct.c:2226-2463); out is nxi x nyi. */
int oflct_interpcc2d(const double *fdata, double xmiss, int nx, int ny,
                     const double *xwant, int nxi, const double *ywant,
                     int nyi, double *out);

/* Uniform Fourier shift (warp.c:757-881) and non-uniform warp
 * (warp.c:883-1011); transp as in the reference (1 for the CLI). */
int oflct_shift_frac2d(const double *arr, double delx, double dely,
                       double *out, int nx, int ny, int transp);
int oflct_warp_frac2d(const double *arr, const double *delx,
                      const double *dely, double *out, int nx, int ny,
                      int transp, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
