/*
 * flct_gpu.h -- C ABI of the GB300-native FLCT hot path (libflctgpu.so).
 *
 * The reference (FLCT 1.01) has no library API: its hot path lives inside
 * the `flct` and `warp` programs.  Each entry point below replaces one part
 * of those programs, cited as file:line in the reference project:
 *
 *   flct_gpu_velocity*      the whole computation between reading the two
 *                           images and writing vx, vy, vm:
 *                           source/flct.c:535-1133 (parameter derivation,
 *                           threshold, skip grid, per-pixel windows,
 *                           cross_cor, skip-grid interpolation, xmiss reset)
 *   flct_gpu_cross_cor_batch  cross_cor, source/flct.c:1325-1327, for many
 *                           windows of one size at once
 *   flct_gpu_interpcc2d     interpcc2d, source/flct.c:2226-2227
 *   flct_gpu_shift_frac2d   shift_frac2d, source/warp.c:757-758
 *   flct_gpu_warp_frac2d    warp_frac2d, source/warp.c:883-884
 *
 * Conventions
 *   - Arrays are C order [nx][ny] (nx = slow axis), i.e. the transposed
 *     layout the reference works in after read2images (flct.c:136-145).
 *     vx is the velocity along the fast axis (the IDL x axis).
 *   - Inputs and outputs are double, as inside the reference.
 *   - Errors are returned as flct_status, never by exiting; the message of
 *     the last failure on a context is available from flct_gpu_last_error.
 *   - There is no CPU fallback: without a usable GPU every compute entry
 *     point returns FLCT_ERR_NO_DEVICE.
 *   - A context owns its device workspace and streams.  Calls on one context
 *     must not overlap; separate contexts are independent.
 */
#ifndef FLCT_GPU_H
#define FLCT_GPU_H

#if defined(__GNUC__)
#define FLCT_API __attribute__((visibility("default")))
#else
#define FLCT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FLCT_OK = 0,
    FLCT_ERR_ARG = 1,              /* null pointer, bad size or bad option */
    FLCT_ERR_SKIP_NONPOSITIVE = 2, /* -s N with N <= 0 (flct.c:433-438) */
    FLCT_ERR_SKIP_OFFSET = 3,      /* |p| or |q| >= N (flct.c:441-448) */
    FLCT_ERR_SKIP_TOO_BIG = 4,     /* N >= nx or ny (flct.c:559-563) */
    FLCT_ERR_BOX_SIZE = 5,         /* sliding box size <= 0 (flct.c:575-579) */
    FLCT_ERR_GRID_TOO_SMALL = 6,   /* interpolation grid < 3 points on an axis */
    FLCT_ERR_NO_DEVICE = 7,        /* no usable CUDA device */
    FLCT_ERR_CUDA = 8,             /* a CUDA call failed (see last_error) */
    FLCT_ERR_ALLOC = 9,            /* device or host allocation failed */
    FLCT_ERR_UNSUPPORTED = 10,     /* option or size not available on GPU */
    FLCT_ERR_WARP_DIMS = 11,       /* shift arrays neither 1x1 nor nx x ny */
    FLCT_ERR_TIMEOUT = 12          /* a bounded device-side wait expired */
} flct_status;

/* Which window-correlation kernel computes the windows. */
typedef enum {
    FLCT_FORM_FP32 = 0,     /* FP32 shared-memory/register radix FFT */
    FLCT_FORM_TC_FP16 = 1,  /* tensor-core DFT, FP16 hi+lo split operands */
    FLCT_FORM_TC_BF16 = 2,  /* tensor-core DFT, BF16 hi+lo split operands */
    FLCT_FORM_AUTO = 3      /* the autotuner's choice for the box size */
} flct_form;

/* The parsed flct command line (flct.c:337-487).  skip == 0 means no -s. */
typedef struct {
    double deltat;      /* time between the images */
    double deltas;      /* length unit of one pixel */
    double sigma;       /* Gaussian width in pixels; <= 0: global-shift mode */
    double thresh;      /* -t value, any trailing 'a' removed */
    int thresh_abs;     /* 1 if the -t value carried the 'a' suffix */
    int skip;           /* -s N (0: off; negative: error, like "-s 0") */
    int poffset;        /* p of -s NpPqQ as typed (negative wraps) */
    int qoffset;        /* q of -s NpPqQ as typed (negative wraps) */
    int interpolate;    /* 'i' in the -s string */
    int filter;         /* 1 if -k given */
    double kr;          /* -k roll-off, units of the Nyquist wavenumber */
    int hires;          /* 1 if -h given */
    int quiet;          /* 1 if -q given (the library itself never prints) */
    int form;           /* flct_form */
} flct_params;

typedef struct flct_ctx flct_ctx;

/* Timing of the most recent compute call on a context (device time from
 * CUDA events on the context's stream). */
typedef struct {
    float ms_total;      /* the whole call on its stream, first to last operation */
    float ms_window;     /* the window-correlation kernel(s) */
    float ms_prepass;    /* threshold, mask, split and box-sum passes */
    float ms_interp;     /* skip-grid interpolation */
    float ms_h2d;        /* host-to-device copies (host-buffer entry points) */
    float ms_d2h;        /* device-to-host copies (host-buffer entry points) */
    long long windows;   /* correlation windows computed */
    int launches;        /* kernels launched by the call */
    int box;             /* box side n = 2*nsize of the last call */
    int form;            /* flct_form actually used */
    float ms_fit;        /* FP64 peak fit, velocity and mask pass */
} flct_timing;

/* ---- context ------------------------------------------------------- */

/* Create a context on CUDA device `device`.  Returns FLCT_ERR_NO_DEVICE if
 * the device does not exist or is not a Blackwell GB300-class part the
 * kernels were built for. */
FLCT_API flct_status flct_gpu_create(int device, flct_ctx **out);
FLCT_API void flct_gpu_destroy(flct_ctx *ctx);
FLCT_API const char *flct_gpu_last_error(const flct_ctx *ctx);
FLCT_API const char *flct_gpu_status_string(flct_status s);
FLCT_API flct_status flct_gpu_last_timing(const flct_ctx *ctx, flct_timing *t);
/* Library version string, e.g. "0.1.0 sm_103a". */
FLCT_API const char *flct_gpu_version(void);

/* ---- velocity (the flct program) ------------------------------------ */

/* Size of the vx/vy/vm outputs: nx*ny, or 1 in the global-shift mode
 * (sigma <= 0, where flct returns one shift for the whole frame). */
FLCT_API long long flct_gpu_output_len(const flct_params *p, int nx, int ny);

/* Host buffers: copies in, computes, copies out (synchronous). */
FLCT_API flct_status flct_gpu_velocity(flct_ctx *ctx, const flct_params *p,
                              const double *f1, const double *f2, int nx,
                              int ny, double *vx, double *vy, double *vm);

/* Device buffers on the caller's CUDA stream (cudaStream_t passed as a
 * void*; NULL means the CUDA default stream, as everywhere in CUDA).
 * Asynchronous with respect to the host: returns once everything is
 * enqueued.  flct_gpu_last_timing waits for the call to finish. */
FLCT_API flct_status flct_gpu_velocity_device(flct_ctx *ctx, const flct_params *p,
                                     const double *d_f1, const double *d_f2,
                                     int nx, int ny, double *d_vx,
                                     double *d_vy, double *d_vm,
                                     void *stream);

/* One pair of a heterogeneous batch (device pointers). */
typedef struct {
    const double *f1;
    const double *f2;
    int nx, ny;
    flct_params params;
    double *vx, *vy, *vm;
} flct_pair;

/* Every window of every pair; pairs may differ in size and sigma.  Device
 * pointers, caller's stream, asynchronous. */
FLCT_API flct_status flct_gpu_velocity_batch(flct_ctx *ctx, int npairs,
                                    const flct_pair *pairs, void *stream);

/* ---- the reference's internal functions ------------------------------ */

/* cross_cor on nwin windows of n x n (host buffers, back to back).  Returns
 * shiftx (slow axis) and shifty (fast axis) per window exactly as cross_cor
 * does (peak - n/2 after the 3x3 fit).  form selects the kernel. */
FLCT_API flct_status flct_gpu_cross_cor_batch(flct_ctx *ctx, const double *g1,
                                     const double *g2, int n, int nwin,
                                     int filter, double kr, int form,
                                     double *shiftx, double *shifty);

/* interpcc2d (host buffers); out is nxi x nyi. */
FLCT_API flct_status flct_gpu_interpcc2d(flct_ctx *ctx, const double *fdata,
                                double xmiss, int nx, int ny,
                                const double *xwant, int nxi,
                                const double *ywant, int nyi, double *out);

/* shift_frac2d / warp_frac2d (host buffers), transp as in the reference
 * (1 for the CLI's transposed storage).  warp_frac2d's per-pixel spectral
 * sum runs on the tensor cores (split FP16 over the half spectrum, within
 * 1e-6 of max |arr| of the FP64 result); the environment variable
 * FLCT_WARP_SUM=fp32, read at each call, selects the FP32 CUDA-core sum.
 * A tensor-core wait that runs out returns FLCT_ERR_TIMEOUT. */
FLCT_API flct_status flct_gpu_shift_frac2d(flct_ctx *ctx, const double *arr,
                                  double delx, double dely, double *out,
                                  int nx, int ny, int transp);
FLCT_API flct_status flct_gpu_warp_frac2d(flct_ctx *ctx, const double *arr,
                                 const double *delx, const double *dely,
                                 double *out, int nx, int ny, int transp);

/* ---- without device allocation ---------------------------------------- */

/* Largest nxi and nyi flct_gpu_interpcc2d_noalloc accepts. */
#define FLCT_NOALLOC_MAX_AXIS 16384

/* interpcc2d for callers that cannot allocate GPU memory: programs that hand
 * all device memory to their own pool or fix their device-memory budget at
 * start-up, and so cannot let a library call cudaMalloc.  It has no
 * counterpart in the reference; it computes what flct_gpu_interpcc2d
 * computes, on device pointers (fdata nx x ny, xwant nxi, ywant nyi, out
 * nxi x nyi) on `stream` (NULL: the CUDA default stream), and allocates
 * nothing: its only scratch is a fixed 1.2 MB array inside the library that
 * every GPU which loads the library keeps until the process exits.
 *   - nxi or nyi above FLCT_NOALLOC_MAX_AXIS: FLCT_ERR_UNSUPPORTED;
 *     nx or ny below 3: FLCT_ERR_GRID_TOO_SMALL; no sm_103 device current:
 *     FLCT_ERR_NO_DEVICE; a device pointer that lives on another device
 *     than the current one: FLCT_ERR_ARG.
 *   - The first call in a CUDA context (the device's primary context, a
 *     context the caller made, or the new primary context after a
 *     cudaDeviceReset) looks up that array's device address once, with
 *     that context current; make that first call before any stream capture
 *     begins.
 *   - All calls share the one array: calls that overlap on the GPU (other
 *     streams, other host threads) race and must be serialised by the
 *     caller.
 *   - An error the caller's earlier work left pending is neither reported
 *     nor cleared; a launch error of this call is returned as
 *     FLCT_ERR_CUDA.
 *   - Asynchronous: returns once the work is enqueued. */
FLCT_API flct_status flct_gpu_interpcc2d_noalloc(const double *d_fdata, double xmiss,
                                                 int nx, int ny,
                                                 const double *d_xwant, int nxi,
                                                 const double *d_ywant, int nyi,
                                                 double *d_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
