/* flct_main.c -- the `flct` program on the GPU: the reference's command line
 * (source/flct.c:283-530), vel_ccor files in and out, and the velocity
 * computed through the C ABI (flct_gpu_velocity).  There is no CPU path:
 * without a usable GPU the program reports it and exits 1.
 *
 *   flct ifile ofile deltat deltas sigma [-t thr[a]] [-k kr]
 *        [-s N[pP][qQ][i]] [-h] [-q]
 *
 * Options are recognised by their first two characters and may come in any
 * order after the five required arguments, as in the reference.  Fatal
 * conditions print the reference's message and exit with status 1.
 * FLCT_GPU_DEVICE selects the CUDA device (default 0) and FLCT_GPU_FORM the
 * window form (fp32, tc_fp16, tc_bf16 or auto, the default). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "flct_gpu.h"
#include "vcio.h"

static const char *kVersion = "1.01   ";

static void usage(const char *prog) {
    printf("flct: Version %s (GB300 GPU build)\n\n", kVersion);
    printf("Syntax: %s ifile ofile deltat deltas sigma -t thr -k kr -s N[pP][qQ][i] -h -q\n\n", prog);
    printf("ifile - contains 2 images for local correlation tracking\n");
    printf("ofile - contains output vx, vy, vm (x,y velocity and mask\n");
    printf("   arrays).  Mask array 0 where velocity not computed.\n");
    printf("deltat - amount of time between images\n");
    printf("deltas - units of length of the side of a single pixel\n");
    printf("   (note velocity is computed in units of deltas/deltat)\n");
    printf("sigma - images modulated by gaussian of width sigma pixels\n");
    printf("(set sigma=0. to just get the overall shift between 2 images)\n");
    printf("Optional parameters:\n");
    printf("-t thr - if avg abs value image pixel < thr, skip calc\n");
    printf("   (thr between 0 & 1 is relative to the max. abs. pixel value;\n");
    printf("   append an 'a' to force absolute units)\n");
    printf("-s NpPqQ - skip calc except every N pixels in x and y,\n");
    printf("   P and Q pixel offsets; append 'i' to interpolate skipped points\n");
    printf("-k kr - filter subimages w/gaussian w/ roll-off wavenumber kr\n");
    printf("-h  - 'hires' flag - Use cub. conv. interp. to find shift\n");
    printf("-q  - flag to suppress printing all non-error messages\n");
}

static int form_from_env(void) {
    const char *f = getenv("FLCT_GPU_FORM");
    if (!f || !strcmp(f, "auto")) return FLCT_FORM_AUTO;
    if (!strcmp(f, "fp32")) return FLCT_FORM_FP32;
    if (!strcmp(f, "tc_fp16")) return FLCT_FORM_TC_FP16;
    if (!strcmp(f, "tc_bf16")) return FLCT_FORM_TC_BF16;
    return FLCT_FORM_AUTO;
}

int main(int argc, char *argv[]) {
    if (argc < 6 || argc > 14) {
        usage(argv[0]);
        return 1;
    }
    char infile[100], outfile[100], buf[100];
    strncpy(infile, argv[1], 99);
    infile[99] = '\0';
    strncpy(outfile, argv[2], 99);
    outfile[99] = '\0';
    flct_params p;
    memset(&p, 0, sizeof(p));
    p.deltat = atof(argv[3]);
    p.deltas = atof(argv[4]);
    p.sigma = atof(argv[5]);
    p.form = form_from_env();
    int quiet = 0, skipon = 0;
    for (int k = 6; k < argc; ++k) {
        if (!strncmp("-h", argv[k], 2)) p.hires = 1;
        if (!strncmp("-q", argv[k], 2)) quiet = 1;
        if (!strncmp("-t", argv[k], 2) && k + 1 < argc) {
            strncpy(buf, argv[k + 1], 99);
            buf[99] = '\0';
            char *a = strchr(buf, 'a');
            p.thresh_abs = a != NULL;
            if (a) *a = '\0';
            p.thresh = atof(buf);
        }
        if (!strncmp("-s", argv[k], 2) && k + 1 < argc) {
            strncpy(buf, argv[k + 1], 99);
            buf[99] = '\0';
            char *c = strchr(buf, 'i');
            p.interpolate = c != NULL;
            if (c) *c = '\0';
            p.qoffset = 0;
            p.poffset = 0;
            if ((c = strchr(buf, 'q')) != NULL) {
                p.qoffset = atoi(c + 1);
                *c = '\0';
            }
            if ((c = strchr(buf, 'p')) != NULL) {
                p.poffset = atoi(c + 1);
                *c = '\0';
            }
            p.skip = atoi(buf);
            if (p.skip <= 0) {
                printf("flct: skip =%d is zero or negative, fatal\n", p.skip);
                return 1;
            }
            if (abs(p.poffset) >= p.skip || abs(p.qoffset) >= p.skip) {
                printf("flct: p=%d,q=%d, abs(p) or abs(q) >= skip=%d\n", p.poffset, p.qoffset, p.skip);
                return 1;
            }
            skipon = 1;
        }
        if (!strncmp("-k", argv[k], 2) && k + 1 < argc) {
            p.kr = atof(argv[k + 1]);
            p.filter = 1;
        }
    }
    p.quiet = quiet;
    if (!quiet) {
        printf("flct: Version %s (GB300 GPU build of the C ABI %s)\n", kVersion, flct_gpu_version());
        printf("flct: infile = %s\n", infile);
        printf("flct: outfile = %s\n", outfile);
        printf("flct: deltat = %g\n", p.deltat);
        printf("flct: deltas = %g\n", p.deltas);
        printf("flct: sigma = %g\n", p.sigma);
        printf("flct: threshold image value for LCT is %g\n", p.thresh);
        if (p.thresh_abs) printf("flct: threshold forced to be in abs. units\n");
        if (skipon) printf("flct: skip = %d pixels with p=%d, q=%d\n", p.skip, p.poffset, p.qoffset);
        if (p.interpolate) printf("flct: skipped pixels interpolated with cubic convolution\n");
        if (p.filter) printf("flct: filter rolloff value for input images is %g\n", p.kr);
        if (p.hires) printf("flct: hires option turned on\n");
    }
    int nx = 0, ny = 0;
    double *f[2] = {NULL, NULL};
    if (vc_read(infile, 2, &nx, &ny, f, "read2images")) return 1;
    if (!quiet) printf("flct: from input file, nx = %d, ny = %d\n", nx, ny);

    const char *dev = getenv("FLCT_GPU_DEVICE");
    flct_ctx *ctx = NULL;
    flct_status s = flct_gpu_create(dev ? atoi(dev) : 0, &ctx);
    if (s != FLCT_OK) {
        printf("flct: %s (a GB300 / sm_103 GPU is required; there is no CPU path)\n", flct_gpu_status_string(s));
        return 1;
    }
    const long long nout = flct_gpu_output_len(&p, nx, ny);
    double *v[3];
    for (int k = 0; k < 3; ++k) v[k] = (double *)malloc(sizeof(double) * (size_t)(nout > 0 ? nout : 1));
    s = flct_gpu_velocity(ctx, &p, f[0], f[1], nx, ny, v[0], v[1], v[2]);
    if (s != FLCT_OK) {
        printf("%s\n", flct_gpu_last_error(ctx));
        flct_gpu_destroy(ctx);
        return 1;
    }
    if (!quiet) {
        flct_timing t;
        if (flct_gpu_last_timing(ctx, &t) == FLCT_OK)
            printf("flct: %lld correlation windows in %.3f ms on the GPU\n", t.windows, (double)t.ms_total);
    }
    flct_gpu_destroy(ctx);
    const int onx = nout == 1 ? 1 : nx, ony = nout == 1 ? 1 : ny;
    if (vc_write(outfile, 3, onx, ony, v, "write3images")) return 1;
    if (!quiet) printf("\nflct: finished\n");
    for (int k = 0; k < 3; ++k) free(v[k]);
    free(f[0]);
    free(f[1]);
    return 0;
}
