/* warp_main.c -- the `warp` program on the GPU: the reference's command
 * line (source/warp.c:69-201), vel_ccor files in and out, and the shift or
 * warp computed through the C ABI (flct_gpu_shift_frac2d /
 * flct_gpu_warp_frac2d).  There is no CPU path.
 *
 *   warp ifile sfile ofile [-q]
 *
 * sfile holds two arrays (delx, dely): of the image's size they warp it
 * pixel by pixel, 1 x 1 they shift it uniformly, anything else is fatal.
 * FLCT_GPU_DEVICE selects the CUDA device (default 0). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "flct_gpu.h"
#include "vcio.h"

int main(int argc, char *argv[]) {
    if (argc < 4 || argc > 6) {
        printf("warp: Version 1.01    (GB300 GPU build)\n\n");
        printf("Syntax: %s ifile sfile ofile [-q]\n\n", argv[0]);
        printf("ifile - contains 1 image for shifting\n");
        printf("sfile - contains 2 values (or arrays) of shifts (or warps)\n");
        printf("ofile - contains output image of shifted or warped array\n");
        printf("-q - optional flag to omit all non-error messages\n");
        return 1;
    }
    char ifile[100], sfile[100], ofile[100];
    strncpy(ifile, argv[1], 99);
    ifile[99] = '\0';
    strncpy(sfile, argv[2], 99);
    sfile[99] = '\0';
    strncpy(ofile, argv[3], 99);
    ofile[99] = '\0';
    int quiet = argc == 5 && !strncmp("-q", argv[argc - 1], 2);
    if (!quiet) {
        printf("warp: Version 1.01    (GB300 GPU build of the C ABI %s)\n", flct_gpu_version());
        printf("warp: ifile = %s\n", ifile);
        printf("warp: sfile = %s\n", sfile);
        printf("warp: ofile = %s\n", ofile);
    }
    int nx = 0, ny = 0, nxd = 0, nyd = 0;
    double *img[1] = {NULL}, *del[2] = {NULL, NULL};
    if (vc_read(ifile, 1, &nx, &ny, img, "readimage")) return 1;
    if (!quiet) printf("warp: from input file, nx = %d, ny = %d\n", nx, ny);
    if (vc_read(sfile, 2, &nxd, &nyd, del, "read2images")) return 1;
    const int warp = nxd == nx && nyd == ny, shift = nxd == 1 && nyd == 1;
    if (!warp && !shift) {
        printf("warp: bad shift arrays: nx=%d, nxdel=%d, ny=%d, nydel=%d\n", nx, nxd, ny, nyd);
        return 1;
    }
    const char *dev = getenv("FLCT_GPU_DEVICE");
    flct_ctx *ctx = NULL;
    flct_status s = flct_gpu_create(dev ? atoi(dev) : 0, &ctx);
    if (s != FLCT_OK) {
        printf("warp: %s (a GB300 / sm_103 GPU is required; there is no CPU path)\n", flct_gpu_status_string(s));
        return 1;
    }
    double *out[1];
    out[0] = (double *)malloc(sizeof(double) * (size_t)nx * (size_t)ny);
    /* transp = 1: the reference's C programs work on transposed arrays */
    s = warp ? flct_gpu_warp_frac2d(ctx, img[0], del[0], del[1], out[0], nx, ny, 1)
             : flct_gpu_shift_frac2d(ctx, img[0], del[0][0], del[1][0], out[0], nx, ny, 1);
    if (s != FLCT_OK) {
        printf("%s\n", flct_gpu_last_error(ctx));
        flct_gpu_destroy(ctx);
        return 1;
    }
    flct_gpu_destroy(ctx);
    if (vc_write(ofile, 1, nx, ny, out, "writeimage")) return 1;
    if (!quiet) printf("\nwarp: finished\n");
    free(out[0]);
    free(img[0]);
    free(del[0]);
    free(del[1]);
    return 0;
}
