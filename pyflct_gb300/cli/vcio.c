/* vcio.c -- vel_ccor file reading and writing (see vcio.h). */
#include "vcio.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint32_t be32(const unsigned char *b) {
    return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}

static void put_be32(unsigned char *b, uint32_t v) {
    b[0] = (unsigned char)(v >> 24);
    b[1] = (unsigned char)(v >> 16);
    b[2] = (unsigned char)(v >> 8);
    b[3] = (unsigned char)v;
}

int vc_read(const char *path, int count, int *nx, int *ny, double **arrays, const char *who) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        printf("%s: cannot open file %s\n", who, path);
        return 1;
    }
    unsigned char h[12];
    if (fread(h, 1, 12, f) != 12 || (int32_t)be32(h) != VC_MAGIC) {
        printf("%s: input file is not a vel_ccor i/o file\n", who);
        fclose(f);
        return 1;
    }
    /* IDL NX (fast axis) first: it becomes the C fast dimension ny */
    *ny = (int32_t)be32(h + 4);
    *nx = (int32_t)be32(h + 8);
    if (*nx < 1 || *ny < 1) {
        printf("%s: bad array dimensions %d x %d in %s\n", who, *ny, *nx, path);
        fclose(f);
        return 1;
    }
    const size_t n = (size_t)(*nx) * (size_t)(*ny);
    unsigned char *buf = (unsigned char *)malloc(n * 4);
    if (!buf) {
        printf("%s: memory request for arr failed\n", who);
        fclose(f);
        return 1;
    }
    for (int a = 0; a < count; ++a) {
        arrays[a] = (double *)malloc(n * sizeof(double));
        if (!arrays[a]) {
            printf("%s: memory request for arr failed\n", who);
            free(buf);
            fclose(f);
            return 1;
        }
        if (fread(buf, 4, n, f) != n) {
            printf("%s: file %s holds fewer than %d arrays of %d x %d\n", who, path, count, *ny, *nx);
            free(buf);
            fclose(f);
            return 1;
        }
        for (size_t k = 0; k < n; ++k) {
            const uint32_t u = be32(buf + 4 * k);
            float v;
            memcpy(&v, &u, 4);
            arrays[a][k] = (double)v;
        }
    }
    free(buf);
    fclose(f);
    return 0;
}

int vc_write(const char *path, int count, int nx, int ny, double *const *arrays, const char *who) {
    FILE *f = fopen(path, "wb");
    if (!f) {
        printf("%s: cannot open file %s\n", who, path);
        return 1;
    }
    unsigned char h[12];
    put_be32(h, (uint32_t)VC_MAGIC);
    put_be32(h + 4, (uint32_t)ny);
    put_be32(h + 8, (uint32_t)nx);
    const size_t n = (size_t)nx * (size_t)ny;
    unsigned char *buf = (unsigned char *)malloc(n * 4);
    int bad = fwrite(h, 1, 12, f) != 12 || !buf;
    for (int a = 0; a < count && !bad; ++a) {
        for (size_t k = 0; k < n; ++k) {
            const float v = (float)arrays[a][k];
            uint32_t u;
            memcpy(&u, &v, 4);
            put_be32(buf + 4 * k, u);
        }
        bad = fwrite(buf, 4, n, f) != n;
    }
    free(buf);
    if (fclose(f) != 0) bad = 1;
    if (bad) printf("%s: write to %s failed\n", who, path);
    return bad;
}
