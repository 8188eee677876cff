/* vcio.h -- vel_ccor files, the reference's flct / warp file format
 * (source/flct.c:1158-1268, 2016-2109; source/warp.c:362-535):
 *   int32 magic 2136967593, int32 NX, int32 NY (IDL order: fast axis
 *   first), then `count` float32 arrays of NX*NY values, all big-endian.
 * In memory the arrays are C order [nx][ny] with nx = NY (slow axis) and
 * ny = NX, which is what the reference's transp = 1 reading gives. */
#ifndef PYFLCT_GB300_VCIO_H
#define PYFLCT_GB300_VCIO_H

#define VC_MAGIC 2136967593

/* Reads `count` arrays (malloc'ed doubles, caller frees).  On failure prints
 * the reference's message prefixed by `who` ("read2images", "readimage")
 * and returns nonzero. */
int vc_read(const char *path, int count, int *nx, int *ny, double **arrays, const char *who);

/* Writes `count` arrays of nx*ny values, converted to float32. */
int vc_write(const char *path, int count, int nx, int ny, double *const *arrays, const char *who);

#endif
