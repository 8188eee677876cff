// global.cuh -- the sigma <= 0 mode of flct: one correlation of the two
// whole frames (flct.c:581-586, 666-675, 802-808).
//
// The frames are mean-subtracted (FP64 means), packed as z = g1 + i g2 in
// FP32 (hi + lo split, scaled by a power of two), transformed by batched
// direct DFTs along each axis (any size; exact twiddle tables built on the
// host), separated into conj(A) B with the mirror trick and the -k filter,
// transformed back, and |c| searched for its first strict maximum in the
// half-shifted frame.  The peak record then goes through the same k_fit /
// k_fit_hires as the sliding windows.
#pragma once
#include "common.cuh"
#include "window_common.cuh"

namespace flct {

constexpr int kGsumBlocks = 256;

// Per-block FP64 partial sums of both frames (fixed order), then the final
// sum of the partials in one block.
__global__ void k_gsum_part(const double* f1, const double* f2, long n, double* part);
__global__ void k_gsum_final(const double* part, int nparts, double inv_n, double* means);

// z = (f1 - m1) + i (f2 - m2) in FP32; |g| maxima (float bits) for the scale.
__global__ void k_gz(const double* f1, const double* f2, long n, const double* means, float2* z,
                     unsigned* maxbits, unsigned* status);

// out[l][k] = sum_j in[l][j] tw[(j k) mod L]^dir, lines of length L
// contiguous (stride L); with `scale` the inputs are first multiplied by
// (pow2_scale(scale[0]), pow2_scale(scale[1])) per component.
cudaError_t launch_dft_rows(bool inverse, const float2* in, float2* out, int L, int lines, const float2* tw,
                            const unsigned* scale, cudaStream_t st);

// out[c][r] = in[r][c] for an R x C array.
__global__ void k_transpose(const float2* in, float2* out, int R, int C);

// C = conj(A) B filt, A and B separated from Z and its mirror, on the
// transposed spectrum Zt[ky][kx] (ny x nx).
__global__ void k_gprod(const float2* zt, float2* ct, int nx, int ny, const float* fx2, const float* fy2);

// First strict maximum of |Re c| in the half-shifted frame, as a key
// (value bits << 32 | ~index), NaN skipped.
__global__ void k_gpeak(const float2* c, int nx, int ny, unsigned long long* key);

// The peak record (3x3, or the 6x6 -h patch) and a one-item work list.
__global__ void k_gpatch(const float2* c, int nx, int ny, const unsigned long long* key, PeakRec* rec,
                         PeakRecH* rech, int* work, int* nwork);

}  // namespace flct
