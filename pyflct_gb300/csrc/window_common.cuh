// window_common.cuh -- the FP64 passes around the window-correlation
// kernels, shared by every window form.
//
// GB300's FP64 pipe is narrow, and an FP64 instruction executed by one lane
// of a warp costs as much pipe time as one executed by all 32.  So the
// per-window FP64 work of the reference's loop body runs here with one
// window per lane instead of inside the window kernels:
//   k_means  FP64 local means from the box sums (flct.c:815-827), split into
//            float hi + lo for the FP32 window load;
//   k_fit    the 3x3 Taylor fit around the integer peak (flct.c:1536-1553,
//            1639-1640), velocity (flct.c:901-905), mask, skip-grid copy and
//            the final xmiss reset (flct.c:918-942, 1125-1133).
#pragma once
#include "common.cuh"
#include "fixsum.cuh"

namespace flct {

constexpr int kMaxBox = 64;  // largest box side with a compiled window kernel

// What a window kernel hands to k_fit: |c| at the 3x3 stencil around the
// integer peak (half-shifted frame, row-major) and the peak itself.
struct PeakRec {
    float v[9];
    unsigned meta;  // peak_meta(I, J, dofit)
};

// The -h (hires) form of PeakRec: |c| on the 6x6 patch rows I-2..I+3,
// columns J-2..J+3 around the integer peak (0 outside the box), which holds
// every value the reference's 21x21 cubic-convolution zoom around the peak
// reads, border extrapolations included (flct.c:1564-1600, 2257-2336).
constexpr int kHiresPatch = 6;
struct PeakRecH {
    float v[kHiresPatch * kHiresPatch];
    unsigned meta;  // peak_meta(I, J, have)
};

// I and J take 15 bits each (the sigma-0 mode correlates whole frames of up
// to kMaxGlobalAxis per side), the flag bit 30.
constexpr int kMaxGlobalAxis = 32767;
__host__ __device__ __forceinline__ unsigned peak_meta(int I, int J, bool flag) {
    return (unsigned)I | ((unsigned)J << 15) | ((flag ? 1u : 0u) << 30);
}
__host__ __device__ __forceinline__ int meta_I(unsigned m) { return (int)(m & 0x7fffu); }
__host__ __device__ __forceinline__ int meta_J(unsigned m) { return (int)((m >> 15) & 0x7fffu); }
__host__ __device__ __forceinline__ bool meta_flag(unsigned m) { return (m >> 30) & 1u; }

struct MeansArgs {
    const int* work;
    const int* nwork;
    int ny;
    int gs, xo, yo, gj;   // grid step and offsets; box sums are [grid row][grid column]
    const BoxSum* bs1;    // exact box sums [gi][gj] (fixsum.cuh)
    const BoxSum* bs2;
    double inv_n2;
    float4* means;
};

struct FitArgs {
    const int* work;
    const int* nwork;
    const PeakRec* peaks;
    int n;                 // box side (square boxes)
    int n1;                // fast-axis side when the box is not square (sigma 0), else 0
    int ny;
    double vscale;         // deltas / deltat (flct.c:343, 901-905)
    int skip, xoff, yoff, jcnt;
    double *vx, *vy, *vm;  // outputs [nx*ny] or null (window-only calls)
    float2* grid;          // skip-grid (vx, vy) for the interpolation, or null
    double *shx, *shy;     // raw shifts per work item or null
    const PeakRecH* peaks_h;  // -h: patches instead of peaks (k_fit_hires)
    const unsigned* pub_src;  // when pub_dst is set: the call's work count and status,
    unsigned* pub_dst;        // copied to page-locked host memory by one thread
};


// One image pair of a batched window launch.  The pair's work items,
// means and peak records sit at [base, base + its work count) of the
// batch's arrays; seg_start (device, prefix sums of the work counts, one
// more entry than segments) maps a launch-wide item index to its pair.
struct WinSeg {
    const float2* s1;
    const float2* s2;
    int nx, ny;
    int base;
    int pad;
};

// Largest k in [0, nseg) with start[k] <= w (skips pairs without work).
__device__ __forceinline__ int seg_find(const int* __restrict__ start, int nseg, int w) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(start + mid) <= w) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_means(MeansArgs a);
__global__ void k_fit(FitArgs a);
__global__ void k_fit_hires(FitArgs a);
// the same kernels over many frame pairs at once (MultiArgs, common.cuh)
__global__ void k_means_multi(MultiArgs<MeansArgs> m);
__global__ void k_fit_multi(MultiArgs<FitArgs> m);
__global__ void k_fit_hires_multi(MultiArgs<FitArgs> m);

// Batched launches: for every group g, start[first[g] + g + k] (k = 0..nseg)
// = prefix sums of the work counts (int at ctr + 64 * pair) of the group's
// pairs seg_pair[first[g] .. first[g+1]).
__global__ void k_batch_starts(const unsigned char* ctr, const int* seg_pair, const int* first, int ngroups,
                               int* start);

}  // namespace flct
