// window_common.cuh -- the FP64 passes around the window-correlation
// kernels, shared by every window form.
//
// GB300's FP64 pipe is narrow, and an FP64 instruction executed by one lane
// of a warp costs as much pipe time as one executed by all 32.  So the
// per-window FP64 work of the reference's loop body runs with one window
// per lane instead of one lane per window: the local means (flct.c:815-827)
// in the column pass of the box sums (k_box_cols, one grid point per lane
// group), and
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

// Where the window of pixel (i, j) finds its local means: one float4
// (f1 hi, f2 hi, f1 lo, f2 lo) per grid point [gi][gj], grid point (q, m) =
// pixel (xo + q gs, yo + m gs).
struct MeanGrid {
    int gs, xo, yo, gj;
};
__host__ __device__ __forceinline__ int mean_slot(const MeanGrid& g, int i, int j) {
    return ((i - g.xo) / g.gs) * g.gj + (j - g.yo) / g.gs;
}

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


__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// Shifts of work item w to velocity, mask and the skip-grid copy
// (flct.c:901-942, 1125-1133), or to the raw-shift outputs.
__device__ __forceinline__ void store_shift(const FitArgs& a, int w, double shx, double shy) {
    if (a.shx) {
        a.shx[w] = shx;
        a.shy[w] = shy;
    }
    if (a.vx) {
        const int pix = a.work[w];
        const int i = pix / a.ny, j = pix - (pix / a.ny) * a.ny;
        // transposed storage: vx from the fast-axis shift (flct.c:901-905),
        // scaled by deltas / deltat in one product
        double vxx = dm(shy, a.vscale);
        double vyy = dm(shx, a.vscale);
        double vmm = 1.;
        if (a.grid) {
            const int ic = (i - a.xoff) / a.skip, jc = (j - a.yoff) / a.skip;
            a.grid[(size_t)ic * a.jcnt + jc] = make_float2(split_double_fast(vxx).x, split_double_fast(vyy).x);
        }
        // xmiss tests on the bit patterns (xmiss is a normal number)
        const long long xm = __double_as_longlong(kXmiss);
        if (__double_as_longlong(vxx) == xm) {
            vmm = 0.;
            vxx = 0.;
        }
        if (__double_as_longlong(vyy) == xm) vyy = 0.;
        a.vx[pix] = vxx;
        a.vy[pix] = vyy;
        a.vm[pix] = vmm;
    }
}

// The 3x3 Taylor fit (flct.c:1536-1553, 1607-1630) of v[3p+q] = f at
// (peak-1+p, peak-1+q), in the reference's operation order without FMA
// contraction, except that both shifts multiply by one reciprocal of the
// determinant (one FP64 division instead of two).
__device__ __forceinline__ void fit3x3(const double* v, double* sx, double* sy) {
    const double fx = dm(0.5, ds(v[7], v[1]));
    const double fy = dm(0.5, ds(v[5], v[3]));
    const double fxx = ds(da(v[7], v[1]), dm(2., v[4]));
    const double fyy = ds(da(v[5], v[3]), dm(2., v[4]));
    const double fxy = dm(0.25, ds(ds(da(v[8], v[0]), v[6]), v[2]));
    const double den = ds(dm(fxy, fxy), dm(fxx, fyy));
    const double inv = 1.0 / den;  // one division for both shifts
    *sx = dm(ds(dm(fyy, fx), dm(fy, fxy)), inv);
    *sy = dm(ds(dm(fxx, fy), dm(fx, fxy)), inv);
}

// Fit, velocity and stores of work item w from its peak record.
__device__ __forceinline__ void fit_item(const FitArgs& a, int w, const PeakRec& r) {
    const int half = a.n / 2, half1 = (a.n1 ? a.n1 : a.n) / 2;
    const int I = meta_I(r.meta), J = meta_J(r.meta);
    double sx = 0., sy = 0.;
    if (meta_flag(r.meta)) {
        double v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = f2d(r.v[k]);
        fit3x3(v, &sx, &sy);
    }
    store_shift(a, w, da((double)(I - half), sx), da((double)(J - half1), sy));
}

// One image pair of a batched window launch.  The pair's work items and
// peak records sit at [base, base + its work count) of the batch's arrays,
// its means at base + mean_slot(mg, i, j); seg_start (device, prefix sums
// of the work counts, one more entry than segments) maps a launch-wide
// item index to its pair.
struct WinSeg {
    const float4* s12;  // the pair's split frames (WinArgs::s12)
    int nx, ny;
    int base;
    MeanGrid mg;
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

__global__ void k_fit(FitArgs a);
__global__ void k_fit_hires(FitArgs a);
// the same kernels over many frame pairs at once (MultiArgs, common.cuh)
__global__ void k_fit_multi(MultiArgs<FitArgs> m);
__global__ void k_fit_hires_multi(MultiArgs<FitArgs> m);

// Batched launches: for every group g, start[first[g] + g + k] (k = 0..nseg)
// = prefix sums of the work counts (int at ctr + 64 * pair) of the group's
// pairs seg_pair[first[g] .. first[g+1]).
__global__ void k_batch_starts(const unsigned char* ctr, const int* seg_pair, const int* first, int ngroups,
                               int* start);

}  // namespace flct
