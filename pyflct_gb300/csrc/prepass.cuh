// prepass.cuh -- argument structs and launch helpers for prepass.cu.
#pragma once
#include "common.cuh"
#include "fixsum.cuh"

namespace flct {

struct ClassifyArgs {
    const double* f1;
    const double* f2;
    int nx, ny;
    double thr_val;           // absolute threshold, used when thr_ptr is null
    const double* thr_ptr;    // device threshold from k_thresh_final
    int skip, xoff, yoff, interpolate, jcnt;
    float4* s12;              // both frames' float split per pixel: (f1 hi, f2 hi, f1 lo, f2 lo)
    int* work;
    int* nwork;
    double *vx, *vy, *vm;
    float2* grid;             // skip-grid (vx, vy) for the interpolation, or null
    unsigned* status;
    int r0, r1;               // rows to classify (the work list gets their windows)
    int* work2;               // when set: windows of rows >= rsplit go to this list
    int* nwork2;
    int rsplit;
};

// Classification: pixels per thread, and per tile (256 threads).
constexpr int kClassPpt = 4;
constexpr int kClassPix = 256 * kClassPpt;

// Row pass of the box sums: warps per block, and the longest input span a
// warp converts into shared memory per pass.
constexpr int kBoxWarps = 4;
constexpr int kRowSpan = 544;
// Column pass: grid rows per thread, runs start at multiples of it (the
// units of a run's box sums depend on the rows it reads)
constexpr int kColRun = 4;
// Column pass: lanes that share one run's rows (a power of two <= 32)
constexpr int kColLanes = 4;

// Local means for the boxes the grid needs, from exact box sums
// (fixsum.cuh).  Grid point (q, m) is pixel (xo + q gs, yo + m gs) (gs = 1,
// xo = yo = 0 without -s); its box starts at (box_start(xo + q gs),
// box_start(yo + m gs)).
struct BoxArgs {
    const double* f1;
    const double* f2;
    int nx, ny, n, nsize;
    int gs, xo, yo, gi, gj;   // grid step, offsets and counts (slow, fast axis)
    int pass_r;               // row pass: grid columns per warp pass
    BoxSum *rt1, *rt2;        // row sums [nx][gj]
    int *re1, *re2;           // their exponents, compact [nx][gj]
    float4* means;            // local means [gi][gj]: (f1 hi, f2 hi, f1 lo, f2 lo)
    double inv_n2;            // 1 / n^2
    int r0, r1;               // frame rows of the row pass
    int q0, q1;               // grid rows of the column pass
};

// Interpolation tiles: kTileR x kTileC pixels per block of kInterpThreads.
constexpr int kTileR = 32, kTileC = 32, kInterpThreads = 256;

// The velocity pipeline's skip-grid interpolation (FP32 arithmetic).
struct InterpArgs {
    int nx, ny, skip, xoff, yoff;
    int gx, gy;               // grid counts along the slow / fast axis
    const float2* grid;       // (vx, vy) per grid point [gx][gy]
    double *vx, *vy, *vm;
    int i0, i1;               // output rows to interpolate
    int pairs;                // ny even and vx, vy, vm 16-byte aligned: pixel pairs as 16-byte stores
    const unsigned* pub_src;  // the call's counters to host memory (publish_counters)
    unsigned* pub_dst;
};

// max |f| of both frames (IEEE bit patterns, NaN skipped) into out[0..1]
struct AbsmaxArgs {
    const double* f1;
    const double* f2;
    long n;
    unsigned long long* out;
};
// the relative threshold thresh * max(f1max, f2max) into *thr
struct ThreshArgs {
    const double* f1;
    const double* f2;
    const unsigned long long* mx;
    double thresh;
    double* thr;
};

__global__ void k_absmax(AbsmaxArgs a);
__global__ void k_thresh_final(ThreshArgs a);
__global__ void k_classify(ClassifyArgs a);
__global__ void k_box_rows(BoxArgs a);
__global__ void k_box_cols(BoxArgs a);
// the same kernels over many frame pairs at once (MultiArgs, common.cuh)
__global__ void k_absmax_multi(MultiArgs<AbsmaxArgs> m);
__global__ void k_thresh_final_multi(MultiArgs<ThreshArgs> m);
__global__ void k_classify_multi(MultiArgs<ClassifyArgs> m);
__global__ void k_box_rows_multi(MultiArgs<BoxArgs> m);
__global__ void k_box_cols_multi(MultiArgs<BoxArgs> m);
__global__ void k_interp_grid_multi(MultiArgs<InterpArgs> m);
__global__ void k_interp_axis(int n, int gcount, int off, int skip, const double* want, int* zero,
                              double* wts, unsigned char* ok);
__global__ void k_interp_grid(InterpArgs a);
__global__ void k_interp_general(const double* f, int gx, int gy, double xmiss, const int* zx,
                                 const double* wx, const unsigned char* okx, int nxi, const int* zy,
                                 const double* wy, const unsigned char* oky, int nyi, double* out);

}  // namespace flct
