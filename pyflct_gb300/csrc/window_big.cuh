// window_big.cuh -- the window-correlation kernel for boxes above 64
// (window_big.cu).
#pragma once
#include "common.cuh"
#include "window_common.cuh"

namespace flct {

constexpr int kMaxBigBox = 128;  // largest box side of the big-box kernel

struct BigArgs {
    const float4* s12;    // both frames split per pixel (WinArgs::s12)
    const float4* means;  // per grid point at mean_slot(mg, i, j), or null: zero means
    MeanGrid mg;
    const int* work;
    const int* nwork;
    int nx, ny, nsize, n;
    int use_filter;
    int direct;           // windows given directly: box w starts at row w*n, unit weights
    PeakRec* peaks;
    PeakRecH* peaks_h;    // -h records instead (else null)
    const WinSeg* segs;   // batched launch (see WinArgs), else null
    const int* seg_start;
    int nseg;
    float2 tw[kMaxBigBox];             // e^{-2 pi i m / n}, m < n
    float gauss[2 * kMaxBigBox + 1];   // weight of offset d at d + n
    float filt2[kMaxBigBox];           // squared k-space filter by frequency index
};

__global__ void k_window_big(BigArgs a);
size_t window_big_smem(int n);
cudaError_t launch_window_big(const BigArgs& a, int grid, cudaStream_t st, bool pdl);
int window_big_blocks_per_sm(int n);

}  // namespace flct
