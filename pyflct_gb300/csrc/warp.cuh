// warp.cuh -- launchers for warp.cu (uniform shift and non-uniform warp).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace flct {

constexpr int kWarpMaxAxis = 16384;  // axis tables live in shared memory

// mode 0: circulant tab[(c - k) mod L]; mode 1: DFT tab[(c k) mod L]
cudaError_t launch_axis_fast(int mode, bool real_in, const void* in, int nrows, int L, const float2* tab,
                             float2* out, cudaStream_t st);
cudaError_t launch_axis_slow(int mode, const float2* in, int ncols, int L, const float2* tab, float2* out,
                             cudaStream_t st);
// scratch: 2n double2
cudaError_t launch_shift_vector(int n, double darg, double2* scratch, float2* v, cudaStream_t st);
cudaError_t launch_twiddles(int L, int sign, float2* tw, cudaStream_t st);
// shift_frac2d by transforms, for axes where shift_fft_axis holds (powers of
// two, 64 .. kWarpMaxAxis): scratch 2 (nx + ny) double2, tw nx + ny float2,
// buf1 / buf2 nx * ny float2 each; out nx * ny doubles on the device
bool shift_fft_axis(int n);
cudaError_t launch_shift_fft(const double* in, int nx, int ny, double dxarg, double dyarg, double2* scratch,
                             float2* tw, float2* buf1, float2* buf2, double* out, int nsm, cudaStream_t st);
// F = forward 2-D DFT of a real nx x ny image by transforms, both axes
// shift_fft_axis: tw nx + ny float2, buf1 nx * ny float2 scratch, F nx * ny
// float2 (natural [ii][jj] order)
cudaError_t launch_dft2_fft(const double* in, int nx, int ny, float2* tw, float2* buf1, float2* F, int nsm,
                            cudaStream_t st);
cudaError_t launch_real_part(const float2* in, long n, double* out, cudaStream_t st);
cudaError_t launch_warp_phase(const double* delx, const double* dely, int nx, int ny, int transp, float4* ph,
                              cudaStream_t st);
cudaError_t launch_warp_sum(const float2* F, const float4* ph, int nx, int ny, double* out, cudaStream_t st);
// the same sum on the tensor cores (split FP16, half spectrum): hs is
// warp_tc_split_bytes(nx, ny) of scratch, misc two words (the spectrum's
// largest |component| and the status word, misc[1]: kStatusTimeout bits);
// stall_ns > 0 is a test hook (the first MMA wait gives up after stall_ns)
size_t warp_tc_split_bytes(int nx, int ny);
cudaError_t launch_warp_sum_tc(const float2* F, const float4* ph, int nx, int ny, void* hs, unsigned* misc,
                               double* out, cudaStream_t st, unsigned long long stall_ns = 0);

}  // namespace flct
