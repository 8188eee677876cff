// warp_math.cuh -- wavenumbers and phase factors shared by the warp kernels.
#pragma once
#include <cuda_runtime.h>

namespace flct {

// Integer wavenumber of FFT index k (make_freq, warp.c:316-360): 0..n/2
// ascending (the Nyquist index n/2 of an even axis is +n/2), then the
// negative wavenumbers rising to -1.
__device__ __forceinline__ int freq_of(int k, int n) { return (k <= n / 2) ? k : k - n; }

// cos/sin of 2 pi * frac(kf * (h + l)) with kf an integer wavenumber:
// the product is formed exactly enough in float-float (fma error term) and
// reduced to (-1/2, 1/2] turn before the trigonometric evaluation.
__device__ __forceinline__ float2 turn_cs(float kf, float h, float l) {
    const float p = kf * h;
    const float e = fmaf(kf, h, -p);  // exact error of the product
    const float fr = (p - rintf(p)) + fmaf(kf, l, e);
    float s, c;
    sincospif(2.0f * fr, &s, &c);
    return make_float2(c, s);
}

}  // namespace flct
