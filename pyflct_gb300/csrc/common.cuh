// common.cuh -- shared definitions for the FLCT CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace flct {

// Missing-value marker of the reference (flct.c:279).
constexpr double kXmiss = -999999.;

// Status bits a kernel may raise in the context's device status word.
enum : unsigned {
    kStatusRange = 1u,    // an input magnitude does not fit FP32
    kStatusTimeout = 2u,  // a bounded wait gave up
};

// Box start along one axis: centred on i, pinned inside [0, n)
// (flct.c:773-788).  With 2*nsize < n the two pins never both apply.
__host__ __device__ __forceinline__ int box_start(int i, int n, int nsize) {
    int lo0 = (0 > (i - (nsize - 1))) ? 0 : i - (nsize - 1);
    int hi0 = ((n - 1) < (i + nsize)) ? n - 1 : i + nsize;
    return (hi0 == n - 1) ? n - 1 - (2 * nsize - 1) : lo0;
}

// Split a double into float hi + float lo (hi = nearest float, lo = nearest
// float to the remainder): a - (hi + lo) is below 2^-48 |a|.
__device__ __forceinline__ float2 split_double(double a) {
    float hi = __double2float_rn(a);
    float lo = __double2float_rn(__dsub_rn(a, (double)hi));
    return make_float2(hi, lo);
}

// Power-of-two factor bringing a non-negative float (given as its bits) into
// [1, 4): exact scaling that leaves every ratio and argmax unchanged.
__device__ __forceinline__ float pow2_scale(unsigned bits) {
    if (bits == 0u) return 1.0f;
    unsigned e = bits >> 23;
    if (e >= 255u) return 1.0f;                 // inf / NaN: leave as is
    if (e == 0u) return 18446744073709551616.0f; // subnormal: 2^64
    if (e > 253u) e = 253u;
    return __uint_as_float((254u - e) << 23);
}

}  // namespace flct
