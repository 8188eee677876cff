// common.cuh -- shared definitions for the FLCT CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace flct {

// Missing-value marker of the reference (flct.c:279).
constexpr double kXmiss = -999999.;
constexpr float kXmissF = -999999.f;  // exact in FP32

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

// Finite test on a double's bit pattern (integer operations only).
__device__ __forceinline__ bool finite_d(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// Split a double into float hi + float lo (hi = nearest float, lo = nearest
// float to the remainder): a - (hi + lo) is below 2^-48 |a|.
__device__ __forceinline__ float2 split_double(double a) {
    float hi = __double2float_rn(a);
    float lo = __double2float_rn(__dsub_rn(a, (double)hi));
    return make_float2(hi, lo);
}

// split_double with integer operations on the normal-range path (GB300's
// FP64 pipe is narrow, and conversions to and from double run on it).
// Bit-identical to split_double except that a zero remainder is +0:
//   hi = x rounded to 24 bits (ties to even), D = the signed 29-bit rest of
//   the mantissa, lo = float(D) * 2^(e-52) (exact: a power-of-two scale of
//   a normal float).  Exponents outside [-74, 126], zeros' signs and
//   non-finite values take the FP64 path.
// (The rare paths are out of line so the compiler cannot execute their
// FP64 instructions speculatively on every call.)
static __device__ __noinline__ float2 split_double_slow(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b << 1) == 0ull) return make_float2(__int_as_float((int)((b >> 32) & 0x80000000u)), 0.0f);
    return split_double(x);
}
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }

__device__ __forceinline__ float2 split_double_fast(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu) - 1023;
    if (e < -74 || e > 126) return split_double_slow(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const unsigned long long mi = (b & 0xfffffffffffffull) | (1ull << 52);
    unsigned top = (unsigned)(mi >> 29);             // 24 bits with the implicit one
    const unsigned rem = (unsigned)(mi & 0x1fffffffu);
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (top & 1u));
    top += up ? 1u : 0u;                             // 2^24 carries into the exponent below
    const float hi = __uint_as_float(sign | ((unsigned)(e + 126) << 23) + top);
    const int D = (int)rem - (up ? (1 << 29) : 0);
    const float lo = (D == 0) ? 0.0f : __int2float_rn(D) * __uint_as_float(sign | ((unsigned)(e - 52 + 127) << 23));
    return make_float2(hi, lo);
}

// kern<<<grid, block, smem, st>>>(args...), launched as a programmatic
// dependent of the stream's previous kernel when pdl is set (the kernel
// then calls grid_dep_wait before it reads that kernel's results).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_kernel(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                 bool pdl, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<Args&&>(args)...);
}

// Per-pair launches of one kernel merged into one grid (batched calls):
// pair p owns blocks [start[p], start[p + 1]) and runs with args[p], its
// block index and grid size relative to its own blocks.
template <class A>
struct MultiArgs {
    const A* args;
    const int* start;  // npairs + 1 block prefix sums
    int npairs;
};

// The pair that owns this block (pairs without blocks are skipped).
template <class A>
__device__ __forceinline__ int multi_owner(const MultiArgs<A>& m) {
    int lo = 0, hi = m.npairs - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(m.start + mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The kernel NAME(ARGS a) over one pair, and NAME_multi over many: the body
// NAME_body(a, vb, vg) sees its block index and grid size as vb and vg.
#define FLCT_MULTI_KERNEL(BOUNDS, NAME, ARGS)                                                    \
    __global__ void BOUNDS NAME(ARGS a) { NAME##_body(a, (int)blockIdx.x, (int)gridDim.x); }    \
    __global__ void BOUNDS NAME##_multi(MultiArgs<ARGS> m) {                                     \
        const int p_ = multi_owner(m);                                                           \
        const ARGS a_ = m.args[p_];                                                              \
        const int s_ = __ldg(m.start + p_);                                                      \
        NAME##_body(a_, (int)blockIdx.x - s_, __ldg(m.start + p_ + 1) - s_);                     \
    }

// A kernel launched as a programmatic dependent (its launch overlaps the
// tail of the kernel before it on the stream) waits here until that kernel
// has finished and its writes are visible; launched normally, this returns
// at once.  Every kernel that may be so launched calls it before its first
// global read or write of anything an earlier operation on the stream
// touches.  The rule carries the ordering when the operation before the
// launch is not a kernel (an event wait joining another stream, a memset)
// and in captured graphs, where the programmatic edge becomes a graph edge.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The call's work count and status word (final once this kernel starts: no
// later kernel writes them) to mapped page-locked host memory, so that no
// copy node ends the call.
__device__ __forceinline__ void publish_counters(const unsigned* src, unsigned* dst) {
    if (dst && blockIdx.x == 0 && threadIdx.x == 0) {
        dst[0] = src[0];
        dst[1] = src[1];
        __threadfence_system();
    }
}

// Exact float -> double with integer operations for normal floats and
// zeros; subnormals, infinities and NaN take the conversion instruction.
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned E = (u >> 23) & 0xffu;
    const unsigned long long s = (unsigned long long)(u >> 31) << 63;
    if (E == 0u && (u & 0x7fffffu) == 0u) return __longlong_as_double((long long)s);
    if (E == 0u || E == 255u) return f2d_slow(f);
    return __longlong_as_double(
        (long long)(s | ((unsigned long long)(E + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
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
