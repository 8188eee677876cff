// fp32_peak.cu -- FP32 CUDA-core throughput microbenchmark (libflctprobe.so).
//
// The roofline of the FP32 window form is the FP32 pipe.  This measures its
// peak on the GPU at hand instead of deriving it from the clock: every
// thread runs kChains independent FMA chains (scalar fma.rn.f32, or packed
// fma.rn.f32x2 on register pairs) for `iters` iterations, on a persistent
// grid of blocks_per_sm x SMs CTAs, timed with CUDA events on one stream.
// The result is 2 flops per lane-FMA over the kernel's event time.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_ffma(float* out, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-3f + c;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 16; ++r)
#pragma unroll
            for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(256) k_ffma2(float* out, int iters, float a, float b) {
    unsigned long long x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
        const float lo = threadIdx.x * 1e-3f + c, hi = lo + 0.5f;
        x[c] = (unsigned long long)__float_as_uint(lo) | ((unsigned long long)__float_as_uint(hi) << 32);
    }
    const unsigned long long A = (unsigned long long)__float_as_uint(a) | ((unsigned long long)__float_as_uint(a) << 32);
    const unsigned long long B = (unsigned long long)__float_as_uint(b) | ((unsigned long long)__float_as_uint(b) << 32);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 16; ++r)
#pragma unroll
            for (int c = 0; c < kChains; ++c)
                asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[c]) : "l"(A), "l"(B));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += __uint_as_float((unsigned)x[c]) + __uint_as_float((unsigned)(x[c] >> 32));
    if (s == 12345.678f) out[blockIdx.x] = s;
}

}  // namespace

// Measured FP32 FMA throughput in TFLOP/s: scalar (fma.rn.f32) and packed
// (fma.rn.f32x2) forms, best of `reps` timed launches each after one
// warm-up.  Returns 0 on success, else the CUDA error code.
extern "C" __attribute__((visibility("default"))) int flct_probe_fp32_peak(int reps, double* scalar_tflops,
                                                                          double* packed_tflops) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    float* out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(float) * 65536);
    if (e != cudaSuccess) return (int)e;
    cudaStream_t st;
    cudaEvent_t e0, e1;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = nsm * 8, iters = 4096;
    const double lane_fmas = (double)blocks * threads * iters * 16 * kChains;
    double best[2] = {0.0, 0.0};
    for (int form = 0; form < 2; ++form) {
        for (int r = 0; r <= reps; ++r) {
            cudaEventRecord(e0, st);
            if (form == 0) k_ffma<<<blocks, threads, 0, st>>>(out, iters, 0.999f, 1e-4f);
            else k_ffma2<<<blocks, threads, 0, st>>>(out, iters, 0.999f, 1e-4f);
            cudaEventRecord(e1, st);
            e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            // packed: two lane-FMAs per instruction and lane
            const double fl = 2.0 * lane_fmas * (form ? 2.0 : 1.0);
            if (r > 0 && ms > 0.f) best[form] = fl / (ms * 1e-3) / 1e12 > best[form] ? fl / (ms * 1e-3) / 1e12 : best[form];
        }
        if (e != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(out);
    if (e != cudaSuccess) return (int)e;
    *scalar_tflops = best[0];
    *packed_tflops = best[1];
    return 0;
}
