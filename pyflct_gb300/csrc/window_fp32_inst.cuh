// window_fp32_inst.cuh -- explicit instantiation of the FP32 window kernel
// for one box size, both shape variants (each per-size .cu file includes
// this once per size, so the sizes compile in parallel).
#pragma once
#include "window_fp32.cuh"

#define FLCT_INSTANTIATE_WINDOW_FP32_V(N, V)                                                      \
    namespace flct {                                                                              \
    template <>                                                                                   \
    cudaError_t launch_window_fp32<N, V>(const WinArgs& a, int grid, cudaStream_t st, bool pdl) { \
        using S = WinShape<N, V>;                                                                 \
        cudaError_t e = cudaFuncSetAttribute(k_window_fp32<N, V>,                                 \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                             (int)S::smem);                                       \
        if (e != cudaSuccess) return e;                                                           \
        return launch_kernel(k_window_fp32<N, V>, dim3(grid), dim3(S::THREADS), S::smem, st, pdl, a); \
    }                                                                                             \
    template <>                                                                                   \
    int window_fp32_blocks_per_sm<N, V>() {                                                       \
        using S = WinShape<N, V>;                                                                 \
        int nb = 0;                                                                               \
        if (cudaFuncSetAttribute(k_window_fp32<N, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 (int)S::smem) != cudaSuccess)                                    \
            return 0;                                                                             \
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_window_fp32<N, V>, S::THREADS,   \
                                                          S::smem) != cudaSuccess)                \
            return 0;                                                                             \
        return nb;                                                                                \
    }                                                                                             \
    }
#define FLCT_INSTANTIATE_WINDOW_FP32(N) FLCT_INSTANTIATE_WINDOW_FP32_V(N, 0) FLCT_INSTANTIATE_WINDOW_FP32_V(N, 1)
