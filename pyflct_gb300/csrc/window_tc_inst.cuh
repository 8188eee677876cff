// Launchers of the tensor-core window kernel for one box size; included by
// the per-size translation units win_tc_<n>.cu.
#pragma once
#include "window_tc.cuh"

namespace flct {

// Dynamic shared memory of a launch: the kernel's need, raised if needed so
// that no more CTAs fit on an SM than its tensor memory holds (each CTA
// allocates TCOLS of the SM's 512 columns and keeps them while it runs).
template <int N, typename T>
int tc_launch_smem() {
    using C = TcCfg<N>;
    int smem = C::SMEM;
    const int cap = 512 / C::TCOLS;
    for (;;) {
        int nb = 0;
        if (cudaFuncSetAttribute(k_window_tc<N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_window_tc<N, T>, 256, smem) != cudaSuccess)
            return -1;
        if (nb <= cap || smem + 4096 > 232448) return smem;
        smem += 4096;
    }
}

template <int N, typename T>
cudaError_t launch_window_tc(const TcArgs& a, int grid, cudaStream_t st, bool pdl) {
    static int smem = 0;
    if (smem == 0) smem = tc_launch_smem<N, T>();
    if (smem < 0) return cudaErrorInvalidConfiguration;
    cudaError_t e = cudaFuncSetAttribute(k_window_tc<N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return launch_kernel(k_window_tc<N, T>, dim3(grid), dim3(256), (size_t)smem, st, pdl, a);
}

template <int N, typename T>
int window_tc_blocks_per_sm() {
    const int smem = tc_launch_smem<N, T>();
    if (smem < 0) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_window_tc<N, T>, 256, smem) != cudaSuccess) return 0;
    const int cap = 512 / TcCfg<N>::TCOLS;
    return nb > cap ? cap : nb;
}

}  // namespace flct

#define FLCT_TC_INST(n)                                                                              \
    namespace flct {                                                                                 \
    template cudaError_t launch_window_tc<n, __half>(const TcArgs&, int, cudaStream_t, bool);        \
    template cudaError_t launch_window_tc<n, __nv_bfloat16>(const TcArgs&, int, cudaStream_t, bool); \
    template int window_tc_blocks_per_sm<n, __half>();                                               \
    template int window_tc_blocks_per_sm<n, __nv_bfloat16>();                                        \
    }
