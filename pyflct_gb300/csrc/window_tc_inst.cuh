// Launchers of the tensor-core window kernel for one box size; included by
// the per-size translation units win_tc_<n>.cu.
#pragma once
#include <cstdio>
#include <cstdlib>

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
    // all of the SM's unified L1 / shared memory as shared memory, so that
    // as many CTAs fit as the registers allow
    if (cudaFuncSetAttribute(k_window_tc<N, T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return -1;
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
    // CTAs per SM from the kernel's registers and shared memory against the
    // SM's register file and shared memory (the occupancy query above has
    // answered 1 where both allow 2 for this kernel)
    cudaFuncAttributes fa{};
    int dev = 0, sm_smem = 0, reserved = 0, regs_sm = 0;
    if (cudaFuncGetAttributes(&fa, k_window_tc<N, T>) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess)
        return nb > cap ? cap : nb;
    const int regs = (fa.numRegs + 7) / 8 * 8;
    const int by_regs = regs_sm / (regs * 256);
    const int by_smem = sm_smem / (smem + reserved);
    int own = by_regs < by_smem ? by_regs : by_smem;
    if (own > cap) own = cap;
    if (getenv("FLCT_DEBUG"))
        fprintf(stderr,
                "k_window_tc<%d>: occupancy query %d CTAs/SM; registers %d (%d/SM) -> %d, shared %d B (+%d, %d/SM) "
                "-> %d, tensor memory -> %d\n",
                N, nb, fa.numRegs, regs_sm, by_regs, smem, reserved, sm_smem, by_smem, cap);
    return own > nb ? own : (nb > cap ? cap : nb);
}

}  // namespace flct

#ifdef FLCT_TC_PROFILE
// Profiling builds only: per-stage clock sums of the box-n kernel (thread 0
// of every CTA), read and cleared.
#define FLCT_TC_PROFILE_READ(n)                                                                          \
    extern "C" __attribute__((visibility("default"))) int flct_debug_tc_clocks_##n(unsigned long long* out) { \
        if (cudaMemcpyFromSymbol(out, flct::g_tc_stage_clk, 12 * sizeof(unsigned long long)) != cudaSuccess) \
            return 1;                                                                                    \
        const unsigned long long z[12] = {};                                                             \
        return cudaMemcpyToSymbol(flct::g_tc_stage_clk, z, sizeof(z)) == cudaSuccess ? 0 : 1;           \
    }
#else
#define FLCT_TC_PROFILE_READ(n)
#endif

#define FLCT_TC_INST(n)                                                                              \
    FLCT_TC_PROFILE_READ(n)                                                                          \
    namespace flct {                                                                                 \
    template cudaError_t launch_window_tc<n, __half>(const TcArgs&, int, cudaStream_t, bool);        \
    template cudaError_t launch_window_tc<n, __nv_bfloat16>(const TcArgs&, int, cudaStream_t, bool); \
    template int window_tc_blocks_per_sm<n, __half>();                                               \
    template int window_tc_blocks_per_sm<n, __nv_bfloat16>();                                        \
    }
