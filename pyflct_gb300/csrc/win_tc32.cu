// Tensor-core window kernel instantiations (32 x 32 boxes, FP16 and BF16 split).
#include "window_tc.cuh"

namespace flct {

template <typename T>
cudaError_t launch_window_tc32(const TcArgs& a, int grid, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_window_tc32<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TcSmem::bytes);
    if (e != cudaSuccess) return e;
    k_window_tc32<T><<<grid, 128, TcSmem::bytes, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
int window_tc32_blocks_per_sm() {
    int nb = 0;
    if (cudaFuncSetAttribute(k_window_tc32<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcSmem::bytes) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_window_tc32<T>, 128, TcSmem::bytes) != cudaSuccess)
        return 0;
    // each CTA holds 256 of the SM's 512 tensor-memory columns
    return nb > 2 ? 2 : nb;
}

template cudaError_t launch_window_tc32<__half>(const TcArgs&, int, cudaStream_t);
template cudaError_t launch_window_tc32<__nv_bfloat16>(const TcArgs&, int, cudaStream_t);
template int window_tc32_blocks_per_sm<__half>();
template int window_tc32_blocks_per_sm<__nv_bfloat16>();

}  // namespace flct
