// FP32 window kernel instantiations for box sizes: 32 36
#include "window_fp32_inst.cuh"
FLCT_INSTANTIATE_WINDOW_FP32(32)
FLCT_INSTANTIATE_WINDOW_FP32(36)
