// FP32 window kernel instantiations for box sizes: 20 24 28
#include "window_fp32_inst.cuh"
FLCT_INSTANTIATE_WINDOW_FP32(20)
FLCT_INSTANTIATE_WINDOW_FP32(24)
FLCT_INSTANTIATE_WINDOW_FP32(28)
