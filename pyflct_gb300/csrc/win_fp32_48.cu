// FP32 window kernel instantiations for box sizes: 48 52
#include "window_fp32_inst.cuh"
FLCT_INSTANTIATE_WINDOW_FP32(48)
FLCT_INSTANTIATE_WINDOW_FP32(52)
