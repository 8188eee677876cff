// FP32 window kernel instantiations for box sizes: 56 60
#include "window_fp32_inst.cuh"
FLCT_INSTANTIATE_WINDOW_FP32(56)
FLCT_INSTANTIATE_WINDOW_FP32(60)
