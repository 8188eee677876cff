// FP32 window kernel instantiations for box sizes: 64
#include "window_fp32_inst.cuh"
FLCT_INSTANTIATE_WINDOW_FP32(64)
