// FP32 window kernel instantiations for box sizes: 40 44
#include "window_fp32_inst.cuh"
FLCT_INSTANTIATE_WINDOW_FP32(40)
FLCT_INSTANTIATE_WINDOW_FP32(44)
