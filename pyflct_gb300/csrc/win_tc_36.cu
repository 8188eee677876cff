// Tensor-core window kernel, box 36 (FP16 and BF16 split).
#include "window_tc_inst.cuh"
FLCT_TC_INST(36)
