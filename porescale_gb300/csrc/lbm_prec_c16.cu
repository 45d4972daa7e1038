// lbm_prec_c16.cu -- 16-bit total + colour storage (PS_PREC_F16C) with FP32
// arithmetic; its own translation unit so it compiles alongside the others.
#include "lbm_prec_impl.cuh"

PS_DEFINE_PREC(4)
