// lbm_prec_lp.cu -- FP32 storage, and FP16 / BF16 deviation storage, all
// with FP32 arithmetic.
#include "lbm_prec_impl.cuh"

PS_DEFINE_PREC(1)
PS_DEFINE_PREC(2)
PS_DEFINE_PREC(3)
