// lbm_prec_lp.cu -- FP32 storage, and FP16 / BF16 deviation storage, all
// with FP32 arithmetic.
#include "lbm_prec_impl.cuh"

#define PS_TILES_LP(X, P) X(P, 128, 256) X(P, 256, 256)
PS_DEFINE_PREC(1, PS_TILES_LP)
PS_DEFINE_PREC(2, PS_TILES_LP)
PS_DEFINE_PREC(3, PS_TILES_LP)
