// lbm_prec_f64.cu -- FP64 storage, FP64 arithmetic (the plain path).
// Compiled with --fmad=false: every multiply and add rounds separately, as
// in the reference's expressions, so the FP64 lattice reproduces the FP64
// CPU restatement bit for bit.
#include "lbm_prec_impl.cuh"

PS_DEFINE_PREC(0)
