// lbm_launch.h -- host-callable launchers of the LBM kernels, one set per
// storage precision (implemented in lbm_prec_f64.cu and lbm_prec_lp.cu so
// that the FP64 kernels can be compiled without FMA contraction).
#pragma once
#include <cuda_runtime.h>

#include "lbm_kernels.cuh"

namespace ps {

struct LbmLaunchArgs {
  const void* K;        // LbmConst<R> of the storage precision (host copy)
  GeomDev G;
  BufDev src, dst;
  void* cc;             // colour field (R per voxel) used by the step kernels
  cudaStream_t stream;
};

// one batched step over many lattices sharing the constants K: tiles_c /
// tiles_d list (lattice, first node) per collide / density CTA
struct BatchLaunchArgs {
  const void* K;
  const VolTable* T;
  const int2* tiles_c;
  int ntc;
  const int2* tiles_d;
  int ntd;
  cudaStream_t stream;
};

// returns cudaErrorInvalidValue when (tx, ty, occ) is not a compiled
// configuration (tx / ty threads per CTA of the collide / density kernel,
// occ minimum resident collide CTAs per SM, 0 = compiler's choice)
cudaError_t lbm_step_launch(int prec, int tx, int ty, int occ, const LbmLaunchArgs& a);
cudaError_t lbm_fields_launch(int prec, const LbmLaunchArgs& a, double* rr, double* rb, double* cf, double* cc);
cudaError_t lbm_get_state_launch(int prec, const LbmLaunchArgs& a, double* fr, double* fb);
cudaError_t lbm_set_state_launch(int prec, const LbmLaunchArgs& a, const double* fr, const double* fb);
cudaError_t lbm_obs_launch(int prec, const LbmLaunchArgs& a, const double* cc, double* partial, int nblocks,
                           double* out);
// 1 when (tx, ty, occ) is a compiled step configuration, else 0
size_t lbm_step_smem(int prec, int tx, int ty, int occ);

// per-precision implementations
#define PS_DECL_PREC(P)                                                                                     \
  cudaError_t lbm_step_launch_##P(int tx, int ty, int zchunk, const LbmLaunchArgs& a);                     \
  cudaError_t lbm_fused_launch_##P(int tx, int occ, const LbmLaunchArgs& a, const FusedArgs& f);           \
  cudaError_t lbm_march_launch_##P(int pw, const MarchArgs& A, const LbmLaunchArgs& a);                    \
  int lbm_march_resident_##P(int pw, int rows, int nx);                                                   \
  cudaError_t lbm_wave_graph_##P(int tx, int ty, int occ, const LbmLaunchArgs* a, int steps, const int* first, \
                                 int S, int window, cudaGraph_t* g);                                        \
  cudaError_t lbm_batch_step_launch_##P(int tx, int ty, int occ, const BatchLaunchArgs& b);                \
  cudaError_t lbm_fields_launch_##P(const LbmLaunchArgs& a, double* rr, double* rb, double* cf, double* cc); \
  cudaError_t lbm_get_state_launch_##P(const LbmLaunchArgs& a, double* fr, double* fb);                    \
  cudaError_t lbm_set_state_launch_##P(const LbmLaunchArgs& a, const double* fr, const double* fb);        \
  cudaError_t lbm_obs_launch_##P(const LbmLaunchArgs& a, const double* cc, double* partial, int nblocks,   \
                                 double* out);                                                              \
  cudaError_t lbm_wall_load_launch_##P(const LbmLaunchArgs& a, double fq1, double fq2, double ppp, double rsdti2, \
                                      double* out);                                                         \
  size_t lbm_step_smem_##P(int tx, int ty, int occ);
PS_DECL_PREC(0)
PS_DECL_PREC(1)
PS_DECL_PREC(2)
PS_DECL_PREC(3)
#undef PS_DECL_PREC

}  // namespace ps
