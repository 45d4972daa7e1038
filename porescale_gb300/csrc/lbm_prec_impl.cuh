// lbm_prec_impl.cuh -- launcher bodies for one storage precision PREC.
// Included by lbm_prec_f64.cu (PREC 0) and lbm_prec_lp.cu (PREC 1..3).
#pragma once
#include "lbm_launch.h"

namespace ps {
namespace detail {

template <int PREC, int BC, int BD>
cudaError_t step_blk(const LbmLaunchArgs& a)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nl;
  if (n == 0) return cudaSuccess;
  const LbmConst<R>& C = *static_cast<const LbmConst<R>*>(a.K);
  R* cc = static_cast<R*>(a.cc);
  k_lbm_dens<PREC, BD><<<(unsigned)((n + BD - 1) / BD), BD, 0, a.stream>>>(C, a.G, a.src, a.dst, cc);
  k_lbm_coll<PREC, BC><<<(unsigned)((n + BC - 1) / BC), BC, 0, a.stream>>>(C, a.G, a.src, a.dst, cc);
  return cudaGetLastError();
}

// fused step: BLK threads, TY rows per CTA, zchunk planes per CTA
template <int PREC, int BLK>
cudaError_t step_fused(int ty, int zchunk, const LbmLaunchArgs& a)
{
  using R = typename Store<PREC>::R;
  const GeomDev& G = a.G;
  if (G.nl == 0) return cudaSuccess;
  const size_t smem = FusedSmem<R>::bytes(ty, G.nx);
  static size_t attr = 0;  // per instantiation: largest dynamic smem opted in so far
  if (smem > 48 * 1024 && smem > attr) {
    cudaError_t e = cudaFuncSetAttribute(k_lbm_fused<PREC, BLK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = smem;
  }
  if (zchunk <= 0) zchunk = G.nz;
  dim3 grid((G.ny + ty - 1) / ty, (G.nz + zchunk - 1) / zchunk);
  const LbmConst<R>& C = *static_cast<const LbmConst<R>*>(a.K);
  k_lbm_fused<PREC, BLK><<<grid, BLK, smem, a.stream>>>(C, G, a.src, a.dst, ty, zchunk);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t fields(const LbmLaunchArgs& a, double* rr, double* rb, double* cf, double* cc)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nl;
  if (n == 0) return cudaSuccess;
  k_lbm_fields<PREC><<<(unsigned)((n + 255) / 256), 256, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K), a.G,
                                                                          a.src, rr, rb, cf, cc);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t get_state(const LbmLaunchArgs& a, double* fr, double* fb)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nl;
  if (n == 0) return cudaSuccess;
  k_lbm_get_state<PREC><<<(unsigned)((n + 255) / 256), 256, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K),
                                                                             a.G, a.src, fr, fb);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t set_state(const LbmLaunchArgs& a, const double* fr, const double* fb)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nl;
  if (n == 0) return cudaSuccess;
  k_lbm_set_state<PREC><<<(unsigned)((n + 255) / 256), 256, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K),
                                                                             a.G, a.dst, fr, fb);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t obs(const LbmLaunchArgs& a, const double* cc, double* partial, int nblocks, double* out)
{
  using R = typename Store<PREC>::R;
  k_lbm_obs<PREC><<<nblocks, 256, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K), a.G, a.src, cc, a.Kd_dev,
                                                 partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_obs_final<<<1, 64, 0, a.stream>>>(partial, nblocks, out);
  return cudaGetLastError();
}

}  // namespace detail
}  // namespace ps

// Defines the per-precision entry points declared in lbm_launch.h for
// precision P.  A step configuration is (tx, ty, zchunk): tx threads per
// CTA; ty >= 1 rows per CTA for the fused kernel (zchunk planes per CTA), or
// ty == 0 for the two-launch form (tx threads for the collide kernel, 256
// for the density kernel).
#define PS_DEFINE_PREC(P)                                                                                  \
  namespace ps {                                                                                           \
  cudaError_t lbm_step_launch_##P(int tx, int ty, int zchunk, const LbmLaunchArgs& a)                      \
  {                                                                                                        \
    if (ty == 0) {                                                                                         \
      if (tx == 128) return detail::step_blk<P, 128, 256>(a);                                              \
      if (tx == 256) return detail::step_blk<P, 256, 256>(a);                                              \
      return cudaErrorInvalidValue;                                                                        \
    }                                                                                                      \
    if (tx == 128) return detail::step_fused<P, 128>(ty, zchunk, a);                                       \
    if (tx == 256) return detail::step_fused<P, 256>(ty, zchunk, a);                                       \
    return cudaErrorInvalidValue;                                                                          \
  }                                                                                                        \
  cudaError_t lbm_fields_launch_##P(const LbmLaunchArgs& a, double* rr, double* rb, double* cf, double* cc) \
  {                                                                                                        \
    return detail::fields<P>(a, rr, rb, cf, cc);                                                           \
  }                                                                                                        \
  cudaError_t lbm_get_state_launch_##P(const LbmLaunchArgs& a, double* fr, double* fb)                    \
  {                                                                                                        \
    return detail::get_state<P>(a, fr, fb);                                                                \
  }                                                                                                        \
  cudaError_t lbm_set_state_launch_##P(const LbmLaunchArgs& a, const double* fr, const double* fb)        \
  {                                                                                                        \
    return detail::set_state<P>(a, fr, fb);                                                                \
  }                                                                                                        \
  cudaError_t lbm_obs_launch_##P(const LbmLaunchArgs& a, const double* cc, double* partial, int nblocks,   \
                                 double* out)                                                              \
  {                                                                                                        \
    return detail::obs<P>(a, cc, partial, nblocks, out);                                                   \
  }                                                                                                        \
  size_t lbm_step_smem_##P(int tx, int ty, int nx)                                                         \
  {                                                                                                        \
    if (tx != 128 && tx != 256) return 0;                                                                  \
    if (ty == 0) return 1;                                                                                 \
    return FusedSmem<typename Store<P>::R>::bytes(ty, nx);                                                 \
  }                                                                                                        \
  }
