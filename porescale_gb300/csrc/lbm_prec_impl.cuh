// lbm_prec_impl.cuh -- launcher bodies for one storage precision PREC.
// Included by lbm_prec_f64.cu (PREC 0) and lbm_prec_lp.cu (PREC 1..3).
#pragma once
#include "lbm_launch.h"

namespace ps {
namespace detail {

template <int PREC, int BC, int BD, int MINB = 0>
cudaError_t step_blk(const LbmLaunchArgs& a)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nl;
  if (n == 0) return cudaSuccess;
  const LbmConst<R>& C = *static_cast<const LbmConst<R>*>(a.K);
  R* cc = static_cast<R*>(a.cc);
  k_lbm_dens<PREC, BD><<<(unsigned)((n + BD - 1) / BD), BD, 0, a.stream>>>(C, a.G, a.src, a.dst, cc);
  k_lbm_coll<PREC, BC, MINB><<<(unsigned)((n + BC - 1) / BC), BC, 0, a.stream>>>(C, a.G, a.src, a.dst, cc);
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
// precision P.  A step configuration is (tx, ty, occ): tx threads per CTA
// of the collide kernel, ty of the density kernel, occ the minimum resident
// collide CTAs per SM requested from the register allocator (0 = its own
// choice).
#define PS_DEFINE_PREC(P)                                                                                  \
  namespace ps {                                                                                           \
  cudaError_t lbm_step_launch_##P(int tx, int ty, int zchunk, const LbmLaunchArgs& a)                      \
  {                                                                                                        \
    const int occ = zchunk;                                                                                \
    if (occ == 0) {                                                                                        \
      if (tx == 128 && ty == 256) return detail::step_blk<P, 128, 256>(a);                                 \
      if (tx == 256 && ty == 256) return detail::step_blk<P, 256, 256>(a);                                 \
      if (tx == 128 && ty == 128) return detail::step_blk<P, 128, 128>(a);                                 \
      if (tx == 256 && ty == 512) return detail::step_blk<P, 256, 512>(a);                                 \
    }                                                                                                      \
    if (tx == 128 && ty == 256 && occ == 6) return detail::step_blk<P, 128, 256, 6>(a);                    \
    if (tx == 128 && ty == 256 && occ == 8) return detail::step_blk<P, 128, 256, 8>(a);                    \
    if (tx == 256 && ty == 256 && occ == 3) return detail::step_blk<P, 256, 256, 3>(a);                    \
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
  size_t lbm_step_smem_##P(int tx, int ty, int occ)                                                        \
  {                                                                                                        \
    const bool base = (tx == 128 && (ty == 256 || ty == 128)) || (tx == 256 && (ty == 256 || ty == 512)); \
    const bool hi = (tx == 128 && ty == 256 && (occ == 6 || occ == 8)) || (tx == 256 && ty == 256 && occ == 3); \
    return (occ == 0 && base) || hi ? 1 : 0;                                                               \
  }                                                                                                        \
  }
