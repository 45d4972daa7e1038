// lbm_prec_impl.cuh -- launcher bodies for one storage precision PREC.
// Included by lbm_prec_f64.cu (PREC 0) and lbm_prec_lp.cu (PREC 1..3).
#pragma once
#include <algorithm>
#include <vector>

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
  const int i1 = (int)n;
  k_lbm_dens<PREC, BD><<<(unsigned)((n + BD - 1) / BD), BD, 0, a.stream>>>(C, a.G, a.src, a.dst, cc, 0, i1);
  k_lbm_coll<PREC, BC, MINB><<<(unsigned)((n + BC - 1) / BC), BC, 0, a.stream>>>(C, a.G, a.src, a.dst, cc, 0, i1);
  return cudaGetLastError();
}

// Wavefront graph of `steps` steps over z-slabs (slab k = fluid nodes
// [first[k], first[k+1])), a[s] the buffers of step s.  Only the true
// dependencies order the launches:
//   density(s, k)  after collide(s-1, k-1..k+1)  (their pushes land in slab
//                  k; it also overwrites the colour and reference densities
//                  those collides read);
//   collide(s, k)  after density(s, k-1..k+1)    (27-point colour stencil,
//                  receivers' reference densities).
// Slab indices wrap (periodic z).  So step s+1 follows step s a few slabs
// behind, and a density launch reads the populations the collides before
// it have just written while they are still in L2, and the collide after it
// re-reads them from there.  window >= 2 adds collide(s, k) after
// density(s+1, k - window) for k > window, which keeps the collides of a
// step from running far ahead of the next step's densities (those targets
// depend only on lower slabs, so no cycle forms).  Empty slabs are empty
// graph nodes.
template <int PREC, int BC, int BD, int MINB = 0>
cudaError_t wave_graph(const LbmLaunchArgs* a, int steps, const int* first, int S, int window, cudaGraph_t* out)
{
  using R = typename Store<PREC>::R;
  *out = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> dn((size_t)S * steps), cn((size_t)S * steps);
  auto add = [&](cudaGraphNode_t* node, const std::vector<cudaGraphNode_t>& deps, void* fn, int blk, int i0, int i1,
                 const LbmLaunchArgs& la) -> cudaError_t {
    if (i1 <= i0) return cudaGraphAddEmptyNode(node, g, deps.data(), deps.size());
    R* cc = static_cast<R*>(la.cc);
    const LbmConst<R>& C = *static_cast<const LbmConst<R>*>(la.K);
    GeomDev G = la.G;
    BufDev src = la.src, dst = la.dst;
    void* args[] = {(void*)&C, (void*)&G, (void*)&src, (void*)&dst, (void*)&cc, (void*)&i0, (void*)&i1};
    cudaKernelNodeParams kp = {};
    kp.func = fn;
    kp.gridDim = dim3((unsigned)((i1 - i0 + blk - 1) / blk));
    kp.blockDim = dim3((unsigned)blk);
    kp.kernelParams = args;
    return cudaGraphAddKernelNode(node, g, deps.data(), deps.size(), &kp);
  };
  auto nb3 = [&](const std::vector<cudaGraphNode_t>& v, int s, int k) {
    std::vector<cudaGraphNode_t> d;
    for (int o = -1; o <= 1; o++) {
      const cudaGraphNode_t n = v[(size_t)s * S + (k + o + S) % S];
      if (std::find(d.begin(), d.end(), n) == d.end()) d.push_back(n);
    }
    return d;
  };
  for (int s = 0; s < steps && e == cudaSuccess; s++) {
    for (int k = 0; k < S && e == cudaSuccess; k++) {
      std::vector<cudaGraphNode_t> deps;
      if (s > 0) deps = nb3(cn, s - 1, k);
      e = add(&dn[(size_t)s * S + k], deps, (void*)k_lbm_dens<PREC, BD>, BD, first[k], first[k + 1], a[s]);
      // the window edges of the previous step's collides that wait for this density
      if (e == cudaSuccess && s > 0 && window > 0 && k >= 1 && k + window < S)
        e = cudaGraphAddDependencies(g, &dn[(size_t)s * S + k], &cn[(size_t)(s - 1) * S + k + window], nullptr, 1);
    }
    for (int k = 0; k < S && e == cudaSuccess; k++)
      e = add(&cn[(size_t)s * S + k], nb3(dn, s, k), (void*)k_lbm_coll<PREC, BC, MINB>, BC, first[k], first[k + 1],
              a[s]);
  }
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return e;
  }
  *out = g;
  return cudaSuccess;
}

// resident CTAs per SM x SMs: the persistent grid of a batched kernel
template <typename Kern>
int persistent_grid(Kern kern, int blk)
{
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, blk, 0);
  return std::max(1, sms * std::max(1, occ));
}

template <int PREC, int BC, int BD, int MINB = 0>
cudaError_t step_batch_blk(const BatchLaunchArgs& b)
{
  using R = typename Store<PREC>::R;
  const LbmConst<R>& C = *static_cast<const LbmConst<R>*>(b.K);
  static const int gd = persistent_grid(k_lbm_dens_batch<PREC, BD>, BD);
  static const int gc = persistent_grid(k_lbm_coll_batch<PREC, BC, MINB>, BC);
  if (b.ntd > 0)
    k_lbm_dens_batch<PREC, BD><<<std::min(gd, b.ntd), BD, 0, b.stream>>>(C, *b.T, b.tiles_d, b.ntd);
  if (b.ntc > 0)
    k_lbm_coll_batch<PREC, BC, MINB><<<std::min(gc, b.ntc), BC, 0, b.stream>>>(C, *b.T, b.tiles_c, b.ntc);
  return cudaGetLastError();
}

template <int PREC, int BLK, int MINB = 0>
cudaError_t step_fused_blk(const LbmLaunchArgs& a, const FusedArgs& f)
{
  using R = typename Store<PREC>::R;
  if (f.nitems == 0) return cudaSuccess;
  // every CTA resident: the cooperative launch refuses a larger grid
  static const int gmax = persistent_grid(k_lbm_fused<PREC, BLK, MINB>, BLK);
  cudaError_t e = cudaMemsetAsync(f.ctr, 0, sizeof(unsigned) * (size_t)(1 + f.nslab), a.stream);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)std::min(gmax, f.nitems));
  cfg.blockDim = dim3(BLK);
  cfg.stream = a.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_lbm_fused<PREC, BLK, MINB>, *static_cast<const LbmConst<R>*>(a.K), a.G, a.src,
                            a.dst, static_cast<R*>(a.cc), f);
}

// one marching step (k_lbm_march): items of `rows` band rows x `planes`
// chunk planes over a persistent grid of one CTA per SM with PW producer and
// CW consumer warps.  FP64 has no marching form (its step is bound by the
// FP64 pipe, not by memory).
template <int PREC, int PW, int CW>
cudaError_t step_march_blk(const LbmLaunchArgs& a, const MarchArgs& A0)
{
  if constexpr (PREC == 0) {
    return cudaErrorInvalidValue;
  } else {
    using R = typename Store<PREC>::R;
    if (a.G.nl == 0) return cudaSuccess;
    MarchArgs A = A0;
    A.nband = (a.G.ny + A.rows - 1) / A.rows;
    A.nitems = A.nband * ((a.G.nz + A.planes - 1) / A.planes);
    const size_t smem = march_smem_bytes<R>(A.rows, a.G.nx);
    cudaError_t e = cudaFuncSetAttribute(k_lbm_march<PREC, PW, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_lbm_march<PREC, PW, CW><<<(unsigned)std::min(sms, A.nitems), 32 * (PW + CW), smem, a.stream>>>(
        *static_cast<const LbmConst<R>*>(a.K), a.G, a.src, a.dst, A);
    return cudaGetLastError();
  }
}

// resident CTAs per SM of the marching kernel with its ring for `rows` band
// rows (0: the ring does not fit, or the collide order would overflow 16 bits)
template <int PREC, int PW, int CW>
int march_resident(int rows, int nx)
{
  if constexpr (PREC == 0) {
    return 0;
  } else {
    using R = typename Store<PREC>::R;
    const size_t smem = march_smem_bytes<R>(rows, nx);
    if (smem > 227 * 1024 || (size_t)rows * nx > 65535) return 0;
    if (cudaFuncSetAttribute(k_lbm_march<PREC, PW, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_march<PREC, PW, CW>, 32 * (PW + CW), smem) !=
        cudaSuccess)
      return 0;
    return n;
  }
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
  k_lbm_get_state<PREC><<<(unsigned)((n + kStateBlk - 1) / kStateBlk), kStateBlk, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K),
                                                                             a.G, a.src, fr, fb);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t set_state(const LbmLaunchArgs& a, const double* fr, const double* fb)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nl;
  if (n == 0) return cudaSuccess;
  k_lbm_set_state<PREC><<<(unsigned)((n + kStateBlk - 1) / kStateBlk), kStateBlk, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K),
                                                                             a.G, a.dst, fr, fb);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t obs(const LbmLaunchArgs& a, const double* cc, double* partial, int nblocks, double* out)
{
  using R = typename Store<PREC>::R;
  k_lbm_obs<PREC><<<nblocks, 256, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K), a.G, a.src, cc, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_obs_final<<<1, 64, 0, a.stream>>>(partial, nblocks, out);
  return cudaGetLastError();
}

template <int PREC>
cudaError_t wall_load(const LbmLaunchArgs& a, double fq1, double fq2, double ppp, double rsdti2, double* out)
{
  using R = typename Store<PREC>::R;
  const long long n = a.G.nvox;
  k_lbm_wall_load<PREC><<<(unsigned)((n + 127) / 128), 128, 0, a.stream>>>(*static_cast<const LbmConst<R>*>(a.K),
                                                                           a.G, a.src, fq1, fq2, ppp, rsdti2, out);
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
    }                                                                                                      \
    if (tx == 128 && ty == 256 && occ == 6) return detail::step_blk<P, 128, 256, 6>(a);                    \
    if (tx == 128 && ty == 256 && occ == 7) return detail::step_blk<P, 128, 256, 7>(a);                    \
    if (tx == 128 && ty == 256 && occ == 8) return detail::step_blk<P, 128, 256, 8>(a);                    \
    if (tx == 256 && ty == 256 && occ == 3) return detail::step_blk<P, 256, 256, 3>(a);                    \
    return cudaErrorInvalidValue;                                                                          \
  }                                                                                                        \
  cudaError_t lbm_wave_graph_##P(int tx, int ty, int occ, const LbmLaunchArgs* a, int steps, const int* first, \
                                 int S, int window, cudaGraph_t* g)                                         \
  {                                                                                                        \
    if (occ == 0) {                                                                                        \
      if (tx == 128 && ty == 256) return detail::wave_graph<P, 128, 256>(a, steps, first, S, window, g);   \
      if (tx == 256 && ty == 256) return detail::wave_graph<P, 256, 256>(a, steps, first, S, window, g);   \
      if (tx == 128 && ty == 128) return detail::wave_graph<P, 128, 128>(a, steps, first, S, window, g);   \
    }                                                                                                      \
    if (tx == 128 && ty == 256 && occ == 6) return detail::wave_graph<P, 128, 256, 6>(a, steps, first, S, window, g); \
    if (tx == 128 && ty == 256 && occ == 7) return detail::wave_graph<P, 128, 256, 7>(a, steps, first, S, window, g); \
    if (tx == 128 && ty == 256 && occ == 8) return detail::wave_graph<P, 128, 256, 8>(a, steps, first, S, window, g); \
    if (tx == 256 && ty == 256 && occ == 3) return detail::wave_graph<P, 256, 256, 3>(a, steps, first, S, window, g); \
    return cudaErrorInvalidValue;                                                                          \
  }                                                                                                        \
  cudaError_t lbm_fused_launch_##P(int tx, int occ, const LbmLaunchArgs& a, const FusedArgs& f)           \
  {                                                                                                        \
    if (tx == 128 && occ == 0) return detail::step_fused_blk<P, 128>(a, f);                                \
    if (tx == 256 && occ == 0) return detail::step_fused_blk<P, 256>(a, f);                                \
    if (tx == 128 && occ == 6) return detail::step_fused_blk<P, 128, 6>(a, f);                             \
    if (tx == 128 && occ == 8) return detail::step_fused_blk<P, 128, 8>(a, f);                             \
    return cudaErrorInvalidValue;                                                                          \
  }                                                                                                        \
  cudaError_t lbm_batch_step_launch_##P(int tx, int ty, int occ, const BatchLaunchArgs& b)                \
  {                                                                                                        \
    if (occ == 0) {                                                                                        \
      if (tx == 128 && ty == 256) return detail::step_batch_blk<P, 128, 256>(b);                           \
      if (tx == 256 && ty == 256) return detail::step_batch_blk<P, 256, 256>(b);                           \
      if (tx == 128 && ty == 128) return detail::step_batch_blk<P, 128, 128>(b);                           \
    }                                                                                                      \
    if (tx == 128 && ty == 256 && occ == 6) return detail::step_batch_blk<P, 128, 256, 6>(b);              \
    if (tx == 128 && ty == 256 && occ == 8) return detail::step_batch_blk<P, 128, 256, 8>(b);              \
    if (tx == 256 && ty == 256 && occ == 3) return detail::step_batch_blk<P, 256, 256, 3>(b);              \
    return cudaErrorInvalidValue;                                                                          \
  }                                                                                                        \
  cudaError_t lbm_march_launch_##P(int pw, const MarchArgs& A, const LbmLaunchArgs& a)                     \
  {                                                                                                        \
    if (pw == 4) return detail::step_march_blk<P, 4, 20>(a, A);                                            \
    if (pw == 8) return detail::step_march_blk<P, 8, 16>(a, A);                                            \
    if (pw == 12) return detail::step_march_blk<P, 12, 12>(a, A);                                          \
    return cudaErrorInvalidValue;                                                                          \
  }                                                                                                        \
  int lbm_march_resident_##P(int pw, int rows, int nx)                                                    \
  {                                                                                                        \
    if (pw == 4) return detail::march_resident<P, 4, 20>(rows, nx);                                        \
    if (pw == 8) return detail::march_resident<P, 8, 16>(rows, nx);                                        \
    if (pw == 12) return detail::march_resident<P, 12, 12>(rows, nx);                                      \
    return 0;                                                                                              \
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
  cudaError_t lbm_wall_load_launch_##P(const LbmLaunchArgs& a, double fq1, double fq2, double ppp, double rsdti2, \
                                      double* out)                                                          \
  {                                                                                                        \
    return detail::wall_load<P>(a, fq1, fq2, ppp, rsdti2, out);                                            \
  }                                                                                                        \
  size_t lbm_step_smem_##P(int tx, int ty, int occ)                                                        \
  {                                                                                                        \
    const bool base = (tx == 128 && (ty == 256 || ty == 128)) || (tx == 256 && ty == 256);                \
    const bool hi = (tx == 128 && ty == 256 && (occ == 6 || occ == 7 || occ == 8)) || (tx == 256 && ty == 256 && occ == 3); \
    return (occ == 0 && base) || hi ? 1 : 0;                                                               \
  }                                                                                                        \
  }
