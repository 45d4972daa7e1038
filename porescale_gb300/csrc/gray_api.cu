// gray_api.cu -- C ABI of the gray partial-bounce-back lattice and its
// adjoint permeability gradient (declared in include/porescale.h).
//
// Forward: nsteps of k_gray_step from the rest state.  Gradient: the same
// forward storing a checkpoint every `segment` steps, then the adjoint
// backwards segment by segment: each segment's states are recomputed from
// its checkpoint into a device buffer (segment x 19 x n doubles) and the
// adjoint steps consume them newest first.  Compiled without FMA
// contraction so that the results are reproducible bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "gray_kernels.cuh"
#include "ps_common.h"

namespace ps {
namespace {

using gray::GrayConst;
using gray::GrayGeom;
constexpr int kBlk = 128;

struct Gray {
  ps_gray_params p{};
  GrayConst C{};
  GrayGeom G{};
  cudaStream_t stream = nullptr;
  double* s = nullptr;      // solid fraction per voxel
  double* f[2] = {nullptr, nullptr};
  double* part = nullptr;   // momentum partial sums
  int cur = 0;              // buffer holding the last forward state
  bool ran = false;
  long long dev_bytes = 0;
  unsigned blocks() const { return (unsigned)((G.n + kBlk - 1) / kBlk); }
  size_t state_bytes() const { return sizeof(double) * 19 * (size_t)G.n; }
};

void free_gray(Gray* g)
{
  if (!g) return;
  cudaFree(g->s);
  cudaFree(g->f[0]);
  cudaFree(g->f[1]);
  cudaFree(g->part);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}
struct GrayDel {
  void operator()(Gray* g) const { free_gray(g); }
};

int galloc(Gray* g, double** p, size_t bytes)
{
  cudaError_t e = cudaMalloc((void**)p, bytes > 0 ? bytes : 16);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  g->dev_bytes += (long long)bytes;
  return PS_OK;
}

const double kT[3] = {1.0 / 3.0, 1.0 / 18.0, 1.0 / 36.0};
int wclass(int i) { return i == 0 ? 0 : (i < 7 ? 1 : 2); }

gray::Vals19 rest_state()  // shifted populations of rho = 1, u = 0
{
  gray::Vals19 r;
  for (int i = 0; i < 19; i++) r.v[i] = 0.0;
  return r;
}

cudaError_t fill(Gray* g, double* f, const gray::Vals19& v)
{
  gray::k_gray_fill<<<g->blocks(), kBlk, 0, g->stream>>>(g->G, v, f);
  return cudaGetLastError();
}

cudaError_t step(Gray* g, const double* src, double* dst)
{
  gray::k_gray_step<kBlk><<<g->blocks(), kBlk, 0, g->stream>>>(g->C, g->G, src, dst, g->s);
  return cudaGetLastError();
}

// permeability along idir of state f: nu (<j> + F/2) / F (lattice units)
int permeability(Gray* g, const double* f, double* k)
{
  const unsigned nb = g->blocks();
  gray::k_gray_momentum<kBlk><<<nb, kBlk, 0, g->stream>>>(g->G, f, g->part);
  PS_CUDA(cudaGetLastError());
  std::vector<double> h((size_t)nb * 3);
  PS_CUDA(cudaMemcpyAsync(h.data(), g->part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, g->stream));
  PS_CUDA(cudaStreamSynchronize(g->stream));
  const int d = g->p.idir - 1;
  double j = 0.0;
  for (unsigned b = 0; b < nb; b++) j += h[(size_t)b * 3 + d];
  const double nu = (g->p.tau - 0.5) / 3.0, F = g->p.F[d];
  *k = nu * (j / (double)g->G.n + 0.5 * F) / F;
  return PS_OK;
}

}  // namespace
}  // namespace ps

using namespace ps;

extern "C" {

int ps_gray_create(const ps_gray_params* p, int32_t nx, int32_t ny, int32_t nz, void** handle)
{
  if (!p || !handle) return fail(PS_ERR_ARG, "ps_gray_create: null argument");
  *handle = nullptr;
  if (nx < 1 || ny < 1 || nz < 1) return fail(PS_ERR_ARG, "ps_gray_create: bad box %d x %d x %d", nx, ny, nz);
  if (!(p->tau > 0.5) || !(p->magic > 0.0)) return fail(PS_ERR_ARG, "ps_gray_create: need tau > 1/2 and magic > 0");
  if (p->idir < 1 || p->idir > 3 || !(p->F[p->idir - 1] != 0.0))
    return fail(PS_ERR_ARG, "ps_gray_create: the body force along idir must be nonzero");
  if (p->nsteps < 1 || p->segment < 1) return fail(PS_ERR_ARG, "ps_gray_create: need nsteps >= 1 and segment >= 1");
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
    return fail(PS_ERR_NODEVICE, "ps_gray_create: no CUDA device");
  std::unique_ptr<Gray, GrayDel> g(new Gray);
  g->p = *p;
  g->G.nx = nx;
  g->G.ny = ny;
  g->G.nz = nz;
  g->G.n = (long long)nx * ny * nz;
  // TRT rates: lp = 1/tau, lm from the magic product (1/lp - 1/2)(1/lm - 1/2)
  const double lp = 1.0 / p->tau, lm = 1.0 / (0.5 + p->magic / (p->tau - 0.5));
  g->C.lp = lp;
  g->C.lm = lm;
  for (int c = 0; c < 3; c++) g->C.F[c] = p->F[c];
  for (int i = 0; i < 19; i++) {
    const double t = kT[wclass(i)];
    const double cF = gray::gcx(i) * p->F[0] + gray::gcy(i) * p->F[1] + gray::gcz(i) * p->F[2];
    g->C.t[i] = t;
    g->C.fF[i] = (1.0 - 0.5 * lm) * 3.0 * t * cF;
  }
  PS_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  if (int r = galloc(g.get(), &g->s, sizeof(double) * (size_t)g->G.n)) return r;
  if (int r = galloc(g.get(), &g->f[0], g->state_bytes())) return r;
  if (int r = galloc(g.get(), &g->f[1], g->state_bytes())) return r;
  if (int r = galloc(g.get(), &g->part, sizeof(double) * 3 * (size_t)g->blocks())) return r;
  PS_CUDA(cudaMemsetAsync(g->s, 0, sizeof(double) * (size_t)g->G.n, g->stream));
  PS_CUDA(cudaStreamSynchronize(g->stream));
  *handle = g.release();
  return PS_OK;
}

int ps_gray_destroy(void* h)
{
  free_gray(static_cast<Gray*>(h));
  return PS_OK;
}

int ps_gray_set_field(void* h, const double* s)
{
  if (!h || !s) return fail(PS_ERR_ARG, "ps_gray_set_field: null argument");
  Gray* g = static_cast<Gray*>(h);
  for (long long v = 0; v < g->G.n; v++)
    if (!(s[v] >= 0.0 && s[v] <= 1.0)) return fail(PS_ERR_ARG, "ps_gray_set_field: s[%lld] = %g outside [0, 1]", v, s[v]);
  PS_CUDA(cudaMemcpyAsync(g->s, s, sizeof(double) * (size_t)g->G.n, cudaMemcpyHostToDevice, g->stream));
  PS_CUDA(cudaStreamSynchronize(g->stream));
  g->ran = false;
  return PS_OK;
}

int ps_gray_permeability(void* h, double* k)
{
  if (!h || !k) return fail(PS_ERR_ARG, "ps_gray_permeability: null argument");
  Gray* g = static_cast<Gray*>(h);
  PS_CUDA(fill(g, g->f[0], rest_state()));
  int c = 0;
  for (int t = 0; t < g->p.nsteps; t++, c ^= 1) PS_CUDA(step(g, g->f[c], g->f[c ^ 1]));
  g->cur = c;
  g->ran = true;
  return permeability(g, g->f[c], k);
}

int ps_gray_gradient(void* h, double* k, double* dk_ds)
{
  if (!h || !k || !dk_ds) return fail(PS_ERR_ARG, "ps_gray_gradient: null argument");
  Gray* g = static_cast<Gray*>(h);
  const int T = g->p.nsteps, K = std::min(g->p.segment, T);
  const int nseg = (T + K - 1) / K;
  const size_t sb = g->state_bytes();
  // checkpoints, the states of one segment, two adjoint buffers, the gradient
  double *ck = nullptr, *seg = nullptr, *a[2] = {nullptr, nullptr}, *gs = nullptr;
  auto release = [&]() {
    cudaFree(ck);
    cudaFree(seg);
    cudaFree(a[0]);
    cudaFree(a[1]);
    cudaFree(gs);
  };
  cudaError_t e = cudaMalloc((void**)&ck, sb * (size_t)nseg);
  if (e == cudaSuccess) e = cudaMalloc((void**)&seg, sb * (size_t)K);
  if (e == cudaSuccess) e = cudaMalloc((void**)&a[0], sb);
  if (e == cudaSuccess) e = cudaMalloc((void**)&a[1], sb);
  if (e == cudaSuccess) e = cudaMalloc((void**)&gs, sizeof(double) * (size_t)g->G.n);
  if (e != cudaSuccess) {
    release();
    return fail(PS_ERR_NOMEM, "ps_gray_gradient: %.2f GB of checkpoints and segment states do not fit (%s); use a "
                "shorter segment", (double)sb * (nseg + K + 2) / 1e9, cudaGetErrorString(e));
  }
  const size_t n = (size_t)g->G.n;
  auto run = [&]() -> int {
    // forward with a checkpoint at the start of every segment
    PS_CUDA(fill(g, g->f[0], rest_state()));
    int c = 0;
    for (int t = 0; t < T; t++, c ^= 1) {
      if (t % K == 0)
        PS_CUDA(cudaMemcpyAsync(ck + (size_t)(t / K) * 19 * n, g->f[c], sb, cudaMemcpyDeviceToDevice, g->stream));
      PS_CUDA(step(g, g->f[c], g->f[c ^ 1]));
    }
    g->cur = c;
    g->ran = true;
    if (int r = permeability(g, g->f[c], k)) return r;
    // terminal adjoint: d k / d f_i(T) = nu c_i,idir / (F n)
    const int d = g->p.idir - 1;
    const double nu = (g->p.tau - 0.5) / 3.0, F = g->p.F[d];
    gray::Vals19 term;
    for (int i = 0; i < 19; i++) {
      const int ci = d == 0 ? gray::gcx(i) : (d == 1 ? gray::gcy(i) : gray::gcz(i));
      term.v[i] = nu * (double)ci / (F * (double)n);
    }
    PS_CUDA(fill(g, a[0], term));
    PS_CUDA(cudaMemsetAsync(gs, 0, sizeof(double) * n, g->stream));
    int ac = 0;
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
      const int t0 = sgi * K, t1 = std::min(T, t0 + K);
      PS_CUDA(cudaMemcpyAsync(seg, ck + (size_t)sgi * 19 * n, sb, cudaMemcpyDeviceToDevice, g->stream));
      for (int t = t0; t + 1 < t1; t++)
        PS_CUDA(step(g, seg + (size_t)(t - t0) * 19 * n, seg + (size_t)(t - t0 + 1) * 19 * n));
      for (int t = t1 - 1; t >= t0; t--, ac ^= 1) {
        gray::k_gray_adjoint<kBlk><<<g->blocks(), kBlk, 0, g->stream>>>(g->C, g->G, seg + (size_t)(t - t0) * 19 * n,
                                                                         a[ac], a[ac ^ 1], g->s, gs);
        PS_CUDA(cudaGetLastError());
      }
    }
    PS_CUDA(cudaMemcpyAsync(dk_ds, gs, sizeof(double) * n, cudaMemcpyDeviceToHost, g->stream));
    PS_CUDA(cudaStreamSynchronize(g->stream));
    return PS_OK;
  };
  const int r = run();
  cudaStreamSynchronize(g->stream);
  release();
  return r;
}

int ps_gray_get_state(void* h, double* f)
{
  if (!h || !f) return fail(PS_ERR_ARG, "ps_gray_get_state: null argument");
  Gray* g = static_cast<Gray*>(h);
  if (!g->ran) return fail(PS_ERR_STATE, "ps_gray_get_state: no forward run yet");
  const size_t n = (size_t)g->G.n;
  std::vector<double> soa(19 * n);
  PS_CUDA(cudaMemcpyAsync(soa.data(), g->f[g->cur], g->state_bytes(), cudaMemcpyDeviceToHost, g->stream));
  PS_CUDA(cudaStreamSynchronize(g->stream));
  for (size_t v = 0; v < n; v++)
    for (int i = 0; i < 19; i++) f[19 * v + i] = kT[wclass(i)] + soa[(size_t)i * n + v];
  return PS_OK;
}

}  // extern "C"
