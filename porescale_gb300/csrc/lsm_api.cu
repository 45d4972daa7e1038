// lsm_api.cu -- C ABI of the lattice-spring static solve (include/porescale.h).
//
// Replaces the reference's damped-Verlet relaxation and calc_stress
// (XX_P.f:1377-1545, 1628-1997; YZ_P.f likewise) by a conjugate-gradient
// solve of the same linear spring network: the tied node planes of the
// loaded axis become one periodic plane with a displacement jump, the
// unknowns are the unique solid nodes, and the operator is applied
// matrix-free from per-material cube matrices (lsm_cube.h).  Precisions:
//   PS_LSM_F64    FP64 CG;
//   PS_LSM_MIXED  FP32 CG inside FP64 iterative refinement: the residual,
//                 dot products and solution update are FP64, the inner
//                 operator products and vectors FP32.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lsm_cube.h"
#include "lsm_kernels.cuh"
#include "ps_common.h"
#include "ps_coupling.h"

namespace ps {
namespace {

using lsm::LsmGeom;

constexpr int kBlk = 256;
// ps_lsm_batch_solve (mixed precision): host threads and streams running
// groups at a time, and the FP32 CG vector bytes a group of networks may
// hold (measured on 48 networks each of 24^3 ... 64^3 and on the 48
// subvolumes of 48^3 ... 128^3: 8, 16 and 40 MB; 40 MB was best or level)
constexpr int kBatchThreads = 8;
constexpr long long kGroupBytes = 40LL << 20;

// A captured batch of CG iterations (CUDA graph) for one vector set
struct CgGraph {
  cudaGraphExec_t exec = nullptr;
  const void* x = nullptr;
  double tol2 = -1.0;
};

struct Springs {
  ps_lsm_params p{};
  CgGraph g64, g32;
  int nx = 0, ny = 0, nz = 0, nvox = 0, pa = 0, jc = 0;
  long long nnode = 0, ncube = 0, ns_ref = 0;
  std::vector<uint8_t> mat, node;
  cudaStream_t stream = nullptr;
  uint8_t *d_mat = nullptr, *d_node = nullptr;
  int* d_surf = nullptr;  // surface nodes (node class 1) in node order
  int nsurf = 0;
  double *d_K64 = nullptr, *d_S64 = nullptr;  // per-material cube matrices of this handle
  double* d_Kab = nullptr;                      // material-independent Ka, Kb (modulus gradients)
  double* fext = nullptr;                       // external nodal load [3][nvox] (fluid wall load)
  bool has_load = false;
  // FP64 vectors (3*nvox each)
  double *b = nullptr, *x = nullptr, *r = nullptr, *p64 = nullptr, *q64 = nullptr;
  // FP32 inner vectors
  float *x32 = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr;
  double *part = nullptr, *scal = nullptr;
  // damped dynamics (ps_lsm_dyn_step): velocity and acceleration [3][nvox]
  // (the displacement is x) and the spring forces of the jump alone
  double *dv = nullptr, *da = nullptr, *bj = nullptr;
  bool periodic = false;  // PS_LOAD_NONE: no tied plane, every axis periodic
  unsigned* ctr = nullptr;  // last-CTA counter of the CG reductions
  int nblk = 0;
  bool solved = false;
  ps_lsm_result last{};
  long long dev_bytes = 0;

  LsmGeom geom() const
  {
    return LsmGeom{nx, ny, nz, nvox, d_mat, d_node, d_K64, d_S64, {(float)p.alf1, (float)p.alf2},
                   {(float)p.bet1, (float)p.bet2}, {p.alf1, p.alf2}, {p.bet1, p.bet2}, d_surf, nsurf};
  }
};

void free_springs(Springs* S)
{
  if (!S) return;
  cudaFree(S->d_mat);
  cudaFree(S->d_node);
  cudaFree(S->d_surf);
  cudaFree(S->d_K64);
  cudaFree(S->d_S64);
  cudaFree(S->d_Kab);
  cudaFree(S->fext);
  cudaFree(S->b);
  cudaFree(S->x);
  cudaFree(S->r);
  cudaFree(S->p64);
  cudaFree(S->q64);
  cudaFree(S->x32);
  cudaFree(S->r32);
  cudaFree(S->p32);
  cudaFree(S->q32);
  cudaFree(S->ctr);
  cudaFree(S->dv);
  cudaFree(S->da);
  cudaFree(S->bj);
  cudaFree(S->part);
  cudaFree(S->scal);
  if (S->g64.exec) cudaGraphExecDestroy(S->g64.exec);
  if (S->g32.exec) cudaGraphExecDestroy(S->g32.exec);
  if (S->stream) cudaStreamDestroy(S->stream);
  delete S;
}

template <typename T>
int dalloc(Springs* S, T** p, size_t bytes)
{
  cudaError_t e = cudaMalloc((void**)p, bytes > 0 ? bytes : 16);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  S->dev_bytes += (long long)bytes;
  return PS_OK;
}

// ---- small device helpers -------------------------------------------------
__global__ void k_masked_sum3(int nv, const uint8_t* node, const double* u, double* part)
{
  __shared__ double red[3][kBlk / 32];
  const int v = blockIdx.x * kBlk + threadIdx.x;
  double s[3] = {0.0, 0.0, 0.0};
  if (v < nv && node[v])
    for (int c = 0; c < 3; c++) s[c] = u[c * nv + v];
  for (int c = 0; c < 3; c++) {
    double t = s[c];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < kBlk / 32; w++) t += red[threadIdx.x][w];
    part[blockIdx.x * 3 + threadIdx.x] = t;
  }
}
__global__ void k_sum3(const double* part, int n, double inv_count, double* out)
{
  if (threadIdx.x >= 3) return;
  double s = 0.0;
  for (int i = 0; i < n; i++) s += part[3 * i + threadIdx.x];
  out[threadIdx.x] = s * inv_count;
}
// u -= mean on existing nodes (removes the rigid translation component)
__global__ void k_sub_mean(int nv, const uint8_t* node, const double* mean, double* u)
{
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv || !node[v]) return;
  for (int c = 0; c < 3; c++) u[c * nv + v] -= mean[c];
}
__global__ void k_axpy_res(int n3, const double* b, const double* q, double* r, double* part)
{
  __shared__ double red[kBlk / 32];
  const int i = blockIdx.x * kBlk + threadIdx.x;
  double t = 0.0;
  if (i < n3) {
    const double ri = b[i] - q[i];
    r[i] = ri;
    t = ri * ri;
  }
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kBlk / 32; w++) s += red[w];
    part[blockIdx.x] = s;
  }
}
__global__ void k_sq_norm(int n3, const double* r, double* part)
{
  __shared__ double red[kBlk / 32];
  const int i = blockIdx.x * kBlk + threadIdx.x;
  double t = i < n3 ? r[i] * r[i] : 0.0;
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kBlk / 32; w++) s += red[w];
    part[blockIdx.x] = s;
  }
}
// inner start: r32 = r64 * s, p32 = r32, x32 = 0
__global__ void k_ir_start(int n3, double s, const double* r64, float* r32, float* p32, float* x32)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  const float v = (float)(r64[i] * s);
  r32[i] = v;
  p32[i] = v;
  x32[i] = 0.f;
}
// refinement update x64 += s * x32
__global__ void k_ir_update(int n3, double s, const float* x32, double* x)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  x[i] += s * (double)x32[i];
}
__global__ void k_set_scal(double* scal, double rr, double bb)
{
  scal[0] = rr;
  scal[3] = 0.0;
  scal[5] = bb;
  scal[6] = 0.0;
  scal[7] = 0.0;
}

int blocks_for(long long n) { return (int)((n + kBlk - 1) / kBlk); }
// CTAs of the CG kernels: one per tile of kMvPer nodes (bulk), kSfPer
// surface nodes (at least one CTA, whose last CTA ends the p.q sum) or
// kVecPer elements per thread
int mv_tiles(long long n) { return (int)((n + lsm::kMvPer * kBlk - 1) / (lsm::kMvPer * kBlk)); }
int sf_tiles(long long n) { return std::max(1, (int)((n + lsm::kSfPer * kBlk - 1) / (lsm::kSfPer * kBlk))); }
int vec_tiles(long long n) { return (int)((n + lsm::kVecPer * kBlk - 1) / (lsm::kVecPer * kBlk)); }

// ---- host-side solve ---------------------------------------------------------
// q = A u in FP64 (bulk then surface kernel; their p.q partials in part[])
int matvec64(Springs* S, const double* u, double* q)
{
  const int tm = mv_tiles(S->nvox);
  lsm::k_lsm_matvec<double, kBlk><<<tm, kBlk, 0, S->stream>>>(S->geom(), u, q, S->part);
  lsm::k_lsm_matvec_surf<double, kBlk><<<sf_tiles(S->nsurf), kBlk, 0, S->stream>>>(S->geom(), u, q, S->part + tm);
  PS_CUDA(cudaGetLastError());
  return PS_OK;
}

int sum_parts(Springs* S, int n, double* d_out)
{
  lsm::k_sum<<<1, 1024, 0, S->stream>>>(S->part, n, d_out);
  return cudaGetLastError() == cudaSuccess ? PS_OK : cuda_fail(cudaGetLastError(), "k_sum");
}

int project_mean(Springs* S, double* u)
{
  const int nb = blocks_for(S->nvox);
  k_masked_sum3<<<nb, kBlk, 0, S->stream>>>(S->nvox, S->d_node, u, S->part);
  k_sum3<<<1, 32, 0, S->stream>>>(S->part, nb, 1.0 / (double)std::max(1LL, S->nnode), S->scal + 8);
  k_sub_mean<<<nb, kBlk, 0, S->stream>>>(S->nvox, S->d_node, S->scal + 8, u);
  PS_CUDA(cudaGetLastError());
  return PS_OK;
}

int read_scal(Springs* S, double* h, int n)
{
  PS_CUDA(cudaMemcpyAsync(h, S->scal, sizeof(double) * n, cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  return PS_OK;
}

// CG on A x = r0 from x = 0 (T = double: x,r,p,q are the FP64 vectors; T =
// float: the FP32 inner vectors).  Stops at |r| <= tol |r0| or maxit.
// Returns iterations in *its and the final |r|^2 / |r0|^2 in *rel2.
template <typename T>
int cg(Springs* S, T* x, T* r, T* p, T* q, double tol, long long maxit, long long* its, double* rel2)
{
  const int n3 = 3 * S->nvox;
  const int nb = blocks_for(S->nvox), nb3 = blocks_for(n3);
  const LsmGeom G = S->geom();
  // |r0|^2 (x = 0 and p = r0 set by the caller)
  lsm::k_sq_norm_t<T, kBlk><<<nb3, kBlk, 0, S->stream>>>(n3, r, S->part);
  if (int e = sum_parts(S, nb3, S->scal + 0)) return e;
  double h[8];
  if (int e = read_scal(S, h, 1)) return e;
  const double rr0 = h[0];
  k_set_scal<<<1, 1, 0, S->stream>>>(S->scal, rr0, rr0);
  PS_CUDA(cudaGetLastError());
  long long it = 0;
  const double tol2 = tol * tol;
  const int batch = 16;
  bool done = rr0 == 0.0;
  // the iteration needs no host decision (alpha, beta and the stop flag live
  // on the device), so a batch of iterations is captured once into a CUDA
  // graph and replayed until the stop flag is set
  CgGraph& cgg = sizeof(T) == 8 ? S->g64 : S->g32;
  if (!done && (!cgg.exec || cgg.tol2 != tol2 || cgg.x != (const void*)x)) {
    if (cgg.exec) cudaGraphExecDestroy(cgg.exec);
    cgg.exec = nullptr;
    cudaGraph_t graph = nullptr;
    PS_CUDA(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
    const int tm = mv_tiles(S->nvox), ts = sf_tiles(S->nsurf), tv = vec_tiles(n3);
    for (int k = 0; k < batch; k++) {
      lsm::k_cg_mv<T, kBlk><<<tm, kBlk, 0, S->stream>>>(G, S->scal, p, q, S->part);
      lsm::k_cg_mv_surf<T, kBlk><<<ts, kBlk, 0, S->stream>>>(G, S->scal, p, q, S->part, tm, S->ctr, tol2);
      lsm::k_cg_xr<T, kBlk><<<tv, kBlk, 0, S->stream>>>(n3, S->scal, x, r, p, q, S->part, S->ctr);
      lsm::k_cg_p<T, kBlk><<<tv, kBlk, 0, S->stream>>>(n3, S->scal, r, p);
    }
    cudaError_t ce = cudaStreamEndCapture(S->stream, &graph);
    if (ce != cudaSuccess) return cuda_fail(ce, "CG batch capture");
    ce = cudaGraphInstantiate(&cgg.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return cuda_fail(ce, "CG batch instantiate");
    cgg.tol2 = tol2;
    cgg.x = x;
  }
  while (!done && it < maxit) {
    PS_CUDA(cudaGraphLaunch(cgg.exec, S->stream));
    if (int e = read_scal(S, h, 7)) return e;
    done = h[6] > 0.0;
    it += batch;
  }
  if (int e = read_scal(S, h, 8)) return e;
  *its = (long long)h[7];
  *rel2 = rr0 > 0 ? h[0] / rr0 : 0.0;
  return PS_OK;
}

int residual(Springs* S, double* rnorm2)
{
  const int n3 = 3 * S->nvox;
  const int nb3 = blocks_for(n3);
  if (int e = matvec64(S, S->x, S->q64)) return e;
  k_axpy_res<<<nb3, kBlk, 0, S->stream>>>(n3, S->b, S->q64, S->r, S->part);
  PS_CUDA(cudaGetLastError());
  if (int e = project_mean(S, S->r)) return e;
  k_sq_norm<<<nb3, kBlk, 0, S->stream>>>(n3, S->r, S->part);
  if (int e = sum_parts(S, nb3, S->scal + 16)) return e;
  PS_CUDA(cudaMemcpyAsync(rnorm2, S->scal + 16, sizeof(double), cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  return PS_OK;
}

int compute_stress(Springs* S, ps_lsm_result* out)
{
  const int nb = blocks_for(S->nvox);
  const double jump = 2.0 * S->p.gstrain;
  lsm::k_lsm_stress<kBlk><<<nb, kBlk, 0, S->stream>>>(S->geom(), S->pa, S->jc, jump, S->x, S->part);
  PS_CUDA(cudaGetLastError());
  std::vector<double> h((size_t)nb * 9);
  PS_CUDA(cudaMemcpyAsync(h.data(), S->part, sizeof(double) * 9 * nb, cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  double sig[9] = {0};
  for (int b = 0; b < nb; b++)
    for (int i = 0; i < 9; i++) sig[i] += h[(size_t)b * 9 + i];
  for (int i = 0; i < 9; i++) out->sigma[i] = sig[i];
  const double vcell = (double)S->nx * S->ny * S->nz;
  const double nax = S->pa == 0 ? S->nx : S->ny;
  const double s = S->pa == 0 ? sig[0] : sig[5];  // asigmap(1,1) or asigmap(2,3)
  out->strain = jump / nax;
  out->modulus = jump != 0.0 ? s / (vcell * jump / nax) : 0.0;
  return PS_OK;
}

// ---- no-allocation stress reduction -------------------------------------
// Scratch of ps_lsm_stress_noalloc: one 9-component partial sum per CTA of
// the stress kernel plus the 9 final sums.  It is a file-scope device array,
// so the entry point never allocates; every GPU that loads the library holds
// it (about 590 KB) until the process exits.
constexpr int kNoAllocMaxBlocks = PS_LSM_NOALLOC_MAX_CUBES / kBlk;
static __device__ __align__(256) double g_stress_scratch[9 * kNoAllocMaxBlocks + 9];

// fixed-order sum of n partials (9 components each) into out[0..8]
__global__ void k_stress_final(const double* part, int n, double* out)
{
  if (threadIdx.x >= 9) return;
  double s = 0.0;
  for (int b = 0; b < n; b++) s += part[(long long)b * 9 + threadIdx.x];
  out[threadIdx.x] = s;
}

// device address of g_stress_scratch on the current device.  Looked up on
// every call, with the caller's device current: the host-side symbol is
// only a stand-in, and an address kept from an earlier call would be stale
// after the application resets the device or recreates its primary
// context.  The lookup allocates nothing.
int noalloc_scratch(double** out)
{
  double* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void**)&p, g_stress_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_stress_scratch)");
  *out = p;
  return PS_OK;
}

// fext = the load on existing nodes; counts loaded corners that are not
// nodes of this network
__global__ void k_take_load(int nv, const uint8_t* node, const double* box, double* fext, unsigned long long* lost)
{
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const bool ok = node[v] != 0;
  bool loaded = false;
  for (int c = 0; c < 3; c++) {
    const double f = box[(size_t)c * nv + v];
    loaded |= f != 0.0;
    fext[(size_t)c * nv + v] = ok ? f : 0.0;
  }
  if (loaded && !ok) atomicAdd(lost, 1ull);
}

__global__ void k_add(int n, const double* a, double* b)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] += a[i];
}

// Surface term of calc_ab's beta (S1:4262-4437) for pore labels
// [p0, p0 + 32): a pore voxel of label p with a solid (label 0) axis
// neighbour d contributes -u_face . c_d, u_face the mean displacement of the
// 4 corner nodes of the shared face.  Per-block FP64 partial sums
// part[32 b + (p - p0)].
__global__ void __launch_bounds__(256) k_beta_surface(const LsmGeom G, const int32_t* __restrict__ lab, int p0,
                                                      const double* __restrict__ u, double* __restrict__ part)
{
  const int v = blockIdx.x * 256 + threadIdx.x;
  int p = -1;
  double val = 0.0;
  if (v < G.nvox) {
    const int l = lab[v];
    if (l >= p0 && l < p0 + 32 && l > 0) {
      p = l - p0;
      const int nx = G.nx, ny = G.ny, nz = G.nz, nv = G.nvox;
      const int c3[3] = {v % nx, (v / nx) % ny, v / (nx * ny)};
      const int n3[3] = {nx, ny, nz};
      for (int d = 0; d < 6; d++) {  // +x, -x, +y, -y, +z, -z (reference l = 2..7)
        const int ax = d >> 1, sg = (d & 1) ? -1 : 1;
        int w[3] = {c3[0], c3[1], c3[2]};
        w[ax] = lsm::wrap_add(c3[ax], sg, n3[ax]);
        if (lab[w[0] + nx * (w[1] + ny * w[2])] != 0) continue;
        // face corners: offset (sg + 1) / 2 along ax, 0/1 along the others
        const int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
        double up[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < 4; q++) {
          int cn[3];
          cn[ax] = lsm::wrap_add(c3[ax], (sg + 1) / 2, n3[ax]);
          cn[a1] = lsm::wrap_add(c3[a1], q & 1, n3[a1]);
          cn[a2] = lsm::wrap_add(c3[a2], q >> 1, n3[a2]);
          const int nb = cn[0] + nx * (cn[1] + ny * cn[2]);
          for (int c = 0; c < 3; c++) up[c] += u[(size_t)c * nv + nb];
        }
        val -= 0.25 * up[ax] * (double)sg;
      }
    }
  }
  __shared__ double red[32][8];
  for (int q = 0; q < 32; q++) {
    double t = (p == q) ? val : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int w = 0; w < 8; w++) t += red[threadIdx.x][w];
    part[(long long)blockIdx.x * 32 + threadIdx.x] = t;
  }
}

// right-hand side of the tied system (imposed jump plus any wall load),
// without its translation component; |b|^2 to *bb; x = 0
int prepare(Springs* S, double* bb)
{
  const int nv = S->nvox, n3 = 3 * nv;
  const int nb = blocks_for(nv), nb3 = blocks_for(n3);
  lsm::k_lsm_rhs<<<nb, kBlk, 0, S->stream>>>(S->geom(), S->pa, S->jc, 2.0 * S->p.gstrain, S->b);
  PS_CUDA(cudaGetLastError());
  if (S->has_load) {  // fluid wall load; its net force is removed with the mean below
    k_add<<<nb3, kBlk, 0, S->stream>>>(n3, S->fext, S->b);
    PS_CUDA(cudaGetLastError());
  }
  if (int e = project_mean(S, S->b)) return e;
  k_sq_norm<<<nb3, kBlk, 0, S->stream>>>(n3, S->b, S->part);
  if (int e = sum_parts(S, nb3, S->scal + 17)) return e;
  PS_CUDA(cudaMemcpyAsync(bb, S->scal + 17, sizeof(double), cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaMemsetAsync(S->x, 0, sizeof(double) * n3, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  return PS_OK;
}

// true FP64 residual, stress and modulus of the current solution into *out
int finish(Springs* S, double bb, double rtol, ps_lsm_result* out)
{
  double rn2 = 0.0;
  if (int e = residual(S, &rn2)) return e;
  const double rel = bb > 0.0 ? std::sqrt(rn2 / bb) : 0.0;
  out->relres = rel;
  out->converged = rel <= rtol * 1.0000001 ? 1 : 0;
  out->nnode = S->nnode;
  out->ncube = S->ncube;
  if (int e = compute_stress(S, out)) return e;
  S->solved = true;
  S->last = *out;
  return PS_OK;
}

// Runs f(s) for every network s = 0..n-1 on up to 8 host threads (each
// network has its own stream, so the per-network launches and waits of the
// refinement overlap instead of queueing behind one another); returns the
// first error code, its message moved to the calling thread.
template <typename F>
int each_network(int n, F f)
{
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int> next{0};
  std::mutex mu;
  int err = PS_OK;
  std::string msg;
  auto work = [&]() {
    cudaSetDevice(dev);
    for (int s = next++; s < n; s = next++) {
      {
        std::lock_guard<std::mutex> g(mu);
        if (err) return;
      }
      const int e = f(s);
      if (e) {
        std::lock_guard<std::mutex> g(mu);
        if (!err) {
          err = e;
          msg = last_error();
        }
        return;
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < std::min(n, 8); t++) th.emplace_back(work);
  work();
  for (std::thread& t : th) t.join();
  if (err) last_error() = msg;
  return err;
}

// The table's list of the networks a batched launch covers (in the given
// order) and the first bulk / surface / element tile of each.
void set_live(lsm::LsmTable& tab, const std::vector<int>& live)
{
  tab.nlive = (int)live.size();
  int a = 0, b = 0, c = 0;
  for (int k = 0; k < tab.nlive; k++) {
    const lsm::LsmSys& d = tab.s[live[k]];
    tab.live[k] = live[k];
    tab.f1[k] = a;
    tab.fs[k] = b;
    tab.f3[k] = c;
    a += d.nt1;
    b += d.nts;
    c += d.nt3;
  }
  tab.f1[tab.nlive] = a;
  tab.fs[tab.nlive] = b;
  tab.f3[tab.nlive] = c;
}

// ---- batched CG over several networks ---------------------------------------
// CG on A x = r0 (x = 0, p = r0 set by the caller) for every network of the
// list at once: the iteration of cg<T> with each kernel launched once for
// all networks (the launch table lists them with their first tiles), 16
// iterations per captured graph, until every network has converged or
// maxit is reached.  When the networks still running hold under 3/4 of the
// bulk tiles the graph was captured with, the graph is captured anew over
// them, so the slowest networks' last iterations do not launch the
// finished networks' tiles.
template <typename T>
int batch_cg(const std::vector<Springs*>& sys, double tol, long long maxit, cudaStream_t st)
{
  const int n = (int)sys.size();
  lsm::LsmTable tab;
  memset(&tab, 0, sizeof tab);
  tab.n = n;
  for (int s = 0; s < n; s++) {
    Springs* S = sys[s];
    lsm::LsmSys& d = tab.s[s];
    d.G = S->geom();
    if (sizeof(T) == 8) {
      d.x = S->x;
      d.r = S->r;
      d.p = S->p64;
      d.q = S->q64;
    } else {
      d.x = S->x32;
      d.r = S->r32;
      d.p = S->p32;
      d.q = S->q32;
    }
    d.part = S->part;
    d.scal = S->scal;
    d.ctr = S->ctr;
    d.n3 = 3 * S->nvox;
    d.nt1 = mv_tiles(S->nvox);
    d.nts = sf_tiles(S->nsurf);
    d.nt3 = vec_tiles(d.n3);
    // |r0|^2 into scal[0] on the network's own stream
    lsm::k_sq_norm_t<T, kBlk><<<blocks_for(d.n3), kBlk, 0, S->stream>>>(d.n3, static_cast<const T*>(d.r), S->part);
    if (int e = sum_parts(S, blocks_for(d.n3), S->scal)) return e;
    PS_CUDA(cudaStreamSynchronize(S->stream));
  }
  double* ddone = nullptr;
  cudaGraphExec_t exec = nullptr;
  auto release = [&]() {
    cudaFree(ddone);
    if (exec) cudaGraphExecDestroy(exec);
  };
  const double tol2 = tol * tol;
  const int batch = 16;
  std::vector<double> done((size_t)n, 0.0);
  // the graph over the networks not yet converged
  auto rebuild = [&]() -> int {
    std::vector<int> live;
    for (int s = 0; s < n; s++)
      if (!(done[s] > 0.0)) live.push_back(s);
    set_live(tab, live);
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    if (live.empty()) return PS_OK;
    cudaGraph_t graph = nullptr;
    PS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < batch; k++) {
      lsm::k_cg_mv_batch<T, kBlk><<<(unsigned)tab.f1[tab.nlive], kBlk, 0, st>>>(tab);
      lsm::k_cg_mv_surf_batch<T, kBlk><<<(unsigned)tab.fs[tab.nlive], kBlk, 0, st>>>(tab, tol2);
      lsm::k_cg_xr_batch<T, kBlk><<<(unsigned)tab.f3[tab.nlive], kBlk, 0, st>>>(tab);
      lsm::k_cg_p_batch<T, kBlk><<<(unsigned)tab.f3[tab.nlive], kBlk, 0, st>>>(tab);
    }
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) return cuda_fail(ce, "batched CG capture");
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      exec = nullptr;
      return cuda_fail(ce, "batched CG instantiate");
    }
    return PS_OK;
  };
  auto run = [&]() -> int {
    PS_CUDA(cudaMalloc((void**)&ddone, sizeof(double) * 2 * n));
    lsm::k_cg_init_batch<<<1, lsm::kLsmBatchMax, 0, st>>>(tab);
    PS_CUDA(cudaGetLastError());
    if (int e = rebuild()) return e;
    for (long long it = 0; it < maxit && exec; it += batch) {
      PS_CUDA(cudaGraphLaunch(exec, st));
      lsm::k_cg_done_batch<<<1, lsm::kLsmBatchMax, 0, st>>>(tab, ddone);
      std::vector<double> now((size_t)n, 0.0);
      PS_CUDA(cudaMemcpyAsync(now.data(), ddone, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      PS_CUDA(cudaStreamSynchronize(st));
      size_t live = 0;  // node tiles of the networks still running
      for (int s = 0; s < n; s++)
        if (!(now[s] > 0.0)) live += (size_t)tab.s[s].nt1;
      done = now;
      if (live == 0 || 4 * live < 3 * (size_t)tab.f1[tab.nlive])
        if (int e = rebuild()) return e;
    }
    return PS_OK;
  };
  const int r = run();
  cudaStreamSynchronize(st);
  release();
  return r;
}

// FP64 iterative refinement around FP32 CG on the network's own stream
// (after prepare(), |b|^2 = bb): rounds of an inner CG to 1e-4 on r / |r|
// until the FP64 residual is below rtol, maxit inner iterations are spent
// or 60 rounds are done; the counts go to out.
int mixed_ir(Springs* S, double bb, double rtol, long long maxit, ps_lsm_result* out)
{
  const int n3 = 3 * S->nvox, nb3 = blocks_for(n3);
  const double inner_tol = 1e-4;
  long long budget = maxit, iters = 0, inner = 0;
  int refinements = 0;
  for (refinements = 0; refinements < 60; refinements++) {
    double rn2 = 0.0;
    if (refinements == 0) {
      PS_CUDA(cudaMemcpyAsync(S->r, S->b, sizeof(double) * n3, cudaMemcpyDeviceToDevice, S->stream));
      rn2 = bb;
    } else if (int e = residual(S, &rn2)) {
      return e;
    }
    if (!(bb > 0.0) || rn2 <= rtol * rtol * bb || budget <= 0) break;
    const double rn = std::sqrt(rn2);
    k_ir_start<<<nb3, kBlk, 0, S->stream>>>(n3, 1.0 / rn, S->r, S->r32, S->p32, S->x32);
    PS_CUDA(cudaGetLastError());
    long long it = 0;
    double rel2 = 0.0;
    if (int e = cg<float>(S, S->x32, S->r32, S->p32, S->q32, inner_tol, budget, &it, &rel2)) return e;
    inner += it;
    budget -= it;
    k_ir_update<<<nb3, kBlk, 0, S->stream>>>(n3, rn, S->x32, S->x);
    PS_CUDA(cudaGetLastError());
    iters++;
  }
  out->iterations = iters;
  out->inner_iterations = inner;
  out->refinements = refinements;
  return PS_OK;
}

// ---- batched mixed-precision solve -------------------------------------------
// ps_lsm_solve's FP64 refinement around FP32 CG for every network of the
// list, the inner CGs advanced together by the batched kernels, with no
// barrier between refinement rounds: a network whose inner CG has
// converged (or spent its iteration budget) leaves the batch at the next
// poll (every 16 iterations), is refined on a worker thread and its own
// stream (x += |r| x32, the FP64 residual, the next inner system) while the
// others keep iterating, and joins the batch again at the poll after that.
// The captured iterations cover every network not yet finished, so that a
// network joining or leaving changes only its scalars (a network outside
// the batch has its stop flag set and its tiles return at once); the graph
// is rebuilt over the unfinished networks when they hold under 3/4 of its
// tiles.  Each network does the arithmetic of ps_lsm_solve's loop in the
// same order (same tiles, same scalars), so the results equal the
// individual solves'.
// bb[s] = |b|^2; the per-network counts go to out[s].  nworkers host
// threads do the refinement steps.
int batch_mixed(const std::vector<Springs*>& sys, const std::vector<double>& bb, double rtol, long long maxit,
                ps_lsm_result* out, cudaStream_t st, int nworkers)
{
  const int n = (int)sys.size();
  lsm::LsmTable tab;
  memset(&tab, 0, sizeof tab);
  tab.n = n;
  for (int s = 0; s < n; s++) {
    Springs* S = sys[s];
    lsm::LsmSys& d = tab.s[s];
    d.G = S->geom();
    d.x = S->x32;
    d.r = S->r32;
    d.p = S->p32;
    d.q = S->q32;
    d.part = S->part;
    d.scal = S->scal;
    d.ctr = S->ctr;
    d.n3 = 3 * S->nvox;
    d.nt1 = mv_tiles(S->nvox);
    d.nts = sf_tiles(S->nsurf);
    d.nt3 = vec_tiles(d.n3);
  }
  std::vector<long long> budget((size_t)n, maxit);
  std::vector<double> rn((size_t)n, 0.0);
  std::vector<char> begun((size_t)n, 0);
  // the step between two inner solves of network s; *next = true when
  // another inner solve follows (its r32, p32, x32 and |r0|^2 in scal[0] set)
  auto refine = [&](int s, bool* next) -> int {
    Springs* S = sys[s];
    const int n3 = 3 * S->nvox, nb3 = blocks_for(n3);
    double rn2 = 0.0;
    *next = false;
    if (!begun[s]) {
      begun[s] = 1;
      PS_CUDA(cudaMemcpyAsync(S->r, S->b, sizeof(double) * n3, cudaMemcpyDeviceToDevice, S->stream));
      rn2 = bb[s];
    } else {
      double h8[8];
      if (int e = read_scal(S, h8, 8)) return e;
      const long long its = (long long)h8[7];
      out[s].inner_iterations += its;
      out[s].iterations++;
      budget[s] -= its;
      k_ir_update<<<nb3, kBlk, 0, S->stream>>>(n3, rn[s], S->x32, S->x);
      PS_CUDA(cudaGetLastError());
      if (int e = residual(S, &rn2)) return e;
    }
    if (!(bb[s] > 0.0) || rn2 <= rtol * rtol * bb[s] || budget[s] <= 0 || out[s].refinements >= 60) return PS_OK;
    rn[s] = std::sqrt(rn2);
    k_ir_start<<<nb3, kBlk, 0, S->stream>>>(n3, 1.0 / rn[s], S->r, S->r32, S->p32, S->x32);
    lsm::k_sq_norm_t<float, kBlk><<<nb3, kBlk, 0, S->stream>>>(n3, S->r32, S->part);
    if (int e = sum_parts(S, nb3, S->scal + 0)) return e;
    PS_CUDA(cudaStreamSynchronize(S->stream));
    out[s].refinements++;
    *next = true;
    return PS_OK;
  };

  // worker threads: refinement steps of the networks in `todo`; the
  // networks with another inner solve go to `ready`
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int> todo;
  std::vector<int> ready;
  std::vector<char> fin((size_t)n, 0);  // no further inner solve
  int pending = n, err = PS_OK;
  bool quit = false;
  std::string msg;
  for (int s = 0; s < n; s++) todo.push_back(s);
  int dev = 0;
  cudaGetDevice(&dev);
  auto worker = [&]() {
    cudaSetDevice(dev);
    for (;;) {
      int s;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return quit || !todo.empty(); });
        if (todo.empty()) return;
        s = todo.front();
        todo.pop_front();
      }
      bool next = false;
      const int e = refine(s, &next);
      {
        std::lock_guard<std::mutex> g(mu);
        if (e && !err) {
          err = e;
          msg = last_error();
        }
        if (!e && next) ready.push_back(s);
        if (!e && !next) fin[s] = 1;
        pending--;
      }
      cv.notify_all();
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < std::min(n, nworkers); t++) th.emplace_back(worker);

  double* ddone = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<int> run;  // networks in the batch
  const double tol2 = 1e-4 * 1e-4;
  const int batch = 16;
  // the captured iterations over the networks in `cover`
  auto rebuild = [&](const std::vector<int>& cover) -> int {
    set_live(tab, cover);
    if (cover.empty()) {
      if (exec) cudaGraphExecDestroy(exec);
      exec = nullptr;
      return PS_OK;
    }
    cudaGraph_t graph = nullptr;
    PS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < batch; k++) {
      lsm::k_cg_mv_batch<float, kBlk><<<(unsigned)tab.f1[tab.nlive], kBlk, 0, st>>>(tab);
      lsm::k_cg_mv_surf_batch<float, kBlk><<<(unsigned)tab.fs[tab.nlive], kBlk, 0, st>>>(tab, tol2);
      lsm::k_cg_xr_batch<float, kBlk><<<(unsigned)tab.f3[tab.nlive], kBlk, 0, st>>>(tab);
      lsm::k_cg_p_batch<float, kBlk><<<(unsigned)tab.f3[tab.nlive], kBlk, 0, st>>>(tab);
    }
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) return cuda_fail(ce, "batched CG capture");
    // the graphs differ only in grid sizes and the table's list: update the
    // instantiated one in place (microseconds) rather than instantiating anew
    cudaGraphExecUpdateResultInfo info;
    if (exec && cudaGraphExecUpdate(exec, graph, &info) != cudaSuccess) {
      cudaGetLastError();  // clear the failed update
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    if (!exec) {
      ce = cudaGraphInstantiate(&exec, graph, 0);
      if (ce != cudaSuccess) {
        cudaGraphDestroy(graph);
        exec = nullptr;
        return cuda_fail(ce, "batched CG instantiate");
      }
    }
    cudaGraphDestroy(graph);
    return PS_OK;
  };
  auto drive = [&]() -> int {
    PS_CUDA(cudaMalloc((void**)&ddone, sizeof(double) * 2 * n));
    std::vector<double> now((size_t)2 * n, 0.0);
    {  // every network starts outside the batch
      lsm::LsmList all{};
      all.n = n;
      for (int s = 0; s < n; s++) all.s[s] = s;
      lsm::k_cg_stop_batch<<<1, lsm::kLsmBatchMax, 0, st>>>(tab, all);
      PS_CUDA(cudaGetLastError());
    }
    for (;;) {
      std::vector<int> admit, cover;
      {
        std::unique_lock<std::mutex> lk(mu);
        if (run.empty()) cv.wait(lk, [&] { return err || !ready.empty() || pending == 0; });
        if (err) return PS_OK;  // the worker's error is returned below
        admit.swap(ready);
        if (run.empty() && admit.empty() && pending == 0) return PS_OK;
        for (int s = 0; s < n; s++)
          if (!fin[s]) cover.push_back(s);
      }
      if (!admit.empty()) {
        lsm::LsmList L{};
        L.n = (int)admit.size();
        for (int i = 0; i < L.n; i++) L.s[i] = admit[i];
        lsm::k_cg_admit_batch<<<1, lsm::kLsmBatchMax, 0, st>>>(tab, L);
        PS_CUDA(cudaGetLastError());
        run.insert(run.end(), admit.begin(), admit.end());
        std::sort(run.begin(), run.end());
      }
      size_t live = 0;
      for (int s : cover) live += (size_t)tab.s[s].nt1;
      if (!exec || 4 * live < 3 * (size_t)tab.f1[tab.nlive])
        if (int e = rebuild(cover)) return e;
      if (!exec || run.empty()) continue;
      PS_CUDA(cudaGraphLaunch(exec, st));
      lsm::k_cg_done_batch<<<1, lsm::kLsmBatchMax, 0, st>>>(tab, ddone);
      PS_CUDA(cudaMemcpyAsync(now.data(), ddone, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
      PS_CUDA(cudaStreamSynchronize(st));
      std::vector<int> stay, leave;
      lsm::LsmList stop{};
      for (int s : run) {
        const bool conv = now[s] > 0.0, spent = (long long)now[n + s] >= budget[s];
        if (!conv && spent) stop.s[stop.n++] = s;
        (conv || spent ? leave : stay).push_back(s);
      }
      if (stop.n) {
        lsm::k_cg_stop_batch<<<1, lsm::kLsmBatchMax, 0, st>>>(tab, stop);
        PS_CUDA(cudaGetLastError());
        PS_CUDA(cudaStreamSynchronize(st));
      }
      run.swap(stay);
      if (!leave.empty()) {
        {
          std::lock_guard<std::mutex> g(mu);
          for (int s : leave) todo.push_back(s);
          pending += (int)leave.size();
        }
        cv.notify_all();
      }
    }
  };
  const int rc = drive();
  {  // drop queued steps (none unless an error ended the loop); the
     // workers finish the steps they are running and return
    std::lock_guard<std::mutex> g(mu);
    pending -= (int)todo.size();
    todo.clear();
    quit = true;
  }
  cv.notify_all();
  for (std::thread& t : th) t.join();
  cudaStreamSynchronize(st);
  cudaFree(ddone);
  if (exec) cudaGraphExecDestroy(exec);
  if (rc) return rc;
  if (err) {
    last_error() = msg;
    return err;
  }
  return PS_OK;
}

// Calls f(k, v, dup) for the reference's nodes k = 0, 1, ... in their order:
// k-j-i over the node grid, which for a tied load has the loaded axis padded
// to planes 0..N (plane N duplicates plane 0 plus the jump, XX:446-523) and
// for PS_LOAD_NONE is the periodic box (S1:541-602).  v is the node's box
// index, dup marks a node on the duplicate plane.  A node exists when one of
// its cubes is solid; along the loaded axis there are no cubes beyond the
// ends (no wrap there).
template <typename F>
void for_ref_nodes(const Springs* S, F f)
{
  const int n3[3] = {S->nx, S->ny, S->nz};
  const int pad = S->periodic ? -1 : S->pa;
  const int M[3] = {S->nx + (pad == 0 ? 1 : 0), S->ny + (pad == 1 ? 1 : 0), S->nz};
  long long k = 0;
  for (int z = 0; z < M[2]; z++)
    for (int y = 0; y < M[1]; y++)
      for (int xx = 0; xx < M[0]; xx++) {
        const int c[3] = {xx, y, z};
        int w[3];
        for (int d = 0; d < 3; d++) w[d] = c[d] % n3[d];
        const int v = w[0] + S->nx * (w[1] + S->ny * w[2]);
        bool exists = false;
        for (int e = 0; e < 8 && !exists; e++) {
          int cc[3];
          bool ok = true;
          for (int d = 0; d < 3; d++) {
            cc[d] = c[d] - ((e >> d) & 1);
            if (d == pad) ok = ok && cc[d] >= 0 && cc[d] < n3[d];
            else cc[d] = (cc[d] + n3[d]) % n3[d];
          }
          exists = ok && S->mat[cc[0] + S->nx * (cc[1] + S->ny * cc[2])] != 0;
        }
        if (!exists) continue;
        f(k, v, pad >= 0 && c[pad] == n3[pad]);
        k++;
      }
}

// velocity, acceleration and jump-force vectors of the dynamics, allocated
// (velocity and acceleration zero) on first use
int ensure_dyn(Springs* S)
{
  if (S->dv) return PS_OK;
  const size_t b64 = sizeof(double) * 3 * (size_t)S->nvox;
  if (int r = dalloc(S, &S->dv, b64)) return r;
  if (int r = dalloc(S, &S->da, b64)) return r;
  if (int r = dalloc(S, &S->bj, b64)) return r;
  PS_CUDA(cudaMemsetAsync(S->dv, 0, b64, S->stream));
  PS_CUDA(cudaMemsetAsync(S->da, 0, b64, S->stream));
  lsm::k_lsm_rhs<<<blocks_for(S->nvox), kBlk, 0, S->stream>>>(S->geom(), S->pa, S->jc, 2.0 * S->p.gstrain, S->bj);
  PS_CUDA(cudaGetLastError());
  PS_CUDA(cudaStreamSynchronize(S->stream));
  return PS_OK;
}

}  // namespace
}  // namespace ps

using namespace ps;

extern "C" {

int ps_lsm_create(const ps_lsm_params* p, const int32_t* ind, int32_t nx, int32_t ny, int32_t nz, void** handle)
{
  if (!p || !ind || !handle) return fail(PS_ERR_ARG, "ps_lsm_create: null argument");
  *handle = nullptr;
  if (nx < 2 || ny < 2 || nz < 2) return fail(PS_ERR_ARG, "ps_lsm_create: box %d x %d x %d too small", nx, ny, nz);
  if ((long long)nx * ny * nz * 3 > (1LL << 31) - 1) return fail(PS_ERR_ARG, "ps_lsm_create: box too large");
  if (p->load != PS_LOAD_XSTRETCH && p->load != PS_LOAD_YZSHEAR && p->load != PS_LOAD_NONE)
    return fail(PS_ERR_ARG, "ps_lsm_create: bad load %d", p->load);
  if (p->load == PS_LOAD_NONE && p->gstrain != 0.0)
    return fail(PS_ERR_ARG, "ps_lsm_create: PS_LOAD_NONE imposes no strain (gstrain must be 0)");
  if (p->precision != PS_LSM_F64 && p->precision != PS_LSM_MIXED)
    return fail(PS_ERR_ARG, "ps_lsm_create: bad precision %d", p->precision);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(PS_ERR_NODEVICE, "ps_lsm_create: no CUDA device");
  std::unique_ptr<Springs, void (*)(Springs*)> S(new Springs, free_springs);
  S->p = *p;
  S->nx = nx;
  S->ny = ny;
  S->nz = nz;
  S->nvox = nx * ny * nz;
  // PS_LOAD_NONE: the x-stretch layout with a zero jump; only the node
  // order of the state calls differs (no duplicate plane)
  S->pa = p->load == PS_LOAD_YZSHEAR ? 1 : 0;
  S->jc = p->load == PS_LOAD_YZSHEAR ? 2 : 0;
  S->periodic = p->load == PS_LOAD_NONE;
  const int nv = S->nvox;
  S->mat.assign(nv, 0);
  S->node.assign(nv, 0);
  for (int v = 0; v < nv; v++) S->mat[v] = ind[v] == 0 ? 1 : (ind[v] == 3 ? 2 : 0);
  long long nn = 0, nc = 0;
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const int v = x + nx * (y + ny * z);
        if (S->mat[v]) nc++;
        bool solid = false;  // a node exists when one of its 8 cubes is solid
        for (int e = 0; e < 8 && !solid; e++) {
          const int cx = (x - (e & 1) + nx) % nx, cy = (y - ((e >> 1) & 1) + ny) % ny, cz = (z - (e >> 2) + nz) % nz;
          solid = S->mat[cx + nx * (cy + ny * cz)] != 0;
        }
        S->node[v] = solid;
        nn += solid;
      }
  S->nnode = nn;
  S->ncube = nc;
  // node classes on the device (lsm_kernels.cuh): 1 surface node, 2 / 3
  // bulk node of material 1 / 2 (its 8 cubes all of that material)
  std::vector<uint8_t> cls(S->node);
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const int v = x + nx * (y + ny * z);
        if (!cls[v]) continue;
        const int m = S->mat[v];
        bool bulk = m != 0;
        for (int e = 1; e < 8 && bulk; e++) {
          const int cx = (x - (e & 1) + nx) % nx, cy = (y - ((e >> 1) & 1) + ny) % ny, cz = (z - (e >> 2) + nz) % nz;
          bulk = S->mat[cx + nx * (cy + ny * cz)] == m;
        }
        if (bulk) cls[v] = (uint8_t)(1 + m);
      }
  std::vector<int> surf;
  for (int v = 0; v < nv; v++)
    if (cls[v] == 1) surf.push_back(v);
  S->nsurf = (int)surf.size();
  // cube matrices, per material
  static const lsm::CubeMatrices M = [] {  // built once, thread-safe
    lsm::CubeMatrices m;
    lsm::build_cube_matrices(m);
    return m;
  }();
  std::vector<double> K64(2 * 24 * 24), S64(2 * 9 * 24), Kab(2 * 24 * 24);
  for (int i = 0; i < 24; i++)
    for (int j = 0; j < 24; j++) {
      Kab[i * 24 + j] = M.Ka[i][j];
      Kab[576 + i * 24 + j] = M.Kb[i][j];
    }
  const double al[2] = {p->alf1, p->alf2}, be[2] = {p->bet1, p->bet2};
  for (int m = 0; m < 2; m++) {
    for (int i = 0; i < 24; i++)
      for (int j = 0; j < 24; j++) K64[(m * 24 + i) * 24 + j] = al[m] * M.Ka[i][j] + be[m] * M.Kb[i][j];
    for (int i = 0; i < 9; i++)
      for (int j = 0; j < 24; j++) S64[(m * 9 + i) * 24 + j] = al[m] * M.Sa[i][j] + be[m] * M.Sb[i][j];
  }
  PS_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
  S->nblk = blocks_for(3LL * nv);
  if (int r = dalloc(S.get(), &S->d_mat, nv)) return r;
  if (int r = dalloc(S.get(), &S->d_node, nv)) return r;
  PS_CUDA(cudaMemcpyAsync(S->d_mat, S->mat.data(), nv, cudaMemcpyHostToDevice, S->stream));
  PS_CUDA(cudaMemcpyAsync(S->d_node, cls.data(), nv, cudaMemcpyHostToDevice, S->stream));
  if (int r = dalloc(S.get(), &S->d_surf, sizeof(int) * std::max<size_t>(1, surf.size()))) return r;
  if (!surf.empty())
    PS_CUDA(cudaMemcpyAsync(S->d_surf, surf.data(), sizeof(int) * surf.size(), cudaMemcpyHostToDevice, S->stream));
  const size_t b64 = sizeof(double) * 3 * (size_t)nv, b32 = sizeof(float) * 3 * (size_t)nv;
  for (double** v : {&S->b, &S->x, &S->r, &S->p64, &S->q64})
    if (int r = dalloc(S.get(), v, b64)) return r;
  if (p->precision == PS_LSM_MIXED)
    for (float** v : {&S->x32, &S->r32, &S->p32, &S->q32})
      if (int r = dalloc(S.get(), v, b32)) return r;
  if (int r = dalloc(S.get(), &S->ctr, sizeof(unsigned))) return r;
  PS_CUDA(cudaMemsetAsync(S->ctr, 0, sizeof(unsigned), S->stream));
  if (int r = dalloc(S.get(), &S->part, sizeof(double) * 9 * (size_t)(S->nblk + 1))) return r;
  if (int r = dalloc(S.get(), &S->scal, sizeof(double) * 32)) return r;
  PS_CUDA(cudaMemsetAsync(S->scal, 0, sizeof(double) * 32, S->stream));
  if (int r = dalloc(S.get(), &S->d_K64, sizeof(double) * K64.size())) return r;
  if (int r = dalloc(S.get(), &S->d_S64, sizeof(double) * S64.size())) return r;
  if (int r = dalloc(S.get(), &S->d_Kab, sizeof(double) * Kab.size())) return r;
  PS_CUDA(cudaMemcpyAsync(S->d_K64, K64.data(), sizeof(double) * K64.size(), cudaMemcpyHostToDevice, S->stream));
  PS_CUDA(cudaMemcpyAsync(S->d_S64, S64.data(), sizeof(double) * S64.size(), cudaMemcpyHostToDevice, S->stream));
  PS_CUDA(cudaMemcpyAsync(S->d_Kab, Kab.data(), sizeof(double) * Kab.size(), cudaMemcpyHostToDevice, S->stream));
  PS_CUDA(cudaMemsetAsync(S->x, 0, b64, S->stream));  // the dynamic state starts at zero displacement
  PS_CUDA(cudaStreamSynchronize(S->stream));
  *handle = S.release();
  return PS_OK;
}

int ps_lsm_destroy(void* h)
{
  if (!h) return PS_OK;
  Springs* S = static_cast<Springs*>(h);
  if (S->stream) cudaStreamSynchronize(S->stream);
  free_springs(S);
  return PS_OK;
}

int ps_lsm_get_info(void* h, ps_lsm_info* o)
{
  if (!h || !o) return fail(PS_ERR_ARG, "ps_lsm_get_info: null argument");
  Springs* S = static_cast<Springs*>(h);
  memset(o, 0, sizeof *o);
  o->nnode = S->nnode;
  o->ncube = S->ncube;
  o->nvox = S->nvox;
  o->nx = S->nx;
  o->ny = S->ny;
  o->nz = S->nz;
  o->load = S->p.load;
  o->precision = S->p.precision;
  o->device_bytes = S->dev_bytes;
  return PS_OK;
}

int ps_lsm_solve(void* h, double rtol, int32_t maxit, ps_lsm_result* out)
{
  if (!h || !out) return fail(PS_ERR_ARG, "ps_lsm_solve: null argument");
  if (!(rtol > 0.0) || maxit < 1) return fail(PS_ERR_ARG, "ps_lsm_solve: need rtol > 0 and maxit >= 1");
  Springs* S = static_cast<Springs*>(h);
  memset(out, 0, sizeof *out);
  const int n3 = 3 * S->nvox;
  const int nb3 = blocks_for(n3);
  double bb = 0.0;
  if (int e = prepare(S, &bb)) return e;
  long long iters = 0, inner = 0;
  double rel = 0.0;
  int refinements = 0;
  if (S->p.precision == PS_LSM_F64) {
    PS_CUDA(cudaMemcpyAsync(S->r, S->b, sizeof(double) * n3, cudaMemcpyDeviceToDevice, S->stream));
    PS_CUDA(cudaMemcpyAsync(S->p64, S->b, sizeof(double) * n3, cudaMemcpyDeviceToDevice, S->stream));
    double rel2 = 0.0;
    if (int e = cg<double>(S, S->x, S->r, S->p64, S->q64, rtol, maxit, &iters, &rel2)) return e;
    inner = iters;
  } else {
    if (int e = mixed_ir(S, bb, rtol, maxit, out)) return e;
    iters = out->iterations;
    inner = out->inner_iterations;
    refinements = out->refinements;
  }
  out->iterations = iters;
  out->inner_iterations = inner;
  out->refinements = refinements;
  if (int e = finish(S, bb, rtol, out)) return e;
  rel = out->relres;
  return out->converged ? PS_OK : fail(PS_ERR_NOTCONV, "ps_lsm_solve: relative residual %.3e above %.3e", rel, rtol);
}

// Modulus gradients with respect to the four spring constants.  The
// stiffness is linear in each constant (K = sum over cubes of alf_m Ka +
// bet_m Kb), the converged displacement minimises the spring energy W under
// the tie, so dW/dk = 1/2 u^T (dK/dk) u at fixed u; with modulus = 2 W /
// (V strain^2) (periodic box under the imposed strain), d modulus / dk =
// u^T (dK/dk) u / (V strain^2).
int ps_lsm_gradients(void* h, double* grad)
{
  if (!h || !grad) return fail(PS_ERR_ARG, "ps_lsm_gradients: null argument");
  Springs* S = static_cast<Springs*>(h);
  if (!S->solved) return fail(PS_ERR_STATE, "ps_lsm_gradients: no solution yet");
  if (!(S->p.gstrain != 0.0)) return fail(PS_ERR_STATE, "ps_lsm_gradients: needs a nonzero imposed strain");
  const int nb = blocks_for(S->nvox);
  const double jump = 2.0 * S->p.gstrain;
  lsm::k_lsm_energy<kBlk><<<nb, kBlk, 0, S->stream>>>(S->geom(), S->pa, S->jc, jump, S->x, S->d_Kab, S->part);
  PS_CUDA(cudaGetLastError());
  std::vector<double> hp((size_t)nb * 4);
  PS_CUDA(cudaMemcpyAsync(hp.data(), S->part, sizeof(double) * 4 * nb, cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  double q[4] = {0, 0, 0, 0};  // u^T Ka u, u^T Kb u for material 1, then material 2
  for (int b = 0; b < nb; b++)
    for (int i = 0; i < 4; i++) q[i] += hp[(size_t)b * 4 + i];
  const double vcell = (double)S->nx * S->ny * S->nz;
  const double strain = jump / (S->pa == 0 ? S->nx : S->ny);
  const double den = vcell * strain * strain;
  for (int i = 0; i < 4; i++) grad[i] = q[i] / den;
  // the energy form of the modulus: 2 W / (V strain^2), W = 1/2 sum k q_k
  grad[4] = (S->p.alf1 * q[0] + S->p.bet1 * q[1] + S->p.alf2 * q[2] + S->p.bet2 * q[3]) / den;
  return PS_OK;
}

int ps_lsm_set_wall_load(void* h, void* lattice, double rsi)
{
  if (!h) return fail(PS_ERR_ARG, "ps_lsm_set_wall_load: null handle");
  Springs* S = static_cast<Springs*>(h);
  S->solved = false;
  if (!lattice) {
    S->has_load = false;
    return PS_OK;
  }
  const double* box = nullptr;
  int dims[3] = {0, 0, 0};
  if (int e = lbm_wall_load_box(lattice, rsi, &box, dims)) return e;
  if (dims[0] != S->nx || dims[1] != S->ny || dims[2] != S->nz)
    return fail(PS_ERR_ARG, "ps_lsm_set_wall_load: lattice box %dx%dx%d differs from the network's %dx%dx%d", dims[0],
                dims[1], dims[2], S->nx, S->ny, S->nz);
  const int nv = S->nvox;
  if (!S->fext)
    if (int r = dalloc(S, &S->fext, sizeof(double) * 3 * (size_t)nv)) return r;
  // the lost-corner counter lives in the scalar block (slot 24)
  unsigned long long* lost = reinterpret_cast<unsigned long long*>(S->scal + 24);
  PS_CUDA(cudaMemsetAsync(lost, 0, sizeof(unsigned long long), S->stream));
  k_take_load<<<blocks_for(nv), kBlk, 0, S->stream>>>(nv, S->d_node, box, S->fext, lost);
  PS_CUDA(cudaGetLastError());
  unsigned long long nlost = 0;
  PS_CUDA(cudaMemcpyAsync(&nlost, lost, sizeof nlost, cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  if (nlost) {
    S->has_load = false;
    return fail(PS_ERR_ARG, "ps_lsm_set_wall_load: %llu loaded corners are not nodes of the spring network", nlost);
  }
  S->has_load = true;
  return PS_OK;
}

int ps_lsm_alpha_beta(void* h, const int32_t* lab, int32_t npores, int32_t iipore, double pres, double* alpha,
                      double* beta)
{
  if (!h || !lab || !alpha || (npores > 0 && !beta)) return fail(PS_ERR_ARG, "ps_lsm_alpha_beta: null argument");
  if (npores < 0 || !(pres != 0.0)) return fail(PS_ERR_ARG, "ps_lsm_alpha_beta: need npores >= 0 and pres != 0");
  Springs* S = static_cast<Springs*>(h);
  if (!S->solved) return fail(PS_ERR_STATE, "ps_lsm_alpha_beta: no solution yet");
  const int nv = S->nvox;
  const double vcell = (double)S->nx * S->ny * S->nz;
  long long npore = 0;
  for (int v = 0; v < nv; v++) npore += lab[v] == iipore;
  const double epsi = (double)npore / vcell;
  // alpha_i = -epsi I + asigmap / vcell / pres (S1:4257)
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) alpha[3 * r + c] = (r == c ? -epsi : 0.0) + S->last.sigma[3 * r + c] / vcell / pres;
  if (npores == 0) return PS_OK;
  int32_t* d_lab = nullptr;
  PS_CUDA(cudaMallocAsync((void**)&d_lab, sizeof(int32_t) * (size_t)nv, S->stream));
  int rc = PS_OK;
  const int nb = (nv + 255) / 256;
  double* part = nullptr;
  std::vector<double> hp((size_t)nb * 32);
  cudaError_t e = cudaMallocAsync((void**)&part, sizeof(double) * hp.size(), S->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_lab, lab, sizeof(int32_t) * (size_t)nv, cudaMemcpyHostToDevice, S->stream);
  for (int p0 = 1; e == cudaSuccess && p0 <= npores; p0 += 32) {
    k_beta_surface<<<nb, 256, 0, S->stream>>>(S->geom(), d_lab, p0, S->x, part);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, S->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
    for (int q = 0; e == cudaSuccess && q < 32 && p0 + q <= npores; q++) {
      double t = 0.0;
      for (int b = 0; b < nb; b++) t += hp[(size_t)b * 32 + q];
      beta[p0 + q - 1] = t / vcell / pres;  // S1:4439
    }
  }
  if (e != cudaSuccess) rc = cuda_fail(e, "ps_lsm_alpha_beta");
  cudaFreeAsync(part, S->stream);
  cudaFreeAsync(d_lab, S->stream);
  cudaStreamSynchronize(S->stream);
  return rc;
}

int ps_lsm_batch_solve(void* const* handles, int32_t n, double rtol, int32_t maxit, ps_lsm_result* out)
{
  if (!handles || !out) return fail(PS_ERR_ARG, "ps_lsm_batch_solve: null argument");
  if (n < 1 || n > lsm::kLsmBatchMax) return fail(PS_ERR_ARG, "ps_lsm_batch_solve: %d networks (1..%d)", n, lsm::kLsmBatchMax);
  if (!(rtol > 0.0) || maxit < 1) return fail(PS_ERR_ARG, "ps_lsm_batch_solve: need rtol > 0 and maxit >= 1");
  std::vector<Springs*> sys;
  for (int s = 0; s < n; s++) {
    if (!handles[s]) return fail(PS_ERR_ARG, "ps_lsm_batch_solve: network %d is null", s);
    Springs* S = static_cast<Springs*>(handles[s]);
    for (Springs* o : sys)
      if (o == S) return fail(PS_ERR_ARG, "ps_lsm_batch_solve: network %d appears twice", s);
    if (S->p.precision != static_cast<Springs*>(handles[0])->p.precision)
      return fail(PS_ERR_ARG, "ps_lsm_batch_solve: networks differ in precision");
    sys.push_back(S);
    memset(out + s, 0, sizeof(ps_lsm_result));
  }
  std::vector<double> bb((size_t)n, 0.0);
  if (int e = each_network(n, [&](int s) { return prepare(sys[s], &bb[s]); })) return e;
  cudaStream_t st = nullptr;
  PS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = PS_OK;
  if (sys[0]->p.precision == PS_LSM_F64) {
    rc = each_network(n, [&](int s) {
      Springs* S = sys[s];
      const size_t b3 = sizeof(double) * 3 * (size_t)S->nvox;
      cudaError_t e = cudaMemcpyAsync(S->r, S->b, b3, cudaMemcpyDeviceToDevice, S->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(S->p64, S->b, b3, cudaMemcpyDeviceToDevice, S->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
      return e == cudaSuccess ? PS_OK : cuda_fail(e, "ps_lsm_batch_solve");
    });
    if (rc == PS_OK) rc = batch_cg<double>(sys, rtol, maxit, st);
    for (int s = 0; s < n && rc == PS_OK; s++) {
      double h8[8];
      if ((rc = read_scal(sys[s], h8, 8))) break;
      out[s].iterations = out[s].inner_iterations = (long long)h8[7];
    }
  } else {
    // Groups of networks whose FP32 CG vectors (x, r, p, q: 48 bytes per
    // box voxel) fit kGroupBytes together, so that a batched iteration
    // finds them in L2 between its launches; up to kBatchThreads groups run
    // at a time, each on its own host thread and stream.  A network above
    // the budget is a group of its own and runs the individual solve's
    // refinement (its launches fill the GPU by themselves); smaller ones
    // share the batched launches.
    std::vector<int> order(n);
    for (int s = 0; s < n; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sys[a]->nvox > sys[b]->nvox; });
    std::vector<std::vector<int>> grp;
    long long used = 0;
    for (int s : order) {
      const long long bytes = 48LL * sys[s]->nvox;
      if (grp.empty() || used + bytes > kGroupBytes) {
        grp.emplace_back();
        used = 0;
      }
      grp.back().push_back(s);
      used += bytes;
    }
    const int ng = (int)grp.size(), nth = std::min(ng, kBatchThreads);
    std::vector<int> grc((size_t)ng, PS_OK);
    std::vector<std::string> gmsg((size_t)ng);
    std::atomic<int> next{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto run_groups = [&]() {
      cudaSetDevice(dev);
      cudaStream_t gs = nullptr;
      if (cudaStreamCreateWithFlags(&gs, cudaStreamNonBlocking) != cudaSuccess) gs = nullptr;
      for (int g = next++; g < ng; g = next++) {
        std::sort(grp[g].begin(), grp[g].end());
        if (grp[g].size() == 1) {
          const int s = grp[g][0];
          grc[g] = mixed_ir(sys[s], bb[s], rtol, maxit, out + s);
        } else if (!gs) {
          grc[g] = fail(PS_ERR_CUDA, "ps_lsm_batch_solve: no stream for a batch");
        } else {
          std::vector<Springs*> gsys;
          std::vector<double> gbb;
          std::vector<ps_lsm_result> gout(grp[g].size());
          for (size_t i = 0; i < grp[g].size(); i++) {
            gsys.push_back(sys[grp[g][i]]);
            gbb.push_back(bb[grp[g][i]]);
            gout[i] = out[grp[g][i]];
          }
          grc[g] = batch_mixed(gsys, gbb, rtol, maxit, gout.data(), gs, 1);
          for (size_t i = 0; i < gout.size(); i++) out[grp[g][i]] = gout[i];
        }
        if (grc[g]) gmsg[g] = last_error();
      }
      if (gs) cudaStreamDestroy(gs);
    };
    std::vector<std::thread> gth;
    for (int t = 1; t < nth; t++) gth.emplace_back(run_groups);
    run_groups();
    for (std::thread& t : gth) t.join();
    for (int g = 0; g < ng && rc == PS_OK; g++)
      if (grc[g]) {
        rc = grc[g];
        last_error() = gmsg[g];
      }
  }
  cudaStreamDestroy(st);
  if (rc != PS_OK) return rc;
  if (int e = each_network(n, [&](int s) { return finish(sys[s], bb[s], rtol, out + s); })) return e;
  int bad = -1;
  for (int s = 0; s < n && bad < 0; s++)
    if (!out[s].converged) bad = s;
  return bad < 0 ? PS_OK
                 : fail(PS_ERR_NOTCONV, "ps_lsm_batch_solve: network %d at relative residual %.3e above %.3e", bad,
                        out[bad].relres, rtol);
}

int ps_lsm_get_disp(void* h, double* u)
{
  if (!h || !u) return fail(PS_ERR_ARG, "ps_lsm_get_disp: null argument");
  Springs* S = static_cast<Springs*>(h);
  if (!S->solved) return fail(PS_ERR_STATE, "ps_lsm_get_disp: no solution yet");
  const int nv = S->nvox;
  std::vector<double> x((size_t)3 * nv);
  PS_CUDA(cudaMemcpyAsync(x.data(), S->x, sizeof(double) * 3 * nv, cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  const double jump = 2.0 * S->p.gstrain;
  for_ref_nodes(S, [&](long long k, int v, bool dup) {
    for (int d = 0; d < 3; d++) u[3 * k + d] = x[(size_t)d * nv + v] + (dup && d == S->jc ? jump : 0.0);
  });
  return PS_OK;
}

int ps_lsm_set_dyn_state(void* h, const double* r, const double* v, const double* a)
{
  if (!h) return fail(PS_ERR_ARG, "ps_lsm_set_dyn_state: null handle");
  Springs* S = static_cast<Springs*>(h);
  if (int e = ensure_dyn(S)) return e;
  const int nv = S->nvox;
  double* dst[3] = {S->x, S->dv, S->da};
  const double* src[3] = {r, v, a};
  std::vector<double> box((size_t)3 * nv);
  for (int q = 0; q < 3; q++) {
    std::fill(box.begin(), box.end(), 0.0);
    if (src[q])
      for_ref_nodes(S, [&](long long k, int vv, bool dup) {
        if (dup) return;  // follows its partner
        for (int d = 0; d < 3; d++) box[(size_t)d * nv + vv] = src[q][3 * k + d];
      });
    PS_CUDA(cudaMemcpyAsync(dst[q], box.data(), sizeof(double) * box.size(), cudaMemcpyHostToDevice, S->stream));
    PS_CUDA(cudaStreamSynchronize(S->stream));
  }
  S->solved = true;
  return PS_OK;
}

int ps_lsm_get_dyn_state(void* h, double* r, double* v, double* a)
{
  if (!h) return fail(PS_ERR_ARG, "ps_lsm_get_dyn_state: null handle");
  Springs* S = static_cast<Springs*>(h);
  if (int e = ensure_dyn(S)) return e;
  const int nv = S->nvox;
  const double jump = 2.0 * S->p.gstrain;
  const double* src[3] = {S->x, S->dv, S->da};
  double* dst[3] = {r, v, a};
  std::vector<double> box((size_t)3 * nv);
  for (int q = 0; q < 3; q++) {
    if (!dst[q]) continue;
    PS_CUDA(cudaMemcpyAsync(box.data(), src[q], sizeof(double) * box.size(), cudaMemcpyDeviceToHost, S->stream));
    PS_CUDA(cudaStreamSynchronize(S->stream));
    for_ref_nodes(S, [&](long long k, int vv, bool dup) {
      for (int d = 0; d < 3; d++)
        dst[q][3 * k + d] = box[(size_t)d * nv + vv] + (q == 0 && dup && d == S->jc ? jump : 0.0);
    });
  }
  return PS_OK;
}

int ps_lsm_dyn_step(void* h, int32_t nsteps, double dt, double rsi, double damp)
{
  if (!h) return fail(PS_ERR_ARG, "ps_lsm_dyn_step: null handle");
  if (nsteps < 0 || !(dt > 0.0) || !std::isfinite(dt) || !std::isfinite(rsi) || !std::isfinite(damp))
    return fail(PS_ERR_ARG, "ps_lsm_dyn_step: need nsteps >= 0, dt > 0 and finite rsi, damp");
  Springs* S = static_cast<Springs*>(h);
  if (int e = ensure_dyn(S)) return e;
  const int nv = S->nvox, n3 = 3 * nv;
  const int nb3 = blocks_for(n3);
  const double* f = S->has_load ? S->fext : nullptr;
  const double* bj = S->p.gstrain != 0.0 ? S->bj : nullptr;
  for (int s = 0; s < nsteps; s++) {
    lsm::k_dyn_kick_drift<<<nb3, kBlk, 0, S->stream>>>(n3, dt, f, S->x, S->dv, S->da);
    if (int e = matvec64(S, S->x, S->q64)) return e;
    lsm::k_dyn_force_kick<<<nb3, kBlk, 0, S->stream>>>(n3, dt, rsi, damp, bj, S->q64, f, S->dv, S->da);
  }
  PS_CUDA(cudaGetLastError());
  PS_CUDA(cudaStreamSynchronize(S->stream));
  S->solved = true;
  return PS_OK;
}

void* ps_lsm_stream(void* h) { return h ? (void*)static_cast<Springs*>(h)->stream : nullptr; }

// Stress and modulus of a caller-supplied displacement field, computed
// without any device allocation: the per-CTA partial sums go to the
// library's static scratch array instead of memory from cudaMalloc.  Meant
// for callers that cannot allocate device memory when they re-evaluate the
// moduli: a host application whose own pool has already reserved the
// device's memory (a cudaMalloc there fails or competes with the pool), and
// a driver stepping several streams, where freeing device memory waits for
// all work on the device and would stall the other streams.  The handle must
// already exist (ps_lsm_create allocates; this call does not).
//
// The scratch array is shared by every call in the process and keeps the
// last call's partial sums; each call rewrites the slots it reads before
// reading them.  Calls that overlap on the GPU (from several host threads or
// streams) race on it and must be serialised by the caller.  Every call
// looks up the array's device address on the current device
// (cudaGetSymbolAddress, which allocates nothing), so a device reset between
// calls leaves no stale address behind.
int ps_lsm_stress_noalloc(void* h, const double* d_u, double* out)
{
  if (!h || !d_u || !out) return fail(PS_ERR_ARG, "ps_lsm_stress_noalloc: null argument");
  Springs* S = static_cast<Springs*>(h);
  if ((long long)S->nvox > PS_LSM_NOALLOC_MAX_CUBES)
    return fail(PS_ERR_ARG, "ps_lsm_stress_noalloc: %d voxel cubes exceed the no-allocation maximum of %d",
                S->nvox, PS_LSM_NOALLOC_MAX_CUBES);
  double* scratch = nullptr;
  if (int e = noalloc_scratch(&scratch)) return e;
  const int nb = blocks_for(S->nvox);
  const double jump = 2.0 * S->p.gstrain;
  lsm::k_lsm_stress<kBlk><<<nb, kBlk, 0, S->stream>>>(S->geom(), S->pa, S->jc, jump, d_u, scratch);
  PS_CUDA(cudaGetLastError());
  k_stress_final<<<1, 32, 0, S->stream>>>(scratch, nb, scratch + 9 * kNoAllocMaxBlocks);
  PS_CUDA(cudaGetLastError());
  double sig[9];
  PS_CUDA(cudaMemcpyAsync(sig, scratch + 9 * kNoAllocMaxBlocks, sizeof sig, cudaMemcpyDeviceToHost, S->stream));
  PS_CUDA(cudaStreamSynchronize(S->stream));
  const double vcell = (double)S->nx * S->ny * S->nz;
  const double nax = S->pa == 0 ? S->nx : S->ny;
  for (int i = 0; i < 9; i++) out[i] = sig[i];
  // no imposed strain (a handle that only carries a wall load): modulus 0,
  // as ps_lsm_solve reports it
  out[9] = jump != 0.0 ? (S->pa == 0 ? sig[0] : sig[5]) / (vcell * jump / nax) : 0.0;
  return PS_OK;
}

}  // extern "C"
