// lbm_kernels.cuh -- device side of the colour-gradient D3Q19 lattice.
//
// Data layout in HBM (one lattice):
//   * dense box nx*ny*nz, voxel v = x + nx*(y + ny*z);
//   * populations structure-of-arrays pop[component][direction][v] for the
//     two components (red, blue), double-buffered (src/dst swap every step);
//   * the buffers hold POST-COLLISION populations of the previous step, so a
//     step is a pull: node x reads direction d from x - c_d, or, when that
//     link is a wall link, its own reflected population opp(d) (half-way
//     bounce-back).  This is the reference's push streaming (ips) and
//     bounce-back (ipb2, ipb4) seen from the receiving node;
//   * mask[v]: bit 31 = fluid node, bit d-1 (d = 1..18) = incoming link d
//     open (the link from x - c_d is one of the reference's ips entries),
//     bits 18..23 = node on the low/high x, y, z face of the box (periodic
//     wrap), so neighbour addresses need no division;
//   * pvox[i]: the fluid voxels in ascending voxel order -- every thread of
//     the step kernels owns one fluid node, so no lane idles on solid voxels
//     and consecutive lanes read consecutive voxels;
//   * cc[v]: the stencil colour of the current step (wetting colour on
//     non-fluid voxels, written once at creation);
//   * 16-bit storage keeps each population as a deviation from the rest
//     equilibrium t_d * rho_ref of its own component and node; rho_ref is the
//     component density of the node at the step that wrote it, stored in
//     FP32 next to the populations (rho[component][v]).
//
// One step = two launches over the fluid list:
//   k_lbm_dens  pulls the populations, writes the colour (and for 16-bit
//               storage the component densities of the new buffer);
//   k_lbm_coll  pulls again, collides with the 27-point colour stencil and
//               writes the post-collision populations.
// The colour of all 26 neighbours must be that of the same step, which is
// what separates the two launches.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "lbm_node.cuh"

namespace ps {

// D3Q19 velocities (reference `velocities19` order) and opposites
__host__ __device__ constexpr int cvx(int d)
{
  return d == 1 || d == 7 || d == 9 || d == 11 || d == 13 ? 1
         : d == 2 || d == 8 || d == 10 || d == 12 || d == 14 ? -1
                                                             : 0;
}
__host__ __device__ constexpr int cvy(int d)
{
  return d == 3 || d == 7 || d == 8 || d == 15 || d == 17 ? 1
         : d == 4 || d == 9 || d == 10 || d == 16 || d == 18 ? -1
                                                              : 0;
}
__host__ __device__ constexpr int cvz(int d)
{
  return d == 5 || d == 11 || d == 12 || d == 15 || d == 16 ? 1
         : d == 6 || d == 13 || d == 14 || d == 17 || d == 18 ? -1
                                                               : 0;
}
__host__ __device__ constexpr int opp(int d)
{
  // axis pairs (1,2) (3,4) (5,6); each diagonal quartet g..g+3 is (a, b, -b, -a)
  return d == 0 ? 0 : (d <= 6 ? (d % 2 == 1 ? d + 1 : d - 1) : (2 * (7 + 4 * ((d - 7) / 4)) + 3 - d));
}
// weight class of direction d: 0 rest, 1 axis, 2 diagonal
__host__ __device__ constexpr int wcls(int d) { return d == 0 ? 0 : (d < 7 ? 1 : 2); }

static_assert(opp(7) == 10 && opp(8) == 9 && opp(11) == 14 && opp(12) == 13, "opposites");
static_assert(opp(15) == 18 && opp(16) == 17 && opp(1) == 2 && opp(5) == 6, "opposites");

constexpr uint32_t kFluidBit = 1u << 31;
constexpr int kWrapShift = 18;  // bits 18..23: x==0, x==nx-1, y==0, y==ny-1, z==0, z==nz-1

// voxel-index offsets of the neighbours at -1, 0, +1 along each axis,
// periodic wrap taken from the mask's face bits
struct NbOff {
  int x[3], y[3], z[3];
};
__device__ __forceinline__ NbOff nb_offsets(uint32_t m, int nx, int nxy, int nz)
{
  NbOff o;
  const int ny_nx = nxy;  // nx*ny
  o.x[0] = (m & (1u << (kWrapShift + 0))) ? nx - 1 : -1;
  o.x[1] = 0;
  o.x[2] = (m & (1u << (kWrapShift + 1))) ? 1 - nx : 1;
  o.y[0] = (m & (1u << (kWrapShift + 2))) ? ny_nx - nx : -nx;
  o.y[1] = 0;
  o.y[2] = (m & (1u << (kWrapShift + 3))) ? nx - ny_nx : nx;
  o.z[0] = (m & (1u << (kWrapShift + 4))) ? (nz - 1) * ny_nx : -ny_nx;
  o.z[1] = 0;
  o.z[2] = (m & (1u << (kWrapShift + 5))) ? (1 - nz) * ny_nx : ny_nx;
  return o;
}

struct GeomDev {
  int nx, ny, nz;
  long long nvox;
  const uint32_t* mask;
  const int32_t* fid;   // voxel -> fluid index (0-based, reference order) or -1
  const int32_t* fvox;  // fluid index -> voxel (reference order)
  const int32_t* pvox;  // fluid voxels in ascending voxel order (processing order)
  long long nl;
};

// one population buffer: pop[k] -> 19*nvox elements, rho[k] -> nvox floats
struct BufDev {
  void* pop[2];
  float* rho[2];
};

// ---- storage policies ----------------------------------------------------
template <int PREC>
struct Store;
template <>
struct Store<0> {  // FP64
  using T = double;
  using R = double;
  static constexpr bool kDev = false;
};
template <>
struct Store<1> {  // FP32
  using T = float;
  using R = float;
  static constexpr bool kDev = false;
};
template <>
struct Store<2> {  // FP16 deviation
  using T = __half;
  using R = float;
  static constexpr bool kDev = true;
};
template <>
struct Store<3> {  // BF16 deviation
  using T = __nv_bfloat16;
  using R = float;
  static constexpr bool kDev = true;
};

// FP16 deviations are stored scaled by 2^10 to keep them in the normal range
template <typename T>
struct DevScale {
  static constexpr float up = 1.0f, down = 1.0f;
};
template <>
struct DevScale<__half> {
  static constexpr float up = 1024.0f, down = 1.0f / 1024.0f;
};

__device__ __forceinline__ float to_f(__half h) { return __half2float(h); }
__device__ __forceinline__ float to_f(__nv_bfloat16 h) { return __bfloat162float(h); }
template <typename T>
__device__ __forceinline__ T from_f(float v);
template <>
__device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

template <int PREC>
struct Pop {
  using S = Store<PREC>;
  using T = typename S::T;
  using R = typename S::R;
  // population d of component k stored at voxel v
  __device__ __forceinline__ static R load(const LbmConst<R>& K, const BufDev& b, int k, int d, long long v,
                                           long long nvox)
  {
    const T* p = static_cast<const T*>(b.pop[k]);
    if constexpr (S::kDev) {
      const float w = K.t[k][wcls(d)];
      return w * __ldg(b.rho[k] + v) + to_f(p[(long long)d * nvox + v]) * DevScale<T>::down;
    } else {
      return __ldg(p + (long long)d * nvox + v);
    }
  }
  // writes the 19 populations of component k at voxel v; rho = density
  // the collision used for that component (the deviation reference, which
  // the density kernel of the same step stored in b.rho[k][v])
  __device__ __forceinline__ static void store(const LbmConst<R>& K, const BufDev& b, int k, long long v,
                                               long long nvox, const R* out, R rho)
  {
    T* p = static_cast<T*>(b.pop[k]);
    if constexpr (S::kDev) {
#pragma unroll
      for (int d = 0; d < 19; d++) {
        const float w = K.t[k][wcls(d)];
        p[(long long)d * nvox + v] = from_f<T>((out[d] - w * rho) * DevScale<T>::up);
      }
    } else {
#pragma unroll
      for (int d = 0; d < 19; d++) p[(long long)d * nvox + v] = out[d];
    }
  }
};

// wrapped neighbour coordinates: idx 0 = c-1, 1 = c, 2 = c+1
__device__ __forceinline__ void nb3(int c, int n, int* o)
{
  o[0] = c == 0 ? n - 1 : c - 1;
  o[1] = c;
  o[2] = c == n - 1 ? 0 : c + 1;
}

// Pulls the 19 post-streaming populations of both components at voxel
// (x,y,z), returns them in f[0..18] (red) and f[19..37] (blue).
template <int PREC>
__device__ __forceinline__ void pull_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& src, int x, int y, int z, uint32_t m,
                                          typename Store<PREC>::R* f)
{
  int xs[3], ys[3], zs[3];
  nb3(x, G.nx, xs);
  nb3(y, G.ny, ys);
  nb3(z, G.nz, zs);
  const long long nxl = G.nx, nxy = (long long)G.nx * G.ny;
  const long long v = x + nxl * y + nxy * z;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    f[19 * k] = Pop<PREC>::load(K, src, k, 0, v, G.nvox);
#pragma unroll
    for (int d = 1; d < 19; d++) {
      long long vs;
      int ds;
      if (m & (1u << (d - 1))) {  // streamed from x - c_d
        vs = xs[1 - cvx(d)] + nxl * ys[1 - cvy(d)] + nxy * zs[1 - cvz(d)];
        ds = d;
      } else {  // reflected at the wall: own population of the opposite direction
        vs = v;
        ds = opp(d);
      }
      f[19 * k + d] = Pop<PREC>::load(K, src, k, ds, vs, G.nvox);
    }
  }
}

// Pull by voxel index and mask only (32-bit addressing): the step kernels'
// form of pull_node.
template <int PREC>
__device__ __forceinline__ void pull_fast(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& src, int v, uint32_t m, const NbOff& o,
                                          typename Store<PREC>::R* f)
{
  const long long nv = G.nvox;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    f[19 * k] = Pop<PREC>::load(K, src, k, 0, v, nv);
#pragma unroll
    for (int d = 1; d < 19; d++) {
      const bool open = m & (1u << (d - 1));
      const int vs = open ? v + o.x[1 - cvx(d)] + o.y[1 - cvy(d)] + o.z[1 - cvz(d)] : v;
      const int ds = open ? d : opp(d);
      f[19 * k + d] = Pop<PREC>::load(K, src, k, ds, vs, nv);
    }
  }
}

template <typename R>
__device__ __forceinline__ void densities(const R* f, R& rr, R& rb)
{
  R a = f[0], b = f[19];
#pragma unroll
  for (int d = 1; d < 19; d++) {
    a = a + f[d];
    b = b + f[19 + d];
  }
  rr = a;
  rb = b;
}

// stencil colour of a fluid node: the reference forms ind*(cf-wet)+wet
template <typename R>
__device__ __forceinline__ R stencil_colour(R rr, R rb, R wet)
{
  const R cf = (rr - rb) / (rr + rb);
  return (cf - wet) + wet;
}

// ---- step kernels ---------------------------------------------------------
// colour (and 16-bit reference densities) of the current step
template <int PREC, int BLK>
__global__ void __launch_bounds__(BLK) k_lbm_dens(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                  const __grid_constant__ GeomDev G, const BufDev src,
                                                  const BufDev dst, typename Store<PREC>::R* __restrict__ cc)
{
  using R = typename Store<PREC>::R;
  const int i = blockIdx.x * BLK + threadIdx.x;
  if (i >= G.nl) return;
  const int v = __ldg(G.pvox + i);
  const uint32_t m = __ldg(G.mask + v);
  const NbOff o = nb_offsets(m, G.nx, G.nx * G.ny, G.nz);
  R f[38];
  pull_fast<PREC>(K, G, src, v, m, o, f);
  R rr, rb;
  densities(f, rr, rb);
  cc[v] = stencil_colour(rr, rb, K.wet);
  if constexpr (Store<PREC>::kDev) {
    dst.rho[0][v] = rr;
    dst.rho[1][v] = rb;
  }
}

// collision, CSF force, recolouring; writes the post-collision populations
template <int PREC, int BLK>
__global__ void __launch_bounds__(BLK) k_lbm_coll(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                  const __grid_constant__ GeomDev G, const BufDev src,
                                                  const BufDev dst, const typename Store<PREC>::R* __restrict__ cc)
{
  using R = typename Store<PREC>::R;
  const int i = blockIdx.x * BLK + threadIdx.x;
  if (i >= G.nl) return;
  const int v = __ldg(G.pvox + i);
  const uint32_t m = __ldg(G.mask + v);
  const NbOff o = nb_offsets(m, G.nx, G.nx * G.ny, G.nz);
  R f[38];
  pull_fast<PREC>(K, G, src, v, m, o, f);
  R rr, rb;
  densities(f, rr, rb);
  auto col = [&](int a, int b, int c) -> R { return cc[v + o.x[a] + o.y[b] + o.z[c]]; };
  R outr[19], outb[19];
  node_update(K, f, f + 19, rr, rb, col, outr, outb);
  Pop<PREC>::store(K, dst, 0, v, G.nvox, outr, rr);
  Pop<PREC>::store(K, dst, 1, v, G.nvox, outb, rb);
}

// ---- colour/density field (observables, fields) ---------------------------
// rr, rb (FP64) and the stencil colour cc (FP64, wetting colour for
// non-fluid voxels) of the current state, dense.
template <int PREC>
__global__ void k_lbm_fields(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                             const __grid_constant__ GeomDev G, const BufDev src, double* rr, double* rb,
                             double* cf, double* cc)
{
  using R = typename Store<PREC>::R;
  const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= G.nvox) return;
  const uint32_t m = G.mask[v];
  if (!(m & kFluidBit)) {
    cc[v] = (double)K.wet;
    return;
  }
  const int x = (int)(v % G.nx), y = (int)((v / G.nx) % G.ny), z = (int)(v / ((long long)G.nx * G.ny));
  R f[38];
  pull_node<PREC>(K, G, src, x, y, z, m, f);
  R a, b;
  densities(f, a, b);
  rr[v] = (double)a;
  rb[v] = (double)b;
  const R c = (a - b) / (a + b);
  cf[v] = (double)c;
  cc[v] = (double)((c - K.wet) + K.wet);
}

// post-streaming populations in the reference layout fr(19,nl), fb(19,nl)
template <int PREC>
__global__ void k_lbm_get_state(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                const __grid_constant__ GeomDev G, const BufDev src, double* fr, double* fb)
{
  using R = typename Store<PREC>::R;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= G.nl) return;
  const long long v = G.fvox[i];
  const int x = (int)(v % G.nx), y = (int)((v / G.nx) % G.ny), z = (int)(v / ((long long)G.nx * G.ny));
  R f[38];
  pull_node<PREC>(K, G, src, x, y, z, G.mask[v], f);
#pragma unroll
  for (int d = 0; d < 19; d++) {
    fr[19 * i + d] = (double)f[d];
    fb[19 * i + d] = (double)f[19 + d];
  }
}

// Inverse of the pull: given post-streaming populations fr, fb (reference
// layout), writes the pre-pull buffer so that pull_node reproduces them.
// Population d at voxel y goes to the node it streams to (y + c_d), or, if
// that link is a wall link, it is the reflection of y's own population
// opp(d).
template <int PREC>
__global__ void k_lbm_set_state(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                const __grid_constant__ GeomDev G, const BufDev dst, const double* fr,
                                const double* fb)
{
  using S = Store<PREC>;
  using R = typename S::R;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= G.nl) return;
  const long long v = G.fvox[i];
  const int x = (int)(v % G.nx), y = (int)((v / G.nx) % G.ny), z = (int)(v / ((long long)G.nx * G.ny));
  int xs[3], ys[3], zs[3];
  nb3(x, G.nx, xs);
  nb3(y, G.ny, ys);
  nb3(z, G.nz, zs);
  const long long nxl = G.nx, nxy = (long long)G.nx * G.ny;
  const double* fk[2] = {fr, fb};
#pragma unroll
  for (int k = 0; k < 2; k++) {
    R out[19];
    R rho = R(0);
    out[0] = (R)fk[k][19 * i];
    for (int d = 1; d < 19; d++) {
      const long long vt = xs[1 + cvx(d)] + nxl * ys[1 + cvy(d)] + nxy * zs[1 + cvz(d)];
      const uint32_t mt = G.mask[vt];
      const bool open = (mt & kFluidBit) && (mt & (1u << (d - 1)));
      double val;
      if (open)
        val = fk[k][19 * (long long)G.fid[vt] + d];
      else
        val = fk[k][19 * i + opp(d)];
      out[d] = (R)val;
    }
    if constexpr (S::kDev) {
      double s = fk[k][19 * i];
      for (int d = 1; d < 19; d++) s += fk[k][19 * i + d];
      rho = (R)s;
      dst.rho[k][v] = rho;
    }
    Pop<PREC>::store(K, dst, k, v, G.nvox, out, rho);
  }
}

// ---- check_state reductions -------------------------------------------------
constexpr int kObsN = 40;  // per-block partial sums
// 0 tmr 1 tmb 2 tm 3 Cpr 4 Cpb 5 nr_cf 6 nb_cf 7 nr 8 nb 9-11 Qr 12-14 Qb
// 15-17 um 18-20 umr 21-23 umb 24-26 tfr 27-29 tfb 30-32 bmt 33-35 rmt
// 36 isneg 37 nneg_rr 38 nneg_rb 39 unused
template <int PREC>
__global__ void __launch_bounds__(256) k_lbm_obs(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                 const __grid_constant__ GeomDev G, const BufDev src,
                                                 const double* cc, const LbmConst<double>* Kd, double* partial)
{
  using R = typename Store<PREC>::R;
  __shared__ double red[kObsN][8];
  double acc[kObsN];
#pragma unroll
  for (int i = 0; i < kObsN; i++) acc[i] = 0.0;
  const LbmConst<double>& D = *Kd;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < G.nl;
       i += (long long)gridDim.x * blockDim.x) {
    const long long v = G.fvox[i];
    const int x = (int)(v % G.nx), y = (int)((v / G.nx) % G.ny), z = (int)(v / ((long long)G.nx * G.ny));
    R fR[38];
    pull_node<PREC>(K, G, src, x, y, z, G.mask[v], fR);
    double f[38];
#pragma unroll
    for (int d = 0; d < 38; d++) f[d] = (double)fR[d];
    double rr = f[0], rb = f[19];
    for (int d = 1; d < 19; d++) {
      rr = rr + f[d];
      rb = rb + f[19 + d];
    }
    const double cf = (rr - rb) / (rr + rb);
    acc[0] += rr;
    acc[1] += rb;
    acc[2] += rr + rb;
    if (cf > 0.99) {
      acc[5] += 1.0;
      acc[3] += rr;
    } else if (cf < -0.99) {
      acc[6] += 1.0;
      acc[4] += rb;
    }
    bool neg = false;
    for (int d = 0; d < 38; d++) neg |= f[d] < 0.0;
    if (neg) acc[36] = 1.0;
    if (rr < 0.0) acc[37] += 1.0;
    if (rb < 0.0) acc[38] += 1.0;
    // raw momenta with the reference's precedence (last term scaled by dti)
    for (int k = 0; k < 2; k++) {
      const double* g = f + 19 * (1 - k);  // k = 0: blue (bmt), 1: red (rmt)
      const double dti = D.dti;
      double jx = g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14] * dti;
      double jy = g[3] - g[4] + g[7] + g[8] - g[9] - g[10] + g[15] - g[16] + g[17] - g[18] * dti;
      double jz = g[5] - g[6] + g[11] + g[12] - g[13] - g[14] + g[15] + g[16] - g[17] - g[18] * dti;
      acc[30 + 3 * k] += jx;
      acc[31 + 3 * k] += jy;
      acc[32 + 3 * k] += jz;
    }
    int xs[3], ys[3], zs[3];
    nb3(x, G.nx, xs);
    nb3(y, G.ny, ys);
    nb3(z, G.nz, zs);
    const long long nxl = G.nx, nxy = (long long)G.nx * G.ny;
    auto ccf = [&](int a, int b, int c) -> double { return cc[xs[a] + nxl * ys[b] + nxy * zs[c]]; };
    double n[3], Fs[3];
    csf_force(D, ccf, n, Fs);
    double g[19];
    for (int d = 0; d < 19; d++) g[d] = f[d] + f[19 + d];
    const double ri = 1.0 / (rr + rb);
    const int ph = rr >= rb ? 0 : 1;
    double bfi[3];
    for (int d = 0; d < 3; d++) bfi[d] = D.dt * (D.bf[ph][d] + Fs[d]) * 0.5;
    const double jx = (g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14] + bfi[0]) * D.dti;
    const double jy = (g[3] - g[4] + g[7] + g[8] - g[9] - g[10] + g[15] - g[16] + g[17] - g[18] + bfi[1]) * D.dti;
    const double jz = (g[5] - g[6] + g[11] + g[12] - g[13] - g[14] + g[15] + g[16] - g[17] - g[18] + bfi[2]) * D.dti;
    const double jm[3] = {jx, jy, jz};
    const int q = ph == 0 ? 9 : 12, uo = ph == 0 ? 18 : 21, to = ph == 0 ? 24 : 27;
    for (int d = 0; d < 3; d++) {
      acc[q + d] += jm[d];
      acc[15 + d] += jm[d] * ri;
      acc[uo + d] += jm[d] * ri;
      acc[to + d] += bfi[d];
    }
    acc[ph == 0 ? 7 : 8] += 1.0;
  }
  // block reduction: warp shuffles, then 8 warps through shared memory
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kObsN; i++) {
    double s = acc[i];
    if (i == 36) {
      for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    } else {
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) red[i][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x < kObsN) {
    const int i = threadIdx.x;
    double s = red[i][0];
    for (int w = 1; w < 8; w++) s = i == 36 ? fmax(s, red[i][w]) : s + red[i][w];
    partial[(long long)blockIdx.x * kObsN + i] = s;
  }
}

// fixed-order sum of the per-block partials (deterministic)
static __global__ void k_obs_final(const double* partial, int nblocks, double* out)
{
  const int i = threadIdx.x;
  if (i >= kObsN) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; b++) s = i == 36 ? fmax(s, partial[(long long)b * kObsN + i]) : s + partial[(long long)b * kObsN + i];
  out[i] = s;
}

}  // namespace ps
