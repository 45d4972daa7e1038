// lbm_kernels.cuh -- device side of the colour-gradient D3Q19 lattice.
//
// Data layout in HBM (one lattice):
//   * fluid nodes only, numbered in ascending voxel order (x fastest, then
//     y, then z): compact index i.  A warp's 32 consecutive nodes are
//     consecutive in memory, and the fluid runs of a row stay contiguous, so
//     nearly every fetched sector is used (a dense box wastes about half of
//     each sector on the solid voxels between fluid runs);
//   * populations structure-of-arrays over directions, pop[direction][i],
//     each element the (red, blue) pair of that population (double2,
//     float2, half2 or bfloat162), double-buffered (src/dst swap every
//     step): one load or store moves both components;
//   * push layout: slot (d, i) holds the POST-STREAMING population d of node
//     i, so a node reads its 19 values from its own slots, contiguously and
//     with no neighbour lookup.  The collision writes population d of node x
//     into slot (d, x + c_d) when that link streams (the reference's ips
//     entries) or, at a wall link, into slot (opp(d), x) (half-way
//     bounce-back, the reference's ipb2 / ipb4 entries);
//   * coord[i] (x | y<<10 | z<<20) and mask[i]: bit d-1 (d = 1..18) =
//     incoming link d open (the link from x - c_d streams; by symmetry the
//     outgoing link opp(d) of x streams), bits 18..23 = node on the low/high
//     x, y, z face of the box;
//   * row tables: rowstart[row] = compact index of the first fluid voxel of
//     row (y, z), and per 32-voxel word of the row its fluid bits and the
//     fluid count before it.  The compact index of fluid voxel (x, y, z) is
//     rowstart + rank of x in its row -- one L1/L2-resident lookup per
//     neighbour row, no per-node neighbour table in HBM;
//   * cc[v]: the stencil colour of the current step on the dense box
//     (wetting colour on non-fluid voxels, written once at creation), read
//     27 times per interface node from L1/L2;
//   * 16-bit storage keeps each population as a deviation from the rest
//     equilibrium t_d * rho_ref of its own component, rho_ref being the
//     component density of the RECEIVING node at the step that wrote it
//     (FP32 pair rho[i] next to the populations): a reader needs only its
//     own two densities.
//
// One step = two launches over the fluid nodes:
//   k_lbm_dens  reads each node's populations, writes the colour (and for
//               16-bit storage the component densities that become the
//               deviation reference of the populations written this step);
//   k_lbm_coll  reads them again, collides with the 27-point colour stencil
//               and writes the post-collision populations to their
//               receivers.
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

constexpr int kWrapShift = 18;  // mask bits 18..23: x==0, x==nx-1, y==0, y==ny-1, z==0, z==nz-1
constexpr int kCoordBits = 10;  // coord packing: x, y in 10 bits, z in 12

struct GeomDev {
  int nx, ny, nz, nwords;  // box; 32-voxel words per row
  long long nvox;
  long long nl;            // fluid nodes
  long long pitch;         // elements per direction array (>= nl)
  const uint32_t* coord;   // [nl] packed coordinates
  const uint32_t* mask;    // [nl] link and face bits
  const int32_t* ref;      // [nl] reference fluid index (i outer, k inner order)
  const int32_t* rowstart; // [ny*nz + 1]
  const uint2* rowbits;    // [ny*nz*nwords] (fluid bits, fluid count before the word)
};

// one population buffer: pop -> 19*pitch (red, blue) pairs, rho -> pitch
// (red, blue) FP32 reference densities (16-bit storage only)
struct BufDev {
  void* pop;
  float2* rho;
};

// ---- storage policies ----------------------------------------------------
template <int PREC>
struct Store;
template <>
struct Store<0> {  // FP64
  using T = double;
  using T2 = double2;
  using R = double;
  static constexpr bool kDev = false;
};
template <>
struct Store<1> {  // FP32
  using T = float;
  using T2 = float2;
  using R = float;
  static constexpr bool kDev = false;
};
template <>
struct Store<2> {  // FP16 deviation
  using T = __half;
  using T2 = __half2;
  using R = float;
  static constexpr bool kDev = true;
};
template <>
struct Store<3> {  // BF16 deviation
  using T = __nv_bfloat16;
  using T2 = __nv_bfloat162;
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

__device__ __forceinline__ float2 to_f2(__half2 h) { return __half22float2(h); }
__device__ __forceinline__ float2 to_f2(__nv_bfloat162 h) { return __bfloat1622float2(h); }
template <typename T2>
__device__ __forceinline__ T2 from_f2(float a, float b);
template <>
__device__ __forceinline__ __half2 from_f2<__half2>(float a, float b) { return __floats2half2_rn(a, b); }
template <>
__device__ __forceinline__ __nv_bfloat162 from_f2<__nv_bfloat162>(float a, float b)
{
  return __floats2bfloat162_rn(a, b);
}

template <int PREC>
struct Pop {
  using S = Store<PREC>;
  using T = typename S::T;
  using T2 = typename S::T2;
  using R = typename S::R;
  // (red, blue) population d in slot (d, i); rho = the deviation references
  // of node i (unused for full-precision storage)
  __device__ __forceinline__ static void load(const LbmConst<R>& K, const BufDev& b, int d, int i, long long pitch,
                                              float2 rho, R& vr, R& vb)
  {
    const T2* p = static_cast<const T2*>(b.pop) + (long long)d * pitch + i;
    if constexpr (S::kDev) {
      const float2 v = to_f2(*p);
      vr = K.t[0][wcls(d)] * rho.x + v.x * DevScale<T>::down;
      vb = K.t[1][wcls(d)] * rho.y + v.y * DevScale<T>::down;
    } else {
      const T2 v = __ldg(p);
      vr = v.x;
      vb = v.y;
    }
  }
  // writes the (red, blue) pair (vr, vb) into slot (d, i) whose node has
  // deviation references rho
  __device__ __forceinline__ static void put(const LbmConst<R>& K, const BufDev& b, int d, int i, long long pitch,
                                             R vr, R vb, float2 rho)
  {
    T2* p = static_cast<T2*>(b.pop) + (long long)d * pitch + i;
    if constexpr (S::kDev) {
      *p = from_f2<T2>((vr - K.t[0][wcls(d)] * rho.x) * DevScale<T>::up,
                       (vb - K.t[1][wcls(d)] * rho.y) * DevScale<T>::up);
    } else {
      T2 v;
      v.x = vr;
      v.y = vb;
      *p = v;
    }
  }
};

// Compact indices of the 18 pull sources x - c_d of node i (src[0] = i).
// Entries of closed links are unspecified.  Each neighbour row needs one
// rank lookup that also serves its x-1 and x+1 voxels: the fluid voxel at
// x-1 has index rank(x) - 1, the one at x+1 has rank(x) + [x fluid].
struct RowRank {
  int base;   // rowstart of the row
  int rank;   // fluid voxels before x in the row
  int fx;     // 1 when voxel x of the row is fluid
};
__device__ __forceinline__ RowRank row_rank(const GeomDev& G, int row, int x)
{
  const uint2 w = __ldg(G.rowbits + (long long)row * G.nwords + (x >> 5));
  const int b = x & 31;
  RowRank r;
  r.base = __ldg(G.rowstart + row);
  r.rank = (int)w.y + __popc(w.x & ((1u << b) - 1u));
  r.fx = (w.x >> b) & 1u;
  return r;
}
__device__ __forceinline__ void pull_sources(const GeomDev& G, int i, uint32_t c, uint32_t m, int* src)
{
  const int x = c & ((1 << kCoordBits) - 1), y = (c >> kCoordBits) & ((1 << kCoordBits) - 1), z = c >> (2 * kCoordBits);
  const int ny = G.ny;
  const int ym = (m & (1u << (kWrapShift + 2))) ? ny - 1 : y - 1;
  const int yp = (m & (1u << (kWrapShift + 3))) ? 0 : y + 1;
  const int zm = (m & (1u << (kWrapShift + 4))) ? G.nz - 1 : z - 1;
  const int zp = (m & (1u << (kWrapShift + 5))) ? 0 : z + 1;
  const bool x0 = m & (1u << (kWrapShift + 0)), x1 = m & (1u << (kWrapShift + 1));
  // index of the voxel at x-1 / x / x+1 of a row from its rank at x
  auto at = [&](const RowRank& r, int row, int dx) -> int {
    if (dx == 0) return r.base + r.rank;
    if (dx < 0) return x0 ? __ldg(G.rowstart + row + 1) - 1 : r.base + r.rank - 1;
    return x1 ? r.base : r.base + r.rank + r.fx;
  };
  src[0] = i;
  {  // own row: x -/+ 1
    const int row = y + ny * z;
    src[1] = x0 ? __ldg(G.rowstart + row + 1) - 1 : i - 1;
    src[2] = x1 ? __ldg(G.rowstart + row) : i + 1;
  }
  {  // row (y-1, z): d = 3 (x), 7 (x-1), 8 (x+1)
    const int row = ym + ny * z;
    const RowRank r = row_rank(G, row, x);
    src[3] = at(r, row, 0);
    src[7] = at(r, row, -1);
    src[8] = at(r, row, 1);
  }
  {  // row (y+1, z): d = 4 (x), 9 (x-1), 10 (x+1)
    const int row = yp + ny * z;
    const RowRank r = row_rank(G, row, x);
    src[4] = at(r, row, 0);
    src[9] = at(r, row, -1);
    src[10] = at(r, row, 1);
  }
  {  // row (y, z-1): d = 5 (x), 11 (x-1), 12 (x+1)
    const int row = y + ny * zm;
    const RowRank r = row_rank(G, row, x);
    src[5] = at(r, row, 0);
    src[11] = at(r, row, -1);
    src[12] = at(r, row, 1);
  }
  {  // row (y, z+1): d = 6 (x), 13 (x-1), 14 (x+1)
    const int row = y + ny * zp;
    const RowRank r = row_rank(G, row, x);
    src[6] = at(r, row, 0);
    src[13] = at(r, row, -1);
    src[14] = at(r, row, 1);
  }
  {  // yz diagonals
    const RowRank a = row_rank(G, ym + ny * zm, x);
    src[15] = a.base + a.rank;
    const RowRank b = row_rank(G, yp + ny * zm, x);
    src[16] = b.base + b.rank;
    const RowRank c2 = row_rank(G, ym + ny * zp, x);
    src[17] = c2.base + c2.rank;
    const RowRank e = row_rank(G, yp + ny * zp, x);
    src[18] = e.base + e.rank;
  }
}

// The 19 post-streaming populations of both components of node i from its
// own slots: f[0..18] red, f[19..37] blue.
template <int PREC>
__device__ __forceinline__ void read_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& src, int i, typename Store<PREC>::R* f)
{
  float2 rho = make_float2(0.f, 0.f);
  if constexpr (Store<PREC>::kDev) rho = __ldg(src.rho + i);
#pragma unroll
  for (int d = 0; d < 19; d++) Pop<PREC>::load(K, src, d, i, G.pitch, rho, f[d], f[19 + d]);
}

// Writes the 19 post-collision (red, blue) populations of node i to their
// receivers (push streaming with half-way bounce-back).  s[] are the pull
// sources of node i (pull_sources): the receiver of an outgoing population
// e is the source of the incoming direction opp(e).
template <int PREC>
__device__ __forceinline__ void push_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& dst, int i, uint32_t m, const int* s,
                                          const typename Store<PREC>::R* outr, const typename Store<PREC>::R* outb)
{
  constexpr bool kDev = Store<PREC>::kDev;
  const float2 zero = make_float2(0.f, 0.f);
  Pop<PREC>::put(K, dst, 0, i, G.pitch, outr[0], outb[0], kDev ? __ldg(dst.rho + i) : zero);
#pragma unroll
  for (int e = 1; e < 19; e++) {
    const int oe = opp(e);
    const bool stream = m & (1u << (oe - 1));
    const int node = stream ? s[oe] : i;
    const int slot = stream ? e : oe;
    Pop<PREC>::put(K, dst, slot, node, G.pitch, outr[e], outb[e], kDev ? __ldg(dst.rho + node) : zero);
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

__device__ __forceinline__ void unpack(uint32_t c, int& x, int& y, int& z)
{
  x = c & ((1 << kCoordBits) - 1);
  y = (c >> kCoordBits) & ((1 << kCoordBits) - 1);
  z = c >> (2 * kCoordBits);
}

// dense-box offsets of the -1 / 0 / +1 neighbours along each axis, periodic
// wrap from the face bits of the mask (for the colour stencil)
struct NbOff {
  int x[3], y[3], z[3];
};
__device__ __forceinline__ NbOff nb_offsets(uint32_t m, int nx, int nxy, int nz)
{
  NbOff o;
  o.x[0] = (m & (1u << (kWrapShift + 0))) ? nx - 1 : -1;
  o.x[1] = 0;
  o.x[2] = (m & (1u << (kWrapShift + 1))) ? 1 - nx : 1;
  o.y[0] = (m & (1u << (kWrapShift + 2))) ? nxy - nx : -nx;
  o.y[1] = 0;
  o.y[2] = (m & (1u << (kWrapShift + 3))) ? nx - nxy : nx;
  o.z[0] = (m & (1u << (kWrapShift + 4))) ? (nz - 1) * nxy : -nxy;
  o.z[1] = 0;
  o.z[2] = (m & (1u << (kWrapShift + 5))) ? (1 - nz) * nxy : nxy;
  return o;
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
  R f[38];
  read_node<PREC>(K, G, src, i, f);
  R rr, rb;
  densities(f, rr, rb);
  int x, y, z;
  unpack(__ldg(G.coord + i), x, y, z);
  cc[x + G.nx * (y + G.ny * z)] = stencil_colour(rr, rb, K.wet);
  if constexpr (Store<PREC>::kDev) dst.rho[i] = make_float2(rr, rb);
}

// collision, CSF force, recolouring; pushes the post-collision populations
// to their receivers
// MINB > 0 asks the register allocator for MINB resident CTAs per SM;
// 0 keeps 640 resident threads per SM (the allocator's unconstrained
// choice for this kernel uses too many registers for that)
template <int PREC, int BLK, int MINB>
__global__ void __launch_bounds__(BLK, MINB > 0 ? MINB : 640 / BLK) k_lbm_coll(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                  const __grid_constant__ GeomDev G, const BufDev src,
                                                  const BufDev dst, const typename Store<PREC>::R* __restrict__ cc)
{
  using R = typename Store<PREC>::R;
  const int i = blockIdx.x * BLK + threadIdx.x;
  if (i >= G.nl) return;
  const uint32_t c = __ldg(G.coord + i), m = __ldg(G.mask + i);
  R f[38];
  read_node<PREC>(K, G, src, i, f);
  R rr, rb;
  densities(f, rr, rb);
  int x, y, z;
  unpack(c, x, y, z);
  const int nxy = G.nx * G.ny;
  const int v = x + G.nx * y + nxy * z;
  const NbOff o = nb_offsets(m, G.nx, nxy, G.nz);
  auto col = [&](int a, int b, int e) -> R { return cc[v + o.x[a] + o.y[b] + o.z[e]]; };
  R outr[19], outb[19];
  node_update(K, f, f + 19, rr, rb, col, outr, outb);
  int s[19];
  pull_sources(G, i, c, m, s);
  push_node<PREC>(K, G, dst, i, m, s, outr, outb);
}

// ---- colour/density field (observables, fields) ---------------------------
// rr, rb, cf in the reference fluid order and the FP64 stencil colour cc on
// the dense box (the wetting colour on non-fluid voxels is set by the host)
template <int PREC>
__global__ void k_lbm_fields(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                             const __grid_constant__ GeomDev G, const BufDev src, double* rr, double* rb,
                             double* cf, double* cc)
{
  using R = typename Store<PREC>::R;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nl) return;
  R f[38];
  read_node<PREC>(K, G, src, i, f);
  R a, b;
  densities(f, a, b);
  const int r = G.ref[i];
  rr[r] = (double)a;
  rb[r] = (double)b;
  const R q = (a - b) / (a + b);
  cf[r] = (double)q;
  int x, y, z;
  unpack(G.coord[i], x, y, z);
  cc[x + G.nx * (y + G.ny * z)] = (double)((q - K.wet) + K.wet);
}

// post-streaming populations in the reference layout fr(19,nl), fb(19,nl)
template <int PREC>
__global__ void k_lbm_get_state(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                const __grid_constant__ GeomDev G, const BufDev src, double* fr, double* fb)
{
  using R = typename Store<PREC>::R;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nl) return;
  R f[38];
  read_node<PREC>(K, G, src, i, f);
  const long long r = G.ref[i];
#pragma unroll
  for (int d = 0; d < 19; d++) {
    fr[19 * r + d] = (double)f[d];
    fb[19 * r + d] = (double)f[19 + d];
  }
}

// post-streaming populations fr, fb (reference layout) into the node's own
// slots; 16-bit storage takes the node's own densities as the reference
template <int PREC>
__global__ void k_lbm_set_state(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                const __grid_constant__ GeomDev G, const BufDev dst, const double* fr,
                                const double* fb)
{
  using S = Store<PREC>;
  using R = typename S::R;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nl) return;
  const long long me = G.ref[i];
  float2 rho = make_float2(0.f, 0.f);
  if constexpr (S::kDev) {
    double sr = fr[19 * me], sb = fb[19 * me];
    for (int d = 1; d < 19; d++) {
      sr += fr[19 * me + d];
      sb += fb[19 * me + d];
    }
    rho = make_float2((float)sr, (float)sb);
    dst.rho[i] = rho;
  }
  for (int d = 0; d < 19; d++) Pop<PREC>::put(K, dst, d, i, G.pitch, (R)fr[19 * me + d], (R)fb[19 * me + d], rho);
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
    const uint32_t cw = G.coord[i], m = G.mask[i];
    R fR[38];
    read_node<PREC>(K, G, src, (int)i, fR);
    int x, y, z;
    unpack(cw, x, y, z);
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
    const int nxy = G.nx * G.ny;
    const int v = x + G.nx * y + nxy * z;
    const NbOff o = nb_offsets(m, G.nx, nxy, G.nz);
    auto ccf = [&](int a, int b, int c) -> double { return cc[v + o.x[a] + o.y[b] + o.z[c]]; };
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
