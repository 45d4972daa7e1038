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
//   * deviation storage keeps each population as a deviation from the rest
//     equilibrium t_d * rho_ref of its own component.  FP32: rho_ref is the
//     component density of the RECEIVING node at the step that wrote it
//     (FP32 pair rho[i] per compact node), so a reader needs only its own
//     two densities.  16-bit: rho_ref is that of the WRITING node (pairs on
//     the dense voxel box, rho[v]), so a population crossing an interface
//     carries its own non-equilibrium part, not the density jump; the
//     writer of slot d of the node at voxel v is voxel v - c_d (or v).
//
// One step = two launches over the fluid nodes:
//   k_lbm_dens  reads each node's populations, writes the colour (and for
//               deviation storage the component densities that become the
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
  int cplane;              // plane stride of the step colour field (nx*ny rounded up to 32)
  long long nvox;
  long long nl;            // fluid nodes
  long long pitch;         // elements per direction array (>= nl)
  const uint32_t* coord;   // [nl] packed coordinates
  const uint32_t* mask;    // [nl] link and face bits
  const int32_t* ref;      // [nl] reference fluid index (i outer, k inner order)
  const int32_t* rowstart; // [ny*nz + 1]
  const uint2* rowbits;    // [ny*nz*nwords] (fluid bits, fluid count before the word)
  int sort;                // step option: the collide kernel orders each CTA's nodes bulk first
};

// one population buffer: pop -> 19*pitch (red, blue) pairs, rho -> pitch
// (red, blue) FP32 densities of the nodes (deviation storage).  recv: the
// 16-bit slots hold deviations from the READING node's densities (a state
// given from outside, whose populations are consistent with each node's own
// densities); steps always write deviations from the writing node's.
struct BufDev {
  void* pop;
  float2* rho;
  int recv;
  // step number of the stochastically rounded 16-bit stores written into
  // this buffer: step, plus *stepbase when set (graph replays, whose kernel
  // arguments are fixed at capture)
  uint32_t step;
  const uint32_t* stepbase;
};

// ---- storage policies ----------------------------------------------------
template <int PREC>
struct Store;
template <>
struct Store<0> {  // FP64
  using T = double;
  using T2 = double2;
  using R = double;
  static constexpr bool kDev = false, kSendRef = false;
};
template <>
struct Store<1> {  // FP32 deviation (receiver reference)
  using T = float;
  using T2 = float2;
  using R = float;
  static constexpr bool kDev = true, kSendRef = false;
};
template <>
struct Store<2> {  // FP16 deviation (sender reference)
  using T = __half;
  using T2 = __half2;
  using R = float;
  static constexpr bool kDev = true, kSendRef = true;
};
template <>
struct Store<3> {  // BF16 deviation (sender reference)
  using T = __nv_bfloat16;
  using T2 = __nv_bfloat162;
  using R = float;
  static constexpr bool kDev = true, kSendRef = true;
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

__device__ __forceinline__ float2 to_f2(float2 h) { return h; }
__device__ __forceinline__ float2 to_f2(__half2 h) { return __half22float2(h); }
__device__ __forceinline__ float2 to_f2(__nv_bfloat162 h) { return __bfloat1622float2(h); }
template <typename T2>
__device__ __forceinline__ T2 from_f2(float a, float b);
template <>
__device__ __forceinline__ float2 from_f2<float2>(float a, float b) { return make_float2(a, b); }
template <>
__device__ __forceinline__ __half2 from_f2<__half2>(float a, float b) { return __floats2half2_rn(a, b); }
template <>
__device__ __forceinline__ __nv_bfloat162 from_f2<__nv_bfloat162>(float a, float b)
{
  return __floats2bfloat162_rn(a, b);
}

// ---- stochastic rounding of the 16-bit stores ------------------------------
// A population of a flow that is steady, or nearly so, takes the same value
// step after step, and round-to-nearest then stores it with the same error
// every step: a bias that never averages out (in a steady two-layer flow,
// round-to-nearest FP16 deviations biased the blue flux by 2e-3).  The
// collide's 16-bit stores therefore round stochastically: a uniform random
// integer below the bits the conversion drops is added to the FP32 bit
// pattern, and the sum is rounded toward zero, so a value rounds up with
// probability equal to its distance from the lower neighbour and the
// rounding error has mean zero.  Values the 16-bit format holds exactly
// (zeros included) are stored unchanged.  The random bits are a hash of
// (node, direction, step), so a state is reproducible and is the same in
// every schedule.
__device__ __forceinline__ uint32_t dither_seed(uint32_t i, uint32_t step)
{
  uint32_t h = (i * 0x9E3779B1u) ^ (step * 0x85EBCA77u + 0x165667B1u);
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return h;
}
// 32 random bits for direction e from the node's seed: the seed times an
// odd constant of its own per direction; the high half of the product
// (bits 16..31) serves the blue value, the red one takes bits 3..15 mixed
// with the seed's high bits (both 13-bit fields for FP16; BF16 takes 16)
__device__ __forceinline__ uint32_t dither_bits(uint32_t seed, int e)
{
  const uint32_t h = seed * (0x9E3779B1u + 0x7F4A7C16u * (uint32_t)e);
  return h ^ (seed >> 16);
}
__device__ __forceinline__ uint32_t step_of(const BufDev& b)
{
  return b.step + (b.stepbase ? __ldg(b.stepbase) : 0u);
}
// (a, b) to a 16-bit pair, stochastically rounded with the random bits r
template <typename T2>
__device__ __forceinline__ T2 from_f2_sr(float a, float b, uint32_t r);
// x stochastically rounded onto FP16's subnormal grid 2^-24 (|x| < 2^-14)
// with 13 random bits r; the result converts exactly
__device__ __forceinline__ float sr_f16_sub(float x, uint32_t r)
{
  const float q = x * 16777216.0f;  // x / 2^-24, exact
  const float fl = floorf(q);
  const float u = (float)r * (1.0f / 8192.0f);  // uniform in [0, 1)
  return (fl + (q - fl > u ? 1.0f : 0.0f)) * 5.9604644775390625e-08f;
}
template <>
__device__ __forceinline__ __half2 from_f2_sr<__half2>(float a, float b, uint32_t r)
{
  // FP16 keeps 10 of FP32's 23 mantissa bits: 13 random bits each, added
  // below the bits the round-toward-zero conversion drops.  Below 2^-14
  // FP16's grid is 2^-24 whatever the exponent (subnormals) and that dither
  // would cover only part of the dropped bits, pulling tiny values toward
  // zero (the minority component's populations at an interface, which
  // matter): those are rounded on the grid directly.  They are rare, so the
  // warp takes that path only when one of its lanes needs it.
  const uint32_t ra = r & 0x1FFFu, rb = (r >> 16) & 0x1FFFu;
  float ad = __uint_as_float(__float_as_uint(a) + ra);
  float bd = __uint_as_float(__float_as_uint(b) + rb);
  const bool sub = fminf(fabsf(a), fabsf(b)) < 6.103515625e-05f;
  if (__any_sync(__activemask(), sub)) {
    if (fabsf(a) < 6.103515625e-05f) ad = sr_f16_sub(a, ra);
    if (fabsf(b) < 6.103515625e-05f) bd = sr_f16_sub(b, rb);
  }
  uint32_t h;
  asm("cvt.rz.f16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(bd), "f"(ad));
  return *reinterpret_cast<__half2*>(&h);
}
template <>
__device__ __forceinline__ __nv_bfloat162 from_f2_sr<__nv_bfloat162>(float a, float b, uint32_t r)
{
  // BF16 keeps 7 mantissa bits: 16 random bits each
  const float ad = __uint_as_float(__float_as_uint(a) + (r & 0xFFFFu));
  const float bd = __uint_as_float(__float_as_uint(b) + (r >> 16));
  uint32_t h;
  asm("cvt.rz.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(bd), "f"(ad));
  return *reinterpret_cast<__nv_bfloat162*>(&h);
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
  // the stored (red, blue) deviations of slot (d, i) (deviation storage)
  __device__ __forceinline__ static void load_dev(const BufDev& b, int d, int i, long long pitch, R& gr, R& gb)
  {
    const float2 v = to_f2(*(static_cast<const T2*>(b.pop) + (long long)d * pitch + i));
    gr = v.x * DevScale<T>::down;
    gb = v.y * DevScale<T>::down;
  }
  __device__ __forceinline__ static void put_dev(const BufDev& b, int d, int i, long long pitch, R gr, R gb)
  {
    *(static_cast<T2*>(b.pop) + (long long)d * pitch + i) = from_f2<T2>(gr * DevScale<T>::up, gb * DevScale<T>::up);
  }
  // writes the (red, blue) pair (vr, vb) into slot (d, i) whose node has
  // deviation references rho; 16-bit storage rounds stochastically with the
  // random bits rnd
  __device__ __forceinline__ static void put(const LbmConst<R>& K, const BufDev& b, int d, int i, long long pitch,
                                             R vr, R vb, float2 rho, uint32_t rnd = 0u)
  {
    T2* p = static_cast<T2*>(b.pop) + (long long)d * pitch + i;
    if constexpr (S::kSendRef) {
      *p = from_f2_sr<T2>((vr - K.t[0][wcls(d)] * rho.x) * DevScale<T>::up,
                          (vb - K.t[1][wcls(d)] * rho.y) * DevScale<T>::up, rnd);
    } else if constexpr (S::kDev) {
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

// Writes the 19 post-collision (red, blue) populations of node i to their
// receivers (push streaming with half-way bounce-back).  s[] are the pull
// sources of node i (pull_sources): the receiver of an outgoing population
// e is the source of the incoming direction opp(e).  kCoh: the receivers'
// reference densities were written by other CTAs of the same launch, so
// they are read through L2 only (no non-coherent or L1 path).
template <typename T>
__device__ __forceinline__ T ld_step(const T* p, bool coherent)
{
  return coherent ? __ldcg(p) : __ldg(p);
}

template <int PREC, bool kCoh = false>
__device__ __forceinline__ void push_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& dst, int i, long long ri, uint32_t m, const int* s,
                                          const typename Store<PREC>::R* outr, const typename Store<PREC>::R* outb)
{
  constexpr bool kDev = Store<PREC>::kDev, kSend = Store<PREC>::kSendRef;
  const float2 zero = make_float2(0.f, 0.f);
  // ri: node i's entry in rho.  Sender reference: every population against
  // node i's own densities; otherwise against each receiver's.
  const float2 own = kDev ? ld_step(dst.rho + ri, kCoh) : zero;
  const uint32_t seed = kSend ? dither_seed((uint32_t)i, step_of(dst)) : 0u;
  Pop<PREC>::put(K, dst, 0, i, G.pitch, outr[0], outb[0], own, kSend ? dither_bits(seed, 0) : 0u);
#pragma unroll
  for (int e = 1; e < 19; e++) {
    const int oe = opp(e);
    const bool stream = m & (1u << (oe - 1));
    const int node = stream ? s[oe] : i;
    const int slot = stream ? e : oe;
    Pop<PREC>::put(K, dst, slot, node, G.pitch, outr[e], outb[e],
                   kDev && !kSend ? ld_step(dst.rho + node, kCoh) : own, kSend ? dither_bits(seed, e) : 0u);
  }
}

// deviation storage: node i's stored deviations and their references
template <int PREC>
__device__ __forceinline__ float2 read_node_dev(const GeomDev& G, const BufDev& src, int i, float* gr, float* gb)
{
#pragma unroll
  for (int d = 0; d < 19; d++) Pop<PREC>::load_dev(src, d, i, G.pitch, gr[d], gb[d]);
  return __ldg(src.rho + i);
}

// deviation storage: pushes out_c[d] = t^c_d S_c + Z_c[d] (node_update_dev)
// to the receivers, each as t^c_d (S_c - rho'_c) + Z_c[d] against the
// receiver's current densities rho' (rn for node i itself)
template <int PREC, bool kCoh = false>
__device__ __forceinline__ void push_node_dev(const LbmConst<float>& K, const GeomDev& G, const BufDev& dst, int i,
                                              uint32_t m, const int* s, float Sr, float Sb, const float* Zr,
                                              const float* Zb, float2 rn)
{
  Pop<PREC>::put_dev(dst, 0, i, G.pitch, K.t[0][0] * (Sr - rn.x) + Zr[0], K.t[1][0] * (Sb - rn.y) + Zb[0]);
#pragma unroll
  for (int e = 1; e < 19; e++) {
    const int oe = opp(e);
    const bool stream = m & (1u << (oe - 1));
    const int node = stream ? s[oe] : i;
    const int slot = stream ? e : oe;
    const float2 rho = stream ? ld_step(dst.rho + node, kCoh) : rn;
    const int w = wcls(e);
    Pop<PREC>::put_dev(dst, slot, node, G.pitch, K.t[0][w] * (Sr - rho.x) + Zr[e], K.t[1][w] * (Sb - rho.y) + Zb[e]);
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
__device__ __forceinline__ NbOff nb_offsets(uint32_t m, int nx, int nxy, int zs, int nz)
{
  NbOff o;
  o.x[0] = (m & (1u << (kWrapShift + 0))) ? nx - 1 : -1;
  o.x[1] = 0;
  o.x[2] = (m & (1u << (kWrapShift + 1))) ? 1 - nx : 1;
  o.y[0] = (m & (1u << (kWrapShift + 2))) ? nxy - nx : -nx;
  o.y[1] = 0;
  o.y[2] = (m & (1u << (kWrapShift + 3))) ? nx - nxy : nx;
  o.z[0] = (m & (1u << (kWrapShift + 4))) ? (nz - 1) * zs : -zs;
  o.z[1] = 0;
  o.z[2] = (m & (1u << (kWrapShift + 5))) ? (1 - nz) * zs : zs;
  return o;
}

// Sender-reference storage (16-bit): slot (d, i) was written by the node at
// x - c_d when the incoming link d is open, else (rest population,
// half-way bounce-back) by node i itself; its deviation is taken from the
// writer's densities at that step, which the writer stored in the same
// buffer's rho.  Those densities live on the dense voxel box (v = voxel of
// node i, o its neighbour offsets), so each writer is a fixed offset away.
// src.recv: every slot against node i's own densities.  f[0..18] red,
// f[19..37] blue.
template <int PREC>
__device__ __forceinline__ void read_node_s(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                            const BufDev& src, int i, uint32_t m, long long v, const NbOff& o,
                                            typename Store<PREC>::R* f)
{
  const float2* rv = src.rho + v;
  const float2 own = __ldg(rv);
  const uint32_t wm = src.recv ? 0u : m;  // links whose slot another node wrote
  Pop<PREC>::load(K, src, 0, i, G.pitch, own, f[0], f[19]);
#pragma unroll
  for (int d = 1; d < 19; d++) {
    const int off = (wm & (1u << (d - 1))) ? o.x[1 - cvx(d)] + o.y[1 - cvy(d)] + o.z[1 - cvz(d)] : 0;
    Pop<PREC>::load(K, src, d, i, G.pitch, __ldg(rv + off), f[d], f[19 + d]);
  }
}

// The (red, blue) densities of node i under sender-reference storage,
// summed on the fly (sum of the stored deviations plus sum of t_d times the
// writers' densities) without holding the 38 populations
template <int PREC>
__device__ __forceinline__ float2 densities_s(const LbmConst<float>& K, const GeomDev& G, const BufDev& src, int i,
                                              uint32_t m, long long v, const NbOff& o)
{
  using T = typename Store<PREC>::T;
  using T2 = typename Store<PREC>::T2;
  const float2* rv = src.rho + v;
  const float2 own = __ldg(rv);
  const uint32_t wm = src.recv ? 0u : m;  // links whose slot another node wrote
  const T2* p = static_cast<const T2*>(src.pop) + i;
  // the stored values summed unscaled, then scaled once (a power of two:
  // the same result as scaling each term)
  float2 g = to_f2(p[0]);
  float sr = g.x, sb = g.y, wr = K.t[0][0] * own.x, wb = K.t[1][0] * own.y;
#pragma unroll
  for (int d = 1; d < 19; d++) {
    const int off = (wm & (1u << (d - 1))) ? o.x[1 - cvx(d)] + o.y[1 - cvy(d)] + o.z[1 - cvz(d)] : 0;
    const float2 rw = __ldg(rv + off);
    g = to_f2(p[(long long)d * G.pitch]);
    sr = sr + g.x;
    sb = sb + g.y;
    wr = wr + K.t[0][wcls(d)] * rw.x;
    wb = wb + K.t[1][wcls(d)] * rw.y;
  }
  return make_float2(wr + sr * DevScale<T>::down, wb + sb * DevScale<T>::down);
}
__device__ __forceinline__ long long voxel_of(const GeomDev& G, uint32_t c)
{
  int x, y, z;
  unpack(c, x, y, z);
  return x + (long long)G.nx * (y + (long long)G.ny * z);
}
__device__ __forceinline__ NbOff box_offsets(const GeomDev& G, uint32_t m)
{
  return nb_offsets(m, G.nx, G.nx * G.ny, G.nx * G.ny, G.nz);
}

// The 19 post-streaming populations of both components of node i from its
// own slots: f[0..18] red, f[19..37] blue.
template <int PREC>
__device__ __forceinline__ void read_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& src, int i, typename Store<PREC>::R* f)
{
  if constexpr (Store<PREC>::kSendRef) {
    const uint32_t c = __ldg(G.coord + i), m = __ldg(G.mask + i);
    read_node_s<PREC>(K, G, src, i, m, voxel_of(G, c), box_offsets(G, m), f);
  } else {
    float2 rho = make_float2(0.f, 0.f);
    if constexpr (Store<PREC>::kDev) rho = __ldg(src.rho + i);
#pragma unroll
    for (int d = 0; d < 19; d++) Pop<PREC>::load(K, src, d, i, G.pitch, rho, f[d], f[19 + d]);
  }
}

// ---- step kernels ---------------------------------------------------------
// per-node bodies, shared by the single-lattice and the batched kernels

// colour (and, for deviation storage, the current densities that the
// collide step encodes against) of fluid node i for this step; returns the
// node's stencil colour, its packed coordinates in *cw and, when iface is
// given, whether both components are present (node_update's interface
// branch; a scheduling hint, node_update decides from its own densities)
template <int PREC>
__device__ __forceinline__ typename Store<PREC>::R dens_colour(const LbmConst<typename Store<PREC>::R>& K,
                                                               const GeomDev& G, const BufDev& src,
                                                               const BufDev& dst, int i, uint32_t* cw,
                                                               bool* iface = nullptr)
{
  using R = typename Store<PREC>::R;
  R rr, rb;
  const uint32_t c = __ldg(G.coord + i);
  *cw = c;
  if constexpr (Store<PREC>::kSendRef) {
    const uint32_t m = __ldg(G.mask + i);
    const long long v = voxel_of(G, c);
    const float2 r2 = densities_s<PREC>(K, G, src, i, m, v, box_offsets(G, m));
    rr = r2.x;
    rb = r2.y;
    dst.rho[v] = r2;
  } else if constexpr (Store<PREC>::kDev) {
    float gr[19], gb[19];
    const float2 ro = read_node_dev<PREC>(G, src, i, gr, gb);
    R sr = gr[0], sb = gb[0];
#pragma unroll
    for (int d = 1; d < 19; d++) {
      sr = sr + gr[d];
      sb = sb + gb[d];
    }
    rr = ro.x + sr;
    rb = ro.y + sb;
    dst.rho[i] = make_float2(rr, rb);
  } else {
    R f[38];
    read_node<PREC>(K, G, src, i, f);
    densities(f, rr, rb);
  }
  if (iface) *iface = !(rb <= K.ee) && !(rr <= K.ee);
  return stencil_colour(rr, rb, K.wet);
}

template <int PREC>
__device__ __forceinline__ void dens_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& src, const BufDev& dst, typename Store<PREC>::R* cc, int i)
{
  uint32_t c;
  const auto q = dens_colour<PREC>(K, G, src, dst, i, &c);
  int x, y, z;
  unpack(c, x, y, z);
  cc[x + G.nx * y + G.cplane * z] = q;
}

// collision, CSF force, recolouring of fluid node i (coordinates c, mask m);
// pushes the post-collision populations to their receivers.  col(a, b, e)
// returns this step's stencil colour at offset (a-1, b-1, e-1).  kCoh: the
// reference densities of this step come from other threads of the same
// launch and are read through L2 (no non-coherent path).
template <int PREC, bool kCoh, typename Col>
__device__ __forceinline__ void coll_node_c(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                            const BufDev& src, const BufDev& dst, int i, uint32_t c, uint32_t m,
                                            Col col)
{
  using R = typename Store<PREC>::R;
  int x, y, z;
  unpack(c, x, y, z);
  // FP32 storage: shifted arithmetic on the deviations.  16-bit storage:
  // full-value arithmetic (about 10% fewer instructions); its rounding of
  // the small increments is deterministic (~4e-9 on populations ~0.05), and
  // the stochastically rounded stores keep it from building up a bias (a
  // deviation-form collide with 16-bit stores measured less accurate in a
  // steady layered flow, and slower).
  if constexpr (PREC == 1) {
    float gr[19], gb[19], Zr[19], Zb[19], Sr, Sb;
    const float2 ro = read_node_dev<PREC>(G, src, i, gr, gb);
    const float2 rn = ld_step(dst.rho + i, kCoh);  // this step's densities (density pass)
    node_update_dev(K, gr, gb, ro.x, ro.y, rn.x, rn.y, col, Sr, Sb, Zr, Zb);
    int s[19];
    pull_sources(G, i, c, m, s);
    push_node_dev<PREC, kCoh>(K, G, dst, i, m, s, Sr, Sb, Zr, Zb, rn);
  } else {
    R f[38];
    long long ri = i;  // node i's entry in rho
    if constexpr (Store<PREC>::kSendRef) {
      ri = x + (long long)G.nx * (y + (long long)G.ny * z);
      read_node_s<PREC>(K, G, src, i, m, ri, box_offsets(G, m), f);
    } else {
      read_node<PREC>(K, G, src, i, f);
    }
    R rr, rb;
    densities(f, rr, rb);
    R outr[19], outb[19];
    node_update(K, f, f + 19, rr, rb, col, outr, outb);
    int s[19];
    pull_sources(G, i, c, m, s);
    push_node<PREC, kCoh>(K, G, dst, i, ri, m, s, outr, outb);
  }
}

// the same with the colour read from the dense colour field cc of the
// two-pass step.  Plain (L1-cached) loads also in the fused schedule: every
// colour plane starts on a 128-byte line, and a collide tile reads only
// planes whose density tiles have all completed, so no line it caches is
// written later in the launch.
template <int PREC, bool kCoh = false>
__device__ __forceinline__ void coll_node(const LbmConst<typename Store<PREC>::R>& K, const GeomDev& G,
                                          const BufDev& src, const BufDev& dst,
                                          const typename Store<PREC>::R* __restrict__ cc, int i)
{
  using R = typename Store<PREC>::R;
  const uint32_t c = __ldg(G.coord + i), m = __ldg(G.mask + i);
  int x, y, z;
  unpack(c, x, y, z);
  const int v = x + G.nx * y + G.cplane * z;
  const NbOff o = nb_offsets(m, G.nx, G.nx * G.ny, G.cplane, G.nz);
  auto col = [&](int a, int b, int e) -> R { return cc[v + o.x[a] + o.y[b] + o.z[e]]; };
  coll_node_c<PREC, kCoh>(K, G, src, dst, i, c, m, col);
}

// Both step kernels work on the fluid nodes [i0, i1): the whole lattice,
// or one z-slab of the wavefront schedule (slabs are contiguous ranges of
// the compact numbering, z being the slowest coordinate).
template <int PREC, int BLK>
__global__ void __launch_bounds__(BLK, (PREC == 0 ? 1024 : 2048) / BLK) k_lbm_dens(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                  const __grid_constant__ GeomDev G, const BufDev src,
                                                  const BufDev dst, typename Store<PREC>::R* __restrict__ cc,
                                                  int i0, int i1)
{
  const int i = i0 + blockIdx.x * BLK + threadIdx.x;
  if (i < i1) dens_node<PREC>(K, G, src, dst, cc, i);
}

// MINB > 0 asks the register allocator for MINB resident CTAs per SM;
// 0 keeps 640 resident threads per SM (the allocator's unconstrained
// choice for this kernel uses too many registers for that).  With G.sort
// (FP32 and 16-bit storage) a CTA first reads its nodes' current densities
// (the density pass wrote them) and collides its bulk nodes before its
// interface nodes, thread t taking the t-th node of that order, so that a
// warp runs one branch of the node update instead of both; every node's
// arithmetic is unchanged.
template <int PREC, int BLK, int MINB>
__global__ void __launch_bounds__(BLK, MINB > 0 ? MINB : 640 / BLK) k_lbm_coll(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                  const __grid_constant__ GeomDev G, const BufDev src,
                                                  const BufDev dst, const typename Store<PREC>::R* __restrict__ cc,
                                                  int i0, int i1)
{
  const int base = i0 + blockIdx.x * BLK;
  int i = base + threadIdx.x;
  if constexpr (Store<PREC>::kDev) {
    if (G.sort) {
      __shared__ int order[BLK], cnt[2];
      if (threadIdx.x == 0) cnt[0] = cnt[1] = 0;
      __syncthreads();
      if (i < i1) {
        const long long ri = Store<PREC>::kSendRef ? voxel_of(G, __ldg(G.coord + i)) : (long long)i;
        const float2 r = __ldg(dst.rho + ri);
        const bool iface = !(r.y <= K.ee) && !(r.x <= K.ee);
        if (iface) order[BLK - 1 - atomicAdd(cnt + 1, 1)] = i;
        else order[atomicAdd(cnt, 1)] = i;
      }
      __syncthreads();
      const int t = threadIdx.x;
      i = (t < cnt[0] || t >= BLK - cnt[1]) ? order[t] : i1;  // the gap: threads past the end
    }
  }
  if (i < i1) coll_node<PREC>(K, G, src, dst, cc, i);
}

// ---- batched step kernels: many lattices (subvolumes) per launch ----------
// Every lattice of a batch shares the constants K; its geometry, buffers
// and colour field come from the descriptor table passed by value (kernel
// parameter space, read through the constant cache with a CTA-uniform
// index).  The work is a list of tiles (lattice, first node) of BLK nodes;
// a persistent grid (resident CTAs x SMs) strides over it.
constexpr int kBatchMaxVolumes = 64;
struct VolDesc {
  GeomDev G;
  BufDev src, dst;
  void* cc;
};
struct VolTable {
  VolDesc v[kBatchMaxVolumes];
};

template <int PREC, int BLK>
__global__ void __launch_bounds__(BLK) k_lbm_dens_batch(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                        const __grid_constant__ VolTable T,
                                                        const int2* __restrict__ tiles, int ntiles)
{
  using R = typename Store<PREC>::R;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 tl = __ldg(tiles + t);
    const VolDesc& D = T.v[tl.x];
    const int i = tl.y + threadIdx.x;
    if (i < D.G.nl) dens_node<PREC>(K, D.G, D.src, D.dst, static_cast<R*>(D.cc), i);
  }
}

template <int PREC, int BLK, int MINB>
__global__ void __launch_bounds__(BLK, MINB > 0 ? MINB : 640 / BLK)
    k_lbm_coll_batch(const __grid_constant__ LbmConst<typename Store<PREC>::R> K, const __grid_constant__ VolTable T,
                     const int2* __restrict__ tiles, int ntiles)
{
  using R = typename Store<PREC>::R;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 tl = __ldg(tiles + t);
    const VolDesc& D = T.v[tl.x];
    const int i = tl.y + threadIdx.x;
    if (i < D.G.nl) coll_node<PREC>(K, D.G, D.src, D.dst, static_cast<const R*>(D.cc), i);
  }
}

// ---- fused step: density and collide tiles in one persistent launch -----
// The fluid nodes are cut into z-slabs; a work list holds the density tiles
// of every slab and the collide tiles of every slab, ordered so that the
// collide tiles of slab k follow the density tiles of slabs k-1, k, k+1
// (periodic).  CTA b takes items b, b + G, b + 2G, ... of the list (G the
// grid, launched cooperatively so that every CTA is resident); a density
// tile publishes its completion on its slab's counter, and a collide tile
// first waits (bounded) for the three counters it needs.  Every item waits
// only for items earlier in the list, each held by a resident CTA that has
// finished its own earlier items, so the lowest unfinished item can always
// proceed and the waits end.  The collide tiles re-read populations that the
// density tiles of the same slab read shortly before (L2 hits), and
// memory-bound density work overlaps compute-bound collide work.
struct FusedArgs {
  const int4* items;     // x = kind (0 density, 1 collide) | slab << 1, y = first node, z = end node
  int nitems;
  int nslab;
  const int* ntd;        // density tiles per slab
  unsigned int* ctr;     // [1 + s] completed density tiles of slab s (zeroed before the launch)
  int* err;              // set to 1 when a wait gave up
  unsigned spin_limit;   // polls before a wait gives up
};
constexpr unsigned kFusedSpinLimit = 1u << 22;  // default spin_limit

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <int PREC, int BLK, int MINB>
__global__ void __launch_bounds__(BLK, MINB > 0 ? MINB : 640 / BLK)
    k_lbm_fused(const __grid_constant__ LbmConst<typename Store<PREC>::R> K, const __grid_constant__ GeomDev G,
                const BufDev src, const BufDev dst, typename Store<PREC>::R* __restrict__ cc, const FusedArgs F)
{
  for (int it = blockIdx.x; it < F.nitems; it += gridDim.x) {
    const int4 w = __ldg(F.items + it);
    const int slab = w.x >> 1;
    const int i = w.y + threadIdx.x;
    if ((w.x & 1) == 0) {
      if (i < w.z) dens_node<PREC>(K, G, src, dst, cc, i);
      __threadfence();  // this tile's colours and densities before its completion count
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(F.ctr + 1 + slab, 1u);
    } else {
      if (threadIdx.x == 0) {
        bool ok = true;
        for (int d = -1; d <= 1 && ok; d++) {
          const int sl = (slab + d + F.nslab) % F.nslab;
          const unsigned target = (unsigned)__ldg(F.ntd + sl);
          unsigned n = 0;
          while (ld_acquire_u32(F.ctr + 1 + sl) < target) {
            if (++n > F.spin_limit) {
              atomicExch(F.err, 1);
              ok = false;
              break;
            }
            __nanosleep(32);
          }
        }
      }
      __syncthreads();
      if (i < w.z) coll_node<PREC, true>(K, G, src, dst, cc, i);
    }
  }
}

// ---- marching step: one persistent launch per step, warp-specialised -----
// The box is cut into items: a band of A.rows y-rows (every x) times a chunk
// of A.planes z-planes; CTA b takes items b, b + grid, ...  Inside a CTA,
// PW producer warps compute the densities and stencil colours of plane p of
// the band plus one halo row on each side (the halo rows are recomputed, so
// no CTA waits for another) into a ring of 4 colour planes in shared memory
// (non-fluid voxels hold the wetting colour), and CW consumer warps collide
// plane p-1 of the band from ring planes p-2..p.  Producers run up to two
// planes ahead of consumers; the hand-off is two mbarriers per ring slot
// (full: the producers wrote it; empty: the consumers are done with it), so
// no barrier spans the whole CTA and memory-bound density work overlaps
// compute-bound collide work.  Consumers re-read a plane's populations
// shortly after the producers read them (L2 hits), so each population comes
// from DRAM about once per step.  Every chunk starts one plane early and
// ends one late (the densities its stencils need).  Producers also write
// each plane's collide order: bulk nodes first when A.sort, so that a
// consumer warp runs one branch of the node update instead of both.  The
// per-node arithmetic is the two-pass step's (dens_colour, coll_node_c), so
// the state is identical.  Every wait is bounded (A.spin polls); one that
// gives up sets *A.err and goes on, so the launch always ends (with an
// invalid state), and every index used comes from the geometry.
struct MarchArgs {
  int rows, planes, nband, nitems;  // band height, chunk depth, bands across y, bands x chunks
  int sort;                         // collide bulk nodes before interface nodes
  unsigned spin;                    // polls before a wait gives up
  int* err;                         // set to 1 when a wait gave up
};

// dynamic shared memory of one CTA: 8 mbarriers, 4 x 2 order counters, 4
// ring planes of (rows + 2) x nx colours, 4 collide orders of rows x nx
template <typename R>
__host__ __device__ constexpr size_t march_smem_bytes(int rows, int nx)
{
  return 64 + 32 + sizeof(R) * 4 * (size_t)(rows + 2) * (size_t)nx + 2 * 4 * (size_t)rows * (size_t)nx;
}

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b)
{
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.release.cta.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(b))
               : "memory");
}
// non-blocking test of the completion of the phase of parity `parity`
__device__ __forceinline__ bool mbar_test(uint64_t* b, unsigned parity)
{
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for that phase, at most A.spin polls about 32 ns apart (2^22 polls:
// a fraction of a second), then gives up and flags the error
__device__ __forceinline__ void mbar_wait(uint64_t* b, unsigned parity, const MarchArgs& A)
{
  for (unsigned n = 0; !mbar_test(b, parity); n++) {
    if (n >= A.spin) {
      atomicExch(A.err, 1);
      return;
    }
    __nanosleep(32);
  }
}
// named barrier among the `count` threads of one role
__device__ __forceinline__ void role_sync(int id, int count)
{
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

template <int PREC, int PW, int CW>
__global__ void __launch_bounds__(32 * (PW + CW), 1)
    k_lbm_march(const __grid_constant__ LbmConst<typename Store<PREC>::R> K, const __grid_constant__ GeomDev G,
                const BufDev src, const BufDev dst, const MarchArgs A)
{
  using R = typename Store<PREC>::R;
  constexpr int NP = 32 * PW, NC = 32 * CW;
  extern __shared__ __align__(16) unsigned char march_smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(march_smem);  // [4]
  uint64_t* empty = full + 4;                                // [4]
  int* cnt = reinterpret_cast<int*>(march_smem + 64);        // [4][2] bulk / interface counters
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  R* ring = reinterpret_cast<R*>(march_smem + 96);
  const int maxb = A.rows * nx;  // band nodes of one plane, at most
  const int slab = (A.rows + 2) * nx;
  uint16_t* order = reinterpret_cast<uint16_t*>(ring + 4 * slab);  // [4][maxb]
  if (threadIdx.x == 0) {
    for (int k = 0; k < 4; k++) {
      mbar_init(full + k, NP);
      mbar_init(empty + k, NC);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool producer = threadIdx.x < NP;
  const R wet = K.wet;
  unsigned t0 = 0;  // ring sequence number of the item's first plane
  for (int item = blockIdx.x; item < A.nitems; item += gridDim.x) {
    const int band = item % A.nband, chunk = item / A.nband;
    const int y0 = band * A.rows;
    const int nr = min(A.rows, ny - y0);  // rows of this band
    const int z0 = chunk * A.planes, z1 = min(nz, z0 + A.planes);
    const int sl = (nr + 2) * nx;  // colours of a ring plane in use
    const int ylo = y0 == 0 ? ny - 1 : y0 - 1, yhi = y0 + nr == ny ? 0 : y0 + nr;
    if (producer) {
      const int tid = threadIdx.x;
      for (int p = z0 - 1; p <= z1; p++) {
        const unsigned t = t0 + (unsigned)(p - (z0 - 1));
        const int s = t & 3;
        if (t >= 4) mbar_wait(empty + s, ((t >> 2) - 1) & 1, A);  // the consumers are done with its last plane
        R* r = ring + s * slab;
        for (int k = tid; k < sl; k += NP) r[k] = wet;
        if (tid == 0) cnt[2 * s] = cnt[2 * s + 1] = 0;
        role_sync(1, NP);
        const int pz = p < 0 ? p + nz : (p >= nz ? p - nz : p);
        const int rb = ny * pz;
        const int a0 = __ldg(G.rowstart + rb + ylo), na = __ldg(G.rowstart + rb + ylo + 1) - a0;
        const int b0 = __ldg(G.rowstart + rb + y0), nb = __ldg(G.rowstart + rb + y0 + nr) - b0;
        const int c0 = __ldg(G.rowstart + rb + yhi), nc = __ldg(G.rowstart + rb + yhi + 1) - c0;
        uint16_t* ord = order + s * maxb;
        const int ntot = na + nb + nc;
        auto one = [&](int k) {
          const bool lo = k < na, hi = k >= na + nb;
          const int i = lo ? a0 + k : (hi ? c0 + (k - na - nb) : b0 + (k - na));
          uint32_t cw;
          bool iface;
          const R q = dens_colour<PREC>(K, G, src, dst, i, &cw, &iface);
          int x, y, z;
          unpack(cw, x, y, z);
          r[(lo ? 0 : (hi ? nr + 1 : y - y0 + 1)) * nx + x] = q;
          if (!lo && !hi) {
            const int j = k - na;
            if (!A.sort) ord[j] = (uint16_t)j;
            else if (iface) ord[nb - 1 - atomicAdd(cnt + 2 * s + 1, 1)] = (uint16_t)j;
            else ord[atomicAdd(cnt + 2 * s, 1)] = (uint16_t)j;
          }
        };
        // two nodes per pass, so that the loads of both are in flight together
        int k = tid;
        for (; k + NP < ntot; k += 2 * NP) {
          one(k);
          one(k + NP);
        }
        if (k < ntot) one(k);
        mbar_arrive(full + s);
      }
    } else {
      const int tid = threadIdx.x - NP;
      for (int q = z0; q < z1; q++) {
        const unsigned tq = t0 + (unsigned)(q - (z0 - 1));  // sequence number of plane q
        mbar_wait(full + ((tq + 1) & 3), ((tq + 1) >> 2) & 1, A);  // plane q+1 written (so q-1, q too)
        const int rb = ny * q;
        const int b0 = __ldg(G.rowstart + rb + y0), nq = __ldg(G.rowstart + rb + y0 + nr) - b0;
        const R *s0 = ring + ((tq - 1) & 3) * slab, *s1 = ring + (tq & 3) * slab, *s2 = ring + ((tq + 1) & 3) * slab;
        const uint16_t* ord = order + (tq & 3) * maxb;
        // a plane has a little more band nodes than colliding threads: the
        // threads that take a second node rotate from plane to plane, so the
        // ring's two planes of slack even the work out
        const int rot = (int)((tq * 97u) % (unsigned)NC);
        for (int j = tid >= rot ? tid - rot : tid - rot + NC; j < nq; j += NC) {
          // an order entry is below nq once the producers wrote this plane;
          // the check keeps a wait that gave up inside the plane's band nodes
          const int o = (int)ord[j];
          if (o >= nq) continue;
          const int i = b0 + o;
          const uint32_t c = __ldg(G.coord + i), m = __ldg(G.mask + i);
          int x, y, z;
          unpack(c, x, y, z);
          const int base = (y - y0 + 1) * nx + x;
          const int ox0 = (m & (1u << (kWrapShift + 0))) ? nx - 1 : -1;
          const int ox2 = (m & (1u << (kWrapShift + 1))) ? 1 - nx : 1;
          auto col = [&](int a, int b, int e) -> R {
            const R* pl = e == 0 ? s0 : (e == 1 ? s1 : s2);
            return pl[base + (b - 1) * nx + (a == 0 ? ox0 : (a == 1 ? 0 : ox2))];
          };
          coll_node_c<PREC, true>(K, G, src, dst, i, c, m, col);
        }
        mbar_arrive(empty + ((tq - 1) & 3));  // plane q-1 is not read again
      }
      // nor are the item's last two planes
      const unsigned tl = t0 + (unsigned)(z1 - (z0 - 1));
      mbar_arrive(empty + ((tl - 1) & 3));
      mbar_arrive(empty + (tl & 3));
    }
    t0 += (unsigned)(z1 - z0 + 2);
  }
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

// The state kernels move between the reference layout (19 consecutive
// doubles per node, nodes in reference order, so consecutive compact nodes
// are far apart) and per-node values through shared memory: each warp
// copies its 32 nodes' 152-byte blocks one block at a time with 19 lanes,
// so every global access is one contiguous block rather than 32 scattered
// 8-byte words per direction.
constexpr int kStateBlk = 128;
__device__ __forceinline__ void state_block_io(double (*sh)[kStateBlk][19], const GeomDev& G, double* fr, double* fb,
                                               bool to_global)
{
  const int lane = threadIdx.x & 31, w0 = threadIdx.x & ~31;
  for (int k = 0; k < 32; k++) {
    const int node = blockIdx.x * kStateBlk + w0 + k;
    if (node >= G.nl) break;  // warp-uniform
    const long long r = G.ref[node];
    if (lane < 19) {
      if (to_global) {
        fr[19 * r + lane] = sh[0][w0 + k][lane];
        fb[19 * r + lane] = sh[1][w0 + k][lane];
      } else {
        sh[0][w0 + k][lane] = fr[19 * r + lane];
        sh[1][w0 + k][lane] = fb[19 * r + lane];
      }
    }
  }
  __syncwarp();
}

// post-streaming populations in the reference layout fr(19,nl), fb(19,nl)
template <int PREC>
__global__ void __launch_bounds__(kStateBlk) k_lbm_get_state(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                             const __grid_constant__ GeomDev G, const BufDev src,
                                                             double* fr_out, double* fb_out)
{
  using R = typename Store<PREC>::R;
  __shared__ double sh[2][kStateBlk][19];
  double* fr = sh[0][threadIdx.x];  // this node's values, written below
  double* fb = sh[1][threadIdx.x];
  const int i = blockIdx.x * kStateBlk + threadIdx.x;
  if (i < G.nl) {
    if constexpr (Store<PREC>::kSendRef) {  // decode t_d rho_writer + g in FP64
      const uint32_t c = __ldg(G.coord + i), m = __ldg(G.mask + i);
      const long long v = voxel_of(G, c);
      const NbOff o = box_offsets(G, m);
#pragma unroll
      for (int d = 0; d < 19; d++) {
        const bool wr = !src.recv && d > 0 && (m & (1u << (d - 1)));  // written by another node
        const float2 rw = __ldg(src.rho + (wr ? v + o.x[1 - cvx(d)] + o.y[1 - cvy(d)] + o.z[1 - cvz(d)] : v));
        R gr, gb;
        Pop<PREC>::load_dev(src, d, i, G.pitch, gr, gb);
        fr[d] = (double)K.t[0][wcls(d)] * (double)rw.x + (double)gr;
        fb[d] = (double)K.t[1][wcls(d)] * (double)rw.y + (double)gb;
      }
    } else if constexpr (Store<PREC>::kDev) {  // decode t_d rho + g in FP64
      float gr[19], gb[19];
      const float2 ro = read_node_dev<PREC>(G, src, i, gr, gb);
#pragma unroll
      for (int d = 0; d < 19; d++) {
        fr[d] = (double)K.t[0][wcls(d)] * (double)ro.x + (double)gr[d];
        fb[d] = (double)K.t[1][wcls(d)] * (double)ro.y + (double)gb[d];
      }
    } else {
      R f[38];
      read_node<PREC>(K, G, src, i, f);
#pragma unroll
      for (int d = 0; d < 19; d++) {
        fr[d] = (double)f[d];
        fb[d] = (double)f[19 + d];
      }
    }
  }
  __syncwarp();
  state_block_io(sh, G, fr_out, fb_out, true);
}

// post-streaming populations fr, fb (reference layout) into the node's own
// slots; deviation storage takes the node's own densities as the reference
// (for sender-reference storage the buffer is then marked recv)
template <int PREC>
__global__ void __launch_bounds__(kStateBlk) k_lbm_set_state(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                             const __grid_constant__ GeomDev G, const BufDev dst,
                                                             const double* fr_in, const double* fb_in)
{
  using S = Store<PREC>;
  using R = typename S::R;
  __shared__ double sh[2][kStateBlk][19];
  state_block_io(sh, G, const_cast<double*>(fr_in), const_cast<double*>(fb_in), false);
  const int i = blockIdx.x * kStateBlk + threadIdx.x;
  if (i >= G.nl) return;
  const double* fr = sh[0][threadIdx.x];  // this node's values
  const double* fb = sh[1][threadIdx.x];
  if constexpr (S::kDev) {
    // the node's own densities are the reference; deviations formed in FP64
    double sr = fr[0], sb = fb[0];
    for (int d = 1; d < 19; d++) {
      sr += fr[d];
      sb += fb[d];
    }
    const float2 rho = make_float2((float)sr, (float)sb);
    dst.rho[S::kSendRef ? voxel_of(G, G.coord[i]) : (long long)i] = rho;
    for (int d = 0; d < 19; d++)
      Pop<PREC>::put_dev(dst, d, i, G.pitch, (R)(fr[d] - (double)K.t[0][wcls(d)] * (double)rho.x),
                         (R)(fb[d] - (double)K.t[1][wcls(d)] * (double)rho.y));
  } else {
    for (int d = 0; d < 19; d++)
      Pop<PREC>::put(K, dst, d, i, G.pitch, (R)fr[d], (R)fb[d], make_float2(0.f, 0.f));
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
                                                 const double* cc, double* partial)
{
  using R = typename Store<PREC>::R;
  __shared__ double red[kObsN][8];
  double acc[kObsN];
#pragma unroll
  for (int i = 0; i < kObsN; i++) acc[i] = 0.0;
  // per-node quantities in the lattice's arithmetic type (FP64 for the FP64
  // lattice, whose observables follow the reference; FP32 for the others,
  // whose populations carry no more), sums over the nodes in FP64
  using A = R;
  const LbmConst<A>& D = K;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < G.nl;
       i += (long long)gridDim.x * blockDim.x) {
    const uint32_t cw = G.coord[i], m = G.mask[i];
    A f[38];
    read_node<PREC>(K, G, src, (int)i, f);
    int x, y, z;
    unpack(cw, x, y, z);
    A rr = f[0], rb = f[19];
    for (int d = 1; d < 19; d++) {
      rr = rr + f[d];
      rb = rb + f[19 + d];
    }
    const A cf = (rr - rb) / (rr + rb);
    acc[0] += (double)rr;
    acc[1] += (double)rb;
    acc[2] += (double)(rr + rb);
    if (cf > A(0.99)) {
      acc[5] += 1.0;
      acc[3] += (double)rr;
    } else if (cf < A(-0.99)) {
      acc[6] += 1.0;
      acc[4] += (double)rb;
    }
    bool neg = false;
    for (int d = 0; d < 38; d++) neg |= f[d] < A(0);
    if (neg) acc[36] = 1.0;
    if (rr < A(0)) acc[37] += 1.0;
    if (rb < A(0)) acc[38] += 1.0;
    // raw momenta with the reference's precedence (last term scaled by dti)
    for (int k = 0; k < 2; k++) {
      const A* g = f + 19 * (1 - k);  // k = 0: blue (bmt), 1: red (rmt)
      const A dti = D.dti;
      const A jx = g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14] * dti;
      const A jy = g[3] - g[4] + g[7] + g[8] - g[9] - g[10] + g[15] - g[16] + g[17] - g[18] * dti;
      const A jz = g[5] - g[6] + g[11] + g[12] - g[13] - g[14] + g[15] + g[16] - g[17] - g[18] * dti;
      acc[30 + 3 * k] += (double)jx;
      acc[31 + 3 * k] += (double)jy;
      acc[32 + 3 * k] += (double)jz;
    }
    const int nxy = G.nx * G.ny;
    const int v = x + G.nx * y + nxy * z;
    const NbOff o = nb_offsets(m, G.nx, nxy, nxy, G.nz);
    auto ccf = [&](int a, int b, int c) -> A { return (A)cc[v + o.x[a] + o.y[b] + o.z[c]]; };
    A n[3], Fs[3];
    csf_force(D, ccf, n, Fs);
    A g[19];
    for (int d = 0; d < 19; d++) g[d] = f[d] + f[19 + d];
    const A ri = A(1) / (rr + rb);
    const int ph = rr >= rb ? 0 : 1;
    A bfi[3];
    for (int d = 0; d < 3; d++) bfi[d] = D.dt * (D.bf[ph][d] + Fs[d]) * A(0.5);
    const A jx = (g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14] + bfi[0]) * D.dti;
    const A jy = (g[3] - g[4] + g[7] + g[8] - g[9] - g[10] + g[15] - g[16] + g[17] - g[18] + bfi[1]) * D.dti;
    const A jz = (g[5] - g[6] + g[11] + g[12] - g[13] - g[14] + g[15] + g[16] - g[17] - g[18] + bfi[2]) * D.dti;
    const A jm[3] = {jx, jy, jz};
    const int q = ph == 0 ? 9 : 12, uo = ph == 0 ? 18 : 21, to = ph == 0 ? 24 : 27;
    for (int d = 0; d < 3; d++) {
      acc[q + d] += (double)jm[d];
      acc[15 + d] += (double)(jm[d] * ri);
      acc[uo + d] += (double)(jm[d] * ri);
      acc[to + d] += (double)bfi[d];
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
// index of the moving direction with velocity (cx, cy, cz)
__device__ __forceinline__ int dir_of(int cx, int cy, int cz)
{
  int r = 0;
#pragma unroll
  for (int d = 1; d < 19; d++)
    if (cvx(d) == cx && cvy(d) == cy && cvz(d) == cz) r = d;
  return r;
}

// Wall load of the fluid on the LSM corner nodes (S1:3849-3882).  Every wall
// link of a fluid node n -- outgoing direction e into the wall, so that the
// incoming link d = opp(e) is closed and slot (d, n) holds the bounced
// post-collision population e -- carries
//   floc = -2 ((f_r + f_b)(e) - ppp fq(d)) c_d rsdti2,
// split equally over the 2 LSM nodes at the ends of the wall edge (diagonal
// e, the reference's ipb2 entries) or the 4 at the corners of the wall face
// (axis e, ipb4).  Corner node v = (X, Y, Z) is the low corner of voxel v.
// Each corner gathers its contributions from the (at most 8) fluid voxels
// that share it, in the reference's accumulation order: all ipb2 entries,
// then all ipb4 entries, each by reference fluid index and then direction,
// so the FP64 sums are those of the reference.  out: [3][nvox].
template <int PREC>
__global__ void __launch_bounds__(128) k_lbm_wall_load(const __grid_constant__ LbmConst<typename Store<PREC>::R> K,
                                                       const __grid_constant__ GeomDev G, const BufDev src,
                                                       double fq1, double fq2, double ppp, double rsdti2,
                                                       double* __restrict__ out)
{
  using R = typename Store<PREC>::R;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= G.nvox) return;
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const int X = (int)(v % nx), Y = (int)((v / nx) % ny), Z = (int)(v / ((long long)nx * ny));
  int idx[8], rf[8], eo[8], n = 0;
#pragma unroll
  for (int e = 0; e < 8; e++) {  // voxel v - e has this corner at its offset e
    const int vx = (e & 1) ? (X == 0 ? nx - 1 : X - 1) : X;
    const int vy = (e & 2) ? (Y == 0 ? ny - 1 : Y - 1) : Y;
    const int vz = (e & 4) ? (Z == 0 ? nz - 1 : Z - 1) : Z;
    const RowRank r = row_rank(G, vy + ny * vz, vx);
    if (r.fx) {
      idx[n] = r.base + r.rank;
      rf[n] = __ldg(G.ref + idx[n]);
      eo[n] = e;
      n++;
    }
  }
  for (int a = 1; a < n; a++)  // by reference fluid index
    for (int b = a; b > 0 && rf[b - 1] > rf[b]; b--) {
      int t = rf[b]; rf[b] = rf[b - 1]; rf[b - 1] = t;
      t = idx[b]; idx[b] = idx[b - 1]; idx[b - 1] = t;
      t = eo[b]; eo[b] = eo[b - 1]; eo[b - 1] = t;
    }
  double acc[3] = {0.0, 0.0, 0.0};
  for (int pass = 0; pass < 2; pass++) {  // 0: edges (ipb2), 1: faces (ipb4)
    const double w = pass == 0 ? 0.5 : 0.25, fq = pass == 0 ? fq2 : fq1;
    for (int k = 0; k < n; k++) {
      const int i = idx[k];
      const uint32_t m = __ldg(G.mask + i);
      // the corner lies on the voxel's high (+1) or low (-1) side per axis
      const int sx = (eo[k] & 1) ? 1 : -1, sy = (eo[k] & 2) ? 1 : -1, sz = (eo[k] & 4) ? 1 : -1;
      int ds[3];
      if (pass == 0) {
        ds[0] = dir_of(sx, sy, 0);
        ds[1] = dir_of(sx, 0, sz);
        ds[2] = dir_of(0, sy, sz);
      } else {
        ds[0] = dir_of(sx, 0, 0);
        ds[1] = dir_of(0, sy, 0);
        ds[2] = dir_of(0, 0, sz);
      }
      for (int a = 1; a < 3; a++)
        for (int b = a; b > 0 && ds[b - 1] > ds[b]; b--) {
          const int t = ds[b]; ds[b] = ds[b - 1]; ds[b - 1] = t;
        }
      float2 rho = make_float2(0.f, 0.f);  // the bounced populations were written by node i
      if constexpr (Store<PREC>::kDev) rho = __ldg(src.rho + (Store<PREC>::kSendRef ? voxel_of(G, G.coord[i]) : (long long)i));
      for (int j = 0; j < 3; j++) {
        const int d = opp(ds[j]);  // incoming link of the bounced population
        if (m & (1u << (d - 1))) continue;
        R vr, vb;
        Pop<PREC>::load(K, src, d, i, G.pitch, rho, vr, vb);
        const double q = ((double)vr + (double)vb) - ppp * fq;
        const double c[3] = {(double)cvx(d), (double)cvy(d), (double)cvz(d)};
#pragma unroll
        for (int t = 0; t < 3; t++) acc[t] = acc[t] + ((-2.0 * q) * c[t]) * rsdti2 * w;
      }
    }
  }
  out[v] = acc[0];
  out[G.nvox + v] = acc[1];
  out[2 * G.nvox + v] = acc[2];
}

// *p = v (the step base of a graph replay)
static __global__ void k_set_u32(uint32_t* p, uint32_t v) { *p = v; }

static __global__ void k_obs_final(const double* partial, int nblocks, double* out)
{
  const int i = threadIdx.x;
  if (i >= kObsN) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; b++) s = i == 36 ? fmax(s, partial[(long long)b * kObsN + i]) : s + partial[(long long)b * kObsN + i];
  out[i] = s;
}

}  // namespace ps
