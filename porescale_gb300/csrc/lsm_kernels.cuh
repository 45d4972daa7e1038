// lsm_kernels.cuh -- device side of the lattice-spring static solve.
//
// Layout in HBM: the unique solid nodes live on the nx*ny*nz node box (the
// reference's duplicate node plane N+1 of the loaded axis is the box's plane
// 0 plus the displacement jump), displacement components as three planes
// u[c*nvox + v] (structure of arrays), v = x + nx*(y + ny*z).  mat[v] is the
// material of the voxel cube whose low corner is node v (0 pore, 1 or 2).
// The stiffness operator is applied matrix-free: each node gathers the
// rows of its corner from the (at most 8) solid cubes around it; nodes
// outside the solid return 0.  Nothing is scattered, so the product is
// deterministic and needs no atomics.
//
// node[v] classifies the node: 0 no node, 1 a node on a pore surface or a
// material interface, 2 / 3 a bulk node (all 8 cubes of material 1 / 2).
// A bulk node's row is the fixed 27-point stencil alpha kBulkKa + beta
// kBulkKb, applied to the neighbours' differences from the node in +-d
// pairs (about 100 operations); the other nodes take the per-cube gather
// (about 650 in FP32).  The two kinds run as two kernels: one over the
// node box for the bulk nodes (and the zero rows of non-nodes), one over
// the list of surface nodes (surf[], in node order), so that the costly
// path runs on full warps and the cheap one at its own occupancy.
#pragma once
#include <stdint.h>

#include "lsm_cube_const.h"

namespace ps {
namespace lsm {

struct LsmGeom {
  int nx, ny, nz, nvox;
  const uint8_t* mat;   // cube material per voxel (0 pore)
  const uint8_t* node;  // 1 where the node exists
  const double* K64;    // per-material cube stiffness [2][24][24] (FP64 matvec)
  const double* S64;    // per-material cube stress rows [2][9][24]
  float alf[2], bet[2];  // spring constants of the two materials (FP32 matvec)
  double alfd[2], betd[2];  // the same in FP64 (FP64 bulk stencil)
  const int* surf;  // the surface nodes (class 1) in node order
  int nsurf;
};

// the bulk stencil's properties that bulk_node relies on: the block of
// offset d equals that of -d, every row sums to zero (a rigid translation
// feels no force) and the node's own block is diagonal, so that row r of
// K p is sum over the 13 pairs of S_d (p_{v+d} + p_{v-d} - 2 p_v), or
// S_own p_v + sum over the pairs of S_d (p_{v+d} + p_{v-d})
constexpr bool bulk_stencil_ok()
{
  for (int d = 0; d < 27; d++)
    for (int j = 0; j < 9; j++)
      if (kBulkKa[d][j] != kBulkKa[26 - d][j] || kBulkKb[d][j] != kBulkKb[26 - d][j]) return false;
  for (int j = 0; j < 9; j++) {
    double a = 0.0, b = 0.0;
    for (int d = 0; d < 27; d++) {
      a += kBulkKa[d][j];
      b += kBulkKb[d][j];
    }
    if (a != 0.0 || b != 0.0) return false;
    if (j % 4 != 0 && (kBulkKa[13][j] != 0.0 || kBulkKb[13][j] != 0.0)) return false;  // diagonal own block
  }
  return true;
}
static_assert(bulk_stencil_ok(), "bulk stencil: symmetric in d, zero row sums, diagonal own block");

// the generated cube matrices in device-readable form; every read below
// has indices fixed by full unrolling, so it folds to a literal and the
// zero entries drop out
__device__ const double kKa[24][24] = {
#define PS_ROW(i) {kCubeKa[i][0], kCubeKa[i][1], kCubeKa[i][2], kCubeKa[i][3], kCubeKa[i][4], kCubeKa[i][5], \
    kCubeKa[i][6], kCubeKa[i][7], kCubeKa[i][8], kCubeKa[i][9], kCubeKa[i][10], kCubeKa[i][11], kCubeKa[i][12], \
    kCubeKa[i][13], kCubeKa[i][14], kCubeKa[i][15], kCubeKa[i][16], kCubeKa[i][17], kCubeKa[i][18], kCubeKa[i][19], \
    kCubeKa[i][20], kCubeKa[i][21], kCubeKa[i][22], kCubeKa[i][23]}
    PS_ROW(0), PS_ROW(1), PS_ROW(2), PS_ROW(3), PS_ROW(4), PS_ROW(5), PS_ROW(6), PS_ROW(7),
    PS_ROW(8), PS_ROW(9), PS_ROW(10), PS_ROW(11), PS_ROW(12), PS_ROW(13), PS_ROW(14), PS_ROW(15),
    PS_ROW(16), PS_ROW(17), PS_ROW(18), PS_ROW(19), PS_ROW(20), PS_ROW(21), PS_ROW(22), PS_ROW(23)
#undef PS_ROW
};
__device__ const double kKb[24][24] = {
#define PS_ROW(i) {kCubeKb[i][0], kCubeKb[i][1], kCubeKb[i][2], kCubeKb[i][3], kCubeKb[i][4], kCubeKb[i][5], \
    kCubeKb[i][6], kCubeKb[i][7], kCubeKb[i][8], kCubeKb[i][9], kCubeKb[i][10], kCubeKb[i][11], kCubeKb[i][12], \
    kCubeKb[i][13], kCubeKb[i][14], kCubeKb[i][15], kCubeKb[i][16], kCubeKb[i][17], kCubeKb[i][18], kCubeKb[i][19], \
    kCubeKb[i][20], kCubeKb[i][21], kCubeKb[i][22], kCubeKb[i][23]}
    PS_ROW(0), PS_ROW(1), PS_ROW(2), PS_ROW(3), PS_ROW(4), PS_ROW(5), PS_ROW(6), PS_ROW(7),
    PS_ROW(8), PS_ROW(9), PS_ROW(10), PS_ROW(11), PS_ROW(12), PS_ROW(13), PS_ROW(14), PS_ROW(15),
    PS_ROW(16), PS_ROW(17), PS_ROW(18), PS_ROW(19), PS_ROW(20), PS_ROW(21), PS_ROW(22), PS_ROW(23)
#undef PS_ROW
};

// the bulk stencil in device-readable form (indices fixed by unrolling, as above)
#define PS_ROW(t, d) {t[d][0], t[d][1], t[d][2], t[d][3], t[d][4], t[d][5], t[d][6], t[d][7], t[d][8]}
#define PS_TAB(t) {PS_ROW(t, 0), PS_ROW(t, 1), PS_ROW(t, 2), PS_ROW(t, 3), PS_ROW(t, 4), PS_ROW(t, 5), \
    PS_ROW(t, 6), PS_ROW(t, 7), PS_ROW(t, 8), PS_ROW(t, 9), PS_ROW(t, 10), PS_ROW(t, 11), PS_ROW(t, 12), \
    PS_ROW(t, 13), PS_ROW(t, 14), PS_ROW(t, 15), PS_ROW(t, 16), PS_ROW(t, 17), PS_ROW(t, 18), PS_ROW(t, 19), \
    PS_ROW(t, 20), PS_ROW(t, 21), PS_ROW(t, 22), PS_ROW(t, 23), PS_ROW(t, 24), PS_ROW(t, 25), PS_ROW(t, 26)}
__device__ const double kBKa[27][9] = PS_TAB(kBulkKa);
__device__ const double kBKb[27][9] = PS_TAB(kBulkKb);
#undef PS_TAB
#undef PS_ROW

// entry (r, c) of the handle's FP64 cube stiffness of material index m
__device__ __forceinline__ double kval(const LsmGeom& G, int m, int r, int c)
{
  return __ldg(G.K64 + (m * 24 + r) * 24 + c);
}

__device__ __forceinline__ int wrap_add(int c, int d, int n) { return c + d < 0 ? c + d + n : (c + d >= n ? c + d - n : c + d); }

// (A p) at node v, written to q; returns p_v . (A p)_v in FP64.  p is
// read through the read-only path (__ldg; q never aliases it), which the
// batched kernels, whose vectors come from a table, need as much as the
// single ones.
template <typename T>
__device__ __forceinline__ double matvec_node(const LsmGeom& G, const T* __restrict__ p, T* __restrict__ q, int v)
{
  double pq = 0.0;
  {
    const int nx = G.nx, ny = G.ny, nz = G.nz, nv = G.nvox;
    const int x = v % nx, y = (v / nx) % ny, z = v / (nx * ny);
    T acc[3] = {T(0), T(0), T(0)};
    if (__ldg(G.node + v)) {
      const int xs[3] = {wrap_add(x, -1, nx), x, wrap_add(x, 1, nx)};
      const int ys[3] = {wrap_add(y, -1, ny), y, wrap_add(y, 1, ny)};
      const int zs[3] = {wrap_add(z, -1, nz), z, wrap_add(z, 1, nz)};
#pragma unroll
      for (int e = 0; e < 8; e++) {  // cube with low corner at node - e; this node is its corner e
        const int ex = e & 1, ey = (e >> 1) & 1, ez = e >> 2;
        const int cv = xs[1 - ex] + nx * (ys[1 - ey] + ny * zs[1 - ez]);
        const int m = __ldg(G.mat + cv);
        if (m == 0) continue;
        if constexpr (sizeof(T) == 4) {
          // FP32: K = alf Ka + bet Kb with Ka, Kb literal (zeros skipped)
          T ta[3] = {T(0), T(0), T(0)}, tb[3] = {T(0), T(0), T(0)};
#pragma unroll
          for (int b = 0; b < 8; b++) {
            if (b == (e ^ 7)) continue;  // no spring couples opposite corners
            const int bx = b & 1, by = (b >> 1) & 1, bz = b >> 2;
            const int nvb = xs[1 - ex + bx] + nx * (ys[1 - ey + by] + ny * zs[1 - ez + bz]);
            const T u[3] = {__ldg(p + nvb), __ldg(p + nv + nvb), __ldg(p + 2 * nv + nvb)};
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
              for (int c = 0; c < 3; c++) {
                const T ka = (T)kKa[3 * e + r][3 * b + c], kb = (T)kKb[3 * e + r][3 * b + c];
                if (ka != T(0)) ta[r] += ka * u[c];
                if (kb != T(0)) tb[r] += kb * u[c];
              }
          }
          const T al = m == 1 ? G.alf[0] : G.alf[1], be = m == 1 ? G.bet[0] : G.bet[1];
#pragma unroll
          for (int r = 0; r < 3; r++) acc[r] += al * ta[r] + be * tb[r];
        } else {
#pragma unroll
          for (int b = 0; b < 8; b++) {
            if (b == (e ^ 7)) continue;  // no spring couples opposite corners
            const int bx = b & 1, by = (b >> 1) & 1, bz = b >> 2;
            const int nvb = xs[1 - ex + bx] + nx * (ys[1 - ey + by] + ny * zs[1 - ez + bz]);
            const T u[3] = {__ldg(p + nvb), __ldg(p + nv + nvb), __ldg(p + 2 * nv + nvb)};
            // FP64: the handle's K of material m; entries zero in both Ka
            // and Kb (known at compile time) are skipped
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
              for (int c = 0; c < 3; c++)
                if (kKa[3 * e + r][3 * b + c] != 0.0 || kKb[3 * e + r][3 * b + c] != 0.0)
                  acc[r] += kval(G, m - 1, 3 * e + r, 3 * b + c) * u[c];
          }
        }
      }
      // the node's p.(Ap) in T (FP32: one conversion instead of three FP64
      // products on GB300's small FP64 pipe); sums across nodes stay FP64
      pq = (double)(__ldg(p + v) * acc[0] + __ldg(p + nv + v) * acc[1] + __ldg(p + 2 * nv + v) * acc[2]);
    }
    q[v] = acc[0];
    q[nv + v] = acc[1];
    q[2 * nv + v] = acc[2];
  }
  return pq;
}
// (A p) at a bulk node v of material index mi (0, 1), written to q; returns
// p_v . (A p)_v.  Every node of the 26 around v exists (its cubes are solid).
template <typename T>
__device__ __forceinline__ double bulk_node(const LsmGeom& G, const T* __restrict__ p, T* __restrict__ q, int v, int x,
                                            int y, int z, int mi)
{
  const int nx = G.nx, ny = G.ny, nz = G.nz, nv = G.nvox;
  const int xs[3] = {wrap_add(x, -1, nx), x, wrap_add(x, 1, nx)};
  const int ys[3] = {wrap_add(y, -1, ny), y, wrap_add(y, 1, ny)};
  const int zs[3] = {wrap_add(z, -1, nz), z, wrap_add(z, 1, nz)};
  T al, be;
  if constexpr (sizeof(T) == 4) {
    al = mi ? G.alf[1] : G.alf[0];
    be = mi ? G.bet[1] : G.bet[0];
  } else {
    al = mi ? G.alfd[1] : G.alfd[0];
    be = mi ? G.betd[1] : G.betd[0];
  }
  const T u0[3] = {__ldg(p + v), __ldg(p + nv + v), __ldg(p + 2 * nv + v)};
  T acc[3] = {T(0), T(0), T(0)};
  // FP64 (bound by GB300's FP64 pipe): the pairs' sums p_{v+d} + p_{v-d}
  // and the node's own diagonal block, whose entries are -2 x the pairs'
  // diagonal entries (off its diagonal the pairs' entries cancel), one
  // operation per pair and component fewer; FP32 keeps the differences
  // from the node, which cancel nothing large
  constexpr bool kSums = sizeof(T) == 8;
  if constexpr (kSums) {
#pragma unroll
    for (int r = 0; r < 3; r++) acc[r] = (al * T(kBKa[13][4 * r]) + be * T(kBKb[13][4 * r])) * u0[r];
  }
#pragma unroll
  for (int d = 0; d < 13; d++) {  // offset d and its mirror 26 - d
    const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
    bool used[3] = {false, false, false};
#pragma unroll
    for (int j = 0; j < 9; j++)
      if (kBKa[d][j] != 0.0 || kBKb[d][j] != 0.0) used[j % 3] = true;
    if (!(used[0] || used[1] || used[2])) continue;
    const int vp = xs[1 + dx] + nx * (ys[1 + dy] + ny * zs[1 + dz]);
    const int vm = xs[1 - dx] + nx * (ys[1 - dy] + ny * zs[1 - dz]);
    T s[3];
#pragma unroll
    for (int c = 0; c < 3; c++)
      if (used[c]) {
        s[c] = __ldg(p + c * nv + vp) + __ldg(p + c * nv + vm);
        if constexpr (!kSums) s[c] -= T(2) * u0[c];
      }
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double ka = kBKa[d][3 * r + c], kb = kBKb[d][3 * r + c];
        if (ka == 0.0 && kb == 0.0) continue;
        T k;
        if (ka == 0.0) k = be * T(kb);
        else if (kb == 0.0) k = al * T(ka);
        else k = al * T(ka) + be * T(kb);
        acc[r] += k * s[c];
      }
  }
  q[v] = acc[0];
  q[nv + v] = acc[1];
  q[2 * nv + v] = acc[2];
  return (double)(u0[0] * acc[0] + u0[1] * acc[1] + u0[2] * acc[2]);
}

// q = A p on the bulk nodes and the non-nodes among the kMvPer * BLK nodes
// from v0 on (one CTA; surface nodes are left to mv_surf_tile); returns
// this thread's part of p.q.  The node coordinates advance by BLK nodes
// per pass without a division.
constexpr int kMvPer = 4;  // nodes per thread and bulk tile
constexpr int kSfPer = 1;  // surface nodes per thread and surface tile
template <typename T, int BLK>
__device__ __forceinline__ double mv_bulk_tile(const LsmGeom& G, const T* __restrict__ p, T* __restrict__ q, int v0)
{
  const int nv = G.nvox, nx = G.nx, ny = G.ny, v1 = min(v0 + kMvPer * BLK, nv);
  double pq = 0.0;
  int v = v0 + (int)threadIdx.x;
  int x = v % nx, y = (v / nx) % ny, z = v / (nx * ny);
  const int ax = BLK % nx, ay = BLK / nx;
#pragma unroll 1
  for (; v < v1; v += BLK) {
    const int cls = __ldg(G.node + v);
    if (cls >= 2) {
      pq += bulk_node<T>(G, p, q, v, x, y, z, cls - 2);
    } else if (cls == 0) {
      q[v] = T(0);
      q[nv + v] = T(0);
      q[2 * nv + v] = T(0);
    }
    x += ax;
    y += ay;
    if (x >= nx) {
      x -= nx;
      y++;
    }
    while (y >= ny) {
      y -= ny;
      z++;
    }
  }
  return pq;
}
// q = A p on the surface nodes surf[i0 .. i0 + kSfPer * BLK)
template <typename T, int BLK>
__device__ __forceinline__ double mv_surf_tile(const LsmGeom& G, const T* __restrict__ p, T* __restrict__ q, int i0)
{
  const int i1 = min(i0 + kSfPer * BLK, G.nsurf);
  double pq = 0.0;
#pragma unroll 1
  for (int i = i0 + (int)threadIdx.x; i < i1; i += BLK) pq += matvec_node<T>(G, p, q, __ldg(G.surf + i));
  return pq;
}

// CG direction update p' = r + beta p (one expression for every caller)
template <typename T>
__device__ __forceinline__ T next_dir(T r, T beta, T p)
{
  return r + beta * p;
}

// FP64 sum of one value per thread over the CTA, stored by thread 0 to *out
template <int BLK>
__device__ __forceinline__ void block_sum_to(double t, double* out)
{
  __shared__ double red[BLK / 32];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < BLK / 32; w++) s += red[w];
    *out = s;
  }
}

// q = A p: k_lsm_matvec over the bulk tiles, then k_lsm_matvec_surf over
// the surface tiles, each with the FP64 partial sums of p.q per CTA in
// dot[blockIdx].  T = storage / arithmetic type of p and q.
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_lsm_matvec(const LsmGeom G, const T* __restrict__ p, T* __restrict__ q,
                                                    double* __restrict__ dot)
{
  const double pq = mv_bulk_tile<T, BLK>(G, p, q, blockIdx.x * kMvPer * BLK);
  block_sum_to<BLK>(pq, dot + blockIdx.x);
}
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK, sizeof(T) == 4 ? 4 : 2) k_lsm_matvec_surf(const LsmGeom G, const T* __restrict__ p,
                                                         T* __restrict__ q, double* __restrict__ dot)
{
  const double pq = mv_surf_tile<T, BLK>(G, p, q, blockIdx.x * kSfPer * BLK);
  block_sum_to<BLK>(pq, dot + blockIdx.x);
}

// b = -sum over cubes of K * (jump of the cube's corners): the right-hand
// side of the tied system.  Cubes whose low corner is on the last plane of
// the loaded axis see their far corners across the tie, shifted by `jump`
// in displacement component jc.
__global__ void k_lsm_rhs(const LsmGeom G, int pa, int jc, double jump, double* __restrict__ b)
{
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= G.nvox) return;
  const int nx = G.nx, ny = G.ny, nz = G.nz, nv = G.nvox;
  const int c3[3] = {v % nx, (v / nx) % ny, v / (nx * ny)};
  const int n3[3] = {nx, ny, nz};
  double acc[3] = {0.0, 0.0, 0.0};
  if (G.node[v]) {
    for (int e = 0; e < 8; e++) {
      const int ee[3] = {e & 1, (e >> 1) & 1, e >> 2};
      int cc[3];
      for (int d = 0; d < 3; d++) cc[d] = wrap_add(c3[d], -ee[d], n3[d]);
      const int m = G.mat[cc[0] + nx * (cc[1] + ny * cc[2])];
      if (m == 0 || cc[pa] != n3[pa] - 1) continue;
      // corners b with bit pa set sit across the tie
      for (int b = 0; b < 8; b++) {
        if (!((b >> pa) & 1)) continue;
        for (int r = 0; r < 3; r++) acc[r] -= kval(G, m - 1, 3 * e + r, 3 * b + jc) * jump;
      }
    }
  }
  b[v] = acc[0];
  b[nv + v] = acc[1];
  b[2 * nv + v] = acc[2];
}

// per-block FP64 sums of sigma+ (9 components) over solid cubes at the
// displacement u (+ the jump across the tie); the strain contribution is
// not needed for the moduli
template <int BLK>
__global__ void __launch_bounds__(BLK) k_lsm_stress(const LsmGeom G, int pa, int jc, double jump,
                                                    const double* __restrict__ u, double* __restrict__ part)
{
  const int v = blockIdx.x * BLK + threadIdx.x;
  double s[9];
  for (int i = 0; i < 9; i++) s[i] = 0.0;
  if (v < G.nvox) {
    const int m = G.mat[v];
    if (m) {
      const int nx = G.nx, ny = G.ny, nz = G.nz, nv = G.nvox;
      const int c3[3] = {v % nx, (v / nx) % ny, v / (nx * ny)};
      const int n3[3] = {nx, ny, nz};
      double ul[24];
      for (int b = 0; b < 8; b++) {
        const int bb[3] = {b & 1, (b >> 1) & 1, b >> 2};
        int w[3];
        for (int d = 0; d < 3; d++) w[d] = wrap_add(c3[d], bb[d], n3[d]);
        const int nb = w[0] + nx * (w[1] + ny * w[2]);
        for (int d = 0; d < 3; d++) ul[3 * b + d] = u[d * nv + nb];
        if (bb[pa] && c3[pa] == n3[pa] - 1) ul[3 * b + jc] += jump;
      }
      for (int r = 0; r < 9; r++) {
        double a = 0.0;
        for (int c = 0; c < 24; c++) a += __ldg(G.S64 + ((m - 1) * 9 + r) * 24 + c) * ul[c];
        s[r] = a;
      }
    }
  }
  __shared__ double red[9][BLK / 32];
  for (int i = 0; i < 9; i++) {
    double t = s[i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[i][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 9) {
    double t = 0.0;
    for (int w = 0; w < BLK / 32; w++) t += red[threadIdx.x][w];
    part[(long long)blockIdx.x * 9 + threadIdx.x] = t;
  }
}

// per-block FP64 sums of the quadratic forms u_c^T Ka u_c and u_c^T Kb u_c
// of every solid cube (24 corner displacements u_c with the jump across the
// tie), by material: part[4 b + 2 (m - 1) + {0: Ka, 1: Kb}].  Kab holds the
// material-independent cube matrices Ka then Kb ([2][24][24]).
template <int BLK>
__global__ void __launch_bounds__(BLK) k_lsm_energy(const LsmGeom G, int pa, int jc, double jump,
                                                    const double* __restrict__ u, const double* __restrict__ Kab,
                                                    double* __restrict__ part)
{
  const int v = blockIdx.x * BLK + threadIdx.x;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  if (v < G.nvox) {
    const int m = G.mat[v];
    if (m) {
      const int nx = G.nx, ny = G.ny, nz = G.nz, nv = G.nvox;
      const int c3[3] = {v % nx, (v / nx) % ny, v / (nx * ny)};
      const int n3[3] = {nx, ny, nz};
      double ul[24];
      for (int b = 0; b < 8; b++) {
        const int bb[3] = {b & 1, (b >> 1) & 1, b >> 2};
        int w[3];
        for (int d = 0; d < 3; d++) w[d] = wrap_add(c3[d], bb[d], n3[d]);
        const int nb = w[0] + nx * (w[1] + ny * w[2]);
        for (int d = 0; d < 3; d++) ul[3 * b + d] = u[d * nv + nb];
        if (bb[pa] && c3[pa] == n3[pa] - 1) ul[3 * b + jc] += jump;
      }
      double ea = 0.0, eb = 0.0;
      for (int r = 0; r < 24; r++) {
        double ar = 0.0, br = 0.0;
        for (int c = 0; c < 24; c++) {
          ar += __ldg(Kab + r * 24 + c) * ul[c];
          br += __ldg(Kab + 576 + r * 24 + c) * ul[c];
        }
        ea += ul[r] * ar;
        eb += ul[r] * br;
      }
      s[2 * (m - 1)] = ea;
      s[2 * (m - 1) + 1] = eb;
    }
  }
  __shared__ double red[4][BLK / 32];
  for (int i = 0; i < 4; i++) {
    double t = s[i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[i][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int w = 0; w < BLK / 32; w++) t += red[threadIdx.x][w];
    part[(long long)blockIdx.x * 4 + threadIdx.x] = t;
  }
}

// ---- damped spring dynamics (lsm_step, S1:1721-1903) ------------------------
// One velocity-Verlet step is three launches: k_dyn_kick_drift, the FP64
// matvec q = K u (k_lsm_matvec), k_dyn_force_kick.  u, v, a: displacement,
// velocity, acceleration [3][nvox]; f: the fluid wall load afdat (already
// an acceleration) or null; bj: the spring forces of the imposed jump alone
// (k_lsm_rhs) or null, so that the spring force at u is bj - K u.
// Expressions keep the reference's order: v + a dt/2 + f dt/2.
__global__ void k_dyn_kick_drift(int n3, double dt, const double* __restrict__ f, double* __restrict__ u,
                                 double* __restrict__ v, const double* __restrict__ a)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  double vi = v[i] + a[i] * dt * 0.5;
  if (f) vi = vi + f[i] * dt * 0.5;
  v[i] = vi;
  u[i] = u[i] + vi * dt;
}
__global__ void k_dyn_force_kick(int n3, double dt, double rsi, double damp, const double* __restrict__ bj,
                                 const double* __restrict__ q, const double* __restrict__ f,
                                 double* __restrict__ v, double* __restrict__ a)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  const double F = bj ? bj[i] - q[i] : -q[i];  // spring force at u
  const double vi = v[i];
  const double ai = F * rsi - damp * vi;       // acceleration, then the viscous term (S1:1888)
  a[i] = ai;
  double vn = vi + ai * dt * 0.5;
  if (f) vn = vn + f[i] * dt * 0.5;
  v[i] = vn;
}

// ---- CG vector kernels (device-resident scalars, no host round trips) ----
// scal[]: 0 rr, 1 pq, 2 alpha, 3 beta, 4 rr_new, 5 bb (|b|^2), 6 done flag
__global__ void k_sum(const double* __restrict__ part, int n, double* __restrict__ out)
{
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) t += red[w];
    *out = t;
  }
}

// per-block partial sums of |r|^2
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_sq_norm_t(int n3, const T* __restrict__ r, double* __restrict__ part)
{
  const int i = blockIdx.x * BLK + threadIdx.x;
  double t = i < n3 ? (double)r[i] * (double)r[i] : 0.0;
  __shared__ double red[BLK / 32];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < BLK / 32; w++) s += red[w];
    part[blockIdx.x] = s;
  }
}

// Sum over all ncta CTAs of a launch of one FP64 value per thread: each CTA
// stores its partial in part[slot] and counts itself in *ctr; the CTA that
// counts last adds the partials part[0 .. nblk) in index order (the same
// order every time; slots below those of this launch hold partials of an
// earlier launch), resets *ctr for the next launch and returns true in its
// thread 0 with the sum in *total.  No CTA waits for another.
template <int BLK>
__device__ __forceinline__ bool grid_sum_last(double t, double* part, int slot, unsigned* ctr, int ncta, int nblk,
                                              double* total)
{
  __shared__ double red[BLK / 32];
  __shared__ int last;
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < BLK / 32; w++) s += red[w];
    part[slot] = s;
    __threadfence();
    last = atomicAdd(ctr, 1u) == (unsigned)(ncta - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double a = 0.0;
  int i = threadIdx.x;
  for (; i + 3 * BLK < nblk; i += 4 * BLK) {  // four independent loads in flight
    const double a0 = __ldcg(part + i), a1 = __ldcg(part + i + BLK), a2 = __ldcg(part + i + 2 * BLK),
                 a3 = __ldcg(part + i + 3 * BLK);
    a += a0;
    a += a1;
    a += a2;
    a += a3;
  }
  for (; i < nblk; i += BLK) a += __ldcg(part + i);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x != 0) return false;
  double s = 0.0;
  for (int w = 0; w < BLK / 32; w++) s += red[w];
  *total = s;
  *ctr = 0u;
  return true;
}

// alpha = rr / pq, or the stop flag (|r|^2 <= tol2 |b|^2, or pq <= 0);
// scal[7] counts the iterations taken
__device__ __forceinline__ void cg_alpha_fin(double* scal, double pq, double tol2)
{
  const double rr = scal[0];
  const bool done = rr <= tol2 * scal[5] || !(pq > 0.0);
  scal[1] = pq;
  scal[6] = done ? 1.0 : 0.0;
  scal[2] = done ? 0.0 : rr / pq;
  if (!done) scal[7] += 1.0;
}
// beta = rr_new / rr; rr = rr_new
__device__ __forceinline__ void cg_beta_fin(double* scal, double rn)
{
  const double ro = scal[0];
  scal[4] = rn;
  scal[3] = !(ro > 0.0) ? 0.0 : rn / ro;
  scal[0] = rn;
}

// One CG iteration is four launches: k_cg_mv and k_cg_mv_surf (q = A p on
// the bulk and the surface nodes, p.q over both grids, the surface
// kernel's last CTA sets alpha or the stop flag), k_cg_xr (x and r along p,
// |r|^2 over the grid, its last CTA sets beta) and k_cg_p (p = r + beta p).
// A converged system (scal[6] set) returns at once, so replayed iterations
// past convergence change nothing.  (Forming p on the fly inside the matvec
// would save the last launch but repeats the update for every neighbour
// read; the matvec is arithmetic-bound, so that is slower.)
// Each CTA covers one tile of kMvPer / kSfPer nodes or kVecPer elements per
// thread (threads striding by BLK): few CTAs, so few partials and counter
// updates per reduction.  The batched kernels use the same tiles, so a
// network sums in the same order either way.
constexpr int kVecPer = 8;  // elements per thread (node tiles: kMvPer)

template <typename T, int BLK>
__device__ __forceinline__ double cg_xr_tile(int n3, T al, T* __restrict__ x, T* __restrict__ r,
                                             const T* __restrict__ p, const T* __restrict__ q, int i0)
{
  // every load of the thread's kVecPer elements before the first store (the
  // batched kernels' vectors come from a table, with no restrict for the
  // compiler to reorder by); the thread's squares summed in T (FP32: one
  // conversion to FP64 per thread), the sums across threads in FP64
  const int i = i0 + (int)threadIdx.x;
  T xv[kVecPer], rv[kVecPer], pv[kVecPer], qv[kVecPer];
#pragma unroll
  for (int k = 0; k < kVecPer; k++)
    if (i + k * BLK < n3) {
      xv[k] = x[i + k * BLK];
      rv[k] = r[i + k * BLK];
      pv[k] = __ldg(p + i + k * BLK);
      qv[k] = __ldg(q + i + k * BLK);
    }
  T rr = T(0);
#pragma unroll
  for (int k = 0; k < kVecPer; k++)
    if (i + k * BLK < n3) {
      const T xi = xv[k] + al * pv[k];
      const T ri = rv[k] - al * qv[k];
      x[i + k * BLK] = xi;
      r[i + k * BLK] = ri;
      rr += ri * ri;
    }
  return (double)rr;
}
template <typename T, int BLK>
__device__ __forceinline__ void cg_p_tile(int n3, T beta, const T* __restrict__ r, T* __restrict__ p, int i0)
{
  const int i = i0 + (int)threadIdx.x;
  T rv[kVecPer], pv[kVecPer];
#pragma unroll
  for (int k = 0; k < kVecPer; k++)
    if (i + k * BLK < n3) {
      rv[k] = __ldg(r + i + k * BLK);
      pv[k] = p[i + k * BLK];
    }
#pragma unroll
  for (int k = 0; k < kVecPer; k++)
    if (i + k * BLK < n3) p[i + k * BLK] = next_dir(rv[k], beta, pv[k]);
}

// q = A p on the bulk tiles (partials of p.q in part[0 .. nt1)), then on
// the surface tiles (part[nt1 ..]), whose last CTA sums both and sets alpha
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_cg_mv(const LsmGeom G, const double* __restrict__ scal,
                                               const T* __restrict__ p, T* __restrict__ q, double* __restrict__ part)
{
  if (scal[6] > 0.0) return;
  const double pq = mv_bulk_tile<T, BLK>(G, p, q, blockIdx.x * kMvPer * BLK);
  block_sum_to<BLK>(pq, part + blockIdx.x);
}
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK, sizeof(T) == 4 ? 4 : 2) k_cg_mv_surf(const LsmGeom G, double* __restrict__ scal,
                                                    const T* __restrict__ p, T* __restrict__ q, double* __restrict__ part,
                                                    int nt1, unsigned* __restrict__ ctr, double tol2)
{
  if (scal[6] > 0.0) return;
  const double pq = mv_surf_tile<T, BLK>(G, p, q, blockIdx.x * kSfPer * BLK);
  double tot;
  if (grid_sum_last<BLK>(pq, part, nt1 + blockIdx.x, ctr, gridDim.x, nt1 + gridDim.x, &tot))
    cg_alpha_fin(scal, tot, tol2);
}

// x += alpha p; r -= alpha q; |r|^2 over the grid, then beta
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_cg_xr(int n3, double* __restrict__ scal, T* __restrict__ x,
                                               T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ q,
                                               double* __restrict__ part, unsigned* __restrict__ ctr)
{
  if (scal[6] > 0.0) return;
  const double rr = cg_xr_tile<T, BLK>(n3, (T)scal[2], x, r, p, q, blockIdx.x * kVecPer * BLK);
  double tot;
  if (grid_sum_last<BLK>(rr, part, blockIdx.x, ctr, gridDim.x, gridDim.x, &tot)) cg_beta_fin(scal, tot);
}

// p = r + beta p
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_cg_p(int n3, const double* __restrict__ scal, const T* __restrict__ r,
                                              T* __restrict__ p)
{
  if (scal[6] > 0.0) return;
  cg_p_tile<T, BLK>(n3, (T)scal[3], r, p, blockIdx.x * kVecPer * BLK);
}

// ---- batched CG: many networks advanced by the same launches ------------
// The descriptor table (kernel parameter) holds each network's geometry,
// CG vectors, partial-sum buffer, counter and scalar block, and the list of
// networks whose tiles a launch covers with the first tile of each: a CTA
// finds its (network, first element) by a binary search of that list in
// the parameter space (no dependent global load before its work starts).
// Every network runs the single-network iteration above on its own
// scalars, its last tile finishing its sums; a converged network's tiles
// return at once.
constexpr int kLsmBatchMax = 64;
struct LsmSys {
  LsmGeom G;
  void *x, *r, *p, *q;
  double* part;   // per-tile partial sums
  double* scal;   // CG scalars (layout of cg_alpha_fin / cg_beta_fin)
  unsigned* ctr;  // last-tile counter
  int n3, nt1, nts, nt3;  // 3 nvox, bulk tiles (kMvPer BLK nodes), surface tiles (kSfPer BLK, at least 1),
                          // element tiles (kVecPer BLK elements)
};
struct LsmTable {
  LsmSys s[kLsmBatchMax];
  int n;
  int nlive;                    // networks of the launches' tiles, in tile order
  int live[kLsmBatchMax];
  int f1[kLsmBatchMax + 1];     // first bulk tile of each listed network (f1[nlive] = grid size)
  int fs[kLsmBatchMax + 1];     // first surface tile
  int f3[kLsmBatchMax + 1];     // first element tile
};

// (network, first node / list entry / element) of this CTA's tile; first[]
// is one of the table's f1, fs, f3 and per the tile's length
__device__ __forceinline__ int2 batch_tile(const LsmTable& B, const int* first, int per)
{
  const int b = (int)blockIdx.x;
  int lo = 0, hi = B.nlive - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return make_int2(B.live[lo], (b - first[lo]) * per);
}

// k_cg_mv over the bulk tiles of the listed networks, then k_cg_mv_surf
// over their surface tiles
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_cg_mv_batch(const __grid_constant__ LsmTable B)
{
  const int2 tl = batch_tile(B, B.f1, kMvPer * BLK);
  const LsmSys& S = B.s[tl.x];
  if (S.scal[6] > 0.0) return;  // converged network (whole CTA)
  const LsmGeom G = S.G;  // fields read once, not at every use through the indexed table
  const double pq = mv_bulk_tile<T, BLK>(G, static_cast<const T*>(S.p), static_cast<T*>(S.q), tl.y);
  block_sum_to<BLK>(pq, S.part + tl.y / (kMvPer * BLK));
}
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK, sizeof(T) == 4 ? 4 : 2) k_cg_mv_surf_batch(const __grid_constant__ LsmTable B,
                                                                                  double tol2)
{
  const int2 tl = batch_tile(B, B.fs, kSfPer * BLK);
  const LsmSys& S = B.s[tl.x];
  if (S.scal[6] > 0.0) return;
  const LsmGeom G = S.G;
  const double pq = mv_surf_tile<T, BLK>(G, static_cast<const T*>(S.p), static_cast<T*>(S.q), tl.y);
  double tot;
  if (grid_sum_last<BLK>(pq, S.part, S.nt1 + tl.y / (kSfPer * BLK), S.ctr, S.nts, S.nt1 + S.nts, &tot))
    cg_alpha_fin(S.scal, tot, tol2);
}

// k_cg_xr over the element tiles of the listed networks
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_cg_xr_batch(const __grid_constant__ LsmTable B)
{
  const int2 tl = batch_tile(B, B.f3, kVecPer * BLK);
  const LsmSys& S = B.s[tl.x];
  if (S.scal[6] > 0.0) return;
  const double rr = cg_xr_tile<T, BLK>(S.n3, (T)S.scal[2], static_cast<T*>(S.x), static_cast<T*>(S.r),
                                       static_cast<const T*>(S.p), static_cast<const T*>(S.q), tl.y);
  double tot;
  if (grid_sum_last<BLK>(rr, S.part, tl.y / (kVecPer * BLK), S.ctr, S.nt3, S.nt3, &tot)) cg_beta_fin(S.scal, tot);
}

// k_cg_p over the element tiles of the listed networks
template <typename T, int BLK>
__global__ void __launch_bounds__(BLK) k_cg_p_batch(const __grid_constant__ LsmTable B)
{
  const int2 tl = batch_tile(B, B.f3, kVecPer * BLK);
  const LsmSys& S = B.s[tl.x];
  if (S.scal[6] > 0.0) return;
  cg_p_tile<T, BLK>(S.n3, (T)S.scal[3], static_cast<const T*>(S.r), static_cast<T*>(S.p), tl.y);
}

// |r0|^2 (already in scal[0]) becomes the reference |b|^2 of the tolerance
__global__ void k_cg_init_batch(const __grid_constant__ LsmTable B)
{
  const int s = threadIdx.x;
  if (s >= B.n) return;
  double* scal = B.s[s].scal;
  scal[3] = 0.0;
  scal[5] = scal[0];
  scal[6] = 0.0;
  scal[7] = 0.0;
}

// done flags of every network into out[s], iteration counts into out[n + s]
__global__ void k_cg_done_batch(const __grid_constant__ LsmTable B, double* out)
{
  const int s = threadIdx.x;
  if (s < B.n) {
    out[s] = B.s[s].scal[6];
    out[B.n + s] = B.s[s].scal[7];
  }
}

// a list of networks of a table
struct LsmList {
  int s[kLsmBatchMax];
  int n;
};
// networks joining the batch with a new inner system whose |r0|^2 is in
// scal[0]: the CG scalars of its first iteration
__global__ void k_cg_admit_batch(const __grid_constant__ LsmTable B, const LsmList L)
{
  const int i = threadIdx.x;
  if (i >= L.n) return;
  double* scal = B.s[L.s[i]].scal;
  scal[3] = 0.0;
  scal[5] = scal[0];
  scal[6] = 0.0;
  scal[7] = 0.0;
}
// networks leaving the batch with their iteration budget spent: their
// tiles of the captured iterations return at once from now on
__global__ void k_cg_stop_batch(const __grid_constant__ LsmTable B, const LsmList L)
{
  const int i = threadIdx.x;
  if (i < L.n) B.s[L.s[i]].scal[6] = 1.0;
}

}  // namespace lsm
}  // namespace ps
