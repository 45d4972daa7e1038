// gray_kernels.cuh -- single-phase D3Q19 TRT lattice with a gray
// partial-bounce-back (PBB) solid field, and its discrete adjoint.
//
// No counterpart in the reference: it extends the reference's single-phase
// branch (one component at a node: S1:3701-3710, the same D3Q19 velocity
// order and TRT rates with the magic product) with the partial bounce-back
// of Walsh, Burwinkle & Saar (Comput. Geosci. 2009):
//   out_i(x) = (1 - s(x)) f*_i(x) + s(x) f_{opp(i)}(x),
// f* the post-collision and f the pre-collision populations, s in [0, 1]
// (0 open fluid, 1 full bounce-back).  Every voxel is a node (dense
// periodic box, FP64).  The state is stored shifted, g_i = f_i - t_i (t_i
// the rest weights at unit density), g[i][v] with v = x + nx (y + ny z):
// at the small velocities of a permeability run f_i - t_i is ~1e-6, so the
// shifted form keeps ~10 more significant bits of the flow than f_i itself;
// that is what lets central differences of k (k ~ <j> / F) resolve the
// adjoint's gradient.  Every map below is written on g (f - e = g - (e - t),
// the partial bounce-back acts on g as on f since t_opp(i) = t_i).
//
// Collision: u = (j + F/2) / rho, equilibrium e_i = t_i rho (1 + 3 c.u +
// 4.5 (c.u)^2 - 1.5 u^2), TRT f*_i = f_i - lp (f - e)^+_i - lm (f - e)^-_i +
// (1 - lm/2) 3 t_i c_i.F (the odd Guo force term, independent of the state,
// so that the momentum gains exactly F per step).
//
// Adjoint of one step f(t) -> f(t+1) = S P C (f(t)) (collision C, PBB P,
// streaming S), evaluated at the forward state f(t):
//   a_out_i(x) = a_i(x + c_i, t+1)                      (S^T: pull)
//   g_s(x)    += sum_i a_out_i (f_opp(i) - f*_i)         (d out / d s)
//   a*_i       = (1 - s) a_out_i;  a_i = s a_out_opp(i)  (P^T)
//   a_i       += a*_i - w_i + dE_rho + c_i . dE_j        (C^T)
// with w = lp (a*)^+ + lm (a*)^-, dE_rho = sum_i w_i de_i/drho and dE_j =
// sum_i w_i de_i/dj (de_i/drho = t_i (1 - 4.5 (c.u)^2 + 1.5 u^2), de_i/dj =
// t_i (3 c_i + 9 (c.u) c_i - 3 u)).
#pragma once
#include <stdint.h>

namespace ps {
namespace gray {

// D3Q19 in the reference's velocities19 order
__host__ __device__ constexpr int gcx(int d)
{
  return d == 1 || d == 7 || d == 9 || d == 11 || d == 13 ? 1 : d == 2 || d == 8 || d == 10 || d == 12 || d == 14 ? -1 : 0;
}
__host__ __device__ constexpr int gcy(int d)
{
  return d == 3 || d == 7 || d == 8 || d == 15 || d == 17 ? 1 : d == 4 || d == 9 || d == 10 || d == 16 || d == 18 ? -1 : 0;
}
__host__ __device__ constexpr int gcz(int d)
{
  return d == 5 || d == 11 || d == 12 || d == 15 || d == 16 ? 1 : d == 6 || d == 13 || d == 14 || d == 17 || d == 18 ? -1 : 0;
}
__host__ __device__ constexpr int gopp(int d)
{
  return d == 0 ? 0 : (d <= 6 ? (d % 2 == 1 ? d + 1 : d - 1) : (2 * (7 + 4 * ((d - 7) / 4)) + 3 - d));
}
// the 9 opposite pairs (a, opp(a)) with a the first of each
__host__ __device__ constexpr int gpair(int k)
{
  return k < 3 ? 1 + 2 * k : (k == 3 ? 7 : k == 4 ? 8 : k == 5 ? 11 : k == 6 ? 12 : k == 7 ? 15 : 16);
}
static_assert(gopp(7) == 10 && gopp(8) == 9 && gopp(16) == 17 && gopp(3) == 4, "gray opposites");

struct GrayConst {
  double lp, lm;      // even / odd relaxation rates
  double F[3];        // body force
  double fF[19];      // (1 - lm/2) 3 t_i c_i . F
  double t[19];       // weights 1/3, 1/18, 1/36
};

struct GrayGeom {
  int nx, ny, nz;
  long long n;  // nodes
};

__device__ __forceinline__ long long gray_nb(const GrayGeom& G, int x, int y, int z, int d)
{
  int a = x + gcx(d), b = y + gcy(d), c = z + gcz(d);
  a = a < 0 ? a + G.nx : (a >= G.nx ? a - G.nx : a);
  b = b < 0 ? b + G.ny : (b >= G.ny ? b - G.ny : b);
  c = c < 0 ? c + G.nz : (c >= G.nz ? c - G.nz : c);
  return a + (long long)G.nx * (b + (long long)G.ny * c);
}

// moments, equilibrium velocity and post-collision populations (shifted,
// g*_i = f*_i - t_i) of one node
struct GrayNode {
  double rho, ux, uy, uz, usq;
  double fs[19];
};

__device__ __forceinline__ void gray_collide(const GrayConst& C, const double* g, GrayNode& N)
{
  double rho1 = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;  // rho - 1 and the momentum, from g
#pragma unroll
  for (int i = 0; i < 19; i++) {
    rho1 = rho1 + g[i];
    jx = jx + (double)gcx(i) * g[i];
    jy = jy + (double)gcy(i) * g[i];
    jz = jz + (double)gcz(i) * g[i];
  }
  const double rho = 1.0 + rho1;
  const double ux = (jx + 0.5 * C.F[0]) / rho, uy = (jy + 0.5 * C.F[1]) / rho, uz = (jz + 0.5 * C.F[2]) / rho;
  const double usq = ux * ux + uy * uy + uz * uz;
  double de[19];  // e_i - t_i
#pragma unroll
  for (int i = 0; i < 19; i++) {
    const double cu = (double)gcx(i) * ux + (double)gcy(i) * uy + (double)gcz(i) * uz;
    de[i] = C.t[i] * rho1 + C.t[i] * rho * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
  }
  N.fs[0] = g[0] - C.lp * (g[0] - de[0]);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int a = gpair(k), b = gopp(a);
    const double fp = 0.5 * (g[a] + g[b]), fm = 0.5 * (g[a] - g[b]);
    const double ep = 0.5 * (de[a] + de[b]), em = 0.5 * (de[a] - de[b]);
    N.fs[a] = g[a] - C.lp * (fp - ep) - C.lm * (fm - em) + C.fF[a];
    N.fs[b] = g[b] - C.lp * (fp - ep) + C.lm * (fm - em) + C.fF[b];
  }
  N.rho = rho;
  N.ux = ux;
  N.uy = uy;
  N.uz = uz;
  N.usq = usq;
}

// one step: collide, partial bounce-back, push to the neighbours
template <int BLK>
__global__ void __launch_bounds__(BLK) k_gray_step(const __grid_constant__ GrayConst C, const GrayGeom G,
                                                   const double* __restrict__ src, double* __restrict__ dst,
                                                   const double* __restrict__ s)
{
  const long long v = (long long)blockIdx.x * BLK + threadIdx.x;
  if (v >= G.n) return;
  const int x = (int)(v % G.nx), y = (int)((v / G.nx) % G.ny), z = (int)(v / ((long long)G.nx * G.ny));
  double f[19];
#pragma unroll
  for (int i = 0; i < 19; i++) f[i] = src[i * G.n + v];
  GrayNode N;
  gray_collide(C, f, N);
  const double sv = s[v], so = 1.0 - sv;
#pragma unroll
  for (int i = 0; i < 19; i++) dst[i * G.n + gray_nb(G, x, y, z, i)] = so * N.fs[i] + sv * f[gopp(i)];
}

// adjoint of one step at forward state f (= f(t)): an = a(t+1) in, at =
// a(t) out, gs += d objective / d s contributions of this step
template <int BLK>
__global__ void __launch_bounds__(BLK) k_gray_adjoint(const __grid_constant__ GrayConst C, const GrayGeom G,
                                                      const double* __restrict__ fst, const double* __restrict__ an,
                                                      double* __restrict__ at, const double* __restrict__ s,
                                                      double* __restrict__ gs)
{
  const long long v = (long long)blockIdx.x * BLK + threadIdx.x;
  if (v >= G.n) return;
  const int x = (int)(v % G.nx), y = (int)((v / G.nx) % G.ny), z = (int)(v / ((long long)G.nx * G.ny));
  double f[19];
#pragma unroll
  for (int i = 0; i < 19; i++) f[i] = fst[i * G.n + v];
  GrayNode N;
  gray_collide(C, f, N);
  double ao[19];
#pragma unroll
  for (int i = 0; i < 19; i++) ao[i] = an[i * G.n + gray_nb(G, x, y, z, i)];
  const double sv = s[v], so = 1.0 - sv;
  double g = 0.0;
#pragma unroll
  for (int i = 0; i < 19; i++) g = g + ao[i] * (f[gopp(i)] - N.fs[i]);
  gs[v] = gs[v] + g;
  double as[19], w[19], a[19];
#pragma unroll
  for (int i = 0; i < 19; i++) {
    as[i] = so * ao[i];
    a[i] = sv * ao[gopp(i)];
  }
  w[0] = C.lp * as[0];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int p = gpair(k), q = gopp(p);
    const double wp = C.lp * (0.5 * (as[p] + as[q])), wm = C.lm * (0.5 * (as[p] - as[q]));
    w[p] = wp + wm;
    w[q] = wp - wm;
  }
  double dr = 0.0, djx = 0.0, djy = 0.0, djz = 0.0;
#pragma unroll
  for (int i = 0; i < 19; i++) {
    const double cx = (double)gcx(i), cy = (double)gcy(i), cz = (double)gcz(i);
    const double cu = cx * N.ux + cy * N.uy + cz * N.uz;
    const double tw = C.t[i] * w[i];
    dr = dr + tw * (1.0 - 4.5 * cu * cu + 1.5 * N.usq);
    djx = djx + tw * (3.0 * cx + 9.0 * cu * cx - 3.0 * N.ux);
    djy = djy + tw * (3.0 * cy + 9.0 * cu * cy - 3.0 * N.uy);
    djz = djz + tw * (3.0 * cz + 9.0 * cu * cz - 3.0 * N.uz);
  }
#pragma unroll
  for (int i = 0; i < 19; i++)
    at[i * G.n + v] = a[i] + (as[i] - w[i]) + (dr + ((double)gcx(i) * djx + (double)gcy(i) * djy + (double)gcz(i) * djz));
}

// per-block sums of the x, y, z momentum of the state (FP64)
template <int BLK>
__global__ void __launch_bounds__(BLK) k_gray_momentum(const GrayGeom G, const double* __restrict__ f,
                                                       double* __restrict__ part)
{
  const long long v = (long long)blockIdx.x * BLK + threadIdx.x;
  double j[3] = {0.0, 0.0, 0.0};
  if (v < G.n) {
#pragma unroll
    for (int i = 1; i < 19; i++) {
      const double q = f[i * G.n + v];
      j[0] = j[0] + (double)gcx(i) * q;
      j[1] = j[1] + (double)gcy(i) * q;
      j[2] = j[2] + (double)gcz(i) * q;
    }
  }
  __shared__ double red[3][BLK / 32];
  for (int c = 0; c < 3; c++) {
    double t = j[c];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < BLK / 32; w++) t += red[threadIdx.x][w];
    part[(long long)blockIdx.x * 3 + threadIdx.x] = t;
  }
}

// one value per direction on every node: the rest state (g = 0) and the
// adjoint's terminal condition
struct Vals19 {
  double v[19];
};
__global__ void k_gray_fill(const GrayGeom G, const Vals19 val, double* __restrict__ f)
{
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= G.n) return;
  for (int i = 0; i < 19; i++) f[i * G.n + v] = val.v[i];
}

}  // namespace gray
}  // namespace ps
