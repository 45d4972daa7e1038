// lbm_node.cuh -- per-node arithmetic of the colour-gradient D3Q19 step.
//
// Three pieces, each a function of one lattice node:
//   mrt_collide   the forced MRT collision with TRT rates  (S1:2407-2620)
//   csf_force     the CSF surface-tension force and unit colour normal from
//                 the 3x3x3 colour neighbourhood            (S1:2626-2796)
//   node_update   branch selection (bulk red / bulk blue / interface), the
//                 interface collision and Latva-Kokko recolouring
//                                                           (S1:3663-3819)
//
// The operation order of every floating-point expression follows the
// reference source, so that the FP64 instantiation compiled without FMA
// contraction (--fmad=false) reproduces the reference arithmetic bit for bit.
// The FP32 instantiation uses the same code with FMA contraction enabled.
//
// Directions are numbered as in the reference's `velocities19` file (0-based
// here): 0 rest, 1..6 axis (+x,-x,+y,-y,+z,-z), 7..18 face diagonals.
#pragma once

#ifdef __CUDACC__
#define PS_HD __host__ __device__ __forceinline__
#else
#define PS_HD inline
#endif

#include <math.h>

namespace ps {

template <typename R>
struct LbmConst {
  R c1d6, c1d12, c5d399, c19d399, c11d2394, c1d63, c1d18, c1d36, c4d1197, c1d252, c1d72, c1d24;
  R cn;  // 1/sqrt(2): cosine factor of the diagonal directions
  R dt, dti, dt2;
  R t[2][3];     // lattice weights (rest, axis, diagonal) of red / blue (S1:1368-1376)
  R cs2[2];      // cr2, cb2
  R S[2][19];    // relaxation vectors Sr, Sb (collmatrTRT)
  R Fp[2][19];   // body-force projections Fpr, Fpb (S1:3428-3430)
  R bf[2][3];    // body forces bfr, bfb
  R B, sig, wet, ee;  // recolouring beta, sig/32, wetting colour, bulk threshold
};

// Forced MRT collision of one node.  f: 19 populations (f[0] is updated in
// place with the post-collision rest population); pcf[1..18] receives the
// post-collision moving populations.
template <typename R>
PS_HD void mrt_collide(const LbmConst<R>& K, R t1, R t2, R t3, R* f, R* pcf, R r, const R* bf,
                       const R* Fp, const R* S)
{
  const R dt = K.dt, dti = K.dti, dt2 = K.dt2;
  // momentum
  R jx = (f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14]) * dti;
  R jy = (f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18]) * dti;
  R jz = (f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18]) * dti;
  // force-shifted velocity
  const R rinv = R(1) / r;
  const R ux = (jx + bf[0] * R(0.5) * dt) * rinv;
  const R uy = (jy + bf[1] * R(0.5) * dt) * rinv;
  const R uz = (jz + bf[2] * R(0.5) * dt) * rinv;
  const R uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
  const R usq = (uxx + uyy + uzz) * R(0.5);

  // second-order equilibrium with sound-speed dependent weights
  R fl[19];
  {
    const R rq = r * R(0.25) * dt2;
    const R e1 = (t2 - usq * K.c1d6 * dt2) * r;
    const R ax = e1 + rq * uxx, ay = e1 + rq * uyy, az = e1 + rq * uzz;
    const R sx = jx * K.c1d6 * dt, sy = jy * K.c1d6 * dt, sz = jz * K.c1d6 * dt;
    fl[0] = f[0] - r * (t1 - usq * dt2);
    fl[1] = f[1] - (ax + sx);
    fl[2] = f[2] - (ax - sx);
    fl[3] = f[3] - (ay + sy);
    fl[4] = f[4] - (ay - sy);
    fl[5] = f[5] - (az + sz);
    fl[6] = f[6] - (az - sz);
    const R ro = r * R(0.125) * dt2;
    const R e2 = (t3 - usq * K.c1d12 * dt2) * r;
    // pairs (a,b): j_a +/- j_b terms and u_a +/- u_b quadratic terms
    const R pxy = (jx + jy) * K.c1d12 * dt, mxy = (jx - jy) * K.c1d12 * dt;
    const R pxz = (jx + jz) * K.c1d12 * dt, mxz = (jx - jz) * K.c1d12 * dt;
    const R pyz = (jy + jz) * K.c1d12 * dt, myz = (jy - jz) * K.c1d12 * dt;
    const R qpxy = ro * (ux + uy) * (ux + uy), qmxy = ro * (ux - uy) * (ux - uy);
    const R qpxz = ro * (ux + uz) * (ux + uz), qmxz = ro * (ux - uz) * (ux - uz);
    const R qpyz = ro * (uy + uz) * (uy + uz), qmyz = ro * (uy - uz) * (uy - uz);
    fl[7] = f[7] - (e2 + pxy + qpxy);
    fl[10] = f[10] - (e2 - pxy + qpxy);
    fl[8] = f[8] - (e2 - mxy + qmxy);
    fl[9] = f[9] - (e2 + mxy + qmxy);
    fl[11] = f[11] - (e2 + pxz + qpxz);
    fl[14] = f[14] - (e2 - pxz + qpxz);
    fl[13] = f[13] - (e2 + mxz + qmxz);
    fl[12] = f[12] - (e2 - mxz + qmxz);
    fl[15] = f[15] - (e2 + pyz + qpyz);
    fl[18] = f[18] - (e2 - pyz + qpyz);
    fl[17] = f[17] - (e2 + myz + qmyz);
    fl[16] = f[16] - (e2 - myz + qmyz);
  }

  // non-conserved moments of the non-equilibrium part (d'Humieres basis),
  // each already multiplied by its relaxation rate
  const R a6 = fl[1] + fl[2] + fl[3] + fl[4] + fl[5] + fl[6];
  const R a12 = fl[7] + fl[8] + fl[9] + fl[10] + fl[11] + fl[12] + fl[13] + fl[14] + fl[15] + fl[16] +
                fl[17] + fl[18];
  const R m_e = (-(R(30) * fl[0]) - R(11) * a6 + R(8) * a12) * S[1];
  const R m_eps = (R(12) * fl[0] - R(4) * a6 + a12) * S[2];
  const R m_qx = (R(4) * (fl[2] - fl[1]) + fl[7] - fl[8] + fl[9] - fl[10] + fl[11] - fl[12] + fl[13] - fl[14]) * S[4];
  const R m_qy = (R(4) * (fl[4] - fl[3]) + fl[7] + fl[8] - fl[9] - fl[10] + fl[15] - fl[16] + fl[17] - fl[18]) * S[6];
  const R m_qz = (R(4) * (fl[6] - fl[5]) + fl[11] + fl[12] - fl[13] - fl[14] + fl[15] + fl[16] - fl[17] - fl[18]) * S[8];
  const R sxy4 = fl[7] + fl[8] + fl[9] + fl[10];
  const R syz4 = fl[15] + fl[16] + fl[17] + fl[18];
  const R sxz4 = fl[11] + fl[12] + fl[13] + fl[14];
  const R dyz = fl[3] + fl[4] - fl[5] - fl[6];
  const R syz2 = fl[3] + fl[4] + fl[5] + fl[6];
  const R m_pxx = (R(2) * (fl[1] + fl[2] - syz4) - syz2 + sxy4 + sxz4) * S[9];
  const R m_rxx = (-(R(4) * (fl[1] + fl[2])) + R(2) * (syz2 - syz4) + sxy4 + sxz4) * S[10];
  const R m_pww = (dyz + sxy4 - sxz4) * S[11];
  const R m_rww = (-(R(2) * dyz) + sxy4 - sxz4) * S[12];
  const R m_pxy = (fl[7] - fl[8] - fl[9] + fl[10]) * S[13];
  const R m_pyz = (fl[15] - fl[16] - fl[17] + fl[18]) * S[14];
  const R m_pxz = (fl[11] - fl[12] - fl[13] + fl[14]) * S[15];
  const R m_mx = (fl[7] - fl[8] + fl[9] - fl[10] - fl[11] + fl[12] - fl[13] + fl[14]) * S[16];
  const R m_my = (-fl[7] - fl[8] + fl[9] + fl[10] + fl[15] - fl[16] + fl[17] - fl[18]) * S[17];
  const R m_mz = (fl[11] + fl[12] - fl[13] - fl[14] - fl[15] - fl[16] + fl[17] + fl[18]) * S[18];

  // back to population space (explicit inverse-basis coefficients)
  R mb[19];
  mb[0] = -(K.c5d399 * m_e) + K.c19d399 * m_eps;
  const R b1 = -(K.c11d2394 * m_e) - K.c1d63 * m_eps;
  mb[1] = b1 - R(0.1) * m_qx + K.c1d18 * (m_pxx - m_rxx);
  mb[2] = mb[1] + m_qx * R(0.2);
  mb[3] = b1 - R(0.1) * m_qy + K.c1d36 * (m_rxx - m_pxx) + K.c1d12 * (m_pww - m_rww);
  mb[4] = mb[3] + m_qy * R(0.2);
  mb[5] = b1 - R(0.1) * m_qz + K.c1d36 * (m_rxx - m_pxx) + K.c1d12 * (m_rww - m_pww);
  mb[6] = mb[5] + m_qz * R(0.2);
  const R b2 = K.c4d1197 * m_e + K.c1d252 * m_eps;
  mb[7] = b2 + (m_qx + m_qy) * R(0.025) + K.c1d36 * m_pxx + K.c1d72 * m_rxx + K.c1d12 * m_pww +
          K.c1d24 * m_rww + m_pxy * R(0.25) + (m_mx - m_my) * R(0.125);
  mb[8] = mb[7] - R(0.05) * m_qx - R(0.5) * m_pxy - R(0.25) * m_mx;
  mb[9] = mb[7] + R(0.25) * m_my - R(0.05) * m_qy - R(0.5) * m_pxy;
  mb[10] = mb[9] + R(0.5) * m_pxy - R(0.05) * m_qx - R(0.25) * m_mx;
  mb[11] = b2 + (m_qx + m_qz) * R(0.025) + K.c1d36 * m_pxx + K.c1d72 * m_rxx - K.c1d12 * m_pww -
           K.c1d24 * m_rww + m_pxz * R(0.25) + (m_mz - m_mx) * R(0.125);
  mb[12] = mb[11] + R(0.25) * m_mx - R(0.5) * m_pxz - R(0.05) * m_qx;
  mb[13] = mb[11] - R(0.05) * m_qz - R(0.5) * m_pxz - R(0.25) * m_mz;
  mb[14] = mb[12] + R(0.5) * m_pxz - R(0.05) * m_qz - R(0.25) * m_mz;
  mb[15] = b2 + (m_qy + m_qz) * R(0.025) - K.c1d18 * m_pxx - K.c1d36 * m_rxx + m_pyz * R(0.25) +
           (m_my - m_mz) * R(0.125);
  mb[16] = mb[15] - R(0.05) * m_qy - R(0.5) * m_pyz - R(0.25) * m_my;
  mb[17] = mb[15] + R(0.25) * m_mz - R(0.05) * m_qz - R(0.5) * m_pyz;
  mb[18] = mb[17] + R(0.5) * m_pyz - R(0.05) * m_qy - R(0.25) * m_my;

  f[0] = f[0] - mb[0] + Fp[0];
#pragma unroll
  for (int i = 1; i < 19; i++) pcf[i] = f[i] - mb[i] + Fp[i];
}

// The same collision in two-relaxation-time population form, used by the
// FP32 paths.  With the reference's rates every even non-conserved moment
// relaxes with wp = s_nu and every odd one with wm = s_q (the TRT magic
// 3/16 pair), and the equilibrium conserves density and momentum exactly,
// so M^-1 S M (f - fe) equals s_nu (f - fe)^+ + s_q (f - fe)^- for each
// opposite pair: the operator of mrt_collide in ~80 operations instead of
// ~300, differing only by rounding.  F is the total body force; its
// projections are formed per pair instead of being passed in.
template <typename R>
PS_HD void trt_collide(const LbmConst<R>& K, R t2, R t3, R* f, R* pcf, R r, const R* F, R wp, R wm)
{
  const R dt = K.dt, dti = K.dti, dt2 = K.dt2;
  const R jx = (f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14]) * dti;
  const R jy = (f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18]) * dti;
  const R jz = (f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18]) * dti;
  const R rinv = R(1) / r;
  const R ux = (jx + F[0] * R(0.5) * dt) * rinv;
  const R uy = (jy + F[1] * R(0.5) * dt) * rinv;
  const R uz = (jz + F[2] * R(0.5) * dt) * rinv;
  const R uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
  const R usq = (uxx + uyy + uzz) * R(0.5);
  // even equilibrium part of each opposite pair (a, b = opp(a))
  const R rq = r * R(0.25) * dt2;
  const R e1 = (t2 - usq * K.c1d6 * dt2) * r;
  const R ro = r * R(0.125) * dt2;
  const R e2 = (t3 - usq * K.c1d12 * dt2) * r;
  const R ev[9] = {e1 + rq * uxx,
                   e1 + rq * uyy,
                   e1 + rq * uzz,
                   e2 + ro * (ux + uy) * (ux + uy),
                   e2 + ro * (ux - uy) * (ux - uy),
                   e2 + ro * (ux + uz) * (ux + uz),
                   e2 + ro * (ux - uz) * (ux - uz),
                   e2 + ro * (uy + uz) * (uy + uz),
                   e2 + ro * (uy - uz) * (uy - uz)};
  // The rest equilibrium is the complement r - sum of the moving ones
  // (r (t1 - usq dt2) in exact arithmetic).  In FP32 the rounded weights
  // t1 + 6 t2 + 12 t3 exceed 1 by ~1.5e-8, which would add wp * 1.5e-8 of
  // mass per node and step; the complement conserves mass up to unbiased
  // rounding.
  const R esum = ((ev[0] + ev[1]) + ev[2]) + (((ev[3] + ev[4]) + (ev[5] + ev[6])) + (ev[7] + ev[8]));
  pcf[0] = f[0] - wp * (f[0] - (r - R(2) * esum));
  // each pair: odd equilibrium part and the body-force projection
  // rk (c_a . F) dt^2 (S1:3428-3430, 3734-3752)
  const R c6 = K.c1d6 * dt, c12 = K.c1d12 * dt;
  const R w6 = K.c1d6 * dt2, w12 = K.c1d12 * dt2;
  auto pair = [&](int a, int b, R even, R odd, R fa) {
    const R la = f[a] - (even + odd), lb = f[b] - (even - odd);
    const R p = (la + lb) * R(0.5), m = (la - lb) * R(0.5);
    pcf[a] = f[a] - wp * p - wm * m + fa;
    pcf[b] = f[b] - wp * p + wm * m - fa;
  };
  pair(1, 2, ev[0], jx * c6, w6 * F[0]);
  pair(3, 4, ev[1], jy * c6, w6 * F[1]);
  pair(5, 6, ev[2], jz * c6, w6 * F[2]);
  pair(7, 10, ev[3], (jx + jy) * c12, w12 * (F[0] + F[1]));
  pair(8, 9, ev[4], (jy - jx) * c12, w12 * (F[1] - F[0]));
  pair(11, 14, ev[5], (jx + jz) * c12, w12 * (F[0] + F[2]));
  pair(12, 13, ev[6], (jz - jx) * c12, w12 * (F[2] - F[0]));
  pair(15, 18, ev[7], (jy + jz) * c12, w12 * (F[1] + F[2]));
  pair(16, 17, ev[8], (jz - jy) * c12, w12 * (F[2] - F[1]));
  f[0] = pcf[0];
}

// trt_collide on shifted populations g = f - T (T_d the storage reference
// t^r_d rho^r_old + t^b_d rho^b_old of the node's populations).  dr1 / dr2
// are t_w r - T_w for the axis / diagonal weight classes (each a small
// difference computed from densities), dsum = sum_d g_d = sum_d (f_d - T_d);
// r is the current density.  gs receives g* = f* - T.  Every intermediate
// is a deviation (~1e-4 in bulk fluid), so FP32 rounding acts on the flow
// itself, not on the O(t_d) rest populations it rides on.
template <typename R>
PS_HD void trt_collide_dev(const LbmConst<R>& K, R dr1, R dr2, R dsum, const R* g, R* gs, R r, const R* F, R wp,
                           R wm)
{
  const R dt = K.dt, dti = K.dti, dt2 = K.dt2;
  const R jx = (g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14]) * dti;
  const R jy = (g[3] - g[4] + g[7] + g[8] - g[9] - g[10] + g[15] - g[16] + g[17] - g[18]) * dti;
  const R jz = (g[5] - g[6] + g[11] + g[12] - g[13] - g[14] + g[15] + g[16] - g[17] - g[18]) * dti;
  const R rinv = R(1) / r;
  const R ux = (jx + F[0] * R(0.5) * dt) * rinv;
  const R uy = (jy + F[1] * R(0.5) * dt) * rinv;
  const R uz = (jz + F[2] * R(0.5) * dt) * rinv;
  const R uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
  const R usq = (uxx + uyy + uzz) * R(0.5);
  // shifted even equilibrium parts e_pair - T_pair
  const R rq = r * R(0.25) * dt2, ro = r * R(0.125) * dt2;
  const R e1 = dr1 - usq * K.c1d6 * dt2 * r;
  const R e2 = dr2 - usq * K.c1d12 * dt2 * r;
  const R ev[9] = {e1 + rq * uxx,
                   e1 + rq * uyy,
                   e1 + rq * uzz,
                   e2 + ro * (ux + uy) * (ux + uy),
                   e2 + ro * (ux - uy) * (ux - uy),
                   e2 + ro * (ux + uz) * (ux + uz),
                   e2 + ro * (ux - uz) * (ux - uz),
                   e2 + ro * (uy + uz) * (uy + uz),
                   e2 + ro * (uy - uz) * (uy - uz)};
  // rest part: the complement, so that the collision conserves sum g exactly
  // up to unbiased rounding
  const R esum = ((ev[0] + ev[1]) + ev[2]) + (((ev[3] + ev[4]) + (ev[5] + ev[6])) + (ev[7] + ev[8]));
  gs[0] = g[0] - wp * (g[0] - (dsum - R(2) * esum));
  const R c6 = K.c1d6 * dt, c12 = K.c1d12 * dt;
  const R w6 = K.c1d6 * dt2, w12 = K.c1d12 * dt2;
  auto pair = [&](int a, int b, R even, R odd, R fa) {
    const R la = g[a] - (even + odd), lb = g[b] - (even - odd);
    const R p = (la + lb) * R(0.5), m = (la - lb) * R(0.5);
    gs[a] = g[a] - wp * p - wm * m + fa;
    gs[b] = g[b] - wp * p + wm * m - fa;
  };
  pair(1, 2, ev[0], jx * c6, w6 * F[0]);
  pair(3, 4, ev[1], jy * c6, w6 * F[1]);
  pair(5, 6, ev[2], jz * c6, w6 * F[2]);
  pair(7, 10, ev[3], (jx + jy) * c12, w12 * (F[0] + F[1]));
  pair(8, 9, ev[4], (jy - jx) * c12, w12 * (F[1] - F[0]));
  pair(11, 14, ev[5], (jx + jz) * c12, w12 * (F[0] + F[2]));
  pair(12, 13, ev[6], (jz - jx) * c12, w12 * (F[2] - F[0]));
  pair(15, 18, ev[7], (jy + jz) * c12, w12 * (F[1] + F[2]));
  pair(16, 17, ev[8], (jz - jy) * c12, w12 * (F[2] - F[1]));
}

// CSF surface tension from the colour neighbourhood.  cc(i,j,k), i,j,k in
// {0,1,2} (offsets -1,0,+1 in x,y,z) returns the stencil colour: the node's
// colour for fluid voxels, the wetting colour for the others.  The colour
// gradient is evaluated on the 8 sub-cubes of the 3x3x3 box; the curvature
// is k2 - k1 with k1 = div of the sub-cube gradients and k2 the gradient of
// their modulus along the normal.  Returns Fs = sig (k2 - k1) n and n.
template <typename R, typename CC>
PS_HD void csf_force(const LbmConst<R>& K, CC cc, R* n, R* Fs)
{
  // Sub-cube s = a + 2b + 4c has its low corner at offset (a,b,c).  Its
  // gradient components are differences of the two 2x2 faces normal to each
  // axis; every face sum is (edge + edge) with edges summed low index first.
  R g[8][3];
  if constexpr (sizeof(R) == 8) {
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const int a = s & 1, b = (s >> 1) & 1, c = s >> 2;
      // x: faces at x=a+1 and x=a, edges along y, summed over z
      const R xh = (cc(a + 1, b, c) + cc(a + 1, b + 1, c)) + (cc(a + 1, b, c + 1) + cc(a + 1, b + 1, c + 1));
      const R xl = (cc(a, b, c) + cc(a, b + 1, c)) + (cc(a, b, c + 1) + cc(a, b + 1, c + 1));
      // y: faces at y=b+1 and y=b, edges along x, summed over z
      const R yh = (cc(a, b + 1, c) + cc(a + 1, b + 1, c)) + (cc(a, b + 1, c + 1) + cc(a + 1, b + 1, c + 1));
      const R yl = (cc(a, b, c) + cc(a + 1, b, c)) + (cc(a, b, c + 1) + cc(a + 1, b, c + 1));
      // z: faces at z=c+1 and z=c, edges along x, summed over y
      const R zh = (cc(a, b, c + 1) + cc(a + 1, b, c + 1)) + (cc(a, b + 1, c + 1) + cc(a + 1, b + 1, c + 1));
      const R zl = (cc(a, b, c) + cc(a + 1, b, c)) + (cc(a, b + 1, c) + cc(a + 1, b + 1, c));
      g[s][0] = xh - xl;
      g[s][1] = yh - yl;
      g[s][2] = zh - zl;
    }
  } else {
    // FP32 paths: the same 2x2 face sums built from shared pair sums (96
    // additions instead of 168); only the rounding order differs
    R v[3][3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int k = 0; k < 3; k++) v[i][j][k] = cc(i, j, k);
    R pz[3][3][2], py[3][2][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int c = 0; c < 2; c++) pz[i][j][c] = v[i][j][c] + v[i][j][c + 1];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int k = 0; k < 3; k++) py[i][b][k] = v[i][b][k] + v[i][b + 1][k];
    R syz[3][2][2], sxz[2][3][2], sxy[2][2][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 2; c++) syz[i][b][c] = pz[i][b][c] + pz[i][b + 1][c];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int c = 0; c < 2; c++) sxz[a][j][c] = pz[a][j][c] + pz[a + 1][j][c];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int k = 0; k < 3; k++) sxy[a][b][k] = py[a][b][k] + py[a + 1][b][k];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const int a = s & 1, b = (s >> 1) & 1, c = s >> 2;
      g[s][0] = syz[a + 1][b][c] - syz[a][b][c];
      g[s][1] = sxz[a][b + 1][c] - sxz[a][b][c];
      g[s][2] = sxy[a][b][c + 1] - sxy[a][b][c];
    }
  }
  R nx = g[0][0], ny = g[0][1], nz = g[0][2];
#pragma unroll
  for (int s = 1; s < 8; s++) {
    nx = nx + g[s][0];
    ny = ny + g[s][1];
    nz = nz + g[s][2];
  }
  constexpr bool kExact = sizeof(R) == 8;  // FP64: IEEE sqrt and divisions as the reference
  const R n2 = nx * nx + ny * ny + nz * nz;
  // divergence of the sub-cube gradients (high half minus low half per axis,
  // in the reference's summation order)
  const R k1 = (g[1][0] + g[3][0] + g[5][0] + g[7][0] - g[0][0] - g[2][0] - g[4][0] - g[6][0]) +
               (g[3][1] + g[7][1] + g[2][1] + g[6][1] - g[0][1] - g[1][1] - g[4][1] - g[5][1]) +
               (g[4][2] + g[5][2] + g[6][2] + g[7][2] - g[0][2] - g[1][2] - g[2][2] - g[3][2]);
  R m[8];
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const R q = g[s][0] * g[s][0] + g[s][1] * g[s][1] + g[s][2] * g[s][2];
    if constexpr (kExact)
      m[s] = sqrt(q);
    else
      m[s] = q > R(0) ? q * rsqrt(q) : R(0);  // FP32 paths: hardware reciprocal square root
  }
  const R mx = m[1] + m[3] + m[5] + m[7] - m[0] - m[2] - m[4] - m[6];
  const R my = m[3] + m[7] + m[2] + m[6] - m[0] - m[1] - m[4] - m[5];
  const R mz = m[4] + m[5] + m[6] + m[7] - m[0] - m[1] - m[2] - m[3];
  R k2 = nx * mx + ny * my + nz * mz;
  if constexpr (kExact) {
    const R nrm = sqrt(n2);
    if (nrm != R(0)) {
      k2 = k2 / nrm;
      nx = nx / nrm;
      ny = ny / nrm;
      nz = nz / nrm;
    }
  } else if (n2 > R(0)) {
    const R inv = rsqrt(n2);
    k2 = k2 * inv;
    nx = nx * inv;
    ny = ny * inv;
    nz = nz * inv;
  }
  const R s = K.sig * (k2 - k1);
  n[0] = nx;
  n[1] = ny;
  n[2] = nz;
  Fs[0] = s * nx;
  Fs[1] = s * ny;
  Fs[2] = s * nz;
}

// One node of the majority-rule step.  fr, fb: post-streaming populations
// (19 each); out_r/out_b receive all 19 post-collision populations (index
// 0 = rest).  rr, rb are the component densities of fr, fb.
//
// The three branches of the reference (bulk red, bulk blue, interface) all
// reduce to one forced collision with branch-dependent inputs, so the
// collision is evaluated once per node: a warp holding nodes of all three
// kinds executes it once instead of three times.  Per node the arithmetic is
// exactly the reference's.
template <typename R, typename CC>
PS_HD void node_update(const LbmConst<R>& K, const R* fr, const R* fb, R rr, R rb, CC cc, R* out_r, R* out_b)
{
  constexpr bool kExact = sizeof(R) == 8;  // FP64: keep every division as written
  const bool bulk_r = rb <= K.ee;
  const bool bulk_b = !bulk_r && rr <= K.ee;
  const bool iface = !bulk_r && !bulk_b;
  // collision inputs
  R f[19], pcf[19], bf[3], n[3] = {R(0), R(0), R(0)};
  R t1, t2, t3, r, ti2 = R(0), ti3 = R(0);
  if constexpr (kExact) {
    R Fp[19], S[19];
    if (iface) {
      R Fs[3];
      csf_force(K, cc, n, Fs);
#pragma unroll
      for (int i = 0; i < 19; i++) f[i] = fr[i] + fb[i];
      const R ri = rr + rb;
      const R ci2 = (K.cs2[0] * rr + K.cs2[1] * rb) / ri;
      t1 = R(1) - R(2) * ci2 * K.dt2;
      ti2 = ci2 * K.c1d6 * K.dt2;
      ti3 = ci2 * K.c1d12 * K.dt2;
      t2 = ti2;
      t3 = ti3;
      r = ri;
      const int ph = rr >= rb ? 0 : 1;
      bf[0] = K.bf[ph][0] + Fs[0];
      bf[1] = K.bf[ph][1] + Fs[1];
      bf[2] = K.bf[ph][2] + Fs[2];
#pragma unroll
      for (int i = 0; i < 19; i++) S[i] = K.S[ph][i];
      const R dt2 = K.dt2;
      Fp[0] = R(0);
      Fp[1] = K.c1d6 * bf[0] * dt2;
      Fp[2] = -Fp[1];
      Fp[3] = K.c1d6 * bf[1] * dt2;
      Fp[4] = -Fp[3];
      Fp[5] = K.c1d6 * bf[2] * dt2;
      Fp[6] = -Fp[5];
      Fp[7] = K.c1d12 * (bf[0] + bf[1]) * dt2;
      Fp[8] = K.c1d12 * (-bf[0] + bf[1]) * dt2;
      Fp[9] = -Fp[8];
      Fp[10] = -Fp[7];
      Fp[11] = K.c1d12 * (bf[0] + bf[2]) * dt2;
      Fp[12] = K.c1d12 * (-bf[0] + bf[2]) * dt2;
      Fp[13] = -Fp[12];
      Fp[14] = -Fp[11];
      Fp[15] = K.c1d12 * (bf[1] + bf[2]) * dt2;
      Fp[16] = K.c1d12 * (-bf[1] + bf[2]) * dt2;
      Fp[17] = -Fp[16];
      Fp[18] = -Fp[15];
    } else {
      const int k = bulk_r ? 0 : 1;
#pragma unroll
      for (int i = 0; i < 19; i++) {
        f[i] = bulk_r ? fr[i] : fb[i];
        Fp[i] = K.Fp[k][i];
        S[i] = K.S[k][i];
      }
      t1 = K.t[k][0];
      t2 = K.t[k][1];
      t3 = K.t[k][2];
      r = bulk_r ? rr : rb;
      bf[0] = K.bf[k][0];
      bf[1] = K.bf[k][1];
      bf[2] = K.bf[k][2];
    }
    mrt_collide(K, t1, t2, t3, f, pcf, r, bf, Fp, S);
  } else {
    // the same inputs without the per-direction arrays (TRT needs two rates)
    int ph;
    if (iface) {
      R Fs[3];
      csf_force(K, cc, n, Fs);
#pragma unroll
      for (int i = 0; i < 19; i++) f[i] = fr[i] + fb[i];
      r = rr + rb;
      const R ci2 = (K.cs2[0] * rr + K.cs2[1] * rb) / r;
      ti2 = ci2 * K.c1d6 * K.dt2;
      ti3 = ci2 * K.c1d12 * K.dt2;
      t2 = ti2;
      t3 = ti3;
      ph = rr >= rb ? 0 : 1;
      bf[0] = K.bf[ph][0] + Fs[0];
      bf[1] = K.bf[ph][1] + Fs[1];
      bf[2] = K.bf[ph][2] + Fs[2];
    } else {
      ph = bulk_r ? 0 : 1;
#pragma unroll
      for (int i = 0; i < 19; i++) f[i] = bulk_r ? fr[i] : fb[i];
      t2 = K.t[ph][1];
      t3 = K.t[ph][2];
      r = bulk_r ? rr : rb;
      bf[0] = K.bf[ph][0];
      bf[1] = K.bf[ph][1];
      bf[2] = K.bf[ph][2];
    }
    trt_collide(K, t2, t3, f, pcf, r, bf, K.S[ph][1], K.S[ph][4]);
  }
  if (iface) {
    // cosine between the colour normal and each direction
    R cs[19];
    cs[1] = n[0];
    cs[2] = -cs[1];
    cs[3] = n[1];
    cs[4] = -cs[3];
    cs[5] = n[2];
    cs[6] = -cs[5];
    cs[7] = (n[0] + n[1]) * K.cn;
    cs[8] = (-n[0] + n[1]) * K.cn;
    cs[9] = -cs[8];
    cs[10] = -cs[7];
    cs[11] = (n[0] + n[2]) * K.cn;
    cs[12] = (-n[0] + n[2]) * K.cn;
    cs[13] = -cs[12];
    cs[14] = -cs[11];
    cs[15] = (n[1] + n[2]) * K.cn;
    cs[16] = (-n[1] + n[2]) * K.cn;
    cs[17] = -cs[16];
    cs[18] = -cs[15];
    // rest population split by mass fraction, moving ones recoloured
    // (Latva-Kokko), S1:3797-3817
    if constexpr (kExact) {
      out_r[0] = f[0] * rr / r;
      out_b[0] = f[0] * rb / r;
#pragma unroll
      for (int i = 1; i < 19; i++) {
        const R w = i < 7 ? ti2 : ti3;
        out_r[i] = (pcf[i] + K.B * w * cs[i] * rb) * rr / r;
        out_b[i] = (pcf[i] - K.B * w * cs[i] * rr) * rb / r;
      }
    } else {
      const R inv = R(1) / r, qr = rr * inv, qb = rb * inv;
      out_r[0] = f[0] * qr;
      out_b[0] = f[0] * qb;
#pragma unroll
      for (int i = 1; i < 19; i++) {
        const R w = K.B * (i < 7 ? ti2 : ti3) * cs[i];
        out_r[i] = (pcf[i] + w * rb) * qr;
        out_b[i] = (pcf[i] - w * rr) * qb;
      }
    }
  } else {
    // collided component, and the other one at its rest equilibrium
#pragma unroll
    for (int i = 0; i < 19; i++) {
      const R c = i == 0 ? f[0] : pcf[i];
      const int w = i == 0 ? 0 : (i < 7 ? 1 : 2);
      out_r[i] = bulk_r ? c : K.t[0][w] * rr;
      out_b[i] = bulk_r ? K.t[1][w] * rb : c;
    }
  }
}

// node_update for the FP32 paths in shifted form.  gr / gb are the node's
// populations as deviations g_c[d] = f_c[d] - t^c_d rho^c_old from the
// reference densities (ror, rob) they were stored against; rr = ror + sum
// g_r and rb = rob + sum g_b are the current densities.  The post-collision
// recoloured populations come out as out_c[d] = t^c_d S_c + Z_c[d]: a
// receiver whose reference density is rho' stores t^c_d (S_c - rho') +
// Z_c[d], again a small number.  Same branches, collision and recolouring
// as node_update; only the representation differs.
template <typename CC>
PS_HD void node_update_dev(const LbmConst<float>& K, const float* gr, const float* gb, float ror, float rob,
                           float rr, float rb, CC cc, float& Sr, float& Sb, float* Zr, float* Zb)
{
  using R = float;
  const bool bulk_r = rb <= K.ee;
  const bool bulk_b = !bulk_r && rr <= K.ee;
  R gs[19];
  if (!bulk_r && !bulk_b) {
    R g[19], n[3], Fs[3], F[3];
    csf_force(K, cc, n, Fs);
    R dsum = R(0);
#pragma unroll
    for (int i = 0; i < 19; i++) {
      g[i] = gr[i] + gb[i];
      dsum = dsum + g[i];
    }
    const R r = rr + rb, dr = rr - ror, db = rb - rob;
    const R ci2 = (K.cs2[0] * rr + K.cs2[1] * rb) / r;
    const R ti2 = ci2 * K.c1d6 * K.dt2, ti3 = ci2 * K.c1d12 * K.dt2;
    // t_w r - T_w = t^r_w (rr - ror) + t^b_w (rb - rob) (the weights are linear in cs^2)
    const R dr1 = K.t[0][1] * dr + K.t[1][1] * db, dr2 = K.t[0][2] * dr + K.t[1][2] * db;
    const int ph = rr >= rb ? 0 : 1;
    F[0] = K.bf[ph][0] + Fs[0];
    F[1] = K.bf[ph][1] + Fs[1];
    F[2] = K.bf[ph][2] + Fs[2];
    trt_collide_dev(K, dr1, dr2, dsum, g, gs, r, F, K.S[ph][1], K.S[ph][4]);
    // recolouring (S1:3797-3817): out_r = (f* + B w cos rb) rr / r with f* =
    // T + g*; T_d = t^r_d (ror + rob) + (t^b_d - t^r_d) rob
    const R inv = R(1) / r, qr = rr * inv, qb = rb * inv, ro = ror + rob;
    Sr = qr * ro;
    Sb = qb * ro;
    R cs[19];
    cs[0] = R(0);
    cs[1] = n[0];
    cs[2] = -cs[1];
    cs[3] = n[1];
    cs[4] = -cs[3];
    cs[5] = n[2];
    cs[6] = -cs[5];
    cs[7] = (n[0] + n[1]) * K.cn;
    cs[8] = (-n[0] + n[1]) * K.cn;
    cs[9] = -cs[8];
    cs[10] = -cs[7];
    cs[11] = (n[0] + n[2]) * K.cn;
    cs[12] = (-n[0] + n[2]) * K.cn;
    cs[13] = -cs[12];
    cs[14] = -cs[11];
    cs[15] = (n[1] + n[2]) * K.cn;
    cs[16] = (-n[1] + n[2]) * K.cn;
    cs[17] = -cs[16];
    cs[18] = -cs[15];
    const bool same_w = K.t[0][1] == K.t[1][1];
#pragma unroll
    for (int i = 0; i < 19; i++) {
      const int wc = i == 0 ? 0 : (i < 7 ? 1 : 2);
      const R w = i == 0 ? R(0) : K.B * (i < 7 ? ti2 : ti3) * cs[i];
      Zr[i] = (gs[i] + w * rb) * qr;
      Zb[i] = (gs[i] - w * rr) * qb;
      if (!same_w) {
        const R dtw = K.t[1][wc] - K.t[0][wc];
        Zr[i] = Zr[i] + qr * dtw * rob;
        Zb[i] = Zb[i] - qb * dtw * ror;
      }
    }
  } else {
    // one component collides against its own reference; the other stays at
    // its rest equilibrium t_d rho (S = its density, no deviation)
    const int c = bulk_r ? 0 : 1;
    const float* g = bulk_r ? gr : gb;
    const R ro = bulk_r ? ror : rob, rc = bulk_r ? rr : rb, d = rc - ro;
    R dsum = R(0);
#pragma unroll
    for (int i = 0; i < 19; i++) dsum = dsum + g[i];
    trt_collide_dev(K, K.t[c][1] * d, K.t[c][2] * d, dsum, g, gs, rc, K.bf[c], K.S[c][1], K.S[c][4]);
    float* Zc = bulk_r ? Zr : Zb;
    float* Zo = bulk_r ? Zb : Zr;
#pragma unroll
    for (int i = 0; i < 19; i++) {
      Zc[i] = gs[i];
      Zo[i] = R(0);
    }
    Sr = bulk_r ? ror : rr;
    Sb = bulk_r ? rb : rob;
  }
}

}  // namespace ps
