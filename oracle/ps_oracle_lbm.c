/*
 * ps_oracle_lbm.c -- TEST INFRASTRUCTURE: FP64 CPU restatement of the
 * colour-gradient two-phase D3Q19 step of porescale (S1 =
 * LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f).  Used only as the parity
 * reference for the GPU kernels and as the timed CPU baseline ("port").
 *
 * Compiled with -ffp-contract=off so that every multiply and add rounds
 * separately, as the reference's source expressions do; expressions keep
 * the reference's left-to-right evaluation order.
 */
#include "ps_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D3Q19 velocity set in the order of the shipped `velocities19` file
 * (index 0 here = reference index 1). */
static const int CV[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},
                              {0, 0, 1},  {0, 0, -1}, {1, 1, 0},  {-1, 1, 0},  {1, -1, 0},
                              {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},  {-1, 0, -1},
                              {0, 1, 1},  {0, -1, 1}, {0, 1, -1}, {0, -1, -1}};

struct or_lbm {
  int nx, ny, nz;
  int64_t nl, nps, npb2, npb4, ns;
  int64_t n_overflow; /* diagonal links whose int32 product of node numbers wraps to 0 */
  or_lbm_params p;
  int32_t *ind;   /* after the reference's reset of values > 1 to 1 */
  int32_t *mijk;  /* fluid number (1-based) or 0 */
  int32_t *mijks; /* LSM node number (1-based) or 0 */
  int32_t *icor;  /* 3*nl */
  int32_t *ips, *ipb2, *ipb4;
  int niv[19];
  /* derived constants */
  double cb2, tr[19], tb[19], Sr[19], Sb[19], Fpr[19], Fpb[19];
  double svr, svb, sigs, dt, dti, dt2;
  double *fr, *fb, *pcfr, *pcfb, *rr, *rb, *cf;
};

static inline int64_t vox(const or_lbm *o, int i, int j, int k) /* 1-based */
{
  return (int64_t)(i - 1) + (int64_t)o->nx * ((int64_t)(j - 1) + (int64_t)o->ny * (int64_t)(k - 1));
}

/* periodic wrap of a 1-based coordinate in 0..n+1, the reference's ipc vectors */
static inline int wrap(int c, int n)
{
  if (c < 1) return c + n;
  if (c > n) return c - n;
  return c;
}

/* S1:2858-2893 collmatrTRT */
void or_collmatr_trt(double sv, double S[19])
{
  double sq = 8.0 * (2.0 - sv) / (8.0 - sv);
  double v[19] = {0.0, sv, sv, 0.0, sq, 0.0, sq, 0.0, sq, sv, sv, sv, sv, sv, sv, sv, sq, sq, sq};
  memcpy(S, v, sizeof v);
}

/* S1:2407-2620 collision (operation order kept) */
void or_collision(double t1, double t2, double t3, double *f, double *pcf, double r,
                  const double bf[3], const double Fp[19], const double S[19], double dt,
                  double dti, double dt2)
{
  const double c1d6 = 1.0 / 6.0, c1d12 = 1.0 / 12.0, c5d399 = 5.0 / 399.0,
               c19d399 = 19.0 / 399.0, c11d2394 = 11.0 / 2394.0, c1d63 = 1.0 / 63.0,
               c1d18 = 1.0 / 18.0, c1d36 = 1.0 / 36.0, c4d1197 = 4.0 / 1197.0,
               c1d252 = 1.0 / 252.0, c1d72 = 1.0 / 72.0, c1d24 = 1.0 / 24.0;
  double j[3], u[3], fe[19], fl[19], mo[19], mb[19];
  j[0] = (f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14]) * dti;
  j[1] = (f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18]) * dti;
  j[2] = (f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18]) * dti;
  double dr1 = 1.0 / r;
  u[0] = (j[0] + bf[0] * 0.5 * dt) * dr1;
  u[1] = (j[1] + bf[1] * 0.5 * dt) * dr1;
  u[2] = (j[2] + bf[2] * 0.5 * dt) * dr1;
  double u1x2 = u[0] * u[0], u2x2 = u[1] * u[1], u3x2 = u[2] * u[2];
  double u2 = (u1x2 + u2x2 + u3x2) * 0.5;
  fe[0] = r * (t1 - u2 * dt2);
  double j1d6 = j[0] * c1d6 * dt, j2d6 = j[1] * c1d6 * dt, j3d6 = j[2] * c1d6 * dt;
  double rd4 = r * 0.25 * dt2;
  double com1 = (t2 - u2 * c1d6 * dt2) * r;
  double fe1 = com1 + rd4 * u1x2, fe2 = com1 + rd4 * u2x2, fe3 = com1 + rd4 * u3x2;
  fe[1] = fe1 + j1d6;
  fe[2] = fe1 - j1d6;
  fe[3] = fe2 + j2d6;
  fe[4] = fe2 - j2d6;
  fe[5] = fe3 + j3d6;
  fe[6] = fe3 - j3d6;
  double j1p2 = (j[0] + j[1]) * c1d12 * dt, j1m2 = (j[0] - j[1]) * c1d12 * dt;
  double j1p3 = (j[0] + j[2]) * c1d12 * dt, j1m3 = (j[0] - j[2]) * c1d12 * dt;
  double j2p3 = (j[1] + j[2]) * c1d12 * dt, j2m3 = (j[1] - j[2]) * c1d12 * dt;
  double rd8 = r * 0.125 * dt2;
  double a12p = rd8 * (u[0] + u[1]) * (u[0] + u[1]);
  double a12m = rd8 * (u[0] - u[1]) * (u[0] - u[1]);
  double a13p = rd8 * (u[0] + u[2]) * (u[0] + u[2]);
  double a13m = rd8 * (u[0] - u[2]) * (u[0] - u[2]);
  double a23p = rd8 * (u[1] + u[2]) * (u[1] + u[2]);
  double a23m = rd8 * (u[1] - u[2]) * (u[1] - u[2]);
  double com2 = (t3 - u2 * c1d12 * dt2) * r;
  fe[7] = com2 + j1p2 + a12p;
  fe[10] = com2 - j1p2 + a12p;
  fe[8] = com2 - j1m2 + a12m;
  fe[9] = com2 + j1m2 + a12m;
  fe[11] = com2 + j1p3 + a13p;
  fe[14] = com2 - j1p3 + a13p;
  fe[13] = com2 + j1m3 + a13m;
  fe[12] = com2 - j1m3 + a13m;
  fe[15] = com2 + j2p3 + a23p;
  fe[18] = com2 - j2p3 + a23p;
  fe[17] = com2 + j2m3 + a23m;
  fe[16] = com2 - j2m3 + a23m;
  for (int i = 0; i < 19; i++) fl[i] = f[i] - fe[i];
  double com3 = fl[1] + fl[2] + fl[3] + fl[4] + fl[5] + fl[6];
  double com4 = fl[7] + fl[8] + fl[9] + fl[10] + fl[11] + fl[12] + fl[13] + fl[14] + fl[15] +
                fl[16] + fl[17] + fl[18];
  mo[0] = 0.0;
  mo[1] = -(30.0 * fl[0]) - 11.0 * com3 + 8.0 * com4;
  mo[2] = 12.0 * fl[0] - 4.0 * com3 + com4;
  mo[3] = 0.0;
  mo[4] = 4.0 * (fl[2] - fl[1]) + fl[7] - fl[8] + fl[9] - fl[10] + fl[11] - fl[12] + fl[13] - fl[14];
  mo[5] = 0.0;
  mo[6] = 4.0 * (fl[4] - fl[3]) + fl[7] + fl[8] - fl[9] - fl[10] + fl[15] - fl[16] + fl[17] - fl[18];
  mo[7] = 0.0;
  mo[8] = 4.0 * (fl[6] - fl[5]) + fl[11] + fl[12] - fl[13] - fl[14] + fl[15] + fl[16] - fl[17] - fl[18];
  double com5 = fl[7] + fl[8] + fl[9] + fl[10];
  double com6 = fl[15] + fl[16] + fl[17] + fl[18];
  double com7 = fl[11] + fl[12] + fl[13] + fl[14];
  double com8 = fl[3] + fl[4] - fl[5] - fl[6];
  double com9 = fl[3] + fl[4] + fl[5] + fl[6];
  mo[9] = 2.0 * (fl[1] + fl[2] - com6) - com9 + com5 + com7;
  mo[10] = -(4.0 * (fl[1] + fl[2])) + 2.0 * (com9 - com6) + com5 + com7;
  mo[11] = com8 + com5 - com7;
  mo[12] = -(2.0 * com8) + com5 - com7;
  mo[13] = fl[7] - fl[8] - fl[9] + fl[10];
  mo[14] = fl[15] - fl[16] - fl[17] + fl[18];
  mo[15] = fl[11] - fl[12] - fl[13] + fl[14];
  mo[16] = fl[7] - fl[8] + fl[9] - fl[10] - fl[11] + fl[12] - fl[13] + fl[14];
  mo[17] = -fl[7] - fl[8] + fl[9] + fl[10] + fl[15] - fl[16] + fl[17] - fl[18];
  mo[18] = fl[11] + fl[12] - fl[13] - fl[14] - fl[15] - fl[16] + fl[17] + fl[18];
  for (int i = 0; i < 19; i++) mo[i] = mo[i] * S[i];
  mb[0] = -(c5d399 * mo[1]) + c19d399 * mo[2];
  double com10 = -(c11d2394 * mo[1]) - c1d63 * mo[2];
  mb[1] = com10 - 0.1 * mo[4] + c1d18 * (mo[9] - mo[10]);
  mb[2] = mb[1] + mo[4] * 0.2;
  mb[3] = com10 - 0.1 * mo[6] + c1d36 * (mo[10] - mo[9]) + c1d12 * (mo[11] - mo[12]);
  mb[4] = mb[3] + mo[6] * 0.2;
  mb[5] = com10 - 0.1 * mo[8] + c1d36 * (mo[10] - mo[9]) + c1d12 * (mo[12] - mo[11]);
  mb[6] = mb[5] + mo[8] * 0.2;
  double com11 = c4d1197 * mo[1] + c1d252 * mo[2];
  mb[7] = com11 + (mo[4] + mo[6]) * 0.025 + c1d36 * mo[9] + c1d72 * mo[10] + c1d12 * mo[11] +
          c1d24 * mo[12] + mo[13] * 0.25 + (mo[16] - mo[17]) * 0.125;
  mb[8] = mb[7] - 0.05 * mo[4] - 0.5 * mo[13] - 0.25 * mo[16];
  mb[9] = mb[7] + 0.25 * mo[17] - 0.05 * mo[6] - 0.5 * mo[13];
  mb[10] = mb[9] + 0.5 * mo[13] - 0.05 * mo[4] - 0.25 * mo[16];
  mb[11] = com11 + (mo[4] + mo[8]) * 0.025 + c1d36 * mo[9] + c1d72 * mo[10] - c1d12 * mo[11] -
           c1d24 * mo[12] + mo[15] * 0.25 + (mo[18] - mo[16]) * 0.125;
  mb[12] = mb[11] + 0.25 * mo[16] - 0.5 * mo[15] - 0.05 * mo[4];
  mb[13] = mb[11] - 0.05 * mo[8] - 0.5 * mo[15] - 0.25 * mo[18];
  mb[14] = mb[12] + 0.5 * mo[15] - 0.05 * mo[8] - 0.25 * mo[18];
  mb[15] = com11 + (mo[6] + mo[8]) * 0.025 - c1d18 * mo[9] - c1d36 * mo[10] + mo[14] * 0.25 +
           (mo[17] - mo[18]) * 0.125;
  mb[16] = mb[15] - 0.05 * mo[6] - 0.5 * mo[14] - 0.25 * mo[17];
  mb[17] = mb[15] + 0.25 * mo[18] - 0.05 * mo[8] - 0.5 * mo[14];
  mb[18] = mb[17] + 0.5 * mo[14] - 0.05 * mo[6] - 0.25 * mo[17];
  f[0] = f[0] - mb[0] + Fp[0];
  for (int i = 1; i < 19; i++) pcf[i] = f[i] - mb[i] + Fp[i];
}

/* S1:2626-2796 calcFs.  c(i,j,k) = ind*(cf-wet)+wet over the periodic 3^3
 * neighbourhood; solid voxels (and voxels outside the fluid list, where the
 * reference reads cf(0)) take the wetting colour. */
static void or_calcfs(const or_lbm *o, int ix, int iy, int iz, double Cg[3], double Fs[3])
{
  const double wet = o->p.wet;
  double c[3][3][3]; /* c[k][j][i], i = x offset */
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        int x = wrap(ix + i - 1, o->nx), y = wrap(iy + j - 1, o->ny), z = wrap(iz + k - 1, o->nz);
        int64_t v = vox(o, x, y, z);
        int32_t m = o->mijk[v];
        if (o->ind[v] != 0 && m != 0)
          c[k][j][i] = (double)o->ind[v] * (o->cf[m - 1] - wet) + wet;
        else
          c[k][j][i] = wet;
      }
#define C(i, j, k) c[(k)-1][(j)-1][(i)-1]
  double r11 = C(1, 1, 1) + C(2, 1, 1), r12 = C(2, 1, 1) + C(3, 1, 1), r13 = C(1, 2, 1) + C(2, 2, 1);
  double r14 = C(2, 2, 1) + C(3, 2, 1), r15 = C(1, 3, 1) + C(2, 3, 1), r16 = C(2, 3, 1) + C(3, 3, 1);
  double r17 = C(1, 1, 1) + C(1, 2, 1), r18 = C(2, 1, 1) + C(2, 2, 1), r19 = C(3, 1, 1) + C(3, 2, 1);
  double r110 = C(1, 2, 1) + C(1, 3, 1), r111 = C(2, 2, 1) + C(2, 3, 1), r112 = C(3, 2, 1) + C(3, 3, 1);
  double r21 = C(1, 1, 2) + C(2, 1, 2), r22 = C(2, 1, 2) + C(3, 1, 2), r23 = C(1, 2, 2) + C(2, 2, 2);
  double r24 = C(2, 2, 2) + C(3, 2, 2), r25 = C(1, 3, 2) + C(2, 3, 2), r26 = C(2, 3, 2) + C(3, 3, 2);
  double r27 = C(1, 1, 2) + C(1, 2, 2), r28 = C(2, 1, 2) + C(2, 2, 2), r29 = C(3, 1, 2) + C(3, 2, 2);
  double r210 = C(1, 2, 2) + C(1, 3, 2), r211 = C(2, 2, 2) + C(2, 3, 2), r212 = C(3, 2, 2) + C(3, 3, 2);
  double r31 = C(1, 1, 3) + C(2, 1, 3), r32 = C(2, 1, 3) + C(3, 1, 3), r33 = C(1, 2, 3) + C(2, 2, 3);
  double r34 = C(2, 2, 3) + C(3, 2, 3), r35 = C(1, 3, 3) + C(2, 3, 3), r36 = C(2, 3, 3) + C(3, 3, 3);
  double r37 = C(1, 1, 3) + C(1, 2, 3), r38 = C(2, 1, 3) + C(2, 2, 3), r39 = C(3, 1, 3) + C(3, 2, 3);
  double r310 = C(1, 2, 3) + C(1, 3, 3), r311 = C(2, 2, 3) + C(2, 3, 3), r312 = C(3, 2, 3) + C(3, 3, 3);
#undef C
  double g12 = r18 + r28, g13 = r13 + r23, g34 = r111 + r211, g24 = r14 + r24;
  double g15 = r21 + r23, g37 = r23 + r25, g48 = r24 + r26, g26 = r22 + r24;
  double g56 = r28 + r38, g57 = r23 + r33, g78 = r211 + r311, g68 = r24 + r34;
  double nm[8][3];
  nm[0][0] = g12 - (r17 + r27);
  nm[1][0] = r19 + r29 - g12;
  nm[2][0] = g34 - (r110 + r210);
  nm[3][0] = r112 + r212 - g34;
  nm[4][0] = g56 - (r27 + r37);
  nm[5][0] = r29 + r39 - g56;
  nm[6][0] = g78 - (r210 + r310);
  nm[7][0] = r212 + r312 - g78;
  nm[0][1] = g13 - (r11 + r21);
  nm[1][1] = g24 - (r12 + r22);
  nm[2][1] = r15 + r25 - g13;
  nm[3][1] = r16 + r26 - g24;
  nm[4][1] = g57 - (r21 + r31);
  nm[5][1] = g68 - (r22 + r32);
  nm[6][1] = r25 + r35 - g57;
  nm[7][1] = r26 + r36 - g68;
  nm[0][2] = g15 - (r11 + r13);
  nm[1][2] = g26 - (r12 + r14);
  nm[2][2] = g37 - (r13 + r15);
  nm[3][2] = g48 - (r14 + r16);
  nm[4][2] = r31 + r33 - g15;
  nm[5][2] = r32 + r34 - g26;
  nm[6][2] = r33 + r35 - g37;
  nm[7][2] = r34 + r36 - g48;
  for (int d = 0; d < 3; d++)
    Cg[d] = nm[0][d] + nm[1][d] + nm[2][d] + nm[3][d] + nm[4][d] + nm[5][d] + nm[6][d] + nm[7][d];
  double normc = sqrt(Cg[0] * Cg[0] + Cg[1] * Cg[1] + Cg[2] * Cg[2]);
  double dn0 = nm[1][0] + nm[3][0] + nm[5][0] + nm[7][0] - nm[0][0] - nm[2][0] - nm[4][0] - nm[6][0];
  double dn1 = nm[3][1] + nm[7][1] + nm[2][1] + nm[6][1] - nm[0][1] - nm[1][1] - nm[4][1] - nm[5][1];
  double dn2 = nm[4][2] + nm[5][2] + nm[6][2] + nm[7][2] - nm[0][2] - nm[1][2] - nm[2][2] - nm[3][2];
  double k1 = dn0 + dn1 + dn2;
  double mm[8];
  for (int i = 0; i < 8; i++) mm[i] = sqrt(nm[i][0] * nm[i][0] + nm[i][1] * nm[i][1] + nm[i][2] * nm[i][2]);
  double dm0 = mm[1] + mm[3] + mm[5] + mm[7] - mm[0] - mm[2] - mm[4] - mm[6];
  double dm1 = mm[3] + mm[7] + mm[2] + mm[6] - mm[0] - mm[1] - mm[4] - mm[5];
  double dm2 = mm[4] + mm[5] + mm[6] + mm[7] - mm[0] - mm[1] - mm[2] - mm[3];
  double k2 = Cg[0] * dm0 + Cg[1] * dm1 + Cg[2] * dm2;
  if (normc != 0.0) {
    k2 = k2 / normc;
    Cg[0] = Cg[0] / normc;
    Cg[1] = Cg[1] / normc;
    Cg[2] = Cg[2] / normc;
  }
  double s = o->sigs * (k2 - k1);
  Fs[0] = s * Cg[0];
  Fs[1] = s * Cg[1];
  Fs[2] = s * Cg[2];
}

or_lbm *or_lbm_create(const or_lbm_params *p, const int32_t *ind_in, int nx, int ny, int nz)
{
  or_lbm *o = (or_lbm *)calloc(1, sizeof(or_lbm));
  o->nx = nx;
  o->ny = ny;
  o->nz = nz;
  o->p = *p;
  int64_t nv = (int64_t)nx * ny * nz;
  /* --- LSM corner dilation for mijks (S1:541-602, 647-660) --- */
  int32_t *ind1 = (int32_t *)malloc(sizeof(int32_t) * nv);
  for (int64_t v = 0; v < nv; v++) ind1[v] = ind_in[v] > 1 ? 1 : ind_in[v];
  int ax = nx + 1, ay = ny + 1, az = nz + 1;
  int32_t *inda = (int32_t *)malloc(sizeof(int32_t) * (int64_t)ax * ay * az);
#define IA(i, j, k) inda[((int64_t)(k)-1) * ax * ay + ((int64_t)(j)-1) * ax + ((i)-1)]
  for (int64_t v = 0; v < (int64_t)ax * ay * az; v++) inda[v] = 1;
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        if (ind1[vox(o, i, j, k)] == 0)
          for (int dk = 0; dk < 2; dk++)
            for (int dj = 0; dj < 2; dj++)
              for (int di = 0; di < 2; di++) IA(i + di, j + dj, k + dk) = 0;
  for (int j = 1; j <= ny + 1; j++)
    for (int k = 1; k <= nz + 1; k++) {
      int a = IA(1, j, k), b = IA(nx + 1, j, k);
      IA(1, j, k) = a < b ? a : b;
    }
  for (int i = 1; i <= nx + 1; i++)
    for (int k = 1; k <= nz + 1; k++) {
      int a = IA(i, 1, k), b = IA(i, ny + 1, k);
      IA(i, 1, k) = a < b ? a : b;
    }
  for (int i = 1; i <= nx + 1; i++)
    for (int j = 1; j <= ny + 1; j++) {
      int a = IA(i, j, 1), b = IA(i, j, nz + 1);
      IA(i, j, 1) = a < b ? a : b;
    }
  o->mijks = (int32_t *)calloc(nv, sizeof(int32_t));
  int64_t ns = 0;
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        if (IA(i, j, k) == 0) o->mijks[vox(o, i, j, k)] = (int32_t)(++ns);
#undef IA
  free(inda);
  o->ns = ns;
  /* --- fluid list, i-j-k order with k fastest (S1:1036-1072) --- */
  o->mijk = (int32_t *)calloc(nv, sizeof(int32_t));
  int64_t nl = 0;
  for (int i = 1; i <= nx; i++)
    for (int j = 1; j <= ny; j++)
      for (int k = 1; k <= nz; k++)
        if (ind_in[vox(o, i, j, k)] == p->iipore) nl++;
  o->nl = nl;
  o->icor = (int32_t *)malloc(sizeof(int32_t) * 3 * (nl > 0 ? nl : 1));
  nl = 0;
  for (int i = 1; i <= nx; i++)
    for (int j = 1; j <= ny; j++)
      for (int k = 1; k <= nz; k++)
        if (ind_in[vox(o, i, j, k)] == p->iipore) {
          o->icor[3 * nl] = i;
          o->icor[3 * nl + 1] = j;
          o->icor[3 * nl + 2] = k;
          o->mijk[vox(o, i, j, k)] = (int32_t)(++nl);
        }
  /* niv: opposite velocities (S1:514-522) */
  for (int a = 0; a < 19; a++)
    for (int b = 0; b < 19; b++)
      if (CV[a][0] + CV[b][0] == 0 && CV[a][1] + CV[b][1] == 0 && CV[a][2] + CV[b][2] == 0) o->niv[a] = b + 1;
  /* --- propagation tables (S1:1077-1340), counted then filled in one pass --- */
  o->ips = (int32_t *)malloc(sizeof(int32_t) * 3 * (18 * nl + 1));
  o->ipb2 = (int32_t *)malloc(sizeof(int32_t) * 4 * (18 * nl + 1));
  o->ipb4 = (int32_t *)malloc(sizeof(int32_t) * 6 * (18 * nl + 1));
  int64_t nps = 0, npb2 = 0, npb4 = 0;
#define MK(x, y, z) o->mijk[vox(o, wrap(x, nx), wrap(y, ny), wrap(z, nz))]
#define MS(x, y, z) o->mijks[vox(o, wrap(x, nx), wrap(y, ny), wrap(z, nz))]
  for (int64_t n = 0; n < nl; n++) {
    int ix = o->icor[3 * n], iy = o->icor[3 * n + 1], iz = o->icor[3 * n + 2];
    for (int d = 1; d < 7; d++) { /* axis links, j = 2..7 */
      int tx = ix + CV[d][0], ty = iy + CV[d][1], tz = iz + CV[d][2];
      if (MK(tx, ty, tz) != 0) {
        o->ips[3 * nps] = (int32_t)(n + 1);
        o->ips[3 * nps + 1] = MK(tx, ty, tz);
        o->ips[3 * nps + 2] = d + 1;
        nps++;
      } else {
        /* the four LSM nodes at the corners of the wall face */
        int h[4][3];
        int ax_ = CV[d][0] != 0 ? 0 : (CV[d][1] != 0 ? 1 : 2);
        int off = (CV[d][ax_] + 1) / 2;
        int q[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
        for (int c = 0; c < 4; c++) {
          int e[3] = {0, 0, 0};
          e[ax_] = off;
          if (ax_ == 0) { e[1] = q[c][0]; e[2] = q[c][1]; }
          else if (ax_ == 1) { e[0] = q[c][0]; e[2] = q[c][1]; }
          else { e[0] = q[c][0]; e[1] = q[c][1]; }
          h[c][0] = ix + e[0];
          h[c][1] = iy + e[1];
          h[c][2] = iz + e[2];
        }
        int32_t *r = o->ipb4 + 6 * npb4;
        r[0] = (int32_t)(n + 1);
        r[1] = o->niv[d];
        for (int c = 0; c < 4; c++) r[2 + c] = MS(h[c][0], h[c][1], h[c][2]);
        npb4++;
      }
    }
    for (int d = 7; d < 19; d++) { /* diagonal links, j = 8..19 */
      int tx = ix + CV[d][0], ty = iy + CV[d][1], tz = iz + CV[d][2];
      int stream = 0;
      if (MK(tx, ty, tz) != 0) {
        int64_t a = MK(ix + CV[d][0], iy, iz), b = MK(ix, iy + CV[d][1], iz), c = MK(ix, iy, iz + CV[d][2]);
        stream = (a * b * c) != 0;
        /* S1:1121 forms this product in 32-bit integers; count the links where
         * that product would wrap to zero (the intended test is used here) */
        if (stream && (uint32_t)((uint32_t)a * (uint32_t)b * (uint32_t)c) == 0u) o->n_overflow++;
      }
      if (stream) {
        o->ips[3 * nps] = (int32_t)(n + 1);
        o->ips[3 * nps + 1] = MK(tx, ty, tz);
        o->ips[3 * nps + 2] = d + 1;
        nps++;
      } else {
        /* the two LSM nodes at the ends of the wall edge */
        int e1[3], e2[3];
        if (CV[d][0] == 0) {
          e1[0] = 0; e1[1] = (CV[d][1] + 1) / 2; e1[2] = (CV[d][2] + 1) / 2;
          e2[0] = 1; e2[1] = e1[1]; e2[2] = e1[2];
        } else if (CV[d][1] == 0) {
          e1[0] = (CV[d][0] + 1) / 2; e1[1] = 0; e1[2] = (CV[d][2] + 1) / 2;
          e2[0] = e1[0]; e2[1] = 1; e2[2] = e1[2];
        } else {
          e1[0] = (CV[d][0] + 1) / 2; e1[1] = (CV[d][1] + 1) / 2; e1[2] = 0;
          e2[0] = e1[0]; e2[1] = e1[1]; e2[2] = 1;
        }
        int32_t *r = o->ipb2 + 4 * npb2;
        r[0] = (int32_t)(n + 1);
        r[1] = o->niv[d];
        r[2] = MS(ix + e1[0], iy + e1[1], iz + e1[2]);
        r[3] = MS(ix + e2[0], iy + e2[1], iz + e2[2]);
        npb2++;
      }
    }
  }
#undef MK
#undef MS
  o->nps = nps;
  o->npb2 = npb2;
  o->npb4 = npb4;
  o->ind = ind1; /* values > 1 reset to 1 (S1:1327-1335) */
  /* --- constants (S1:1355-1382, 3411-3431) --- */
  o->dt = p->dt;
  o->dti = 1.0 / p->dt;
  o->dt2 = p->dt * p->dt;
  o->sigs = 0.03125 * p->sig;
  o->cb2 = p->rr0 * p->cr2 / p->rb0;
  double dt = p->dt;
  double tr1 = 1.0 - 2.0 * p->cr2 * dt * dt, tr2 = p->cr2 * dt * dt * (1.0 / 6.0),
         tr3 = p->cr2 * dt * dt * (1.0 / 12.0);
  double tb1 = 1.0 - 2.0 * o->cb2 * dt * dt, tb2 = o->cb2 * dt * dt * (1.0 / 6.0),
         tb3 = o->cb2 * dt * dt * (1.0 / 12.0);
  for (int i = 0; i < 19; i++) {
    o->tr[i] = i == 0 ? tr1 : (i < 7 ? tr2 : tr3);
    o->tb[i] = i == 0 ? tb1 : (i < 7 ? tb2 : tb3);
  }
  o->svr = 1.0 / (3.0 * p->vir * dt + 0.5);
  o->svb = 1.0 / (3.0 * p->vib * dt + 0.5);
  or_collmatr_trt(o->svr, o->Sr);
  or_collmatr_trt(o->svb, o->Sb);
  for (int i = 0; i < 19; i++) {
    double rk = i == 0 ? 1.0 : (i < 7 ? 1.0 / 6.0 : 1.0 / 12.0);
    double mr = (double)CV[i][0] * p->bfr[0] + (double)CV[i][1] * p->bfr[1] + (double)CV[i][2] * p->bfr[2];
    double mb = (double)CV[i][0] * p->bfb[0] + (double)CV[i][1] * p->bfb[1] + (double)CV[i][2] * p->bfb[2];
    o->Fpr[i] = rk * mr * o->dt2;
    o->Fpb[i] = rk * mb * o->dt2;
  }
  size_t sz = sizeof(double) * 19 * (nl > 0 ? nl : 1);
  o->fr = (double *)calloc(1, sz);
  o->fb = (double *)calloc(1, sz);
  o->pcfr = (double *)calloc(1, sz);
  o->pcfb = (double *)calloc(1, sz);
  o->rr = (double *)calloc(nl + 1, sizeof(double));
  o->rb = (double *)calloc(nl + 1, sizeof(double));
  o->cf = (double *)calloc(nl + 1, sizeof(double));
  return o;
}

void or_lbm_destroy(or_lbm *o)
{
  if (!o) return;
  free(o->ind); free(o->mijk); free(o->mijks); free(o->icor);
  free(o->ips); free(o->ipb2); free(o->ipb4);
  free(o->fr); free(o->fb); free(o->pcfr); free(o->pcfb);
  free(o->rr); free(o->rb); free(o->cf);
  free(o);
}

void or_lbm_sizes(const or_lbm *o, int64_t out[6])
{
  out[0] = o->nl; out[1] = o->nps; out[2] = o->npb2; out[3] = o->npb4; out[4] = o->ns;
  out[5] = o->n_overflow;
}

void or_lbm_tables(const or_lbm *o, int32_t *icor, int32_t *ips, int32_t *ipb2, int32_t *ipb4,
                   int32_t *mijk, int32_t *mijks)
{
  int64_t nv = (int64_t)o->nx * o->ny * o->nz;
  if (icor) memcpy(icor, o->icor, sizeof(int32_t) * 3 * o->nl);
  if (ips) memcpy(ips, o->ips, sizeof(int32_t) * 3 * o->nps);
  if (ipb2) memcpy(ipb2, o->ipb2, sizeof(int32_t) * 4 * o->npb2);
  if (ipb4) memcpy(ipb4, o->ipb4, sizeof(int32_t) * 6 * o->npb4);
  if (mijk) memcpy(mijk, o->mijk, sizeof(int32_t) * nv);
  if (mijks) memcpy(mijks, o->mijks, sizeof(int32_t) * nv);
}

/* densities and colour field (S1:3436-3447, 3934-3945) */
static void or_densities(or_lbm *o, int nthreads)
{
  (void)nthreads;
  int64_t nl = o->nl;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t i = 0; i < nl; i++) {
    const double *a = o->fr + 19 * i, *b = o->fb + 19 * i;
    double sr = a[0], sb = b[0];
    for (int d = 1; d < 19; d++) { sr = sr + a[d]; sb = sb + b[d]; }
    o->rr[i] = sr;
    o->rb[i] = sb;
    o->cf[i] = (sr - sb) / (sr + sb);
  }
}

/* S1:2800-2854 initdistr, icon = 0 */
void or_lbm_init_random(or_lbm *o, double sat)
{
  double seed = 13.081984;
  const double m31 = 2147483647.0, p31 = 2147483648.0;
  for (int64_t i = 0; i < o->nl; i++) {
    seed = fmod(16807.0 * seed, m31);
    double rn = seed / p31;
    double cfield = rn <= sat ? 0.0 : 1.0;
    for (int d = 0; d < 19; d++) {
      o->fr[19 * i + d] = o->tr[d] * cfield * o->p.rr0;
      o->fb[19 * i + d] = o->tb[d] * (1.0 - cfield) * o->p.rb0;
    }
  }
  or_densities(o, 1);
}

void or_lbm_set_state(or_lbm *o, const double *fr, const double *fb)
{
  memcpy(o->fr, fr, sizeof(double) * 19 * o->nl);
  memcpy(o->fb, fb, sizeof(double) * 19 * o->nl);
  or_densities(o, 1);
}

void or_lbm_get_state(const or_lbm *o, double *fr, double *fb)
{
  memcpy(fr, o->fr, sizeof(double) * 19 * o->nl);
  memcpy(fb, o->fb, sizeof(double) * 19 * o->nl);
}

void or_lbm_fields(const or_lbm *o, double *rr, double *rb, double *cf)
{
  if (rr) memcpy(rr, o->rr, sizeof(double) * o->nl);
  if (rb) memcpy(rb, o->rb, sizeof(double) * o->nl);
  if (cf) memcpy(cf, o->cf, sizeof(double) * o->nl);
}

/* one node of the collision loop S1:3663-3819 (majority rule, mtype = 0) */
static void or_node_collide(or_lbm *o, int64_t i)
{
  const or_lbm_params *p = &o->p;
  const double dt = o->dt, dti = o->dti, dt2 = o->dt2;
  const double cn = 1.0 / sqrt(2.0);
  double *fr = o->fr + 19 * i, *fb = o->fb + 19 * i;
  double *pcfr = o->pcfr + 19 * i, *pcfb = o->pcfb + 19 * i;
  double rr = o->rr[i], rb = o->rb[i];
  if (rb <= p->ee) {
    or_collision(o->tr[0], o->tr[1], o->tr[7], fr, pcfr, rr, p->bfr, o->Fpr, o->Sr, dt, dti, dt2);
    fb[0] = o->tb[0] * rb;
    for (int d = 1; d < 19; d++) pcfb[d] = o->tb[d] * rb;
  } else if (rr <= p->ee) {
    or_collision(o->tb[0], o->tb[1], o->tb[7], fb, pcfb, rb, p->bfb, o->Fpb, o->Sb, dt, dti, dt2);
    fr[0] = o->tr[0] * rr;
    for (int d = 1; d < 19; d++) pcfr[d] = o->tr[d] * rr;
  } else {
    double Cg[3], Fs[3], f[19], pcf[19], bfi[3], Fpi[19];
    or_calcfs(o, o->icor[3 * i], o->icor[3 * i + 1], o->icor[3 * i + 2], Cg, Fs);
    for (int d = 0; d < 19; d++) f[d] = fr[d] + fb[d];
    double ri = rr + rb;
    double ci2 = (p->cr2 * rr + o->cb2 * rb) / ri;
    double ti1 = 1.0 - 2.0 * ci2 * dt2, ti2 = ci2 * (1.0 / 6.0) * dt2, ti3 = ci2 * (1.0 / 12.0) * dt2;
    const double *bfp = rr >= rb ? p->bfr : p->bfb;
    const double *S = rr >= rb ? o->Sr : o->Sb;
    for (int d = 0; d < 3; d++) bfi[d] = bfp[d] + Fs[d];
    const double c6 = 1.0 / 6.0, c12 = 1.0 / 12.0;
    Fpi[0] = 0.0;
    Fpi[1] = c6 * bfi[0] * dt2;
    Fpi[2] = -Fpi[1];
    Fpi[3] = c6 * bfi[1] * dt2;
    Fpi[4] = -Fpi[3];
    Fpi[5] = c6 * bfi[2] * dt2;
    Fpi[6] = -Fpi[5];
    Fpi[7] = c12 * (bfi[0] + bfi[1]) * dt2;
    Fpi[8] = c12 * (-bfi[0] + bfi[1]) * dt2;
    Fpi[9] = -Fpi[8];
    Fpi[10] = -Fpi[7];
    Fpi[11] = c12 * (bfi[0] + bfi[2]) * dt2;
    Fpi[12] = c12 * (-bfi[0] + bfi[2]) * dt2;
    Fpi[13] = -Fpi[12];
    Fpi[14] = -Fpi[11];
    Fpi[15] = c12 * (bfi[1] + bfi[2]) * dt2;
    Fpi[16] = c12 * (-bfi[1] + bfi[2]) * dt2;
    Fpi[17] = -Fpi[16];
    Fpi[18] = -Fpi[15];
    or_collision(ti1, ti2, ti3, f, pcf, ri, bfi, Fpi, S, dt, dti, dt2);
    double cosf[18];
    cosf[0] = Cg[0];
    cosf[1] = -cosf[0];
    cosf[2] = Cg[1];
    cosf[3] = -cosf[2];
    cosf[4] = Cg[2];
    cosf[5] = -cosf[4];
    cosf[6] = (Cg[0] + Cg[1]) * cn;
    cosf[7] = (-Cg[0] + Cg[1]) * cn;
    cosf[8] = -cosf[7];
    cosf[9] = -cosf[6];
    cosf[10] = (Cg[0] + Cg[2]) * cn;
    cosf[11] = (-Cg[0] + Cg[2]) * cn;
    cosf[12] = -cosf[11];
    cosf[13] = -cosf[10];
    cosf[14] = (Cg[1] + Cg[2]) * cn;
    cosf[15] = (-Cg[1] + Cg[2]) * cn;
    cosf[16] = -cosf[15];
    cosf[17] = -cosf[14];
    fr[0] = f[0] * rr / ri;
    fb[0] = f[0] * rb / ri;
    for (int d = 1; d < 19; d++) {
      double tw = d < 7 ? ti2 : ti3;
      pcfr[d] = (pcf[d] + p->B * tw * cosf[d - 1] * rb) * rr / ri;
      pcfb[d] = (pcf[d] - p->B * tw * cosf[d - 1] * rr) * rb / ri;
    }
  }
}

void or_lbm_run(or_lbm *o, int nsteps, int nthreads)
{
  if (nthreads < 1) nthreads = 1;
  int64_t nl = o->nl;
  for (int s = 0; s < nsteps; s++) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t i = 0; i < nl; i++) or_node_collide(o, i);
    /* ips streaming S1:3833-3839 */
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t e = 0; e < o->nps; e++) {
      int64_t from = o->ips[3 * e] - 1, to = o->ips[3 * e + 1] - 1;
      int d = o->ips[3 * e + 2] - 1;
      o->fr[19 * to + d] = o->pcfr[19 * from + d];
      o->fb[19 * to + d] = o->pcfb[19 * from + d];
    }
    /* half-way bounce-back S1:3890-3915 */
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t e = 0; e < o->npb2; e++) {
      int64_t n = o->ipb2[4 * e] - 1;
      int d = o->ipb2[4 * e + 1] - 1, dback = o->niv[d] - 1;
      o->fr[19 * n + d] = o->pcfr[19 * n + dback];
      o->fb[19 * n + d] = o->pcfb[19 * n + dback];
    }
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t e = 0; e < o->npb4; e++) {
      int64_t n = o->ipb4[6 * e] - 1;
      int d = o->ipb4[6 * e + 1] - 1, dback = o->niv[d] - 1;
      o->fr[19 * n + d] = o->pcfr[19 * n + dback];
      o->fb[19 * n + d] = o->pcfb[19 * n + dback];
    }
    or_densities(o, nthreads);
  }
}

/* check_state reductions (S1:2988-3202).  out[]:
 *  0 tmr, 1 tmb, 2 tm, 3 Cpr, 4 Cpb, 5 nr, 6 nb (rr>=rb / rr<rb counts),
 *  7..9 Qr/t0, 10..12 Qb/t0, 13..15 um/t0, 16..18 umr, 19..21 umb,
 *  22..24 tfr, 25..27 tfb, 28..30 bmt, 31..33 rmt, 34 isneg,
 *  35 nneg_rr, 36 nneg_rb, 37 permr, 38 permb, 39 nr_cf, 40 nb_cf */
void or_lbm_observables(const or_lbm *o, double *out)
{
  const or_lbm_params *p = &o->p;
  const double dt = o->dt, dti = o->dti;
  double tmr = 0, tmb = 0, tm = 0, Cpr = 0, Cpb = 0, nr = 0, nb = 0;
  for (int64_t i = 0; i < o->nl; i++) {
    tmr = tmr + o->rr[i];
    tmb = tmb + o->rb[i];
    tm = tm + o->rr[i] + o->rb[i];
    if (o->cf[i] > 0.99) { nr = nr + 1.0; Cpr = Cpr + o->rr[i]; }
    else if (o->cf[i] < -0.99) { nb = nb + 1.0; Cpb = Cpb + o->rb[i]; }
  }
  double nr_cf = nr, nb_cf = nb;
  Cpr = p->cr2 * Cpr / nr;
  Cpb = o->cb2 * Cpb / nb;
  nr = 0; nb = 0;
  double Qr[3] = {0, 0, 0}, Qb[3] = {0, 0, 0}, um[3] = {0, 0, 0}, umr[3] = {0, 0, 0}, umb[3] = {0, 0, 0};
  double tfr[3] = {0, 0, 0}, tfb[3] = {0, 0, 0}, bmt[3] = {0, 0, 0}, rmt[3] = {0, 0, 0};
  double isneg = 0, nnr = 0, nnb = 0;
  for (int64_t i = 0; i < o->nl; i++) {
    const double *a = o->fr + 19 * i, *b = o->fb + 19 * i;
    for (int d = 0; d < 19; d++)
      if (b[d] < 0.0 || a[d] < 0.0) isneg = 1;
    if (o->rr[i] < 0.0) nnr += 1;
    if (o->rb[i] < 0.0) nnb += 1;
    /* bubble-test momenta, including the reference's precedence (only the last
     * population is scaled by dti) */
    const double *f = b;
    double jm[3];
    jm[0] = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] * dti;
    jm[1] = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] * dti;
    jm[2] = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] * dti;
    for (int d = 0; d < 3; d++) bmt[d] = bmt[d] + jm[d];
    f = a;
    jm[0] = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] * dti;
    jm[1] = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] * dti;
    jm[2] = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] * dti;
    for (int d = 0; d < 3; d++) rmt[d] = rmt[d] + jm[d];
    double Cg[3], Fs[3], g[19], bfi[3];
    or_calcfs(o, o->icor[3 * i], o->icor[3 * i + 1], o->icor[3 * i + 2], Cg, Fs);
    for (int d = 0; d < 19; d++) g[d] = a[d] + b[d];
    double ri = 1.0 / (o->rr[i] + o->rb[i]);
    int red = o->rr[i] >= o->rb[i];
    const double *bfp = red ? p->bfr : p->bfb;
    for (int d = 0; d < 3; d++) bfi[d] = dt * (bfp[d] + Fs[d]) * 0.5;
    jm[0] = (g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14] + bfi[0]) * dti;
    jm[1] = (g[3] - g[4] + g[7] + g[8] - g[9] - g[10] + g[15] - g[16] + g[17] - g[18] + bfi[1]) * dti;
    jm[2] = (g[5] - g[6] + g[11] + g[12] - g[13] - g[14] + g[15] + g[16] - g[17] - g[18] + bfi[2]) * dti;
    if (red) {
      for (int d = 0; d < 3; d++) {
        Qr[d] = Qr[d] + jm[d];
        um[d] = um[d] + jm[d] * ri;
        umr[d] = umr[d] + jm[d] * ri;
        tfr[d] = tfr[d] + bfi[d];
      }
      nr = nr + 1;
    } else {
      for (int d = 0; d < 3; d++) {
        Qb[d] = Qb[d] + jm[d];
        um[d] = um[d] + jm[d] * ri;
        umb[d] = umb[d] + jm[d] * ri;
        tfb[d] = tfb[d] + bfi[d];
      }
      nb = nb + 1;
    }
  }
  double t0 = (double)o->nx * o->ny * o->nz;
  for (int d = 0; d < 3; d++) { Qr[d] = Qr[d] / t0; Qb[d] = Qb[d] / t0; um[d] = um[d] / t0; }
  /* viscosities as re-derived from the relaxation rates (S1:3419-3420) */
  double vir = dti * (1.0 / o->svr - 0.5) / 3.0, vib = dti * (1.0 / o->svb - 0.5) / 3.0;
  int id = p->idir - 1;
  double permr = Qr[id] * vir / p->bfr[id], permb = Qb[id] * vib / p->bfb[id];
  double v[41] = {tmr, tmb, tm, Cpr, Cpb, nr, nb};
  for (int d = 0; d < 3; d++) {
    v[7 + d] = Qr[d]; v[10 + d] = Qb[d]; v[13 + d] = um[d]; v[16 + d] = umr[d]; v[19 + d] = umb[d];
    v[22 + d] = tfr[d]; v[25 + d] = tfb[d]; v[28 + d] = bmt[d]; v[31 + d] = rmt[d];
  }
  v[34] = isneg; v[35] = nnr; v[36] = nnb; v[37] = permr; v[38] = permb; v[39] = nr_cf; v[40] = nb_cf;
  memcpy(out, v, sizeof v);
}

/* S1:3849-3882: afdat = 0, then for every ipb2 entry (node n, incoming
 * direction d, LSM nodes n3 n4) floc = -2((pcfr + pcfb)(niv(d), n) - ppp
 * fq(d)) vv(:, d) rsdti2 is added with weight 0.5 to both nodes, then for
 * every ipb4 entry with weight 0.25 to its four nodes.  fq (S1:3417) and
 * rsdti2 = rsi dti dti (S1:3413), ppp = 0.99 (S1:3406). */
void or_lbm_wall_load(const or_lbm *o, double rsi, double *afdat)
{
  const double dt2 = o->dt2, dti = o->dti;
  const double c1d6 = 1.0 / 6.0, c1d12 = 1.0 / 12.0, ppp = 0.99;
  double fq[19];
  fq[0] = o->p.rr0 * 0.0;
  for (int d = 1; d < 19; d++) fq[d] = o->p.rr0 * (o->p.cr2 * (d < 7 ? c1d6 : c1d12) * dt2);
  const double rsdti2 = rsi * dti * dti;
  for (int64_t i = 0; i < 3 * o->ns; i++) afdat[i] = 0.0;
  for (int64_t e = 0; e < o->npb2; e++) {
    const int32_t *r = o->ipb2 + 4 * e;
    const int64_t n = r[0] - 1;
    const int d = r[1] - 1, db = o->niv[d] - 1;
    const double q = (o->pcfr[19 * n + db] + o->pcfb[19 * n + db]) - ppp * fq[d];
    for (int c = 0; c < 3; c++) {
      const double floc = -2.0 * q * (double)CV[d][c] * rsdti2;
      afdat[3 * (int64_t)(r[2] - 1) + c] = afdat[3 * (int64_t)(r[2] - 1) + c] + floc * 0.5;
      afdat[3 * (int64_t)(r[3] - 1) + c] = afdat[3 * (int64_t)(r[3] - 1) + c] + floc * 0.5;
    }
  }
  for (int64_t e = 0; e < o->npb4; e++) {
    const int32_t *r = o->ipb4 + 6 * e;
    const int64_t n = r[0] - 1;
    const int d = r[1] - 1, db = o->niv[d] - 1;
    const double q = (o->pcfr[19 * n + db] + o->pcfb[19 * n + db]) - ppp * fq[d];
    for (int c = 0; c < 3; c++) {
      const double floc = -2.0 * q * (double)CV[d][c] * rsdti2;
      for (int k = 2; k < 6; k++) afdat[3 * (int64_t)(r[k] - 1) + c] = afdat[3 * (int64_t)(r[k] - 1) + c] + floc * 0.25;
    }
  }
}
