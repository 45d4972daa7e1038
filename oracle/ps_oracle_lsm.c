/*
 * ps_oracle_lsm.c -- TEST INFRASTRUCTURE: FP64 CPU restatement of the
 * two-solid alpha-beta / bond-bending lattice-spring model of porescale
 * (XX = LSM2S/Cxxxx/XX_P.f, x-stretch; YZ = LSM2S/Cyzyz/YZ_P.f, yz-shear).
 * Used only as the reference for parity tests of the GPU solver and as the CPU baseline.
 *
 * The reference pads the loaded axis with a pore column and ties the node
 * planes 1 and N+1 (their forces are summed and shared) with a displacement
 * jump 2g between them (XX:446-523, 1366-1375, 1511-1520).  Here the padded
 * axis is `pa` (0 for XX, 1 for YZ) and the jump acts on displacement
 * component `jc` (0 for XX, 2 for YZ).  The other two axes are periodic.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ps_oracle.h"

/* D3Q19 (velocities19 order) and the 9 bond vectors (velocities9 order) */
static const int CV[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                              {1, 1, 0},  {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},
                              {-1, 0, -1}, {0, 1, 1},  {0, -1, 1}, {0, 1, -1}, {0, -1, -1}};
static const int IB[9][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, -1, 0},
                             {1, 0, 1}, {1, 0, -1}, {0, 1, 1}, {0, 1, -1}};
/* Angle table (XX:314-362 nta): the two arm directions (1-based D3Q19
 * indices) of the 48 angles at a node; 1-24 are pi/4 angles (axis + face
 * diagonal, two cubes share them), 25-48 pi/3 angles (two face diagonals,
 * inside one cube).  Each group of 8 / 4 walks counter-clockwise around a
 * plane, as in the reference. */
static const int NTA[48][2] = {
    {2, 8},   {8, 4},   {4, 9},   {9, 3},   {3, 11},  {11, 5},  {5, 10},  {10, 2},  /* xy */
    {2, 12},  {12, 6},  {6, 13},  {13, 3},  {3, 15},  {15, 7},  {7, 14},  {14, 2},  /* xz */
    {4, 16},  {16, 6},  {6, 17},  {17, 5},  {5, 19},  {19, 7},  {7, 18},  {18, 4},  /* yz */
    {12, 16}, {16, 13}, {13, 17}, {17, 12}, {14, 18}, {18, 15}, {15, 19}, {19, 14}, /* z = +-1 */
    {8, 12},  {12, 10}, {10, 14}, {14, 8},  {9, 13},  {13, 11}, {11, 15}, {15, 9},  /* x = +-1 */
    {8, 16},  {16, 9},  {9, 18},  {18, 8},  {10, 17}, {17, 11}, {11, 19}, {19, 10}, /* y = +-1 */
};

struct or_lsm {
  int N[3];  /* voxel box */
  int M[3];  /* node grid: M[pa] = N[pa] + 2 */
  int pa, jc;
  double alf[2], bet[2], g;
  int32_t *ind; /* N[0]*N[1]*N[2], as given */
  int32_t *num; /* node numbers over M grid, 1-based or 0 */
  int64_t ns, nbo, nna, ntie;
  int32_t *icors, *bon, *ang, *tie;
  double *sbond, *abond;
  double *r, *v, *a; /* displacement, velocity, acceleration (3*ns) */
  double *load;       /* external nodal load (3*ns) or NULL */
  double anf[48][9], bn[9][3], vb[9][3], vn[19][3], vx[19][3];
};

/* material of voxel (1-based coordinates, may be out of range): 1 = solid
 * phase 1 (ind 0), 2 = solid phase 2 (ind 3), 0 = pore.  Along the padded
 * axis voxels outside 1..N are the reference's pore column. */
static int cube_mat(const or_lsm *o, int c[3])
{
  int w[3];
  for (int d = 0; d < 3; d++) {
    int x = c[d];
    if (d == o->pa) {
      if (x < 1 || x > o->N[d]) return 0;
    } else {
      while (x < 1) x += o->N[d];
      while (x > o->N[d]) x -= o->N[d];
    }
    w[d] = x;
  }
  int32_t t = o->ind[(int64_t)(w[0] - 1) + (int64_t)o->N[0] * ((w[1] - 1) + (int64_t)o->N[1] * (w[2] - 1))];
  return t == 0 ? 1 : (t == 3 ? 2 : 0);
}

/* node number at 1-based node coordinates wrapped on the node grid (the
 * reference's ipc vectors over the padded grid) */
static int32_t node_at(const or_lsm *o, const int p[3])
{
  int w[3];
  for (int d = 0; d < 3; d++) {
    int x = p[d], m = o->M[d];
    if (x < 1) x += m;
    if (x > m) x -= m;
    w[d] = x;
  }
  return o->num[(int64_t)(w[0] - 1) + (int64_t)o->M[0] * ((w[1] - 1) + (int64_t)o->M[1] * (w[2] - 1))];
}

static void cross3(const double a[3], const double b[3], double c[3])
{
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

/* lattice constants (XX:1297-1315; anf = plane normal n, force directions
 * on the two arm ends: n x c_j / |c_j|^2 and -(n x c_k) / |c_k|^2) */
static void lsm_constants(or_lsm *o)
{
  for (int i = 0; i < 19; i++) {
    double n2 = (double)(CV[i][0] * CV[i][0] + CV[i][1] * CV[i][1] + CV[i][2] * CV[i][2]);
    for (int d = 0; d < 3; d++) {
      o->vn[i][d] = i == 0 ? 0.0 : (double)CV[i][d] / sqrt(n2);
      o->vx[i][d] = i == 0 ? 0.0 : (double)CV[i][d] / n2;
    }
  }
  for (int i = 0; i < 9; i++) {
    double n2 = (double)(IB[i][0] * IB[i][0] + IB[i][1] * IB[i][1] + IB[i][2] * IB[i][2]);
    for (int d = 0; d < 3; d++) {
      o->vb[i][d] = (double)IB[i][d];
      o->bn[i][d] = (double)IB[i][d] / sqrt(n2);
    }
  }
  for (int j = 0; j < 48; j++) {
    double cj[3], ck[3], n[3], fj[3], fk[3];
    for (int d = 0; d < 3; d++) {
      cj[d] = CV[NTA[j][0] - 1][d];
      ck[d] = CV[NTA[j][1] - 1][d];
    }
    cross3(cj, ck, n);
    double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int d = 0; d < 3; d++) n[d] /= nn;
    cross3(n, cj, fj);
    cross3(n, ck, fk);
    double j2 = cj[0] * cj[0] + cj[1] * cj[1] + cj[2] * cj[2], k2 = ck[0] * ck[0] + ck[1] * ck[1] + ck[2] * ck[2];
    for (int d = 0; d < 3; d++) {
      o->anf[j][d] = n[d];
      o->anf[j][3 + d] = fj[d] / j2;
      o->anf[j][6 + d] = -fk[d] / k2;
    }
  }
}

/* cubes adjacent to bond j (1-based, velocities9) from node p: offsets of
 * the voxels (relative to p, voxel (x,y,z) has its low corner at node
 * (x,y,z)) sharing that edge or face diagonal (XX:637-790) */
static int bond_cubes(int j, int off[4][3])
{
  static const int T[9][4][3] = {
      {{0, 0, 0}, {0, 0, -1}, {0, -1, 0}, {0, -1, -1}}, /* 1 0 0 */
      {{0, 0, 0}, {-1, 0, 0}, {0, 0, -1}, {-1, 0, -1}}, /* 0 1 0 */
      {{0, 0, 0}, {-1, 0, 0}, {0, -1, 0}, {-1, -1, 0}}, /* 0 0 1 */
      {{0, 0, 0}, {0, 0, -1}, {0}, {0}},                /* 1 1 0 */
      {{0, -1, 0}, {0, -1, -1}, {0}, {0}},              /* 1 -1 0 */
      {{0, 0, 0}, {0, -1, 0}, {0}, {0}},                /* 1 0 1 */
      {{0, 0, -1}, {0, -1, -1}, {0}, {0}},              /* 1 0 -1 */
      {{0, 0, 0}, {-1, 0, 0}, {0}, {0}},                /* 0 1 1 */
      {{0, 0, -1}, {-1, 0, -1}, {0}, {0}},              /* 0 1 -1 */
  };
  int n = j <= 3 ? 4 : 2;
  memcpy(off, T[j - 1], sizeof(int) * 12);
  return n;
}

or_lsm *or_lsm_create(const int32_t *ind, int nx, int ny, int nz, double alf1, double bet1, double alf2,
                      double bet2, double gstrain, int load)
{
  or_lsm *o = (or_lsm *)calloc(1, sizeof(or_lsm));
  o->N[0] = nx;
  o->N[1] = ny;
  o->N[2] = nz;
  o->pa = load == 0 ? 0 : 1;
  o->jc = load == 0 ? 0 : 2;
  o->alf[0] = alf1;
  o->alf[1] = alf2;
  o->bet[0] = bet1;
  o->bet[1] = bet2;
  o->g = gstrain;
  int64_t nv = (int64_t)nx * ny * nz;
  o->ind = (int32_t *)malloc(sizeof(int32_t) * nv);
  memcpy(o->ind, ind, sizeof(int32_t) * nv);
  for (int d = 0; d < 3; d++) o->M[d] = o->N[d] + (d == o->pa ? 2 : 0);
  lsm_constants(o);
  /* nodes: a node is solid when one of the 8 voxels sharing it is solid
   * (XX:477-518); numbered in k-j-i order (XX:565-578) */
  int64_t nm = (int64_t)o->M[0] * o->M[1] * o->M[2];
  o->num = (int32_t *)calloc(nm, sizeof(int32_t));
  int64_t ns = 0;
  for (int k = 1; k <= o->M[2]; k++)
    for (int j = 1; j <= o->M[1]; j++)
      for (int i = 1; i <= o->M[0]; i++) {
        int solid = 0;
        for (int e = 0; e < 8 && !solid; e++) {
          int c[3] = {i - (e & 1), j - ((e >> 1) & 1), k - ((e >> 2) & 1)};
          /* along the padded axis the node planes 1..N+2 see voxels 1..N+1;
           * a voxel index 0 there does not exist (no wrap) */
          if (c[o->pa] < 1) continue;
          if (cube_mat(o, c)) solid = 1;
        }
        if (solid) o->num[(int64_t)(i - 1) + (int64_t)o->M[0] * ((j - 1) + (int64_t)o->M[1] * (k - 1))] = (int32_t)(++ns);
      }
  o->ns = ns;
  o->icors = (int32_t *)malloc(sizeof(int32_t) * 3 * (ns + 1));
  for (int k = 1; k <= o->M[2]; k++)
    for (int j = 1; j <= o->M[1]; j++)
      for (int i = 1; i <= o->M[0]; i++) {
        int32_t n = o->num[(int64_t)(i - 1) + (int64_t)o->M[0] * ((j - 1) + (int64_t)o->M[1] * (k - 1))];
        if (n) {
          o->icors[3 * (n - 1)] = i;
          o->icors[3 * (n - 1) + 1] = j;
          o->icors[3 * (n - 1) + 2] = k;
        }
      }
  /* bonds (XX:626-1020): node order, then j = 1..9; the constant counts
   * the adjacent solid cubes of each phase, 1/4 per edge cube, 1/2 per
   * face-diagonal cube */
  o->bon = (int32_t *)malloc(sizeof(int32_t) * 3 * 9 * (ns + 1));
  o->sbond = (double *)malloc(sizeof(double) * 9 * (ns + 1));
  int64_t nbo = 0;
  for (int64_t i = 0; i < ns; i++) {
    int p[3] = {o->icors[3 * i], o->icors[3 * i + 1], o->icors[3 * i + 2]};
    for (int j = 1; j <= 9; j++) {
      int q[3] = {p[0] + IB[j - 1][0], p[1] + IB[j - 1][1], p[2] + IB[j - 1][2]};
      int32_t to = node_at(o, q);
      if (!to) continue;
      int off[4][3], n1 = 0, n2 = 0;
      int nc = bond_cubes(j, off);
      for (int c = 0; c < nc; c++) {
        int cc[3] = {p[0] + off[c][0], p[1] + off[c][1], p[2] + off[c][2]};
        int m = cube_mat(o, cc);
        if (m == 1) n1++;
        if (m == 2) n2++;
      }
      if (n1 + n2 == 0) continue;
      double w = j <= 3 ? 0.25 : 0.5;
      o->bon[3 * nbo] = (int32_t)(i + 1);
      o->bon[3 * nbo + 1] = to;
      o->bon[3 * nbo + 2] = j;
      o->sbond[nbo] = (double)n1 * w * alf1 + (double)n2 * w * alf2;
      nbo++;
    }
  }
  o->nbo = nbo;
  /* angles (XX:1023-1261): node order, then j = 1..48 */
  o->ang = (int32_t *)malloc(sizeof(int32_t) * 6 * 48 * (ns + 1));
  o->abond = (double *)malloc(sizeof(double) * 48 * (ns + 1));
  int64_t nna = 0;
  for (int64_t i = 0; i < ns; i++) {
    int p[3] = {o->icors[3 * i], o->icors[3 * i + 1], o->icors[3 * i + 2]};
    for (int j = 0; j < 48; j++) {
      const int *cj = CV[NTA[j][0] - 1], *ck = CV[NTA[j][1] - 1];
      int pj[3] = {p[0] + cj[0], p[1] + cj[1], p[2] + cj[2]};
      int pk[3] = {p[0] + ck[0], p[1] + ck[1], p[2] + ck[2]};
      int32_t nj = node_at(o, pj), nk = node_at(o, pk);
      if (!nj || !nk) continue;
      int mn[3];
      for (int d = 0; d < 3; d++) {
        int a = p[d] < pj[d] ? p[d] : pj[d];
        mn[d] = a < pk[d] ? a : pk[d];
      }
      double c1, c2;
      if (NTA[j][0] > 7 && NTA[j][1] > 7) { /* pi/3: one cube */
        int m = cube_mat(o, mn);
        if (!m) continue;
        c1 = m == 1 ? 1.0 : 0.0;
        c2 = m == 2 ? 1.0 : 0.0;
      } else { /* pi/4: the two cubes on either side of the angle's plane */
        int ax = (cj[0] == 0 && ck[0] == 0) ? 0 : ((cj[1] == 0 && ck[1] == 0) ? 1 : 2);
        int other[3] = {mn[0], mn[1], mn[2]};
        other[ax] -= 1;
        int m1 = cube_mat(o, mn), m2 = cube_mat(o, other);
        int i1 = (m1 == 1) + (m2 == 1), i2 = (m1 == 2) + (m2 == 2);
        if (i1 + i2 == 0) continue;
        c1 = (double)i1 * 0.5;
        c2 = (double)i2 * 0.5;
      }
      int32_t *r = o->ang + 6 * nna;
      r[0] = (int32_t)(i + 1);
      r[1] = nj;
      r[2] = nk;
      r[3] = NTA[j][0];
      r[4] = NTA[j][1];
      r[5] = j + 1;
      o->abond[nna] = c1 * bet1 + c2 * bet2;
      nna++;
    }
  }
  o->nna = nna;
  /* tied planes 1 and N+1 of the padded axis (XX:1366-1375) */
  int b1 = (o->pa + 1) % 3, b2 = (o->pa + 2) % 3;
  o->tie = (int32_t *)malloc(sizeof(int32_t) * 2 * ((int64_t)o->M[b1] * o->M[b2] + 1));
  int64_t nt = 0;
  /* the reference loops j (or i) outer, k inner */
  int outer = o->pa == 0 ? 1 : 0;
  for (int s = 1; s <= o->M[outer]; s++)
    for (int k = 1; k <= o->M[2]; k++) {
      int p1[3], p2[3];
      p1[o->pa] = 1;
      p2[o->pa] = o->N[o->pa] + 1;
      p1[outer] = p2[outer] = s;
      p1[2] = p2[2] = k;
      int32_t l1 = node_at(o, p1), l2 = node_at(o, p2);
      if (l1 > 0 && l2 > 0) {
        o->tie[2 * nt] = l1;
        o->tie[2 * nt + 1] = l2;
        nt++;
      }
    }
  o->ntie = nt;
  o->r = (double *)calloc(3 * (ns + 1), sizeof(double));
  o->v = (double *)calloc(3 * (ns + 1), sizeof(double));
  o->a = (double *)calloc(3 * (ns + 1), sizeof(double));
  for (int64_t t = 0; t < nt; t++) {
    o->r[3 * (o->tie[2 * t] - 1) + o->jc] = -gstrain;
    o->r[3 * (o->tie[2 * t + 1] - 1) + o->jc] = gstrain;
  }
  return o;
}

void or_lsm_destroy(or_lsm *o)
{
  if (!o) return;
  free(o->ind); free(o->num); free(o->icors); free(o->bon); free(o->sbond);
  free(o->ang); free(o->abond); free(o->tie); free(o->r); free(o->v); free(o->a);
  free(o->load);
  free(o);
}

void or_lsm_sizes(const or_lsm *o, int64_t out[4])
{
  out[0] = o->ns;
  out[1] = o->nbo;
  out[2] = o->nna;
  out[3] = o->ns - o->ntie;
}

void or_lsm_tables(const or_lsm *o, int32_t *icors, int32_t *bon, double *sbond, int32_t *ang, double *abond)
{
  if (icors) memcpy(icors, o->icors, sizeof(int32_t) * 3 * o->ns);
  if (bon) memcpy(bon, o->bon, sizeof(int32_t) * 3 * o->nbo);
  if (sbond) memcpy(sbond, o->sbond, sizeof(double) * o->nbo);
  if (ang) memcpy(ang, o->ang, sizeof(int32_t) * 6 * o->nna);
  if (abond) memcpy(abond, o->abond, sizeof(double) * o->nna);
}

/* spring forces at displacement u (XX:1404-1500), bonds then angles in
 * table order; `linear` drops the equilibrium vectors, which cancel
 * exactly, to give the exact linear operator used by CG */
static void forces(const or_lsm *o, const double *u, double *a, int linear)
{
  memset(a, 0, sizeof(double) * 3 * o->ns);
  for (int64_t i = 0; i < o->nbo; i++) {
    const int32_t *b = o->bon + 3 * i;
    const double *xn = o->bn[b[2] - 1], *rn = o->vb[b[2] - 1];
    const double *u1 = u + 3 * (b[0] - 1), *u2 = u + 3 * (b[1] - 1);
    double rt[3], f[3];
    for (int d = 0; d < 3; d++) rt[d] = linear ? u2[d] - u1[d] : u2[d] - u1[d] + rn[d];
    double s = rt[0] * xn[0] + rt[1] * xn[1] + rt[2] * xn[2];
    for (int d = 0; d < 3; d++) f[d] = o->sbond[i] * (linear ? s * xn[d] : s * xn[d] - rn[d]);
    for (int d = 0; d < 3; d++) {
      a[3 * (b[0] - 1) + d] += f[d];
      a[3 * (b[1] - 1) + d] -= f[d];
    }
  }
  for (int64_t i = 0; i < o->nna; i++) {
    const int32_t *g = o->ang + 6 * i;
    const double *xrj = o->vx[g[3] - 1], *xrk = o->vx[g[4] - 1];
    double cj[3], ck[3], rtj[3], rtk[3];
    for (int d = 0; d < 3; d++) {
      cj[d] = CV[g[3] - 1][d];
      ck[d] = CV[g[4] - 1][d];
    }
    const double *ui = u + 3 * (g[0] - 1), *uj = u + 3 * (g[1] - 1), *uk = u + 3 * (g[2] - 1);
    for (int d = 0; d < 3; d++) {
      rtj[d] = linear ? uj[d] - ui[d] : uj[d] - ui[d] + cj[d];
      rtk[d] = linear ? uk[d] - ui[d] : uk[d] - ui[d] + ck[d];
    }
    const double *an = o->anf[g[5] - 1];
    double dfi = ((xrk[1] * rtk[2] - xrk[2] * rtk[1] - xrj[1] * rtj[2] + xrj[2] * rtj[1]) * an[0] -
                  (xrk[0] * rtk[2] - xrk[2] * rtk[0] - xrj[0] * rtj[2] + xrj[2] * rtj[0]) * an[1] +
                  (xrk[0] * rtk[1] - xrk[1] * rtk[0] - xrj[0] * rtj[1] + xrj[1] * rtj[0]) * an[2]) *
                 o->abond[i];
    for (int d = 0; d < 3; d++) {
      a[3 * (g[1] - 1) + d] += dfi * an[3 + d];
      a[3 * (g[2] - 1) + d] += dfi * an[6 + d];
      a[3 * (g[0] - 1) + d] -= dfi * an[3 + d] + dfi * an[6 + d];
    }
  }
  /* tie the duplicate planes (XX:1511-1520) */
  for (int64_t t = 0; t < o->ntie; t++) {
    double *a1 = a + 3 * (o->tie[2 * t] - 1), *a2 = a + 3 * (o->tie[2 * t + 1] - 1);
    for (int d = 0; d < 3; d++) {
      a1[d] = a1[d] + a2[d];
      a2[d] = a1[d];
    }
  }
}

void or_lsm_forces(const or_lsm *o, const double *u, double *a) { forces(o, u, a, 0); }

/* The same forces on `nthreads` OpenMP threads, scheduled as the reference
 * schedules its force loops (XX:1406-1500, S1:1785-1879): the bond and the
 * angle lists are cut into 2*nthreads chunks and the odd chunks run before
 * the even ones, so that no two chunks that run together touch the same
 * node.  Chunks are whole node slabs of the slowest axis (z; the tables are
 * in node order), at least two slabs wide; with fewer slabs than that the
 * serial loop runs.  Sums at chunk borders add in another order than the
 * serial loop. */
static void forces_par(const or_lsm *o, const double *u, double *a, int linear, int nthreads)
{
  const int nzn = o->M[2];
  int nch = 2 * nthreads;
  while (nch > 1 && nzn / nch < 2) nch -= 2;
  if (nthreads <= 1 || nch < 2) {
    forces(o, u, a, linear);
    return;
  }
  memset(a, 0, sizeof(double) * 3 * o->ns);
  /* chunk c: elements whose first node (bonds) or centre node (angles) lies
   * in z slabs [c*nzn/nch, (c+1)*nzn/nch) */
  int64_t *bcut = (int64_t *)calloc(nch + 1, sizeof(int64_t)), *acut = (int64_t *)calloc(nch + 1, sizeof(int64_t));
  for (int c = 0; c <= nch; c++) {
    const int zc = (int)((int64_t)c * nzn / nch) + 1; /* 1-based slab */
    int64_t lo = 0, hi = o->nbo;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (o->icors[3 * (o->bon[3 * mid] - 1) + 2] < zc) lo = mid + 1; else hi = mid;
    }
    bcut[c] = c == nch ? o->nbo : lo;
    lo = 0, hi = o->nna;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (o->icors[3 * (o->ang[6 * mid] - 1) + 2] < zc) lo = mid + 1; else hi = mid;
    }
    acut[c] = c == nch ? o->nna : lo;
  }
  for (int parity = 0; parity < 2; parity++) {
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
    for (int c = parity; c < nch; c += 2) {
      for (int64_t i = bcut[c]; i < bcut[c + 1]; i++) {
        const int32_t *b = o->bon + 3 * i;
        const double *xn = o->bn[b[2] - 1], *rn = o->vb[b[2] - 1];
        const double *u1 = u + 3 * (b[0] - 1), *u2 = u + 3 * (b[1] - 1);
        double rt[3], f[3];
        for (int d = 0; d < 3; d++) rt[d] = linear ? u2[d] - u1[d] : u2[d] - u1[d] + rn[d];
        const double sd = rt[0] * xn[0] + rt[1] * xn[1] + rt[2] * xn[2];
        for (int d = 0; d < 3; d++) f[d] = o->sbond[i] * (linear ? sd * xn[d] : sd * xn[d] - rn[d]);
        for (int d = 0; d < 3; d++) {
          a[3 * (b[0] - 1) + d] += f[d];
          a[3 * (b[1] - 1) + d] -= f[d];
        }
      }
      for (int64_t i = acut[c]; i < acut[c + 1]; i++) {
        const int32_t *g = o->ang + 6 * i;
        const double *xrj = o->vx[g[3] - 1], *xrk = o->vx[g[4] - 1];
        double rtj[3], rtk[3];
        const double *ui = u + 3 * (g[0] - 1), *uj = u + 3 * (g[1] - 1), *uk = u + 3 * (g[2] - 1);
        for (int d = 0; d < 3; d++) {
          rtj[d] = linear ? uj[d] - ui[d] : uj[d] - ui[d] + CV[g[3] - 1][d];
          rtk[d] = linear ? uk[d] - ui[d] : uk[d] - ui[d] + CV[g[4] - 1][d];
        }
        const double *an = o->anf[g[5] - 1];
        const double dfi = ((xrk[1] * rtk[2] - xrk[2] * rtk[1] - xrj[1] * rtj[2] + xrj[2] * rtj[1]) * an[0] -
                            (xrk[0] * rtk[2] - xrk[2] * rtk[0] - xrj[0] * rtj[2] + xrj[2] * rtj[0]) * an[1] +
                            (xrk[0] * rtk[1] - xrk[1] * rtk[0] - xrj[0] * rtj[1] + xrj[1] * rtj[0]) * an[2]) *
                           o->abond[i];
        for (int d = 0; d < 3; d++) {
          a[3 * (g[1] - 1) + d] += dfi * an[3 + d];
          a[3 * (g[2] - 1) + d] += dfi * an[6 + d];
          a[3 * (g[0] - 1) + d] -= dfi * an[3 + d] + dfi * an[6 + d];
        }
      }
    }
  }
  free(bcut);
  free(acut);
  for (int64_t t = 0; t < o->ntie; t++) {
    double *a1 = a + 3 * (o->tie[2 * t] - 1), *a2 = a + 3 * (o->tie[2 * t + 1] - 1);
    for (int d = 0; d < 3; d++) {
      a1[d] = a1[d] + a2[d];
      a2[d] = a1[d];
    }
  }
}

/* nsteps of the coupled driver's spring dynamics, lsm_step S1:1721-1903:
 * velocity Verlet with the fluid's wall load afdat (the external load of
 * or_lsm_set_load, already an acceleration: S1 forms it with rsdti2 = rsi
 * dti^2, S1:3413) added to both half kicks, spring accelerations F rsi and
 * viscous damping a -= damp v (damp = 0.25 at S1:1888; the standalone
 * relaxation XX:1533 uses 0.5 and no load).  The load of a tied duplicate
 * plane acts on both nodes of the pair, as the tied forces do.  State: the
 * handle's r, v, a (r starts with the jump).  nthreads > 1 evaluates the
 * forces on that many threads (forces_par). */
void or_lsm_dyn_step(or_lsm *o, int64_t nsteps, double dt, double rsi, double damp, int nthreads)
{
  const int64_t n3 = 3 * o->ns;
  double *f = (double *)calloc(n3 + 3, sizeof(double));
  if (o->load) {
    memcpy(f, o->load, sizeof(double) * n3);
    for (int64_t t = 0; t < o->ntie; t++) {
      double *f1 = f + 3 * (o->tie[2 * t] - 1), *f2 = f + 3 * (o->tie[2 * t + 1] - 1);
      for (int d = 0; d < 3; d++) {
        f1[d] = f1[d] + f2[d];
        f2[d] = f1[d];
      }
    }
  }
  for (int64_t it = 0; it < nsteps; it++) {
    for (int64_t i = 0; i < n3; i++) o->v[i] = o->v[i] + o->a[i] * dt * 0.5 + f[i] * dt * 0.5;
    for (int64_t i = 0; i < n3; i++) o->r[i] = o->r[i] + o->v[i] * dt;
    forces_par(o, o->r, o->a, 0, nthreads);
    for (int64_t i = 0; i < n3; i++) o->a[i] = o->a[i] * rsi;
    for (int64_t i = 0; i < n3; i++) o->a[i] = o->a[i] - damp * o->v[i];
    for (int64_t i = 0; i < n3; i++) o->v[i] = o->v[i] + o->a[i] * dt * 0.5 + f[i] * dt * 0.5;
  }
  free(f);
}

/* r, v, a of the dynamics (3, ns each, node order); NULL skips one */
void or_lsm_get_dyn(const or_lsm *o, double *r, double *v, double *a)
{
  if (r) memcpy(r, o->r, sizeof(double) * 3 * o->ns);
  if (v) memcpy(v, o->v, sizeof(double) * 3 * o->ns);
  if (a) memcpy(a, o->a, sizeof(double) * 3 * o->ns);
}

static void forces_par(const or_lsm *o, const double *u, double *a, int linear, int nthreads);

static int64_t relax_impl(or_lsm *o, double dt, double rs, double damp, int64_t maxsteps, double ftol, int nthreads)
{
  const int64_t n3 = 3 * o->ns;
  const double rsi = 1.0 / rs;
  int64_t it = 0;
  for (; it < maxsteps; it++) {
    for (int64_t i = 0; i < n3; i++) o->v[i] = o->v[i] + o->a[i] * dt * 0.5;
    for (int64_t i = 0; i < n3; i++) o->r[i] = o->r[i] + o->v[i] * dt;
    forces_par(o, o->r, o->a, 0, nthreads);
    double fmax = 0.0;
    for (int64_t i = 0; i < n3; i++) {
      double f = fabs(o->a[i]);
      if (f > fmax) fmax = f;
      o->a[i] = o->a[i] * rsi;
    }
    for (int64_t i = 0; i < n3; i++) o->a[i] = o->a[i] - damp * o->v[i];
    for (int64_t i = 0; i < n3; i++) o->v[i] = o->v[i] + o->a[i] * dt * 0.5;
    if (fmax < ftol) {
      it++;
      break;
    }
  }
  return it;
}

int64_t or_lsm_relax(or_lsm *o, double dt, double rs, double damp, int64_t maxsteps, double ftol)
{
  return relax_impl(o, dt, rs, damp, maxsteps, ftol, 1);
}

int64_t or_lsm_relax_par(or_lsm *o, double dt, double rs, double damp, int64_t maxsteps, double ftol, int nthreads)
{
  return relax_impl(o, dt, rs, damp, maxsteps, ftol, nthreads);
}

/* FP64 CG on the tied system: unknowns are the displacements of all nodes
 * except the second plane of each tied pair, which follows its partner plus
 * the jump.  A = E^T K E, b = E^T F(J) with F the linear spring forces. */
static int64_t cg_impl(or_lsm *o, double rtol, int64_t maxit, double *relres, int nthreads)
{
  const int64_t ns = o->ns, n3 = 3 * ns;
  char *dup = (char *)calloc(ns + 1, 1);
  int32_t *partner = (int32_t *)calloc(ns + 1, sizeof(int32_t));
  for (int64_t t = 0; t < o->ntie; t++) {
    dup[o->tie[2 * t + 1] - 1] = 1;
    partner[o->tie[2 * t + 1] - 1] = o->tie[2 * t] - 1;
  }
  double *x = (double *)calloc(n3, sizeof(double)), *r = (double *)calloc(n3, sizeof(double));
  double *p = (double *)calloc(n3, sizeof(double)), *q = (double *)calloc(n3, sizeof(double));
  double *full = (double *)calloc(n3, sizeof(double)), *f = (double *)calloc(n3, sizeof(double));
  /* b: forces of the pure jump field (tied sum lands on the first plane) */
  for (int64_t i = 0; i < ns; i++)
    if (dup[i]) full[3 * i + o->jc] = 2.0 * o->g;
  forces(o, full, f, 1);
  for (int64_t i = 0; i < ns; i++)
    for (int d = 0; d < 3; d++) r[3 * i + d] = dup[i] ? 0.0 : f[3 * i + d];
  /* external load: equilibrium f(u) + load = 0; a duplicate node's load
   * acts on its tied partner */
  if (o->load)
    for (int64_t i = 0; i < ns; i++)
      for (int d = 0; d < 3; d++) r[3 * (dup[i] ? partner[i] : i) + d] += o->load[3 * i + d];
  int64_t nu = ns - o->ntie;
  /* remove the rigid-translation component */
  for (int d = 0; d < 3; d++) {
    double m = 0.0;
    for (int64_t i = 0; i < ns; i++)
      if (!dup[i]) m += r[3 * i + d];
    m /= (double)nu;
    for (int64_t i = 0; i < ns; i++)
      if (!dup[i]) r[3 * i + d] -= m;
  }
  double bb = 0.0;
  for (int64_t i = 0; i < n3; i++) bb += r[i] * r[i];
  memcpy(p, r, sizeof(double) * n3);
  double rr = bb;
  int64_t it = 0;
  double res = bb > 0 ? 1.0 : 0.0;
  while (it < maxit && rr > rtol * rtol * bb) {
    for (int64_t i = 0; i < ns; i++)
      for (int d = 0; d < 3; d++) full[3 * i + d] = dup[i] ? p[3 * partner[i] + d] : p[3 * i + d];
    forces_par(o, full, f, 1, nthreads);
    for (int64_t i = 0; i < ns; i++)
      for (int d = 0; d < 3; d++) q[3 * i + d] = dup[i] ? 0.0 : -f[3 * i + d];
    double pq = 0.0;
    for (int64_t i = 0; i < n3; i++) pq += p[i] * q[i];
    double al = rr / pq, rn = 0.0;
    for (int64_t i = 0; i < n3; i++) {
      x[i] += al * p[i];
      r[i] -= al * q[i];
      rn += r[i] * r[i];
    }
    double be = rn / rr;
    rr = rn;
    for (int64_t i = 0; i < n3; i++) p[i] = r[i] + be * p[i];
    it++;
  }
  res = bb > 0 ? sqrt(rr / bb) : 0.0;
  if (relres) *relres = res;
  /* displacement field: unknowns, duplicates = partner + jump; the first
   * plane carries -g and the second +g as the reference starts from */
  double sh[3] = {0, 0, 0};
  sh[o->jc] = -o->g;
  for (int64_t i = 0; i < ns; i++)
    for (int d = 0; d < 3; d++) {
      double base = dup[i] ? x[3 * partner[i] + d] + (d == o->jc ? 2.0 * o->g : 0.0) : x[3 * i + d];
      o->r[3 * i + d] = base + sh[d];
    }
  free(dup); free(partner); free(x); free(r); free(p); free(q); free(full); free(f);
  return it;
}

int64_t or_lsm_cg(or_lsm *o, double rtol, int64_t maxit, double *relres)
{
  return cg_impl(o, rtol, maxit, relres, 1);
}

int64_t or_lsm_cg_par(or_lsm *o, double rtol, int64_t maxit, double *relres, int nthreads)
{
  return cg_impl(o, rtol, maxit, relres, nthreads);
}

/* the derived angle table (48 x 9) and the cube-local tables as generated
 * for calc_stress, for comparison with the reference's literal ones */
void or_lsm_anf(double *out)
{
  or_lsm tmp;
  memset(&tmp, 0, sizeof tmp);
  lsm_constants(&tmp);
  memcpy(out, tmp.anf, sizeof tmp.anf);
}

void or_lsm_cube_tables(int32_t *bonds, double *sb, int32_t *angs, double *ab)
{
  int nb = 0, na = 0;
  for (int a = 0; a < 8; a++)
    for (int j = 0; j < 9; j++) {
      int c[3] = {(a & 1) + IB[j][0], ((a >> 1) & 1) + IB[j][1], ((a >> 2) & 1) + IB[j][2]};
      if (c[0] < 0 || c[0] > 1 || c[1] < 0 || c[1] > 1 || c[2] < 0 || c[2] > 1) continue;
      bonds[3 * nb] = a + 1; /* reference corner numbering is 1-based */
      bonds[3 * nb + 1] = c[0] + 2 * c[1] + 4 * c[2] + 1;
      bonds[3 * nb + 2] = j + 1;
      sb[nb] = j < 3 ? 0.25 : 0.5;
      nb++;
    }
  for (int a = 0; a < 8; a++)
    for (int j = 0; j < 48; j++) {
      const int *cj = CV[NTA[j][0] - 1], *ck = CV[NTA[j][1] - 1];
      int p[3] = {a & 1, (a >> 1) & 1, (a >> 2) & 1};
      int qj[3] = {p[0] + cj[0], p[1] + cj[1], p[2] + cj[2]}, qk[3] = {p[0] + ck[0], p[1] + ck[1], p[2] + ck[2]};
      int ok = 1;
      for (int d = 0; d < 3; d++) ok &= qj[d] >= 0 && qj[d] <= 1 && qk[d] >= 0 && qk[d] <= 1;
      if (!ok) continue;
      int32_t *r = angs + 6 * na;
      r[0] = a + 1;
      r[1] = qj[0] + 2 * qj[1] + 4 * qj[2] + 1;
      r[2] = qk[0] + 2 * qk[1] + 4 * qk[2] + 1;
      r[3] = NTA[j][0];
      r[4] = NTA[j][1];
      r[5] = j + 1;
      ab[na] = j >= 24 ? 1.0 : 0.5;
      na++;
    }
}

void or_lsm_get_disp(const or_lsm *o, double *u) { memcpy(u, o->r, sizeof(double) * 3 * o->ns); }
void or_lsm_set_disp(or_lsm *o, const double *u) { memcpy(o->r, u, sizeof(double) * 3 * o->ns); }

/* calc_stress (XX:1628-1997): per solid cube, strain from its 8 corners and
 * the +/- stress from its 24 bonds and 72 angles with the cube's own
 * constants; averaged; modulus = <sigma>(m,n) / (V * 2g / N). */
void or_lsm_stress(const or_lsm *o, double *out)
{
  /* cube-local bonds: corner pairs along a bond vector, in corner order */
  int cb[24][3], ncb = 0;
  double csb[24];
  for (int a = 0; a < 8; a++)
    for (int j = 0; j < 9; j++) {
      int c[3] = {(a & 1) + IB[j][0], ((a >> 1) & 1) + IB[j][1], ((a >> 2) & 1) + IB[j][2]};
      if (c[0] < 0 || c[0] > 1 || c[1] < 0 || c[1] > 1 || c[2] < 0 || c[2] > 1) continue;
      cb[ncb][0] = a;
      cb[ncb][1] = c[0] + 2 * c[1] + 4 * c[2];
      cb[ncb][2] = j;
      csb[ncb] = j < 3 ? 0.25 : 0.5;
      ncb++;
    }
  /* cube-local angles: both arms inside the cube */
  int ca[72][4], nca = 0;
  double cab[72];
  for (int a = 0; a < 8; a++)
    for (int j = 0; j < 48; j++) {
      const int *cj = CV[NTA[j][0] - 1], *ck = CV[NTA[j][1] - 1];
      int p[3] = {a & 1, (a >> 1) & 1, (a >> 2) & 1};
      int qj[3] = {p[0] + cj[0], p[1] + cj[1], p[2] + cj[2]}, qk[3] = {p[0] + ck[0], p[1] + ck[1], p[2] + ck[2]};
      int ok = 1;
      for (int d = 0; d < 3; d++) ok &= qj[d] >= 0 && qj[d] <= 1 && qk[d] >= 0 && qk[d] <= 1;
      if (!ok) continue;
      ca[nca][0] = a;
      ca[nca][1] = qj[0] + 2 * qj[1] + 4 * qj[2];
      ca[nca][2] = qk[0] + 2 * qk[1] + 4 * qk[2];
      ca[nca][3] = j;
      cab[nca] = j >= 24 ? 1.0 : 0.5;
      nca++;
    }
  double sp[3][3] = {{0}}, sm[3][3] = {{0}}, st[3][3] = {{0}};
  int64_t ncub = 0;
  int N0 = o->N[0], N1 = o->N[1], N2 = o->N[2];
  for (int i = 1; i <= N0; i++)
    for (int j = 1; j <= N1; j++)
      for (int k = 1; k <= N2; k++) {
        int c[3] = {i, j, k};
        int m = cube_mat(o, c);
        if (!m) continue;
        ncub++;
        double alf = o->alf[m - 1], bet = o->bet[m - 1];
        int32_t nd[8];
        for (int l = 0; l < 8; l++) {
          int p[3] = {i + (l & 1), j + ((l >> 1) & 1), k + ((l >> 2) & 1)};
          nd[l] = node_at(o, p);
        }
        double cs[3][3] = {{0}}, csp[3][3] = {{0}}, csm[3][3] = {{0}};
        for (int l = 0; l < 8; l++) {
          const double *u = o->r + 3 * (nd[l] - 1);
          double sv[3] = {(l & 1) ? 0.5 : -0.5, ((l >> 1) & 1) ? 0.5 : -0.5, ((l >> 2) & 1) ? 0.5 : -0.5};
          for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) cs[a][b] += sv[a] * u[b] + sv[b] * u[a];
        }
        for (int l = 0; l < ncb; l++) {
          const double *xn = o->bn[cb[l][2]], *rn = o->vb[cb[l][2]];
          const double *u1 = o->r + 3 * (nd[cb[l][0]] - 1), *u2 = o->r + 3 * (nd[cb[l][1]] - 1);
          double rt[3], f[3];
          for (int d = 0; d < 3; d++) rt[d] = u2[d] - u1[d] + rn[d];
          double s = rt[0] * xn[0] + rt[1] * xn[1] + rt[2] * xn[2];
          for (int d = 0; d < 3; d++) f[d] = csb[l] * alf * (s * xn[d] - rn[d]);
          for (int col = 0; col < 3; col++) {
            if (xn[col] > 0)
              for (int d = 0; d < 3; d++) { csp[d][col] += f[d]; csm[d][col] -= f[d]; }
            if (xn[col] < 0)
              for (int d = 0; d < 3; d++) { csp[d][col] -= f[d]; csm[d][col] += f[d]; }
          }
        }
        for (int l = 0; l < nca; l++) {
          int jj = ca[l][3];
          int dj = NTA[jj][0] - 1, dk = NTA[jj][1] - 1;
          const double *xrj = o->vx[dj], *xrk = o->vx[dk], *xnj = o->vn[dj], *xnk = o->vn[dk];
          const double *ui = o->r + 3 * (nd[ca[l][0]] - 1), *uj = o->r + 3 * (nd[ca[l][1]] - 1),
                       *uk = o->r + 3 * (nd[ca[l][2]] - 1);
          double rtj[3], rtk[3];
          for (int d = 0; d < 3; d++) {
            rtj[d] = uj[d] - ui[d] + CV[dj][d];
            rtk[d] = uk[d] - ui[d] + CV[dk][d];
          }
          const double *an = o->anf[jj];
          double dfi = ((xrk[1] * rtk[2] - xrk[2] * rtk[1] - xrj[1] * rtj[2] + xrj[2] * rtj[1]) * an[0] -
                        (xrk[0] * rtk[2] - xrk[2] * rtk[0] - xrj[0] * rtj[2] + xrj[2] * rtj[0]) * an[1] +
                        (xrk[0] * rtk[1] - xrk[1] * rtk[0] - xrj[0] * rtj[1] + xrj[1] * rtj[0]) * an[2]) *
                       (cab[l] * bet);
          for (int col = 0; col < 3; col++) {
            if (xnj[col] > 0)
              for (int d = 0; d < 3; d++) { csp[d][col] -= dfi * an[3 + d]; csm[d][col] += dfi * an[3 + d]; }
            if (xnj[col] < 0)
              for (int d = 0; d < 3; d++) { csp[d][col] += dfi * an[3 + d]; csm[d][col] -= dfi * an[3 + d]; }
          }
          for (int col = 0; col < 3; col++) {
            if (xnk[col] > 0)
              for (int d = 0; d < 3; d++) { csp[d][col] -= dfi * an[6 + d]; csm[d][col] += dfi * an[6 + d]; }
            if (xnk[col] < 0)
              for (int d = 0; d < 3; d++) { csp[d][col] += dfi * an[6 + d]; csm[d][col] -= dfi * an[6 + d]; }
          }
        }
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) {
            sp[a][b] += csp[a][b];
            sm[a][b] += csm[a][b];
            st[a][b] += cs[a][b] * 0.25;
          }
      }
  double vcell = (double)N0 * N1 * N2;
  double nax = (double)o->N[o->pa];
  double strain = 2.0 * o->g;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) out[3 * a + b] = sp[a][b];
  /* Exxxx = asigmap(1,1)/(V*2g/N) (XX:1960); Eyzyz = asigmap(2,3)/(...) (YZ:1936) */
  double s = o->pa == 0 ? sp[0][0] : sp[1][2];
  out[9] = s / (vcell * strain / nax);
  out[10] = strain / nax;
  out[11] = (double)ncub;
}

/* external nodal load (3, ns) in node order for the following or_lsm_cg
 * (the static counterpart of the coupled step's afdat, S1:3849-3886);
 * NULL removes it */
void or_lsm_set_load(or_lsm *o, const double *f)
{
  free(o->load);
  o->load = NULL;
  if (!f) return;
  o->load = (double *)malloc(sizeof(double) * 3 * (o->ns + 1));
  memcpy(o->load, f, sizeof(double) * 3 * o->ns);
}
