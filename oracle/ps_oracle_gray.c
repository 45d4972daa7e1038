/*
 * ps_oracle_gray.c -- CPU FP64 restatement of the gray partial-bounce-back
 * single-phase lattice and of its discrete adjoint.  TEST INFRASTRUCTURE
 * ONLY (see ps_oracle.h).
 *
 * The reference has no gray model: this follows its single-phase branch
 * (S1:3701-3710: D3Q19 in velocities19 order, TRT rates from tau and the
 * magic product) and the published partial bounce-back of Walsh, Burwinkle
 * & Saar (Comput. Geosci. 2009), out_i = (1 - s) f*_i + s f_opp(i), with the
 * odd Guo force term (1 - lm/2) 3 t_i c_i.F and u = (j + F/2)/rho.  The
 * adjoint is derived from that discrete map (transposed streaming, PBB and
 * collision Jacobian); tests pin it against central finite differences.
 * The state is kept shifted, g = f - t (t the rest weights): at the small
 * velocities of permeability runs this keeps ~10 more bits of the flow.
 * Operation order matches the GPU kernels so that states agree bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ps_oracle.h"

static const int GC[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},
                              {0, 0, 1},  {0, 0, -1}, {1, 1, 0},  {-1, 1, 0},  {1, -1, 0},
                              {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},  {-1, 0, -1},
                              {0, 1, 1},  {0, -1, 1}, {0, 1, -1}, {0, -1, -1}};
static const int GOPP[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
static const int GPAIR[9] = {1, 3, 5, 7, 8, 11, 12, 15, 16};

typedef struct {
  int nx, ny, nz;
  int64_t n;
  double lp, lm, F[3], fF[19], t[19];
} gray_ctx;

static void gray_setup(gray_ctx *g, const or_gray_params *p, int nx, int ny, int nz)
{
  g->nx = nx;
  g->ny = ny;
  g->nz = nz;
  g->n = (int64_t)nx * ny * nz;
  g->lp = 1.0 / p->tau;
  g->lm = 1.0 / (0.5 + p->magic / (p->tau - 0.5));
  for (int c = 0; c < 3; c++) g->F[c] = p->F[c];
  for (int i = 0; i < 19; i++) {
    double t = i == 0 ? 1.0 / 3.0 : (i < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
    double cF = GC[i][0] * p->F[0] + GC[i][1] * p->F[1] + GC[i][2] * p->F[2];
    g->t[i] = t;
    g->fF[i] = (1.0 - 0.5 * g->lm) * 3.0 * t * cF;
  }
}

static int64_t gray_nb(const gray_ctx *g, int64_t v, int d)
{
  int x = (int)(v % g->nx), y = (int)((v / g->nx) % g->ny), z = (int)(v / ((int64_t)g->nx * g->ny));
  int a = (x + GC[d][0] + g->nx) % g->nx, b = (y + GC[d][1] + g->ny) % g->ny, c = (z + GC[d][2] + g->nz) % g->nz;
  return a + (int64_t)g->nx * (b + (int64_t)g->ny * c);
}

/* moments and post-collision populations of one node, on the shifted
 * populations g = f - t (f - e = g - (e - t)); fs receives g* = f* - t */
static void gray_collide(const gray_ctx *g, const double *f, double *fs, double *u, double *usq_out)
{
  double rho1 = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
  for (int i = 0; i < 19; i++) {
    rho1 = rho1 + f[i];
    jx = jx + (double)GC[i][0] * f[i];
    jy = jy + (double)GC[i][1] * f[i];
    jz = jz + (double)GC[i][2] * f[i];
  }
  double rho = 1.0 + rho1;
  double ux = (jx + 0.5 * g->F[0]) / rho, uy = (jy + 0.5 * g->F[1]) / rho, uz = (jz + 0.5 * g->F[2]) / rho;
  double usq = ux * ux + uy * uy + uz * uz;
  double de[19];
  for (int i = 0; i < 19; i++) {
    double cu = (double)GC[i][0] * ux + (double)GC[i][1] * uy + (double)GC[i][2] * uz;
    de[i] = g->t[i] * rho1 + g->t[i] * rho * (3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
  }
  fs[0] = f[0] - g->lp * (f[0] - de[0]);
  for (int k = 0; k < 9; k++) {
    int a = GPAIR[k], b = GOPP[a];
    double fp = 0.5 * (f[a] + f[b]), fm = 0.5 * (f[a] - f[b]);
    double ep = 0.5 * (de[a] + de[b]), em = 0.5 * (de[a] - de[b]);
    fs[a] = f[a] - g->lp * (fp - ep) - g->lm * (fm - em) + g->fF[a];
    fs[b] = f[b] - g->lp * (fp - ep) + g->lm * (fm - em) + g->fF[b];
  }
  u[0] = ux;
  u[1] = uy;
  u[2] = uz;
  *usq_out = usq;
}

/* one forward step; f, out in node-major layout f[19 v + i] */
static void gray_step(const gray_ctx *g, const double *s, const double *src, double *dst)
{
  for (int64_t v = 0; v < g->n; v++) {
    double fs[19], u[3], usq;
    const double *f = src + 19 * v;
    gray_collide(g, f, fs, u, &usq);
    double sv = s[v], so = 1.0 - sv;
    for (int i = 0; i < 19; i++) dst[19 * gray_nb(g, v, i) + i] = so * fs[i] + sv * f[GOPP[i]];
  }
}

static double gray_perm(const gray_ctx *g, const or_gray_params *p, const double *f)
{
  int d = p->idir - 1;
  double j = 0.0;
  for (int64_t v = 0; v < g->n; v++)
    for (int i = 1; i < 19; i++) j += (double)GC[i][d] * f[19 * v + i];
  double nu = (p->tau - 0.5) / 3.0, F = p->F[d];
  return nu * (j / (double)g->n + 0.5 * F) / F;
}

static void gray_rest(const gray_ctx *g, double *f) /* shifted: g = 0 */
{
  for (int64_t v = 0; v < g->n; v++)
    for (int i = 0; i < 19; i++) f[19 * v + i] = 0.0;
}

double or_gray_forward(const or_gray_params *p, int nx, int ny, int nz, const double *s, double *f_out)
{
  gray_ctx g;
  gray_setup(&g, p, nx, ny, nz);
  double *a = (double *)malloc(sizeof(double) * 19 * g.n), *b = (double *)malloc(sizeof(double) * 19 * g.n);
  gray_rest(&g, a);
  for (int t = 0; t < p->nsteps; t++) {
    gray_step(&g, s, a, b);
    double *x = a;
    a = b;
    b = x;
  }
  double k = gray_perm(&g, p, a);
  if (f_out)
    for (int64_t v = 0; v < g.n; v++)
      for (int i = 0; i < 19; i++) f_out[19 * v + i] = g.t[i] + a[19 * v + i];
  free(a);
  free(b);
  return k;
}

/* forward storing every state, then the adjoint backwards; dk[v] = dk/ds(v) */
double or_gray_gradient(const or_gray_params *p, int nx, int ny, int nz, const double *s, double *dk)
{
  gray_ctx g;
  gray_setup(&g, p, nx, ny, nz);
  const int T = p->nsteps;
  const int64_t n = g.n;
  double *st = (double *)malloc(sizeof(double) * 19 * n * (size_t)(T + 1));
  gray_rest(&g, st);
  for (int t = 0; t < T; t++) gray_step(&g, s, st + (size_t)t * 19 * n, st + (size_t)(t + 1) * 19 * n);
  double k = gray_perm(&g, p, st + (size_t)T * 19 * n);
  double *an = (double *)malloc(sizeof(double) * 19 * n), *at = (double *)malloc(sizeof(double) * 19 * n);
  int d = p->idir - 1;
  double nu = (p->tau - 0.5) / 3.0, F = p->F[d];
  for (int64_t v = 0; v < n; v++)
    for (int i = 0; i < 19; i++) an[19 * v + i] = nu * (double)GC[i][d] / (F * (double)n);
  for (int64_t v = 0; v < n; v++) dk[v] = 0.0;
  for (int t = T - 1; t >= 0; t--) {
    const double *fstate = st + (size_t)t * 19 * n;
    for (int64_t v = 0; v < n; v++) {
      const double *f = fstate + 19 * v;
      double fs[19], u[3], usq;
      gray_collide(&g, f, fs, u, &usq);
      double ao[19];
      for (int i = 0; i < 19; i++) ao[i] = an[19 * gray_nb(&g, v, i) + i];
      double sv = s[v], so = 1.0 - sv;
      double gsum = 0.0;
      for (int i = 0; i < 19; i++) gsum = gsum + ao[i] * (f[GOPP[i]] - fs[i]);
      dk[v] = dk[v] + gsum;
      double as[19], w[19], a[19];
      for (int i = 0; i < 19; i++) {
        as[i] = so * ao[i];
        a[i] = sv * ao[GOPP[i]];
      }
      w[0] = g.lp * as[0];
      for (int kk = 0; kk < 9; kk++) {
        int pp = GPAIR[kk], q = GOPP[pp];
        double wp = g.lp * (0.5 * (as[pp] + as[q])), wm = g.lm * (0.5 * (as[pp] - as[q]));
        w[pp] = wp + wm;
        w[q] = wp - wm;
      }
      double dr = 0.0, djx = 0.0, djy = 0.0, djz = 0.0;
      for (int i = 0; i < 19; i++) {
        double cx = (double)GC[i][0], cy = (double)GC[i][1], cz = (double)GC[i][2];
        double cu = cx * u[0] + cy * u[1] + cz * u[2];
        double tw = g.t[i] * w[i];
        dr = dr + tw * (1.0 - 4.5 * cu * cu + 1.5 * usq);
        djx = djx + tw * (3.0 * cx + 9.0 * cu * cx - 3.0 * u[0]);
        djy = djy + tw * (3.0 * cy + 9.0 * cu * cy - 3.0 * u[1]);
        djz = djz + tw * (3.0 * cz + 9.0 * cu * cz - 3.0 * u[2]);
      }
      for (int i = 0; i < 19; i++)
        at[19 * v + i] = a[i] + (as[i] - w[i]) + (dr + ((double)GC[i][0] * djx + (double)GC[i][1] * djy + (double)GC[i][2] * djz));
    }
    double *x = an;
    an = at;
    at = x;
  }
  free(st);
  free(an);
  free(at);
  return k;
}
