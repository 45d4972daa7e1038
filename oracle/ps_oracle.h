/*
 * ps_oracle.h -- CPU FP64 restatement of porescale's two hot paths.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity reference for
 * the GPU implementation in porescale_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product never does.
 *
 * Every routine restates the Fortran reference (Eng-RSMY/porescale) in
 * plain C, keeping the reference's loop orders and floating-point
 * operation order so that integer tables are bit-exact and FP64 results
 * are reproducible.  Citations (file:line) are relative to the reference
 * project root:
 *   S1 = LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f
 *   XX = LSM2S/Cxxxx/XX_P.f,  YZ = LSM2S/Cyzyz/YZ_P.f
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists on
 * either build machine, so this restatement cannot be compared with the
 * reference's own outputs ("parity unpinned"); it is pinned instead by
 * physics known-answer tests (mass/momentum conservation, Poiseuille flow,
 * homogeneous-solid elastic moduli) in tests/.
 *
 * Arrays follow the reference's Fortran layouts: ind(nx,ny,nz) with x
 * fastest; fr(19,nl) with the 19 populations of a node contiguous;
 * icor(3,nl), ips(3,nps), ipb2(4,npb2), ipb4(6,npb4) with 1-based values.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double cr2, rr0, rb0, B, sig, vir, vib, wet, ee, dt;
  double bfr[3], bfb[3];
  int32_t idir, iipore;
} or_lbm_params;

typedef struct or_lbm or_lbm;

/* LBM context: builds the S1 tables (S1:526-602 LSM corner dilation for
 * mijks, S1:1026-1340 fluid list and propagation tables). */
or_lbm *or_lbm_create(const or_lbm_params *p, const int32_t *ind, int nx, int ny, int nz);
void or_lbm_destroy(or_lbm *o);
/* sizes: nl, nps, npb2, npb4, ns, n_overflow (diagonal links on which the
 * reference's 32-bit node-number product S1:1121 would wrap to zero) */
void or_lbm_sizes(const or_lbm *o, int64_t out[6]);
void or_lbm_tables(const or_lbm *o, int32_t *icor, int32_t *ips, int32_t *ipb2, int32_t *ipb4,
                   int32_t *mijk, int32_t *mijks);
/* S1:2800-2854 initdistr (Park-Miller colour assignment) + densities */
void or_lbm_init_random(or_lbm *o, double sat);
void or_lbm_set_state(or_lbm *o, const double *fr, const double *fb);
void or_lbm_get_state(const or_lbm *o, double *fr, double *fb);
void or_lbm_fields(const or_lbm *o, double *rr, double *rb, double *cf);
/* full steps, S1:3634-3945 (LSM coupling omitted: it does not feed back) */
void or_lbm_run(or_lbm *o, int nsteps, int nthreads);
/* check_state reductions S1:2988-3202; out layout documented in the .c */
void or_lbm_observables(const or_lbm *o, double *out);
/* wall load afdat(3, ns) of the last step (S1:3849-3882) from the
 * post-collision populations pcfr/pcfb, loops and sums in the reference's
 * order; needs at least one step run */
void or_lbm_wall_load(const or_lbm *o, double rsi, double *afdat);
/* single-node kernels exposed for unit tests */
void or_collision(double t1, double t2, double t3, double *f, double *pcf, double r,
                  const double bf[3], const double Fp[19], const double S[19],
                  double dt, double dti, double dt2);
void or_collmatr_trt(double sv, double S[19]);

/* ---------------- gray partial-bounce-back lattice (extension) ----------
 * single-phase TRT on a dense periodic box, partial bounce-back by the
 * solid fraction s(nx,ny,nz); no reference counterpart (ps_oracle_gray.c) */
typedef struct {
  double tau, magic;
  double F[3];
  int32_t idir, nsteps, segment, reserved;
} or_gray_params;
/* nsteps from rest; returns k = nu (<j_idir> + F/2) / F; f_out (19, n) or NULL */
double or_gray_forward(const or_gray_params *p, int nx, int ny, int nz, const double *s, double *f_out);
/* k and dk/ds by the discrete adjoint (all states kept: small boxes only) */
double or_gray_gradient(const or_gray_params *p, int nx, int ny, int nz, const double *s, double *dk);

/* ---------------- lattice-spring model ---------------- */
typedef struct or_lsm or_lsm;
/* load: 0 = x-stretch (XX_P.f), 1 = yz-shear (YZ_P.f).  ind values:
 * 1 pore, 0 solid phase 1, 3 solid phase 2 (XX:446-523). */
or_lsm *or_lsm_create(const int32_t *ind, int nx, int ny, int nz, double alf1, double bet1,
                      double alf2, double bet2, double gstrain, int load);
void or_lsm_destroy(or_lsm *o);
/* sizes: ns (with duplicate plane), nbo, nna, nunique */
void or_lsm_sizes(const or_lsm *o, int64_t out[4]);
void or_lsm_tables(const or_lsm *o, int32_t *icors, int32_t *bon, double *sbond, int32_t *ang,
                   double *abond);
/* force evaluation (bond + angle springs) at displacement u(3,ns) */
void or_lsm_forces(const or_lsm *o, const double *u, double *a);
/* damped Verlet dynamic relaxation as XX:1377-1545; returns steps done */
int64_t or_lsm_relax(or_lsm *o, double dt, double rs, double damp, int64_t maxsteps, double ftol);
/* FP64 CG on the same operator over unique nodes; returns iterations.
 * or_lsm_cg_par evaluates the forces on nthreads OpenMP threads. */
int64_t or_lsm_cg(or_lsm *o, double rtol, int64_t maxit, double *relres);
int64_t or_lsm_cg_par(or_lsm *o, double rtol, int64_t maxit, double *relres, int nthreads);
/* the relaxation XX:1377-1545 with the forces on nthreads OpenMP threads */
int64_t or_lsm_relax_par(or_lsm *o, double dt, double rs, double damp, int64_t maxsteps, double ftol, int nthreads);
/* the coupled driver's spring dynamics lsm_step (S1:1721-1903): nsteps of
 * velocity Verlet with the external load (or_lsm_set_load) as afdat,
 * accelerations F rsi and damping a -= damp v */
void or_lsm_dyn_step(or_lsm *o, int64_t nsteps, double dt, double rsi, double damp, int nthreads);
void or_lsm_get_dyn(const or_lsm *o, double *r, double *v, double *a);
/* external nodal load (3, ns) added to the CG right-hand side; NULL = none */
void or_lsm_set_load(or_lsm *o, const double *f);
void or_lsm_get_disp(const or_lsm *o, double *u);
void or_lsm_set_disp(or_lsm *o, const double *u);
/* calc_stress XX:1628-1997: out[0..8] = <sigma> (3x3, row major),
 * out[9] = modulus (Exxxx or Eyzyz), out[10] = strain used */
void or_lsm_stress(const or_lsm *o, double *out);
/* derived anf(9,48) table (row per angle) and the generated cube-local
 * bond (24 x 3) / angle (72 x 6) tables with their unit constants */
void or_lsm_anf(double *out);
void or_lsm_cube_tables(int32_t *bonds, double *sb, int32_t *angs, double *ab);

#ifdef __cplusplus
}
#endif
#endif
