/*
 * porescale.h -- C ABI of porescale_gb300, the GB300 (sm_103a) implementation
 * of porescale's two data-parallel hot paths:
 *
 *   (a) the D3Q19 colour-gradient two-phase lattice Boltzmann step, and
 *   (b) the alpha-beta / bond-bending lattice-spring (LSM) static solve.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns
 * PS_OK (0) or a PS_ERR_* code, and never exits or traps; the message of the
 * last failure on the calling thread is available from ps_last_error().
 * Host arrays use the reference's Fortran layouts (column-major, 1-based
 * index values where the reference stores indices), so a Fortran driver can
 * bind them through ISO_C_BINDING without copies (fortran/porescale_gpu.f90).
 *
 * Reference files (paths inside the porescale project):
 *   S1 = LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f
 *   XX = LSM2S/Cxxxx/XX_P.f,  YZ = LSM2S/Cyzyz/YZ_P.f
 *
 * Threading: one handle per host thread.  Each handle owns one CUDA stream;
 * every call on a handle is ordered on that stream, and calls that return
 * host data synchronise it.  The library owns all device memory it uses.
 */
#ifndef PORESCALE_H
#define PORESCALE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---- */
#define PS_OK 0
#define PS_ERR_ARG 1          /* invalid argument or size */
#define PS_ERR_CUDA 2         /* CUDA runtime error (message has details) */
#define PS_ERR_NOMEM 3        /* device or host allocation failed */
#define PS_ERR_TIMEOUT 4      /* a bounded device wait gave up */
#define PS_ERR_NOTCONV 5      /* iterative solve did not reach its tolerance */
#define PS_ERR_NODEVICE 6     /* no CUDA device / wrong architecture */
#define PS_ERR_STATE 7        /* call out of order (e.g. step before state) */

/* ---- LBM population storage precisions ---- */
#define PS_PREC_F64 0   /* FP64 storage, FP64 arithmetic (plain path)            */
#define PS_PREC_F32 1   /* FP32 storage, FP32 arithmetic                         */
#define PS_PREC_F16 2   /* FP16 deviations from rest equilibrium, FP32 arithmetic */
#define PS_PREC_BF16 3  /* BF16 deviations from rest equilibrium, FP32 arithmetic */

/* Physical parameters of the two-phase LBM, as read from INPUT_PARAMETERS
 * (S1:435-469).  `sig` is the value in the file (the library applies the
 * reference's internal factor 1/32, S1:1020).  `dt` is the LSM time step
 * that the reference also applies to the LBM weights (S1:1369-1378). */
typedef struct {
  double cr2, rr0, rb0, B, sig, vir, vib, wet, ee, dt;
  double bfr[3], bfb[3];
  int32_t idir, iipore;
} ps_lbm_params;

/* Sizes of a lattice (settings_19 file, S1:1484-1488). */
typedef struct {
  int64_t nl;    /* fluid nodes (ind == iipore)                  */
  int64_t nps;   /* streaming links (ips)                         */
  int64_t npb2;  /* bounce-back links with 2 wall nodes (ipb2)    */
  int64_t npb4;  /* bounce-back links with 4 wall nodes (ipb4)    */
  int64_t ns;    /* LSM solid nodes after corner dilation (S1:608) */
  int64_t nvox;  /* nx*ny*nz                                      */
  int32_t nx, ny, nz, precision;
  int32_t tile_x, tile_y, occupancy, reserved;  /* step-kernel configuration */
  int64_t device_bytes; /* device memory held by the handle */
} ps_lbm_info;

/* check_state quantities (S1:2988-3202) for the current state. */
typedef struct {
  double tmr, tmb, tm;   /* total red, blue, fluid mass                      */
  double Cpr, Cpb;       /* phase-averaged pressures (cf > 0.99 / < -0.99)   */
  double nr_cf, nb_cf;   /* node counts with cf > 0.99 / cf < -0.99          */
  double nr, nb;         /* node counts with rr >= rb / rr < rb              */
  double Qr[3], Qb[3];   /* red/blue momentum incl. half force, divided by t0 */
  double um[3], umr[3], umb[3];
  double tfr[3], tfb[3]; /* half-force totals                                */
  double bmt[3], rmt[3]; /* blue/red raw momentum (bubble test)              */
  double permr, permb;   /* Qr(idir)*vir/bfr(idir), Qb(idir)*vib/bfb(idir)   */
  double sat_r, sat_b;   /* nr/nl, nb/nl (output.m columns 11-12)            */
  int32_t isneg;         /* any negative population                          */
  int32_t nneg_rr, nneg_rb;
  int32_t reserved;
} ps_lbm_obs;

/* Creates a lattice from the voxel field ind(nx,ny,nz) (x fastest; the
 * values of the reference's `ind` file).  Replaces S1:1026-1382: the fluid
 * list, the ips/ipb2/ipb4 propagation tables (kept bit-exact, see
 * ps_lbm_tables) and the collision constants.  precision = PS_PREC_*. */
int ps_lbm_create(const ps_lbm_params *p, const int32_t *ind, int32_t nx, int32_t ny, int32_t nz,
                  int32_t precision, void **handle);
int ps_lbm_destroy(void *handle);
int ps_lbm_get_info(void *handle, ps_lbm_info *out);
/* Copies the reference tables: icor(3,nl), ips(3,nps), ipb2(4,npb2),
 * ipb4(6,npb4) (S1:1060-1072, 1143-1325); any pointer may be NULL. */
int ps_lbm_tables(void *handle, int32_t *icor, int32_t *ips, int32_t *ipb2, int32_t *ipb4);
/* State in the reference layout fr(19,nl), fb(19,nl) = post-streaming
 * populations (what S1 holds between steps and writes to `iteration2`,
 * S1:3951-3960).  Replaces initdistr's archive read (S1:2845-2851). */
int ps_lbm_set_state(void *handle, const double *fr, const double *fb);
int ps_lbm_get_state(void *handle, double *fr, double *fb);
/* initdistr with icon = 0 (S1:2800-2843): Park-Miller colouring of the
 * fluid nodes with blue fraction `sat`, then rest equilibrium. */
int ps_lbm_init_random(void *handle, double sat);
/* Runs nsteps full steps: collision (majority rule), CSF surface tension,
 * recolouring, streaming and half-way bounce-back, densities.  Replaces the
 * step body S1:3663-3945 (and the identical init pass S1:3454-3621). */
int ps_lbm_step(void *handle, int32_t nsteps);
/* check_state reductions S1:2988-3202 (FP64 sums on the device). */
int ps_lbm_observables(void *handle, ps_lbm_obs *out);
/* Density and colour fields rr(nl), rb(nl), cf(nl) for save_results. */
int ps_lbm_fields(void *handle, double *rr, double *rb, double *cf);
/* Stream handle (cudaStream_t) the lattice launches on, for event timing. */
void *ps_lbm_stream(void *handle);
int ps_lbm_sync(void *handle);
/* Step-kernel configuration: tx threads per CTA of the collide kernel, ty
 * of the density kernel, occ the minimum resident collide CTAs per SM asked
 * of the register allocator (0 = its choice).  Compiled: (128,256,0),
 * (256,256,0), (128,128,0), (256,512,0), (128,256,6), (128,256,8),
 * (256,256,3).  Used by the autotuner; values are validated. */
int ps_lbm_set_tile(void *handle, int32_t tx, int32_t ty, int32_t occ);
/* Times the candidate configurations on the current state (restored
 * afterwards) and keeps the fastest; writes it to *tx, *ty, *occ. */
int ps_lbm_autotune(void *handle, int32_t steps, int32_t *tx, int32_t *ty, int32_t *occ);

/* ---- lattice-spring static solve (hot path b) ---- */
#define PS_LOAD_XSTRETCH 0 /* x stretch with tied x faces: Cxxxx (XX_P.f) */
#define PS_LOAD_YZSHEAR 1  /* yz shear with tied y faces: Cyzyz (YZ_P.f)  */
#define PS_LSM_F64 0       /* FP64 conjugate gradient                                */
#define PS_LSM_MIXED 1     /* FP32 CG inside FP64 iterative refinement              */

/* Spring constants per solid phase (alf = Em/(5-10nu), bet =
 * Em(4nu-1)/(20(2nu^2+nu-1)), XX:411-414) and the imposed half jump g:
 * the loaded faces are tied with a displacement jump 2g (strain 2g/N). */
typedef struct {
  double alf1, bet1, alf2, bet2, gstrain;
  int32_t load, precision;
} ps_lsm_params;

typedef struct {
  int64_t nnode;   /* unique solid nodes (the tied planes counted once) */
  int64_t ncube;   /* solid voxel cubes                                  */
  int64_t nvox;
  int32_t nx, ny, nz, load, precision, reserved;
  int64_t device_bytes;
} ps_lsm_info;

typedef struct {
  double modulus;    /* Exxxx = <sigma>(1,1)/(V 2g/N) or Eyzyz = <sigma>(2,3)/(V 2g/N) */
  double sigma[9];   /* summed cube stress sigma+ (calc_stress asigmap), row = force component */
  double strain;     /* 2g/N */
  double relres;     /* final FP64 relative residual |b - A x| / |b| */
  int64_t iterations;        /* FP64 CG iterations, or outer refinements (mixed) */
  int64_t inner_iterations;  /* CG iterations in the working precision */
  int64_t nnode, ncube;
  int32_t refinements, converged;
} ps_lsm_result;

/* Builds the spring network of the voxel field ind(nx,ny,nz) (0 = solid
 * phase 1, 3 = solid phase 2, other values pore).  Replaces the geometry,
 * bond and angle construction of XX:446-1361 (YZ likewise). */
int ps_lsm_create(const ps_lsm_params *p, const int32_t *ind, int32_t nx, int32_t ny, int32_t nz, void **handle);
int ps_lsm_destroy(void *handle);
int ps_lsm_get_info(void *handle, ps_lsm_info *out);
/* Static equilibrium to |b - A x| <= rtol |b| and the effective modulus.
 * Replaces the damped-Verlet loop XX:1377-1545 and calc_stress
 * XX:1628-1997.  Returns PS_ERR_NOTCONV (result still filled) when the
 * tolerance is not reached within maxit working-precision iterations. */
int ps_lsm_solve(void *handle, double rtol, int32_t maxit, ps_lsm_result *out);
/* Displacements (3, ns) in the reference node order (k-j-i over the padded
 * grid, duplicate plane included, as LSM_displ_field) after a solve. */
int ps_lsm_get_disp(void *handle, double *u);
void *ps_lsm_stream(void *handle);

/* Largest box (voxel cubes) ps_lsm_stress_noalloc accepts: 128^3. */
#define PS_LSM_NOALLOC_MAX_CUBES (2 * 1024 * 1024)
/* Allocation-free stress evaluation -- no counterpart in the reference.
 * For callers that cannot allocate device memory when they need the moduli
 * (a time loop being captured into a CUDA graph, or a driver confined to a
 * fixed device memory budget).  d_u is a DEVICE array of the displacements
 * of the unique nodes of the handle's box, three planes (x, y, z component)
 * of nx*ny*nz values, node (x,y,z) at x + nx*(y + ny*z), without the jump;
 * out (host) receives the 9 summed cube stresses (as ps_lsm_result.sigma)
 * and then the modulus.  Uses a static device scratch array instead of
 * cudaMalloc; boxes above PS_LSM_NOALLOC_MAX_CUBES are rejected
 * (PS_ERR_ARG).  Calls that overlap on the GPU share that array and race;
 * the first call on a device sets it up and should precede any stream
 * capture. */
int ps_lsm_stress_noalloc(void *handle, const double *d_u, double *out);

/* Message of the last error on this thread (always NUL-terminated). */
int ps_last_error(char *buf, int32_t len);
/* Library build information ("porescale_gb300 <version> sm_103a"). */
const char *ps_version(void);

#ifdef __cplusplus
}
#endif
#endif
