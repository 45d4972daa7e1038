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
#define PS_PREC_F16 2   /* FP16 deviations from the rest equilibrium of the node that
                           wrote each population, FP32 arithmetic            */
#define PS_PREC_BF16 3  /* BF16 deviations, as PS_PREC_F16                           */

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
  int32_t tile_x, tile_y, occupancy;  /* step-kernel configuration */
  int32_t schedule;     /* 0: two-pass step; else fused: slab planes + 256 x look-ahead */
  int32_t wave;         /* 0: off; else wavefront graph: slab planes + 256 x window */
  int32_t march;        /* 0: off; else marching step: band rows + 4096 x chunk planes
                           + 2^25 x producer warps / 4 (+ 2^30 when not sorted) */
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
 * (256,256,0), (128,128,0), (128,256,6), (128,256,7), (128,256,8),
 * (256,256,3).  Used by the autotuner; values are validated. */
int ps_lbm_set_tile(void *handle, int32_t tx, int32_t ty, int32_t occ);
/* Fused step schedule: planes > 0 runs each step as ONE persistent launch
 * in which CTAs take density tiles and collide tiles of z-slabs of
 * `planes` planes from a work list (collide tiles of slab k after the
 * density tiles of slabs k-1..k+1, `ahead` slabs of look-ahead); the
 * collide tiles re-read their populations from L2 and density (memory) and
 * collide (compute) work overlap.  Results are identical to the two-pass
 * step.  Needs a configuration with tx 128 or 256 and occ 0, or tx 128
 * and occ 6 / 8.  planes = 0 restores the two-pass step.  A collide tile
 * whose wait gives up (bounded) makes the next synchronising call return
 * PS_ERR_TIMEOUT. */
int ps_lbm_set_fused(void *handle, int32_t planes, int32_t ahead);
/* Bound of the fused and marching schedules' device waits, in polls (of a
 * density-tile counter, about 32 ns apart, or of an mbarrier); 0 restores
 * the default 2^22.  A wait that
 * reaches it gives up, the tile collides with whatever colour field it
 * finds, and the next synchronising call (ps_lbm_sync, ps_lbm_observables,
 * ps_lbm_get_state, ...) returns PS_ERR_TIMEOUT: the state is then invalid
 * until ps_lbm_set_state.  Every index the collide uses comes from the
 * geometry, never from the data, so giving up reads and writes only the
 * lattice's own arrays.  No counterpart in the reference: it exists so
 * that the give-up path can be exercised. */
int ps_lbm_set_wait_limit(void *handle, int32_t polls);
/* Wavefront schedule: planes > 0 runs the steps in graphs of 8 steps whose
 * density and collide launches each cover one z-slab of `planes` planes,
 * ordered only by their data dependencies (density of slab k after the
 * previous step's collides of slabs k-1..k+1; collide of slab k after the
 * densities of k-1..k+1).  Later steps then follow earlier ones a few
 * slabs behind, so populations are re-read from L2 soon after they were
 * written.  window (0, or 2..64) additionally holds a step's collides at
 * most `window` slabs ahead of the next step's densities.  Results are
 * identical to the two-pass step; step counts that are not a multiple of 8
 * finish with two-pass steps.  Turns the fused schedule off (and
 * ps_lbm_set_fused with planes > 0 turns this one off). */
int ps_lbm_set_wave(void *handle, int32_t planes, int32_t window);
/* Marching step: rows > 0 runs each step as ONE persistent launch (one CTA
 * per SM) over items of `rows` y-rows (every x) times `planes` z-planes (0:
 * about three items per SM).  Inside a CTA, `producers` warps (4, 8 or 12;
 * the other 24 - producers warps collide) walk the item in z computing the
 * densities and stencil colours of each plane -- band plus one recomputed
 * halo row per side, so no CTA waits for another -- into a 4-plane ring in
 * shared memory, up to two planes ahead of the colliding warps, which read
 * their populations again from L2.  The hand-off is by mbarriers whose waits
 * are bounded (ps_lbm_set_wait_limit): one that gives up makes the next
 * synchronising call return PS_ERR_TIMEOUT.  sort != 0 collides each plane's
 * bulk nodes before its interface nodes (the producers record which is
 * which), so that a warp runs one branch of the node update rather than
 * both.  Results are identical to the two-pass step.  Needs FP32/16-bit
 * storage; rows = 0 turns it off.  Turns the fused and wavefront schedules
 * off (and they turn this one off). */
int ps_lbm_set_march(void *handle, int32_t rows, int32_t planes, int32_t producers, int32_t sort);
/* Two-pass (and wavefront) collide kernel: on != 0 lets each CTA collide
 * its bulk nodes before its interface nodes (classes read from the density
 * pass's densities), so that a warp runs one branch of the node update
 * rather than both; every node's arithmetic is unchanged (FP32 and 16-bit
 * storage).  No counterpart in the reference: a kernel option. */
int ps_lbm_set_sort(void *handle, int32_t on);
/* Seed of the stochastic rounding of 16-bit stores (default 0): the random
 * bits are a hash of (node, direction, step number + a seed offset), so runs
 * with different seeds are independent samples of the rounding and runs
 * with the same seed are identical.  No counterpart in the reference. */
int ps_lbm_set_rounding_seed(void *handle, uint32_t seed);
/* Times the candidate configurations (two-pass, fused, wavefront) on the current
 * state (restored afterwards) and keeps the fastest; writes its tile to
 * *tx, *ty, *occ (the schedules are in ps_lbm_info.schedule and .wave). */
int ps_lbm_autotune(void *handle, int32_t steps, int32_t *tx, int32_t *ty, int32_t *occ);

/* ---- batches of lattices (extension; no counterpart in the reference) ----
 * Many subvolumes advanced together: each step is one persistent launch of
 * the density kernel and one of the collide kernel over a tile list that
 * covers every lattice of the batch (uneven sizes welcome), and chunks of
 * 20 steps are replayed from a captured CUDA graph.  The lattices stay
 * ordinary handles (state, observables, wall load work on each); they must
 * share the storage precision and the parameters, be distinct, and outlive
 * the batch.  At most PS_BATCH_MAX_VOLUMES per batch. */
#define PS_BATCH_MAX_VOLUMES 64
int ps_batch_create(void *const *lattices, int32_t n, void **handle);
int ps_batch_destroy(void *handle);
/* nsteps steps of every lattice (each must have a state); results are
 * identical to stepping each lattice on its own with the same
 * configuration */
int ps_batch_step(void *handle, int32_t nsteps);
int ps_batch_set_tile(void *handle, int32_t tx, int32_t ty, int32_t occ);
/* times the compiled configurations on the batch (states restored) and
 * keeps the fastest */
int ps_batch_autotune(void *handle, int32_t steps, int32_t *tx, int32_t *ty, int32_t *occ);
void *ps_batch_stream(void *handle);

/* ---- lattice-spring static solve (hot path b) ---- */
#define PS_LOAD_XSTRETCH 0 /* x stretch with tied x faces: Cxxxx (XX_P.f) */
#define PS_LOAD_YZSHEAR 1  /* yz shear with tied y faces: Cyzyz (YZ_P.f)  */
#define PS_LOAD_NONE 2     /* no tie, no imposed strain (gstrain must be 0),
                              every axis periodic: the coupled driver's network
                              (S1:541-660), nodes in its k-j-i order            */
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
/* Several networks solved together (extension): every CG kernel runs once
 * per iteration for all of them (per-network scalars, a converged network
 * stops moving), 16 iterations per captured CUDA graph.  Same precision for
 * all.  PS_LSM_F64: one batched FP64 CG.  PS_LSM_MIXED: the networks in
 * groups by working set, up to eight groups at a time on their own host
 * threads and streams; in a group, FP64 refinement around a batched FP32 CG,
 * each network refined as soon as its inner CG converges (a network too
 * large for a group runs ps_lsm_solve's refinement alone).  The results
 * equal ps_lsm_solve's bit for bit.  out[n] as ps_lsm_solve's;
 * PS_ERR_NOTCONV names the first network above rtol.  At most 64 networks;
 * the calling thread must not use the handles meanwhile. */
int ps_lsm_batch_solve(void *const *handles, int32_t n, double rtol, int32_t maxit, ps_lsm_result *out);
/* Displacements (3, ns) in the reference node order (k-j-i over the padded
 * grid, duplicate plane included, as LSM_displ_field) after a solve. */
int ps_lsm_get_disp(void *handle, double *u);
void *ps_lsm_stream(void *handle);
/* Modulus gradients (extension; no counterpart in the reference).  After
 * a converged ps_lsm_solve, grad[0..3] = d modulus / d(alf1, bet1, alf2,
 * bet2) from the spring energies at the converged displacement (the
 * stiffness is linear in each constant, so dW/dk = u^T (dK/dk) u / 2 at
 * fixed u, and modulus = 2 W / (V strain^2)); grad[4] = 2 W / (V
 * strain^2), the energy form of the modulus, equal to ps_lsm_result.modulus
 * at equilibrium. */
int ps_lsm_gradients(void *handle, double *grad);

/* ---- fluid -> solid coupling (S1:3849-3882 and calc_ab S1:4008-4468) ---- */
/* Wall load of the lattice's current state: afdat(3, ns) in the reference's
 * LSM node order (ps_lbm_info.ns nodes, numbered as mijks by corner
 * dilation of the solid voxels, S1:541-602).  Every wall link (the ipb2 /
 * ipb4 entries) contributes floc = -2 (f_r + f_b - 0.99 fq) c rsi / dt^2
 * from its bounced post-collision populations, split over the 2 nodes of
 * the wall edge or the 4 of the wall face; FP64 sums in the reference's
 * order.  Needs a box of at least 2 voxels per axis and a state. */
int ps_lbm_wall_load(void *handle, double rsi, double *afdat);
/* Makes the wall load of `lattice` (same box, same GPU) an external nodal
 * load of the spring network for the following ps_lsm_solve calls: the
 * solve then balances the imposed strain (gstrain, may be 0) plus this load,
 * its net force removed (the periodic network carries no net force).
 * Fails with PS_ERR_ARG when a loaded corner is not a node of the network.
 * lattice == NULL removes the load.  (Static counterpart of the coupled
 * dynamic step S1:3849-3886: the reference feeds afdat to lsm_step.) */
int ps_lsm_set_wall_load(void *handle, void *lattice, double rsi);
/* calc_ab (S1:4008-4468) on the last solution: alpha(3,3) = -epsi I +
 * sigma / (V pres), epsi = fraction of voxels labelled iipore, sigma =
 * ps_lsm_result.sigma (same layout); beta(npores) = -(sum over the faces
 * between a pore p voxel and a solid voxel (label 0) of the mean face
 * displacement . c) / (V pres).  lab(nx,ny,nz) = pore labels 1..npores, 0
 * solid.  The reference evaluates them with pres = 0.01 rr0 cr2 (S1:3987). */
int ps_lsm_alpha_beta(void *handle, const int32_t *lab, int32_t npores, int32_t iipore, double pres, double *alpha,
                      double *beta);

/* Damped spring dynamics of the coupled driver: nsteps of lsm_step
 * (S1:1721-1903, called once per fluid step at S1:1884), velocity Verlet
 *   v += a dt/2 + afdat dt/2;  r += v dt;  a = F(r) rsi;  a -= damp v;
 *   v += a dt/2 + afdat dt/2
 * with F the spring forces (the imposed jump included), afdat the wall load
 * set by ps_lsm_set_wall_load (used as given, an acceleration: the lattice
 * forms it with rsi / dt^2, S1:3413; none when unset) and damp = 0.25 in S1
 * (0.5 with dt = 0.01 and no load is the standalone relaxation of
 * XX:1377-1545).  The state (r, v, a) starts at zero displacement (the
 * jump on the tied plane) and rest unless ps_lsm_set_dyn_state set it; r is
 * the handle's displacement, so ps_lsm_get_disp and ps_lsm_alpha_beta see
 * it (a later ps_lsm_solve replaces it by the static solution).  FP64 on
 * the GPU in either solve precision.  The spring forces are the linear
 * operator of the static solve (the reference's bond term -rn cancels up to
 * rounding). */
int ps_lsm_dyn_step(void *handle, int32_t nsteps, double dt, double rsi, double damp);
/* r, v, a (3 x ns each, the reference's node order as ps_lsm_get_disp; a
 * tied duplicate node follows its partner, r plus the jump) into the
 * dynamic state; NULL sets that vector to zero.  The `iteration` checkpoint
 * of the coupled driver (S1:3951-3960) restarts through this call. */
int ps_lsm_set_dyn_state(void *handle, const double *r, const double *v, const double *a);
/* the dynamic state in the same layout; NULL skips a vector */
int ps_lsm_get_dyn_state(void *handle, double *r, double *v, double *a);

/* Largest box (voxel cubes) ps_lsm_stress_noalloc accepts: 128^3. */
#define PS_LSM_NOALLOC_MAX_CUBES (2 * 1024 * 1024)
/* Allocation-free stress evaluation -- no counterpart in the reference.
 * For callers that cannot allocate device memory when they need the moduli:
 * an application whose own pool has already reserved the device's memory,
 * or a driver stepping several streams, where freeing device memory would
 * wait for all work on the device.  d_u is a DEVICE array of the displacements
 * of the unique nodes of the handle's box, three planes (x, y, z component)
 * of nx*ny*nz values, node (x,y,z) at x + nx*(y + ny*z), without the jump;
 * its kernels run on the handle's stream (ps_lsm_stream), so work that
 * writes d_u on another stream must be complete or ordered before the
 * call, which returns after that stream is synchronised; out (host)
 * receives the 9 summed cube stresses (as ps_lsm_result.sigma)
 * and then the modulus.  Uses a static device scratch array instead of
 * cudaMalloc; boxes above PS_LSM_NOALLOC_MAX_CUBES are rejected
 * (PS_ERR_ARG).  Calls that overlap on the GPU share that array and race.
 * Every call looks up the array's device address on the current device
 * (cudaGetSymbolAddress, no allocation), so it stays valid across a device
 * reset; a handle with no imposed strain (gstrain 0) gets modulus 0, as
 * from ps_lsm_solve. */
int ps_lsm_stress_noalloc(void *handle, const double *d_u, double *out);

/* ---- gray partial-bounce-back lattice and its adjoint (extension) ---- */
/* Single-phase D3Q19 TRT (the reference's single-phase branch, S1:3701-3710)
 * on a dense periodic box where every voxel carries a solid fraction s in
 * [0, 1] applied by partial bounce-back (Walsh, Burwinkle & Saar 2009):
 * out_i = (1 - s) f*_i + s f_opp(i).  No counterpart in the reference.
 * tau: relaxation time of the even moments; magic: TRT product (3/16);
 * F: body force; idir (1..3): the permeability direction; nsteps from the
 * rest state; segment: checkpoint interval of the adjoint. */
typedef struct {
  double tau, magic;
  double F[3];
  int32_t idir, nsteps, segment, reserved;
} ps_gray_params;

int ps_gray_create(const ps_gray_params *p, int32_t nx, int32_t ny, int32_t nz, void **handle);
int ps_gray_destroy(void *handle);
/* s(nx,ny,nz) in [0, 1] (default 0 everywhere) */
int ps_gray_set_field(void *handle, const double *s);
/* nsteps from rest, then k = nu (<j_idir> + F/2) / F_idir over all voxels
 * (lattice units, FP64) */
int ps_gray_permeability(void *handle, double *k);
/* k and dk/ds(nx,ny,nz) by the discrete adjoint: reverse-time adjoint
 * lattice with a population checkpoint every `segment` steps and the
 * segment's states recomputed in between (device memory: (nsteps/segment +
 * segment + 2) x 152 bytes per voxel).  PS_ERR_NOMEM when that does not
 * fit. */
int ps_gray_gradient(void *handle, double *k, double *dk_ds);
/* populations f(19, nx*ny*nz) of the last forward run */
int ps_gray_get_state(void *handle, double *f);

/* Message of the last error on this thread (always NUL-terminated). */
int ps_last_error(char *buf, int32_t len);
/* Library build information ("porescale_gb300 <version> sm_103a"). */
const char *ps_version(void);

#ifdef __cplusplus
}
#endif
#endif
