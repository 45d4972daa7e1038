! porescale_gpu.f90 -- ISO_C_BINDING interface of libporescale_gpu.so for the
! Fortran drivers of porescale (lsm_lbm_static_alpha_beta_multipore.f,
! alfabeta2solid.f, XX_P.f, YZ_P.f).  Every routine binds one entry point
! declared in include/porescale.h; arrays are passed in the drivers' own
! layouts (ind(ncx,ncy,ncz), fr(19,nl), rdat(3,ns)) without copies.
!
! Build (with any Fortran 2003 compiler):
!   gfortran -c porescale_gpu.f90
!   gfortran driver.f porescale_gpu.o -L<dir> -lporescale_gpu -Wl,-rpath,<dir>
module porescale_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: PS_OK = 0
  integer(c_int), parameter :: PS_PREC_F64 = 0, PS_PREC_F32 = 1, PS_PREC_F16 = 2, PS_PREC_BF16 = 3
  integer(c_int), parameter :: PS_LOAD_XSTRETCH = 0, PS_LOAD_YZSHEAR = 1, PS_LOAD_NONE = 2
  integer(c_int), parameter :: PS_LSM_F64 = 0, PS_LSM_MIXED = 1

  ! ps_lbm_params: the LBM block of INPUT_PARAMETERS (S1:435-469)
  type, bind(c) :: ps_lbm_params
    real(c_double) :: cr2, rr0, rb0, B, sig, vir, vib, wet, ee, dt
    real(c_double) :: bfr(3), bfb(3)
    integer(c_int32_t) :: idir, iipore
  end type

  type, bind(c) :: ps_lbm_info
    integer(c_int64_t) :: nl, nps, npb2, npb4, ns, nvox
    integer(c_int32_t) :: nx, ny, nz, precision, tile_x, tile_y, occupancy, schedule, wave, march
    integer(c_int64_t) :: device_bytes
  end type

  ! ps_lbm_obs: check_state quantities (S1:2988-3202)
  type, bind(c) :: ps_lbm_obs
    real(c_double) :: tmr, tmb, tm, Cpr, Cpb, nr_cf, nb_cf, nr, nb
    real(c_double) :: Qr(3), Qb(3), um(3), umr(3), umb(3), tfr(3), tfb(3), bmt(3), rmt(3)
    real(c_double) :: permr, permb, sat_r, sat_b
    integer(c_int32_t) :: isneg, nneg_rr, nneg_rb, reserved
  end type

  ! gray partial-bounce-back lattice (extension, no reference counterpart)
  type, bind(c) :: ps_gray_params
    real(c_double) :: tau, magic
    real(c_double) :: F(3)
    integer(c_int32_t) :: idir, nsteps, segment, reserved
  end type

  type, bind(c) :: ps_lsm_params
    real(c_double) :: alf1, bet1, alf2, bet2, gstrain
    integer(c_int32_t) :: load, precision
  end type

  type, bind(c) :: ps_lsm_info
    integer(c_int64_t) :: nnode, ncube, nvox
    integer(c_int32_t) :: nx, ny, nz, load, precision, reserved
    integer(c_int64_t) :: device_bytes
  end type

  type, bind(c) :: ps_lsm_result
    real(c_double) :: modulus, sigma(9), strain, relres
    integer(c_int64_t) :: iterations, inner_iterations, nnode, ncube
    integer(c_int32_t) :: refinements, converged
  end type

  interface
    integer(c_int) function ps_lbm_create(p, ind, nx, ny, nz, precision, handle) bind(c, name='ps_lbm_create')
      import :: c_int, c_int32_t, c_ptr, ps_lbm_params
      type(ps_lbm_params), intent(in) :: p
      integer(c_int32_t), intent(in) :: ind(*)
      integer(c_int32_t), value :: nx, ny, nz, precision
      type(c_ptr), intent(out) :: handle
    end function
    integer(c_int) function ps_lbm_destroy(handle) bind(c, name='ps_lbm_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: handle
    end function
    integer(c_int) function ps_lbm_get_info(handle, info) bind(c, name='ps_lbm_get_info')
      import :: c_int, c_ptr, ps_lbm_info
      type(c_ptr), value :: handle
      type(ps_lbm_info), intent(out) :: info
    end function
    integer(c_int) function ps_lbm_tables(handle, icor, ips, ipb2, ipb4) bind(c, name='ps_lbm_tables')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), intent(out) :: icor(*), ips(*), ipb2(*), ipb4(*)
    end function
    integer(c_int) function ps_lbm_set_state(handle, fr, fb) bind(c, name='ps_lbm_set_state')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(in) :: fr(*), fb(*)
    end function
    integer(c_int) function ps_lbm_get_state(handle, fr, fb) bind(c, name='ps_lbm_get_state')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: fr(*), fb(*)
    end function
    integer(c_int) function ps_lbm_init_random(handle, sat) bind(c, name='ps_lbm_init_random')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), value :: sat
    end function
    integer(c_int) function ps_lbm_step(handle, nsteps) bind(c, name='ps_lbm_step')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: nsteps
    end function
    integer(c_int) function ps_lbm_observables(handle, obs) bind(c, name='ps_lbm_observables')
      import :: c_int, c_ptr, ps_lbm_obs
      type(c_ptr), value :: handle
      type(ps_lbm_obs), intent(out) :: obs
    end function
    integer(c_int) function ps_lbm_set_fused(handle, planes, ahead) bind(c, name='ps_lbm_set_fused')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: planes, ahead
    end function
    integer(c_int) function ps_lbm_set_wait_limit(handle, polls) bind(c, name='ps_lbm_set_wait_limit')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: polls
    end function
    integer(c_int) function ps_lbm_set_march(handle, rows, planes, producers, sort) bind(c, name='ps_lbm_set_march')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: rows, planes, producers, sort
    end function
    integer(c_int) function ps_lbm_set_sort(handle, on) bind(c, name='ps_lbm_set_sort')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: on
    end function
    integer(c_int) function ps_lbm_set_rounding_seed(handle, seed) bind(c, name='ps_lbm_set_rounding_seed')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: seed
    end function
    integer(c_int) function ps_lbm_set_wave(handle, planes, window) bind(c, name='ps_lbm_set_wave')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: planes, window
    end function
    integer(c_int) function ps_lbm_autotune(handle, steps, tx, ty, occ) bind(c, name='ps_lbm_autotune')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: steps
      integer(c_int32_t), intent(out) :: tx, ty, occ
    end function
    ! the lattice's CUDA stream (cudaStream_t) and a wait for its work
    type(c_ptr) function ps_lbm_stream(handle) bind(c, name='ps_lbm_stream')
      import :: c_ptr
      type(c_ptr), value :: handle
    end function
    integer(c_int) function ps_lbm_sync(handle) bind(c, name='ps_lbm_sync')
      import :: c_int, c_ptr
      type(c_ptr), value :: handle
    end function
    integer(c_int) function ps_lbm_set_tile(handle, tx, ty, occ) bind(c, name='ps_lbm_set_tile')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: tx, ty, occ
    end function
    ! several subvolumes advanced together (handles(n) from ps_lbm_create)
    integer(c_int) function ps_batch_create(handles, n, batch) bind(c, name='ps_batch_create')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), intent(in) :: handles(*)
      integer(c_int32_t), value :: n
      type(c_ptr), intent(out) :: batch
    end function
    integer(c_int) function ps_batch_step(batch, nsteps) bind(c, name='ps_batch_step')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: batch
      integer(c_int32_t), value :: nsteps
    end function
    integer(c_int) function ps_batch_set_tile(batch, tx, ty, occ) bind(c, name='ps_batch_set_tile')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: batch
      integer(c_int32_t), value :: tx, ty, occ
    end function
    integer(c_int) function ps_batch_autotune(batch, steps, tx, ty, occ) bind(c, name='ps_batch_autotune')
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: batch
      integer(c_int32_t), value :: steps
      integer(c_int32_t), intent(out) :: tx, ty, occ
    end function
    type(c_ptr) function ps_batch_stream(batch) bind(c, name='ps_batch_stream')
      import :: c_ptr
      type(c_ptr), value :: batch
    end function
    integer(c_int) function ps_batch_destroy(batch) bind(c, name='ps_batch_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: batch
    end function
    integer(c_int) function ps_gray_create(p, nx, ny, nz, handle) bind(c, name='ps_gray_create')
      import :: c_int, c_int32_t, c_ptr, ps_gray_params
      type(ps_gray_params), intent(in) :: p
      integer(c_int32_t), value :: nx, ny, nz
      type(c_ptr), intent(out) :: handle
    end function
    integer(c_int) function ps_gray_set_field(handle, s) bind(c, name='ps_gray_set_field')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(in) :: s(*)
    end function
    integer(c_int) function ps_gray_gradient(handle, k, dk_ds) bind(c, name='ps_gray_gradient')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: k, dk_ds(*)
    end function
    integer(c_int) function ps_gray_permeability(handle, k) bind(c, name='ps_gray_permeability')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: k
    end function
    ! f(19, nx*ny*nz) of the last forward run
    integer(c_int) function ps_gray_get_state(handle, f) bind(c, name='ps_gray_get_state')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: f(*)
    end function
    integer(c_int) function ps_gray_destroy(handle) bind(c, name='ps_gray_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: handle
    end function
    integer(c_int) function ps_lbm_fields(handle, rr, rb, cf) bind(c, name='ps_lbm_fields')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: rr(*), rb(*), cf(*)
    end function
    integer(c_int) function ps_lsm_create(p, ind, nx, ny, nz, handle) bind(c, name='ps_lsm_create')
      import :: c_int, c_int32_t, c_ptr, ps_lsm_params
      type(ps_lsm_params), intent(in) :: p
      integer(c_int32_t), intent(in) :: ind(*)
      integer(c_int32_t), value :: nx, ny, nz
      type(c_ptr), intent(out) :: handle
    end function
    integer(c_int) function ps_lsm_get_info(handle, info) bind(c, name='ps_lsm_get_info')
      import :: c_int, c_ptr, ps_lsm_info
      type(c_ptr), value :: handle
      type(ps_lsm_info), intent(out) :: info
    end function
    integer(c_int) function ps_lsm_solve(handle, rtol, maxit, res) bind(c, name='ps_lsm_solve')
      import :: c_int, c_int32_t, c_double, c_ptr, ps_lsm_result
      type(c_ptr), value :: handle
      real(c_double), value :: rtol
      integer(c_int32_t), value :: maxit
      type(ps_lsm_result), intent(out) :: res
    end function
    ! several networks solved by shared launches (handles(n) from ps_lsm_create)
    integer(c_int) function ps_lsm_batch_solve(handles, n, rtol, maxit, res) bind(c, name='ps_lsm_batch_solve')
      import :: c_int, c_int32_t, c_double, c_ptr, ps_lsm_result
      type(c_ptr), intent(in) :: handles(*)
      integer(c_int32_t), value :: n, maxit
      real(c_double), value :: rtol
      type(ps_lsm_result), intent(out) :: res(*)
    end function
    integer(c_int) function ps_lsm_get_disp(handle, u) bind(c, name='ps_lsm_get_disp')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: u(*)
    end function
    type(c_ptr) function ps_lsm_stream(handle) bind(c, name='ps_lsm_stream')
      import :: c_ptr
      type(c_ptr), value :: handle
    end function
    integer(c_int) function ps_lsm_gradients(handle, grad) bind(c, name='ps_lsm_gradients')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: grad(5)
    end function
    ! afdat(3,ns) of the coupled step (S1:3849-3882)
    integer(c_int) function ps_lbm_wall_load(handle, rsi, afdat) bind(c, name='ps_lbm_wall_load')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), value :: rsi
      real(c_double), intent(out) :: afdat(*)
    end function
    integer(c_int) function ps_lsm_set_wall_load(handle, lattice, rsi) bind(c, name='ps_lsm_set_wall_load')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle, lattice
      real(c_double), value :: rsi
    end function
    ! calc_ab (S1:4008-4468): alphai(3,3) (row = force component), betai(npores)
    integer(c_int) function ps_lsm_alpha_beta(handle, lab, npores, iipore, pres, alphai, betai) &
        bind(c, name='ps_lsm_alpha_beta')
      import :: c_int, c_int32_t, c_double, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), intent(in) :: lab(*)
      integer(c_int32_t), value :: npores, iipore
      real(c_double), value :: pres
      real(c_double), intent(out) :: alphai(9), betai(*)
    end function
    ! stress of a device displacement field (d_u: a device address, three
    ! planes of nx*ny*nz) without any device allocation; out(1:9) the summed
    ! cube stresses, out(10) the modulus
    integer(c_int) function ps_lsm_stress_noalloc(handle, d_u, out) bind(c, name='ps_lsm_stress_noalloc')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle, d_u
      real(c_double), intent(out) :: out(10)
    end function
    ! the coupled driver's lsm_step (S1:1721-1903): nsteps of damped velocity
    ! Verlet under the wall load of ps_lsm_set_wall_load
    integer(c_int) function ps_lsm_dyn_step(handle, nsteps, dt, rsi, damp) bind(c, name='ps_lsm_dyn_step')
      import :: c_int, c_int32_t, c_double, c_ptr
      type(c_ptr), value :: handle
      integer(c_int32_t), value :: nsteps
      real(c_double), value :: dt, rsi, damp
    end function
    ! rdat, vdat, adat (3, ns) in and out of the dynamic state (the
    ! iteration checkpoint of the coupled driver)
    integer(c_int) function ps_lsm_set_dyn_state(handle, rdat, vdat, adat) bind(c, name='ps_lsm_set_dyn_state')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(in) :: rdat(3, *), vdat(3, *), adat(3, *)
    end function
    integer(c_int) function ps_lsm_get_dyn_state(handle, rdat, vdat, adat) bind(c, name='ps_lsm_get_dyn_state')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: handle
      real(c_double), intent(out) :: rdat(3, *), vdat(3, *), adat(3, *)
    end function
    integer(c_int) function ps_lsm_destroy(handle) bind(c, name='ps_lsm_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: handle
    end function
    integer(c_int) function ps_last_error(buf, len) bind(c, name='ps_last_error')
      import :: c_int, c_int32_t, c_char
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_int32_t), value :: len
    end function
    ! NUL-terminated version string (convert with c_f_pointer)
    type(c_ptr) function ps_version() bind(c, name='ps_version')
      import :: c_ptr
    end function
  end interface
end module porescale_gpu
