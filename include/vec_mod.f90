!=======================================================================
! vec_mod.f90 -- ISO_C_BINDING interface to the GB300 library (vec.h)
!
! A Fortran host (the reference's src/main.F90) uses this module to call
! the sm_103a kernels in place of its own module procedures, e.g.
!     call d1bydx(fin, fout)    ->  ierr = vec_d1bydx(ctx, fin, fout)
!     call hydro_deriv()        ->  ierr = vec_hydro_deriv(ctx)
! Arrays are passed as the reference stores them: contiguous
! real(kind=8) (nx,ny,nz).  Every function returns 0 or a negative status
! (include/vec.h); nothing aborts inside the library.
! No Fortran compiler is installed where this library is built, so this
! file is shipped uncompiled; it needs gfortran >= 9 (or any F2003 compiler).
!=======================================================================
module vec_mod
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: VEC_OK = 0, VEC_ERR_DIVB = -12, VEC_ERR_FLAG = -7, VEC_ERR_NAN = -20
  integer(c_int), parameter :: VEC_PREC_FP64 = 0, VEC_PREC_SPLIT = 1
  integer(c_int), parameter :: VEC_F_R = 0, VEC_F_T = 1, VEC_F_U = 2, VEC_F_V = 3, &
                               VEC_F_W = 4, VEC_F_BX = 5, VEC_F_BY = 6, VEC_F_BZ = 7, &
                               VEC_F_JSQ = 8, VEC_F_POL = 9, VEC_F_TOR = 10

  ! same member order as struct vec_params
  type, bind(C) :: vec_params
    real(c_double) :: gamma, sigma, theta, ck, cm, f, tayl, psi, zeta, xmax, ymax, sf
    real(c_double) :: rayl, chand, eta_contrast, noise_amp
    integer(c_int32_t) :: nx, ny, nz, nframe, ntotal, ndu06, ndu16, ndurestart
    integer(c_int32_t) :: dalias, kinematic, radbc, constflux, perfect, dynamo
    integer(c_int32_t) :: kappa_uniform, seed_base, precision, diag_cadence
  end type vec_params

  type, bind(C) :: vec_scalars
    real(c_double) :: dt, dt1, dt2, ttime
    integer(c_int32_t) :: iter, nit, first, second
  end type vec_scalars

  type, bind(C) :: vec_diag_out
    real(c_double) :: ubar, vbar, kenergy, menergy, nusselt, divbmax, divbmin
    real(c_double) :: rmin, rmax, tmin, tmax, umin, umax, vmin, vmax, wmin, wmax
    real(c_double) :: bxmin, bxmax, bymin, bymax, bzmin, bzmax
    real(c_double) :: machmin, machmax, alfvenmin, alfvenmax, rmsmin, rmsmax
  end type vec_diag_out

  interface
    integer(c_int) function vec_params_default(p) bind(C, name='vec_params_default')
      import :: c_int, vec_params
      type(vec_params), intent(out) :: p
    end function
    integer(c_int) function vec_params_read_input(path, p) bind(C, name='vec_params_read_input')
      import :: c_int, c_char, vec_params
      character(kind=c_char), dimension(*), intent(in) :: path
      type(vec_params), intent(out) :: p
    end function
    integer(c_int) function vec_create(p, ctx) bind(C, name='vec_create')
      import :: c_int, c_ptr, vec_params
      type(vec_params), intent(in) :: p
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function vec_destroy(ctx) bind(C, name='vec_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    ! field i/o: field = VEC_F_* ; array (nx,ny,nz)
    integer(c_int) function vec_set_field(ctx, field, src) bind(C, name='vec_set_field')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      real(c_double), dimension(*), intent(in) :: src
    end function
    integer(c_int) function vec_get_field(ctx, field, dst) bind(C, name='vec_get_field')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      real(c_double), dimension(*), intent(out) :: dst
    end function
    integer(c_int) function vec_get_scalars(ctx, s) bind(C, name='vec_get_scalars')
      import :: c_int, c_ptr, vec_scalars
      type(c_ptr), value :: ctx
      type(vec_scalars), intent(out) :: s
    end function
    ! set-up: static (initial.F90:25), mag_init (magnetic.f90:5), calcdt (utils.F90:144)
    integer(c_int) function vec_static(ctx) bind(C, name='vec_static')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_mag_init(ctx) bind(C, name='vec_mag_init')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_calcdt(ctx, dt) bind(C, name='vec_calcdt')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: dt
    end function
    ! fft.F90 operators
    integer(c_int) function vec_d1bydx(ctx, fin, fout) bind(C, name='vec_d1bydx')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
    end function
    integer(c_int) function vec_d1bydy(ctx, fin, fout) bind(C, name='vec_d1bydy')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
    end function
    integer(c_int) function vec_d2bydx(ctx, fin, f1out, f2out) bind(C, name='vec_d2bydx')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: f1out, f2out
    end function
    integer(c_int) function vec_d2bydy(ctx, fin, f1out, f2out) bind(C, name='vec_d2bydy')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: f1out, f2out
    end function
    integer(c_int) function vec_dealias(ctx, z) bind(C, name='vec_dealias')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(inout) :: z
    end function
    integer(c_int) function vec_forwardfft(ctx, fin, fout) bind(C, name='vec_forwardfft')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
    end function
    integer(c_int) function vec_inversefft(ctx, fin, fout) bind(C, name='vec_inversefft')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
    end function
    ! dbydz.F90 operators
    integer(c_int) function vec_d1bydz(ctx, fin, fout, dflag) bind(C, name='vec_d1bydz')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
      integer(c_int), value :: dflag
    end function
    integer(c_int) function vec_d1upbydz(ctx, fin, fout, dflag) bind(C, name='vec_d1upbydz')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
      integer(c_int), value :: dflag
    end function
    integer(c_int) function vec_d2bydz(ctx, fin, fout, dflag) bind(C, name='vec_d2bydz')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
      integer(c_int), value :: dflag
    end function
    ! physics on the context state
    integer(c_int) function vec_hydro_deriv(ctx) bind(C, name='vec_hydro_deriv')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_mag_deriv(ctx) bind(C, name='vec_mag_deriv')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_bandj(ctx) bind(C, name='vec_bandj')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_boundary(ctx) bind(C, name='vec_boundary')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_mag_boundary(ctx) bind(C, name='vec_mag_boundary')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_ab3_update(ctx) bind(C, name='vec_ab3_update')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function vec_diag(ctx, d) bind(C, name='vec_diag')
      import :: c_int, c_ptr, vec_diag_out
      type(c_ptr), value :: ctx
      type(vec_diag_out), intent(out) :: d
    end function
    ! the fused time loop (main.F90:340-747) and snapshots (netcdf.F90)
    integer(c_int) function vec_step(ctx, nsteps) bind(C, name='vec_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function vec_last_diag(ctx, d) bind(C, name='vec_last_diag')
      import :: c_int, c_ptr, vec_diag_out
      type(c_ptr), value :: ctx
      type(vec_diag_out), intent(out) :: d
    end function
    integer(c_int) function vec_write_snapshot(ctx, path, iprec, history) bind(C, name='vec_write_snapshot')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), dimension(*), intent(in) :: path, history
      integer(c_int), value :: iprec
    end function
    integer(c_int) function vec_read_restart(ctx, path) bind(C, name='vec_read_restart')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), dimension(*), intent(in) :: path
    end function
    ! additions without a reference counterpart: graphs, ensembles, the
    ! interpolate step (interpolate/fft.F90:834-927)
    integer(c_int) function vec_use_graphs(ctx, on) bind(C, name='vec_use_graphs')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function
    integer(c_int) function vec_ensemble_create(ps, n, ens) bind(C, name='vec_ensemble_create')
      import :: c_int, c_ptr, vec_params
      type(vec_params), dimension(*), intent(in) :: ps
      integer(c_int), value :: n
      type(c_ptr), intent(out) :: ens
    end function
    integer(c_int) function vec_ensemble_destroy(ens) bind(C, name='vec_ensemble_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
    end function
    type(c_ptr) function vec_ensemble_member(ens, i) bind(C, name='vec_ensemble_member')
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
      integer(c_int), value :: i
    end function
    integer(c_int) function vec_ensemble_start(ens) bind(C, name='vec_ensemble_start')
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
    end function
    integer(c_int) function vec_ensemble_step(ens, nsteps) bind(C, name='vec_ensemble_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: ens
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function vec_ensemble_tune(ens, steps, cache) bind(C, name='vec_ensemble_tune')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ens
      integer(c_int), value :: steps
      character(kind=c_char), dimension(*), intent(in) :: cache
    end function
    integer(c_int) function vec_expand(coarse, fine, fin, fout) bind(C, name='vec_expand')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: coarse, fine
      real(c_double), dimension(*), intent(in) :: fin
      real(c_double), dimension(*), intent(out) :: fout
    end function
    integer(c_int) function vec_upsample(coarse, fine) bind(C, name='vec_upsample')
      import :: c_int, c_ptr
      type(c_ptr), value :: coarse, fine
    end function
  end interface
end module vec_mod
