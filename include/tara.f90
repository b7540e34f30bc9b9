! tara.f90 -- ISO_C_BINDING interfaces to libtara's C API (include/tara.h) for
! Fortran hosts that keep a solver's state on the GPU.
!
! The reference's hot-path subroutines (derive2csh, ab2csh, derive2css, ab2css,
! rk42css, derive3com, ab3com, derive2coh, ab2coh, derive2com, ab2com) need no
! interface: libtara exports them under gfortran's default mangling with the
! reference's implicit-interface argument lists, so the reference's callers link
! against them unchanged.  This module covers everything else in tara.h:
! status codes, the device-resident solvers (tara2d_*, tara_ens_*, tara_coh2d_*,
! tara_com2d_*, tara3d_*), particles, transforms, the ini driver, the learned
! closure and the allocation-free RHS.
!
! Conventions:
! * A handle (tara2d*, tara_ens*, ...) is a type(c_ptr) passed by value; the
!   *_create calls return it through an intent(out) type(c_ptr).
! * Host arrays are passed by reference: complex(c_double_complex) for half
!   spectra (Nh,Ny[,Nz], kx fastest, as the reference declares them), and
!   real(c_double) / integer(c_int) otherwise.  Where the C function accepts
!   NULL for an array, the dummy is OPTIONAL (an absent argument is NULL).
! * Device arrays (the *_device, tara_fno_*, filter and noalloc entry points)
!   and CUDA streams are type(c_ptr) by value.
! * Strings are NUL-terminated: pass trim(s)//c_null_char; tara_string turns a
!   returned const char* into a Fortran string.
! * The bind(C) types below have the C structs' members in the same order.
module tara_gb300
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: TARA_OK = 0, TARA_ERR_ARGS = 1, TARA_ERR_CUDA = 2, &
                               TARA_ERR_NONFINITE = 3, TARA_ERR_NOMEM = 4, TARA_ERR_TIMEOUT = 5, &
                               TARA_ERR_INI = 6
  integer(c_int), parameter :: TARA_RHS_PLAIN = 0, TARA_RHS_SCREEN = 1
  integer(c_int), parameter :: TARA_SCHEME_AB2 = 0, TARA_SCHEME_RK4 = 1
  integer(c_int), parameter :: TARA_PREC_FP64 = 0, TARA_PREC_FP32 = 1, TARA_PREC_DF64 = 2
  integer(c_int), parameter :: TARA_ENS_GRAPH = 0, TARA_ENS_PERSISTENT4 = 1, TARA_ENS_PERSISTENT8 = 2
  integer(c_int), parameter :: TARA_FNO_BF16 = 0, TARA_FNO_FP32 = 1, TARA_FNO_BF16_TMEM = 2

  type, bind(C) :: tara2d_config
    integer(c_int) :: nx, ny
    integer(c_int) :: rhs
    integer(c_int) :: scheme
    integer(c_int) :: precision
    real(c_double) :: nu
    real(c_double) :: dt
    real(c_double) :: alpha
    real(c_double) :: lambda
    real(c_double) :: lx, ly
    real(c_double) :: kpi
    integer(c_int) :: batch
  end type tara2d_config

  type, bind(C) :: tara2d_diag_params
    real(c_double) :: kpi, lx, ly, lambda
    integer(c_int) :: screened
  end type tara2d_diag_params

  type, bind(C) :: tara_ens_run
    integer(c_int) :: n
    real(c_double) :: k0
    integer(c_int64_t) :: seed
  end type tara_ens_run

  type, bind(C) :: tara_coh2d_config
    integer(c_int) :: nx, ny
    real(c_double) :: kpi
    real(c_double) :: lx, ly
    real(c_double) :: mux, muy
    real(c_double) :: cs
    real(c_double) :: dt
  end type tara_coh2d_config

  type, bind(C) :: tara_com2d_config
    integer(c_int) :: nx, ny
    integer(c_int) :: defined
    real(c_double) :: kpi
    real(c_double) :: lx, ly
    real(c_double) :: mu, eta
    real(c_double) :: cs
    real(c_double) :: kf, a
    real(c_double) :: dt
  end type tara_com2d_config

  type, bind(C) :: tara3d_config
    integer(c_int) :: nx, ny, nz
    integer(c_int) :: defined
    real(c_double) :: kpi
    real(c_double) :: lx, ly, lz
    real(c_double) :: mu
    real(c_double) :: eta
    real(c_double) :: cs
    real(c_double) :: nu_u, eta_b
    real(c_double) :: dt
  end type tara3d_config

  type, bind(C) :: tara_fno_config
    integer(c_int) :: h, w
    integer(c_int) :: ci, c, co
    integer(c_int) :: mx, my
    integer(c_int) :: layers, p
    integer(c_int) :: max_batch
    integer(c_int) :: mode
    integer(c_int64_t) :: seed
  end type tara_fno_config

  interface
    ! ---- status ---------------------------------------------------------------
    integer(c_int) function tara_last_error() bind(C, name="tara_last_error")
      import
    end function tara_last_error
    type(c_ptr) function tara_last_error_message() bind(C, name="tara_last_error_message")
      import
    end function tara_last_error_message
    subroutine tara_clear_error() bind(C, name="tara_clear_error")
      import
    end subroutine tara_clear_error
    subroutine tara_set_css_params(lx, ly, lambda) bind(C, name="tara_set_css_params")
      import
      real(c_double), value :: lx, ly, lambda
    end subroutine tara_set_css_params
    integer(c_int) function tara_finalize() bind(C, name="tara_finalize")
      import
    end function tara_finalize

    ! ---- device-resident 2D vorticity solver ----------------------------------
    subroutine tara2d_default_config(cfg, nx, ny) bind(C, name="tara2d_default_config")
      import
      type(tara2d_config), intent(out) :: cfg
      integer(c_int), value :: nx, ny
    end subroutine tara2d_default_config
    integer(c_int) function tara2d_create(cfg, h) bind(C, name="tara2d_create")
      import
      type(tara2d_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function tara2d_create
    integer(c_int) function tara2d_destroy(h) bind(C, name="tara2d_destroy")
      import
      type(c_ptr), value :: h
    end function tara2d_destroy
    integer(c_int) function tara2d_set_state(h, omegak, dt_old) bind(C, name="tara2d_set_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(in) :: omegak(*)
      complex(c_double_complex), intent(in), optional :: dt_old(*)
    end function tara2d_set_state
    integer(c_int) function tara2d_get_state(h, omegak, dt_old) bind(C, name="tara2d_get_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: omegak(*)
      complex(c_double_complex), intent(out), optional :: dt_old(*)
    end function tara2d_get_state
    integer(c_int) function tara2d_set_state_run(h, run, omegak, dt_old) bind(C, name="tara2d_set_state_run")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run
      complex(c_double_complex), intent(in) :: omegak(*)
      complex(c_double_complex), intent(in), optional :: dt_old(*)
    end function tara2d_set_state_run
    integer(c_int) function tara2d_get_state_run(h, run, omegak, dt_old) bind(C, name="tara2d_get_state_run")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run
      complex(c_double_complex), intent(out) :: omegak(*)
      complex(c_double_complex), intent(out), optional :: dt_old(*)
    end function tara2d_get_state_run
    integer(c_int) function tara2d_set_state_device(h, omegak_dev, dt_old_dev) &
        bind(C, name="tara2d_set_state_device")
      import
      type(c_ptr), value :: h, omegak_dev, dt_old_dev
    end function tara2d_set_state_device
    integer(c_int) function tara2d_get_state_device(h, omegak_dev) bind(C, name="tara2d_get_state_device")
      import
      type(c_ptr), value :: h, omegak_dev
    end function tara2d_get_state_device
    integer(c_int) function tara2d_step(h, nsteps) bind(C, name="tara2d_step")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function tara2d_step
    integer(c_int) function tara2d_step_timed(h, nsteps, kernel_ms, kernel_launches, total_ms) &
        bind(C, name="tara2d_step_timed")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
      real(c_double), intent(out) :: kernel_ms(3)
      integer(c_int), intent(out) :: kernel_launches(3)
      real(c_double), intent(out), optional :: total_ms
    end function tara2d_step_timed
    integer(c_int) function tara2d_rhs(h, dt_omegak) bind(C, name="tara2d_rhs")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: dt_omegak(*)
    end function tara2d_rhs
    integer(c_int) function tara2d_diag(h, energy, enstrophy) bind(C, name="tara2d_diag")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out), optional :: energy, enstrophy
    end function tara2d_diag
    integer(c_int) function tara2d_diag_run(h, run, energy, enstrophy) bind(C, name="tara2d_diag_run")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run
      real(c_double), intent(out), optional :: energy, enstrophy
    end function tara2d_diag_run
    integer(c_int) function tara2d_synchronize(h) bind(C, name="tara2d_synchronize")
      import
      type(c_ptr), value :: h
    end function tara2d_synchronize
    type(c_ptr) function tara2d_stream(h) bind(C, name="tara2d_stream")
      import
      type(c_ptr), value :: h
    end function tara2d_stream
    integer(c_int) function tara2d_launches_per_step(h) bind(C, name="tara2d_launches_per_step")
      import
      type(c_ptr), value :: h
    end function tara2d_launches_per_step
    integer(c_int) function tara2d_autotune(h, trial_steps, variants3, ms24) bind(C, name="tara2d_autotune")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: trial_steps
      integer(c_int), intent(out), optional :: variants3(3)
      real(c_double), intent(out), optional :: ms24(24)
    end function tara2d_autotune
    integer(c_int) function tara2d_set_variants(h, variants3) bind(C, name="tara2d_set_variants")
      import
      type(c_ptr), value :: h
      integer(c_int), intent(in) :: variants3(3)
    end function tara2d_set_variants
    integer(c_int) function tara2d_diag_reference(h, dp, usq, uysq) bind(C, name="tara2d_diag_reference")
      import
      type(c_ptr), value :: h
      type(tara2d_diag_params), intent(in) :: dp
      real(c_double), intent(out), optional :: usq, uysq
    end function tara2d_diag_reference
    integer(c_int) function tara2d_real_fields(h, dp, psi, omega, ux, uy) bind(C, name="tara2d_real_fields")
      import
      type(c_ptr), value :: h
      type(tara2d_diag_params), intent(in) :: dp
      real(c_double), intent(out), optional :: psi(*), omega(*), ux(*), uy(*)
    end function tara2d_real_fields
    integer(c_int) function tara2d_init_random(h, k0, energy, seed) bind(C, name="tara2d_init_random")
      import
      type(c_ptr), value :: h
      real(c_double), value :: k0, energy
      integer(c_int64_t), value :: seed
    end function tara2d_init_random
    integer(c_int) function tara2d_init_random_run(h, run, k0, energy, seed) bind(C, name="tara2d_init_random_run")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run
      real(c_double), value :: k0, energy
      integer(c_int64_t), value :: seed
    end function tara2d_init_random_run

    ! ---- ensembles of uneven sizes -------------------------------------------
    integer(c_int) function tara_ens_create(nruns, runs, precision, scheme, nu, dt, energy, e) &
        bind(C, name="tara_ens_create")
      import
      integer(c_int), value :: nruns
      type(tara_ens_run), intent(in) :: runs(*)
      integer(c_int), value :: precision, scheme
      real(c_double), value :: nu, dt, energy
      type(c_ptr), intent(out) :: e
    end function tara_ens_create
    integer(c_int) function tara_ens_destroy(e) bind(C, name="tara_ens_destroy")
      import
      type(c_ptr), value :: e
    end function tara_ens_destroy
    integer(c_int) function tara_ens_autotune(e, trial_steps) bind(C, name="tara_ens_autotune")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: trial_steps
    end function tara_ens_autotune
    integer(c_int) function tara_ens_step(e, nsteps) bind(C, name="tara_ens_step")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: nsteps
    end function tara_ens_step
    integer(c_int) function tara_ens_set_form(e, form) bind(C, name="tara_ens_set_form")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: form
    end function tara_ens_set_form
    integer(c_int) function tara_ens_form(e, form, ms3) bind(C, name="tara_ens_form")
      import
      type(c_ptr), value :: e
      integer(c_int), intent(out), optional :: form
      real(c_double), intent(out), optional :: ms3(3)
    end function tara_ens_form
    integer(c_int) function tara_ens_synchronize(e) bind(C, name="tara_ens_synchronize")
      import
      type(c_ptr), value :: e
    end function tara_ens_synchronize
    type(c_ptr) function tara_ens_stream(e) bind(C, name="tara_ens_stream")
      import
      type(c_ptr), value :: e
    end function tara_ens_stream
    integer(c_int) function tara_ens_get_state(e, run, omegak) bind(C, name="tara_ens_get_state")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: run
      complex(c_double_complex), intent(out) :: omegak(*)
    end function tara_ens_get_state
    integer(c_int) function tara_ens_set_state(e, run, omegak) bind(C, name="tara_ens_set_state")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: run
      complex(c_double_complex), intent(in) :: omegak(*)
    end function tara_ens_set_state
    integer(c_int) function tara_ens_diag(e, run, energy, enstrophy) bind(C, name="tara_ens_diag")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: run
      real(c_double), intent(out), optional :: energy, enstrophy
    end function tara_ens_diag
    integer(c_int) function tara_ens_groups(e) bind(C, name="tara_ens_groups")
      import
      type(c_ptr), value :: e
    end function tara_ens_groups
    integer(c_int) function tara_ens_group_info(e, group, n, runs, variants3, tuned_ms24) &
        bind(C, name="tara_ens_group_info")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: group
      integer(c_int), intent(out), optional :: n, runs
      integer(c_int), intent(out), optional :: variants3(3)
      real(c_double), intent(out), optional :: tuned_ms24(24)
    end function tara_ens_group_info
    integer(c_int) function tara_ens_launches_per_step(e) bind(C, name="tara_ens_launches_per_step")
      import
      type(c_ptr), value :: e
    end function tara_ens_launches_per_step

    ! ---- 2D compressible isothermal hydro ------------------------------------
    subroutine tara_coh2d_default_config(cfg, nx, ny) bind(C, name="tara_coh2d_default_config")
      import
      type(tara_coh2d_config), intent(out) :: cfg
      integer(c_int), value :: nx, ny
    end subroutine tara_coh2d_default_config
    integer(c_int) function tara_coh2d_create(cfg, h) bind(C, name="tara_coh2d_create")
      import
      type(tara_coh2d_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function tara_coh2d_create
    integer(c_int) function tara_coh2d_destroy(h) bind(C, name="tara_coh2d_destroy")
      import
      type(c_ptr), value :: h
    end function tara_coh2d_destroy
    ! state3(Nh, Ny, 3) = nk, ukx, uky; hist3 absent for a zero AB2 history
    integer(c_int) function tara_coh2d_set_state(h, state3, hist3) bind(C, name="tara_coh2d_set_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(in) :: state3(*)
      complex(c_double_complex), intent(in), optional :: hist3(*)
    end function tara_coh2d_set_state
    integer(c_int) function tara_coh2d_get_state(h, state3, hist3) bind(C, name="tara_coh2d_get_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: state3(*)
      complex(c_double_complex), intent(out), optional :: hist3(*)
    end function tara_coh2d_get_state
    integer(c_int) function tara_coh2d_rhs(h, d3) bind(C, name="tara_coh2d_rhs")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: d3(*)
    end function tara_coh2d_rhs
    integer(c_int) function tara_coh2d_step(h, nsteps) bind(C, name="tara_coh2d_step")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function tara_coh2d_step
    integer(c_int) function tara_coh2d_synchronize(h) bind(C, name="tara_coh2d_synchronize")
      import
      type(c_ptr), value :: h
    end function tara_coh2d_synchronize
    type(c_ptr) function tara_coh2d_stream(h) bind(C, name="tara_coh2d_stream")
      import
      type(c_ptr), value :: h
    end function tara_coh2d_stream
    integer(c_int) function tara_coh2d_launches_per_step(h) bind(C, name="tara_coh2d_launches_per_step")
      import
      type(c_ptr), value :: h
    end function tara_coh2d_launches_per_step
    integer(c_int) function tara_coh2d_init_vortices(h, lx_ini, ly_ini) bind(C, name="tara_coh2d_init_vortices")
      import
      type(c_ptr), value :: h
      real(c_double), value :: lx_ini, ly_ini
    end function tara_coh2d_init_vortices
    ! out6 = Energy/(2N^2), y_Energy/(2N^2), C0..C3/N^2: one Energy.dat record
    integer(c_int) function tara_coh2d_diag(h, out6) bind(C, name="tara_coh2d_diag")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out) :: out6(6)
    end function tara_coh2d_diag
    integer(c_int) function tara_coh2d_real_fields(h, n, ux, uy, omega) bind(C, name="tara_coh2d_real_fields")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out), optional :: n(*), ux(*), uy(*), omega(*)
    end function tara_coh2d_real_fields

    ! ---- 2D compressible MHD --------------------------------------------------
    subroutine tara_com2d_default_config(cfg, nx, ny) bind(C, name="tara_com2d_default_config")
      import
      type(tara_com2d_config), intent(out) :: cfg
      integer(c_int), value :: nx, ny
    end subroutine tara_com2d_default_config
    integer(c_int) function tara_com2d_create(cfg, h) bind(C, name="tara_com2d_create")
      import
      type(tara_com2d_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function tara_com2d_create
    integer(c_int) function tara_com2d_destroy(h) bind(C, name="tara_com2d_destroy")
      import
      type(c_ptr), value :: h
    end function tara_com2d_destroy
    ! state6(Nh, Ny, 6) = rho, rho ux, rho uy, E, Bx, By; hist6 absent for zero
    integer(c_int) function tara_com2d_set_state(h, state6, hist6) bind(C, name="tara_com2d_set_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(in) :: state6(*)
      complex(c_double_complex), intent(in), optional :: hist6(*)
    end function tara_com2d_set_state
    integer(c_int) function tara_com2d_get_state(h, state6, hist6) bind(C, name="tara_com2d_get_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: state6(*)
      complex(c_double_complex), intent(out), optional :: hist6(*)
    end function tara_com2d_get_state
    integer(c_int) function tara_com2d_rhs(h, d6) bind(C, name="tara_com2d_rhs")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: d6(*)
    end function tara_com2d_rhs
    integer(c_int) function tara_com2d_step(h, nsteps) bind(C, name="tara_com2d_step")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function tara_com2d_step
    integer(c_int) function tara_com2d_synchronize(h) bind(C, name="tara_com2d_synchronize")
      import
      type(c_ptr), value :: h
    end function tara_com2d_synchronize
    type(c_ptr) function tara_com2d_stream(h) bind(C, name="tara_com2d_stream")
      import
      type(c_ptr), value :: h
    end function tara_com2d_stream
    integer(c_int) function tara_com2d_launches_per_step(h) bind(C, name="tara_com2d_launches_per_step")
      import
      type(c_ptr), value :: h
    end function tara_com2d_launches_per_step
    integer(c_int) function tara_com2d_init_reference(h, lx_ini, ly_ini, b0) bind(C, name="tara_com2d_init_reference")
      import
      type(c_ptr), value :: h
      real(c_double), value :: lx_ini, ly_ini, b0
    end function tara_com2d_init_reference
    ! out5 = Energy, B_Field, C2, C3, div_B_Tot: one Energy.dat record
    integer(c_int) function tara_com2d_diag(h, out5) bind(C, name="tara_com2d_diag")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out) :: out5(5)
    end function tara_com2d_diag
    integer(c_int) function tara_com2d_real_fields(h, rho, ux, uy, p, e, bx, by) &
        bind(C, name="tara_com2d_real_fields")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out), optional :: rho(*), ux(*), uy(*), p(*), e(*), bx(*), by(*)
    end function tara_com2d_real_fields

    ! ---- 3D compressible MHD --------------------------------------------------
    subroutine tara3d_default_config(cfg, nx, ny, nz) bind(C, name="tara3d_default_config")
      import
      type(tara3d_config), intent(out) :: cfg
      integer(c_int), value :: nx, ny, nz
    end subroutine tara3d_default_config
    integer(c_int) function tara3d_create(cfg, h) bind(C, name="tara3d_create")
      import
      type(tara3d_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function tara3d_create
    integer(c_int) function tara3d_destroy(h) bind(C, name="tara3d_destroy")
      import
      type(c_ptr), value :: h
    end function tara3d_destroy
    ! state8(Nh, Ny, Nz, 8) = rho, rho ux, rho uy, rho uz, E, Bx, By, Bz
    integer(c_int) function tara3d_set_state(h, state8, hist8) bind(C, name="tara3d_set_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(in) :: state8(*)
      complex(c_double_complex), intent(in), optional :: hist8(*)
    end function tara3d_set_state
    integer(c_int) function tara3d_get_state(h, state8, hist8) bind(C, name="tara3d_get_state")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: state8(*)
      complex(c_double_complex), intent(out), optional :: hist8(*)
    end function tara3d_get_state
    integer(c_int) function tara3d_set_state_real(h, real8) bind(C, name="tara3d_set_state_real")
      import
      type(c_ptr), value :: h
      real(c_double), intent(in) :: real8(*)
    end function tara3d_set_state_real
    integer(c_int) function tara3d_init_orszag_tang(h, amp, kmax, seed) &
        bind(C, name="tara3d_init_orszag_tang")
      import
      type(c_ptr), value :: h
      real(c_double), value :: amp
      integer(c_int), value :: kmax
      integer(c_int64_t), value :: seed
    end function tara3d_init_orszag_tang
    integer(c_int) function tara3d_step(h, nsteps) bind(C, name="tara3d_step")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function tara3d_step
    integer(c_int) function tara3d_rhs(h, d8) bind(C, name="tara3d_rhs")
      import
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: d8(*)
    end function tara3d_rhs
    integer(c_int) function tara3d_synchronize(h) bind(C, name="tara3d_synchronize")
      import
      type(c_ptr), value :: h
    end function tara3d_synchronize
    type(c_ptr) function tara3d_stream(h) bind(C, name="tara3d_stream")
      import
      type(c_ptr), value :: h
    end function tara3d_stream
    ! out4 = Pressure, Energy, T_Energy, B_Field
    integer(c_int) function tara3d_diag(h, out4) bind(C, name="tara3d_diag")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out) :: out4(4)
    end function tara3d_diag

    ! ---- input.ini driver and Fortran I/O helpers ------------------------------
    integer(c_int) function tara_run_ini(ini_path, out_dir, max_steps) bind(C, name="tara_run_ini")
      import
      character(kind=c_char), intent(in) :: ini_path(*), out_dir(*)
      integer(c_int), value :: max_steps
    end function tara_run_ini
    integer(c_int) function tara_ini_get(path, section, key, buf, buflen) bind(C, name="tara_ini_get")
      import
      character(kind=c_char), intent(in) :: path(*), section(*), key(*)
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_int), value :: buflen
    end function tara_ini_get
    integer(c_int) function tara_fortran_read_double(s, val) bind(C, name="tara_fortran_read_double")
      import
      character(kind=c_char), intent(in) :: s(*)
      real(c_double), intent(out) :: val
    end function tara_fortran_read_double
    integer(c_int) function tara_fortran_read_int(s, val) bind(C, name="tara_fortran_read_int")
      import
      character(kind=c_char), intent(in) :: s(*)
      integer(c_long_long), intent(out) :: val
    end function tara_fortran_read_int
    integer(c_int) function tara_fortran_list_record(v, n, buf, buflen) bind(C, name="tara_fortran_list_record")
      import
      real(c_double), intent(in) :: v(*)
      integer(c_int), value :: n
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_int), value :: buflen
    end function tara_fortran_list_record
    integer(c_int) function tara_write_grid_records(path, nx, ny, xs, ys, fields, nfields) &
        bind(C, name="tara_write_grid_records")
      import
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: nx, ny, nfields
      real(c_double), intent(in) :: xs(*), ys(*), fields(*)
    end function tara_write_grid_records

    ! ---- Lagrangian particles -------------------------------------------------
    integer(c_int) function tara_particles_create(h, kpi, lx, ly, np, xp, yp, p) &
        bind(C, name="tara_particles_create")
      import
      type(c_ptr), value :: h
      real(c_double), value :: kpi, lx, ly
      integer(c_int), value :: np
      real(c_double), intent(in) :: xp(*), yp(*)
      type(c_ptr), intent(out) :: p
    end function tara_particles_create
    integer(c_int) function tara_particles_destroy(p) bind(C, name="tara_particles_destroy")
      import
      type(c_ptr), value :: p
    end function tara_particles_destroy
    integer(c_int) function tara_particles_advance(p, dt) bind(C, name="tara_particles_advance")
      import
      type(c_ptr), value :: p
      real(c_double), value :: dt
    end function tara_particles_advance
    integer(c_int) function tara_particles_get(p, xp, yp) bind(C, name="tara_particles_get")
      import
      type(c_ptr), value :: p
      real(c_double), intent(out) :: xp(*), yp(*)
    end function tara_particles_get
    real(c_float) function tara_park_miller_rand(state) bind(C, name="tara_park_miller_rand")
      import
      integer(c_int64_t), intent(inout) :: state
    end function tara_park_miller_rand

    ! ---- standalone transforms ------------------------------------------------
    integer(c_int) function tara_fft2d_r2c(nx, ny, precision, in, out) bind(C, name="tara_fft2d_r2c")
      import
      integer(c_int), value :: nx, ny, precision
      real(c_double), intent(in) :: in(*)
      complex(c_double_complex), intent(out) :: out(*)
    end function tara_fft2d_r2c
    integer(c_int) function tara_fft2d_c2r(nx, ny, precision, in, out) bind(C, name="tara_fft2d_c2r")
      import
      integer(c_int), value :: nx, ny, precision
      complex(c_double_complex), intent(in) :: in(*)
      real(c_double), intent(out) :: out(*)
    end function tara_fft2d_c2r

    ! ---- learned subgrid closure (device arrays as type(c_ptr)) ------------------
    subroutine tara_fno_default_config(cfg) bind(C, name="tara_fno_default_config")
      import
      type(tara_fno_config), intent(out) :: cfg
    end subroutine tara_fno_default_config
    integer(c_int) function tara_fno_create(cfg, f) bind(C, name="tara_fno_create")
      import
      type(tara_fno_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: f
    end function tara_fno_create
    integer(c_int) function tara_fno_destroy(f) bind(C, name="tara_fno_destroy")
      import
      type(c_ptr), value :: f
    end function tara_fno_destroy
    integer(c_size_t) function tara_fno_num_params(f) bind(C, name="tara_fno_num_params")
      import
      type(c_ptr), value :: f
    end function tara_fno_num_params
    integer(c_int) function tara_fno_get_params(f, host) bind(C, name="tara_fno_get_params")
      import
      type(c_ptr), value :: f
      real(c_float), intent(out) :: host(*)
    end function tara_fno_get_params
    integer(c_int) function tara_fno_set_params(f, host) bind(C, name="tara_fno_set_params")
      import
      type(c_ptr), value :: f
      real(c_float), intent(in) :: host(*)
    end function tara_fno_set_params
    integer(c_int) function tara_fno_get_grads(f, host) bind(C, name="tara_fno_get_grads")
      import
      type(c_ptr), value :: f
      real(c_float), intent(out) :: host(*)
    end function tara_fno_get_grads
    integer(c_int) function tara_fno_set_mode(f, mode) bind(C, name="tara_fno_set_mode")
      import
      type(c_ptr), value :: f
      integer(c_int), value :: mode
    end function tara_fno_set_mode
    integer(c_int) function tara_fno_set_fused(f, enable) bind(C, name="tara_fno_set_fused")
      import
      type(c_ptr), value :: f
      integer(c_int), value :: enable
    end function tara_fno_set_fused
    integer(c_int) function tara_fno_forward(f, x_dev, y_dev, nb) bind(C, name="tara_fno_forward")
      import
      type(c_ptr), value :: f, x_dev, y_dev
      integer(c_int), value :: nb
    end function tara_fno_forward
    integer(c_int) function tara_fno_train_step(f, x_dev, t_dev, idx_dev, n_samples, nb, lr, loss) &
        bind(C, name="tara_fno_train_step")
      import
      type(c_ptr), value :: f, x_dev, t_dev, idx_dev
      integer(c_int), value :: n_samples, nb
      real(c_float), value :: lr
      real(c_double), intent(out), optional :: loss
    end function tara_fno_train_step
    integer(c_long_long) function tara_fno_adam_steps(f) bind(C, name="tara_fno_adam_steps")
      import
      type(c_ptr), value :: f
    end function tara_fno_adam_steps
    type(c_ptr) function tara_fno_stream(f) bind(C, name="tara_fno_stream")
      import
      type(c_ptr), value :: f
    end function tara_fno_stream
    integer(c_int) function tara2d_filter(h, run, factor, omega_bar, flux, omega_bar64) bind(C, name="tara2d_filter")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run, factor
      type(c_ptr), value :: omega_bar, flux, omega_bar64
    end function tara2d_filter
    integer(c_int) function tara2d_set_state_real_device(h, run, omega_dev) &
        bind(C, name="tara2d_set_state_real_device")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run
      type(c_ptr), value :: omega_dev
    end function tara2d_set_state_real_device
    integer(c_int) function tara2d_spectrum(h, run, kmax, spec) bind(C, name="tara2d_spectrum")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run, kmax
      real(c_double), intent(out) :: spec(*)
    end function tara2d_spectrum
    integer(c_int) function tara2d_features(h, run, nf, scales, out_dev) bind(C, name="tara2d_features")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: run, nf
      real(c_double), intent(in), optional :: scales(*)
      type(c_ptr), value :: out_dev
    end function tara2d_features
    integer(c_int) function tara_closure_augment(x_dev, t_dev, n_samples, n, nf, x_out, t_out) &
        bind(C, name="tara_closure_augment")
      import
      type(c_ptr), value :: x_dev, t_dev
      integer(c_int), value :: n_samples, n, nf
      type(c_ptr), value :: x_out, t_out
    end function tara_closure_augment
    integer(c_int) function tara_closure_create(coarse, fno, in_scales, out_scale, c) bind(C, name="tara_closure_create")
      import
      type(c_ptr), value :: coarse, fno
      real(c_double), intent(in) :: in_scales(*)
      real(c_double), value :: out_scale
      type(c_ptr), intent(out) :: c
    end function tara_closure_create
    integer(c_int) function tara_closure_destroy(c) bind(C, name="tara_closure_destroy")
      import
      type(c_ptr), value :: c
    end function tara_closure_destroy
    integer(c_int) function tara_closure_step(c, nsteps) bind(C, name="tara_closure_step")
      import
      type(c_ptr), value :: c
      integer(c_int), value :: nsteps
    end function tara_closure_step

    ! ---- allocation-free RHS, measurement, version -------------------------------
    integer(c_int) function tara_derive2csh_noalloc(nx, ny, nu, omegak_dev, dt_omegak_dev, stream) &
        bind(C, name="tara_derive2csh_noalloc")
      import
      integer(c_int), value :: nx, ny
      real(c_double), value :: nu
      type(c_ptr), value :: omegak_dev, dt_omegak_dev, stream
    end function tara_derive2csh_noalloc
    integer(c_int) function tara_measure_dfma_rate(reps, inst_per_s) bind(C, name="tara_measure_dfma_rate")
      import
      integer(c_int), value :: reps
      real(c_double), intent(out) :: inst_per_s
    end function tara_measure_dfma_rate
    integer(c_int) function tara_twiddle_table(n, precision, out, capacity, count) &
        bind(C, name="tara_twiddle_table")
      import
      integer(c_int), value :: n, precision, capacity
      real(c_double), intent(out) :: out(*)
      integer(c_int), intent(out) :: count
    end function tara_twiddle_table
    type(c_ptr) function tara_version() bind(C, name="tara_version")
      import
    end function tara_version
  end interface

contains

  ! The NUL-terminated C string at p (tara_version(), tara_last_error_message())
  ! as a Fortran string; '' for a null pointer.
  function tara_string(p) result(s)
    type(c_ptr), intent(in) :: p
    character(len=:), allocatable :: s
    character(kind=c_char), pointer :: chars(:)
    integer :: i, n
    interface
      integer(c_size_t) function c_strlen(str) bind(C, name="strlen")
        import
        type(c_ptr), value :: str
      end function c_strlen
    end interface
    if (.not. c_associated(p)) then
      s = ''
      return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: s)
    do i = 1, n
      s(i:i) = chars(i)
    end do
  end function tara_string

end module tara_gb300
