! gmcore_gpu_mod -- iso_c_binding interface of the GB300 dynamics step
! (include/gmcore_gpu.h) for the GMCORE Fortran driver.
!
! A Fortran host keeps its namelist, initial conditions, output and restart
! and replaces, under a preprocessor switch,
!   call time_integrate(dt_dyn, blocks)          (src/dynamics/gmcore_mod.F90:577-591)
! by   ierr = gmc_step(ctx, 1)
! and the run prologue (gmcore_mod.F90:97-135) by gmc_prepare, diagnose
! (gmcore_mod.F90:213-341) by gmc_diagnose.  Every entry point of the header
! is bound here with the same name, argument order and meaning; the derived
! types are the C structures field for field.  Arrays cross as gmc_view: the
! array's own bounds (halos included), of which only interior points are
! read or written (view2 / view3 below build one from an array).
!
! Build: gfortran -c gmcore_gpu_mod.F90; link with
!   -L<repo>/gmcore_gb300/lib -lgmcore_gpu -Wl,-rpath,<repo>/gmcore_gb300/lib
module gmcore_gpu_mod

  use iso_c_binding

  implicit none

  private :: c_strlen

  ! status codes
  integer(c_int), parameter :: GMC_OK = 0, GMC_EINVAL = -1, GMC_ECFL = -2, GMC_ENONMONO = -3, &
                               GMC_ENEGTRACER = -4, GMC_ENAN = -5, GMC_ECUDA = -7, &
                               GMC_ENOMEM = -8, GMC_ESTATE = -9, GMC_EIO = -10
  ! namelist options (src/utils/namelist_mod.F90)
  integer(c_int32_t), parameter :: GMC_TIME_EULER = 0, GMC_TIME_PC2 = 1, GMC_TIME_WRFRK3 = 2
  integer(c_int32_t), parameter :: GMC_PV_MIDPOINT = 0, GMC_PV_UPWIND = 1, GMC_PV_TVD = 2
  integer(c_int32_t), parameter :: GMC_TVD_NONE = 0, GMC_TVD_VAN_LEER = 1, GMC_TVD_MC = 2
  integer(c_int32_t), parameter :: GMC_FLUX_PPM = 0, GMC_FLUX_VAN_LEER = 1
  integer(c_int32_t), parameter :: GMC_LIMITER_NONE = 0, GMC_LIMITER_MONO = 1, GMC_LIMITER_PD = 2
  integer(c_int32_t), parameter :: GMC_VCOORD_NONE = 0, GMC_VCOORD_TEST_L26 = 26, GMC_VCOORD_WRF_L32 = 32, &
                                   GMC_VCOORD_WRF_L64 = 64
  integer(c_int32_t), parameter :: GMC_PREC_FP64 = 0, GMC_PREC_MIXED = 1
  integer(c_int32_t), parameter :: GMC_FORCING_NONE = 0, GMC_FORCING_HELD_SUAREZ = 1

  type, bind(c) :: gmc_config
    integer(c_int32_t) :: nlon, nlat, nlev
    integer(c_int32_t) :: baroclinic
    integer(c_int32_t) :: time_scheme
    real(c_double)     :: dt_dyn
    real(c_double)     :: dt_adv
    integer(c_int32_t) :: ke_scheme
    real(c_double)     :: ke_cell_wgt
    integer(c_int32_t) :: pv_scheme
    integer(c_int32_t) :: upwind_order_pv
    real(c_double)     :: upwind_wgt_pv
    integer(c_int32_t) :: pv_pole_stokes
    integer(c_int32_t) :: coriolis_scheme
    integer(c_int32_t) :: ffsl_flux_type
    integer(c_int32_t) :: limiter_type
    integer(c_int32_t) :: use_div_damp
    integer(c_int32_t) :: div_damp_order
    real(c_double)     :: div_damp_coef2
    integer(c_int32_t) :: vert_coord_template
    real(c_double)     :: ptop
    real(c_double)     :: hybrid_coord_p0
    real(c_double)     :: max_wave_speed, max_cfl
    real(c_double)     :: filter_coef_a, filter_coef_b, filter_coef_c, filter_coef_d, filter_coef_e
    integer(c_int32_t) :: lon_halo_width
    integer(c_int32_t) :: ntracer
    integer(c_int32_t) :: precision
    integer(c_int32_t) :: n_members
    real(c_double)     :: radius, omega, g, Rd, cpd, p0
    integer(c_int32_t) :: tvd_limiter_type
    real(c_double)     :: div_damp_coef4
    integer(c_int32_t) :: forcing
    integer(c_int32_t) :: use_smag_damp
    real(c_double)     :: smag_damp_coef
  end type gmc_config

  type, bind(c) :: gmc_diag
    real(c_double) :: tm, te, te_ke, te_ie, te_pe, tav, tpe, tpt
  end type gmc_diag

  type, bind(c) :: gmc_view
    type(c_ptr)        :: data
    integer(c_int32_t) :: lb(3)
    integer(c_int32_t) :: ub(3)
  end type gmc_view

  ! an item of gmc_step_io: a field (name, a C string) or, with name null, a tracer
  type, bind(c) :: gmc_io
    type(c_ptr)        :: name
    integer(c_int32_t) :: tracer
    type(gmc_view)     :: view
  end type gmc_io

  ! history and restart file options: C strings (c_null_ptr: the default)
  type, bind(c) :: gmc_file_opts
    type(c_ptr) :: time_units, start_time, tracer_names, restart_interval
    integer(c_int32_t) :: background
  end type gmc_file_opts

  ! dense FP64 host arrays of a restart (c_loc of contiguous arrays, or c_null_ptr)
  type, bind(c) :: gmc_restart_arrays
    type(c_ptr) :: u_lon, v_lat, pt, phs, gz, gzs, q
  end type gmc_restart_arrays

  type, bind(c) :: gmc_ffsl_fields
    type(c_ptr) :: q, u, v, mfx, mfy, cflx, cfly, divx, divy, qmfx, qmfy
  end type gmc_ffsl_fields

  type, bind(c) :: gmc_stats
    real(c_double)     :: step_ms
    integer(c_int64_t) :: steps
    integer(c_int64_t) :: kernel_launches
    integer(c_int32_t) :: member_layout
    integer(c_int32_t) :: layout_tuned
  end type gmc_stats

  interface

    subroutine gmc_config_default(cfg) bind(c, name='gmc_config_default')
      import
      type(gmc_config), intent(out) :: cfg
    end subroutine gmc_config_default

    integer(c_int) function gmc_create(cfg, ctx) bind(c, name='gmc_create')
      import
      type(gmc_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: ctx
    end function gmc_create

    integer(c_int) function gmc_lon_halo_width(ctx, out) bind(c, name='gmc_lon_halo_width')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: out
    end function gmc_lon_halo_width

    integer(c_int) function gmc_set_field(ctx, member, name, v) bind(c, name='gmc_set_field')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member
      character(kind=c_char), intent(in) :: name(*)
      type(gmc_view), intent(in) :: v
    end function gmc_set_field

    integer(c_int) function gmc_set_tracer(ctx, member, tracer, v) bind(c, name='gmc_set_tracer')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member, tracer
      type(gmc_view), intent(in) :: v
    end function gmc_set_tracer

    integer(c_int) function gmc_prepare(ctx) bind(c, name='gmc_prepare')
      import
      type(c_ptr), value :: ctx
    end function gmc_prepare

    integer(c_int) function gmc_step(ctx, nsteps) bind(c, name='gmc_step')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nsteps
    end function gmc_step

    integer(c_int) function gmc_get_field(ctx, member, name, v) bind(c, name='gmc_get_field')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member
      character(kind=c_char), intent(in) :: name(*)
      type(gmc_view), intent(in) :: v
    end function gmc_get_field

    integer(c_int) function gmc_get_tracer(ctx, member, tracer, v) bind(c, name='gmc_get_tracer')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member, tracer
      type(gmc_view), intent(in) :: v
    end function gmc_get_tracer

    integer(c_int) function gmc_step_io(ctx, member, in, n_in, nsteps, out, n_out) bind(c, name='gmc_step_io')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member, n_in, nsteps, n_out
      type(gmc_io), intent(in) :: in(*)
      type(gmc_io), intent(in) :: out(*)
    end function gmc_step_io

    ! history and restart files (restart_write / restart_read / history_write_h0;
    ! path is a null-terminated C string, e.g. trim(file) // c_null_char)
    integer(c_int) function gmc_restart_write(ctx, member, path, elapsed_seconds, opts) &
        bind(c, name='gmc_restart_write')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member
      character(kind=c_char), intent(in) :: path(*)
      real(c_double), value :: elapsed_seconds
      type(gmc_file_opts), intent(in) :: opts
    end function gmc_restart_write

    integer(c_int) function gmc_restart_read(ctx, member, path, opts, elapsed_seconds) &
        bind(c, name='gmc_restart_read')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member
      character(kind=c_char), intent(in) :: path(*)
      type(gmc_file_opts), intent(in) :: opts
      real(c_double), intent(out) :: elapsed_seconds
    end function gmc_restart_read

    integer(c_int) function gmc_history_write(ctx, member, path, elapsed_seconds, append, opts) &
        bind(c, name='gmc_history_write')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member, append
      character(kind=c_char), intent(in) :: path(*)
      real(c_double), value :: elapsed_seconds
      type(gmc_file_opts), intent(in) :: opts
    end function gmc_history_write

    integer(c_int) function gmc_output_wait(ctx) bind(c, name='gmc_output_wait')
      import
      type(c_ptr), value :: ctx
    end function gmc_output_wait

    integer(c_int) function gmc_restart_write_host(cfg, path, elapsed_seconds, opts, a, errbuf, errlen) &
        bind(c, name='gmc_restart_write_host')
      import
      type(gmc_config), intent(in) :: cfg
      character(kind=c_char), intent(in) :: path(*)
      real(c_double), value :: elapsed_seconds
      type(gmc_file_opts), intent(in) :: opts
      type(gmc_restart_arrays), intent(in) :: a
      character(kind=c_char), intent(out) :: errbuf(*)
      integer(c_int32_t), value :: errlen
    end function gmc_restart_write_host

    integer(c_int) function gmc_restart_read_host(cfg, path, opts, elapsed_seconds, a, errbuf, errlen) &
        bind(c, name='gmc_restart_read_host')
      import
      type(gmc_config), intent(in) :: cfg
      character(kind=c_char), intent(in) :: path(*)
      type(gmc_file_opts), intent(in) :: opts
      real(c_double), intent(out) :: elapsed_seconds
      type(gmc_restart_arrays), intent(in) :: a
      character(kind=c_char), intent(out) :: errbuf(*)
      integer(c_int32_t), value :: errlen
    end function gmc_restart_read_host

    integer(c_int) function gmc_diagnose(ctx, member, out) bind(c, name='gmc_diagnose')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: member
      type(gmc_diag), intent(out) :: out
    end function gmc_diagnose

    integer(c_int) function gmc_time_step(ctx, out) bind(c, name='gmc_time_step')
      import
      type(c_ptr), value :: ctx
      integer(c_int64_t), intent(out) :: out
    end function gmc_time_step

    ! the adv_calc_tracer_hflx_cell operator (adv_mod.F90:109) on device buffers
    integer(c_int) function gmc_ffsl_hflx(ctx, f, dt) bind(c, name='gmc_ffsl_hflx')
      import
      type(c_ptr), value :: ctx
      type(gmc_ffsl_fields), intent(in) :: f
      real(c_double), value :: dt
    end function gmc_ffsl_hflx

    integer(c_int) function gmc_ffsl_hflx_noalloc(ctx, f, dt) bind(c, name='gmc_ffsl_hflx_noalloc')
      import
      type(c_ptr), value :: ctx
      type(gmc_ffsl_fields), intent(in) :: f
      real(c_double), value :: dt
    end function gmc_ffsl_hflx_noalloc

    ! tangent-linear / adjoint of nsteps steps from the prepared state
    ! (views of u_lon, v_lat, gz; FP64 shallow-water model)
    integer(c_int) function gmc_tlm_step(ctx, nsteps, dx0, dxn) bind(c, name='gmc_tlm_step')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nsteps
      type(gmc_view), intent(in) :: dx0(3), dxn(3)
    end function gmc_tlm_step

    integer(c_int) function gmc_adjoint(ctx, nsteps, ckpt_every, lambda_n, lambda_0) bind(c, name='gmc_adjoint')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nsteps, ckpt_every
      type(gmc_view), intent(in) :: lambda_n(3), lambda_0(3)
    end function gmc_adjoint

    integer(c_int) function gmc_set_graphs(ctx, on) bind(c, name='gmc_set_graphs')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: on
    end function gmc_set_graphs

    ! page-lock a host array once (e.g. a state array exchanged every step)
    integer(c_int) function gmc_host_register(ptr, bytes) bind(c, name='gmc_host_register')
      import
      type(c_ptr), value :: ptr
      integer(c_size_t), value :: bytes
    end function gmc_host_register

    integer(c_int) function gmc_host_unregister(ptr) bind(c, name='gmc_host_unregister')
      import
      type(c_ptr), value :: ptr
    end function gmc_host_unregister

    integer(c_int) function gmc_get_stats(ctx, out) bind(c, name='gmc_get_stats')
      import
      type(c_ptr), value :: ctx
      type(gmc_stats), intent(out) :: out
    end function gmc_get_stats

    integer(c_int) function gmc_set_member_layout(ctx, layout) bind(c, name='gmc_set_member_layout')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: layout
    end function gmc_set_member_layout

    integer(c_int) function gmc_set_profiling(ctx, on) bind(c, name='gmc_set_profiling')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: on
    end function gmc_set_profiling

    integer(c_int) function gmc_kernel_profile(ctx, index, name, name_len, total_ms, launches) &
        bind(c, name='gmc_kernel_profile')
      import
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: index
      character(kind=c_char), intent(out) :: name(*)
      integer(c_size_t), value :: name_len
      real(c_double), intent(out) :: total_ms
      integer(c_int64_t), intent(out) :: launches
    end function gmc_kernel_profile

    type(c_ptr) function gmc_last_error(ctx) bind(c, name='gmc_last_error')
      import
      type(c_ptr), value :: ctx
    end function gmc_last_error

    subroutine gmc_destroy(ctx) bind(c, name='gmc_destroy')
      import
      type(c_ptr), value :: ctx
    end subroutine gmc_destroy

    integer(c_int) function gmc_mesh_metric(cfg, name, out, n) bind(c, name='gmc_mesh_metric')
      import
      type(gmc_config), intent(in) :: cfg
      character(kind=c_char), intent(in) :: name(*)
      real(c_double), intent(out) :: out(*)
      integer(c_size_t), value :: n
    end function gmc_mesh_metric

    integer(c_int) function gmc_filter_taps(cfg, which, lat, out, n) bind(c, name='gmc_filter_taps')
      import
      type(gmc_config), intent(in) :: cfg
      integer(c_int32_t), value :: which, lat
      integer(c_int32_t), intent(out) :: out(*)
      integer(c_size_t), value :: n
    end function gmc_filter_taps

    ! pass c_null_ptr for a field to skip it
    integer(c_int) function gmc_make_ic(cfg, kind, seed, noise_k, u_lon, v_lat, pt_or_gz, phs, gzs, q) &
        bind(c, name='gmc_make_ic')
      import
      type(gmc_config), intent(in) :: cfg
      integer(c_int32_t), value :: kind
      integer(c_int64_t), value :: seed
      real(c_double), value :: noise_k
      type(c_ptr), value :: u_lon, v_lat, pt_or_gz, phs, gzs, q
    end function gmc_make_ic

    ! measured FP64 FMA throughput of the current device (TFLOP/s)
    integer(c_int) function gmc_fp64_fma_peak(tflops) bind(c, name='gmc_fp64_fma_peak')
      import
      real(c_double), intent(out) :: tflops
    end function gmc_fp64_fma_peak

    ! measured FP32 FMA throughput of the current device (TFLOP/s)
    integer(c_int) function gmc_fp32_fma_peak(tflops) bind(c, name='gmc_fp32_fma_peak')
      import
      real(c_double), intent(out) :: tflops
    end function gmc_fp32_fma_peak

    integer(c_size_t) function c_strlen(s) bind(c, name='strlen')
      import
      type(c_ptr), value :: s
    end function c_strlen

  end interface

contains

  ! A view of a 3-D Fortran array with its own bounds (halos included).
  function view3(a) result(v)
    real(c_double), target, contiguous, intent(in) :: a(:,:,:)
    type(gmc_view) v
    v%data = c_loc(a)
    v%lb = 1
    v%ub = shape(a)
  end function view3

  ! The same for an array declared with explicit (halo) bounds, e.g.
  ! state%u_lon(lon_lb:lon_ub, lat_lb:lat_ub, lev_lb:lev_ub).
  function view3_bounds(a, lb, ub) result(v)
    integer, intent(in) :: lb(3), ub(3)
    real(c_double), target, intent(in) :: a(lb(1):ub(1), lb(2):ub(2), lb(3):ub(3))
    type(gmc_view) v
    v%data = c_loc(a)
    v%lb = lb
    v%ub = ub
  end function view3_bounds

  ! A 2-D field (surface pressure, surface geopotential): level bounds 1:1.
  function view2_bounds(a, lb, ub) result(v)
    integer, intent(in) :: lb(2), ub(2)
    real(c_double), target, intent(in) :: a(lb(1):ub(1), lb(2):ub(2))
    type(gmc_view) v
    v%data = c_loc(a)
    v%lb = [lb(1), lb(2), 1]
    v%ub = [ub(1), ub(2), 1]
  end function view2_bounds

  ! gmc_last_error as a Fortran string.
  function gmc_error_message(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(:), allocatable :: msg
    type(c_ptr) p
    character(kind=c_char), pointer :: chars(:)
    integer(c_size_t) n, i
    p = gmc_last_error(ctx)
    n = c_strlen(p)
    call c_f_pointer(p, chars, [n])
    allocate(character(n) :: msg)
    do i = 1, n
      msg(i:i) = chars(i)
    end do
  end function gmc_error_message

end module gmcore_gpu_mod
