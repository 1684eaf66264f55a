! ISO_C_BINDING interfaces of the GB300 library (libsam_gpu.so, C ABI in
! sam_gpu.h) for the reference's Fortran driver: one interface per exported
! routine, with the C types and argument order of sam_gpu.h.  Arrays are
! passed as c_ptr base addresses (c_loc of the same arrays sam.f passes
! today); character file names as NUL-terminated c_char arrays.  Every
! function returns 0 on success and a negative SAM_GPU_E* code otherwise;
! sam_gpu_error_message turns the library's last message into a Fortran
! string for stop_on_error.
!
! Build beside sam.f with any Fortran 2003 compiler, e.g.
!   gfortran -c sam_gpu.f90
! and link libsam_gpu.so.  The routine each interface replaces is named in
! its comment (file:line of the reference's subroutine statement).
module sam_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SAM_GPU_OK = 0, SAM_GPU_EINVAL = -1, SAM_GPU_ENOTINIT = -2
  integer(c_int), parameter :: SAM_GPU_EUNSUPPORTED = -3, SAM_GPU_ECUDA = -4, SAM_GPU_ENONFINITE = -5
  integer(c_int), parameter :: SAM_GPU_PREC_FP64 = 64, SAM_GPU_PREC_DD = 48, SAM_GPU_PREC_FP32 = 32
  integer(c_int), parameter :: SAM_GPU_MLP_PARAMS = 5122, SAM_GPU_MLP_FEATURES = 12
  integer(c_int), parameter :: SAM_GPU_MAX_PLANES = 16, SAM_GPU_NOALLOC_MAX_PLANES = 4096

  ! the COMMON values the hot path reads (/static/, /strat/, /gravity_wave/, /tstep/)
  type, bind(C) :: sam_gpu_config
    integer(c_int) :: nx, ny, nz, n_dealias, i_strat, i_cfl, nrk_max, rot_sav, i_les, precision
    real(c_double) :: xl, yl, zl, vis, pr, dt0, cfl0
    real(c_double) :: buoy_fac_x, buoy_fac_z, lapse, cos_theta, sin_theta, c_smag
  end type

  ! /dynamic/ and /statistics/ as the device keeps them
  type, bind(C) :: sam_gpu_stats
    real(c_double) :: time, dt, u_avg(4), u_var(4), u_max(4), energy, cfl_x, cfl_y, cfl_z
    integer(c_int) :: nonfinite, pad
  end type

  interface
    ! ---- context (the COMMON-block analogue; after fft_init, sam.f:51)
    integer(c_int) function sam_gpu_init(cfg) bind(C, name="sam_gpu_init")
      import :: c_int, sam_gpu_config
      type(sam_gpu_config), intent(in) :: cfg
    end function
    integer(c_int) function sam_gpu_finalize() bind(C, name="sam_gpu_finalize")
      import :: c_int
    end function
    integer(c_int) function sam_gpu_dims(out11) bind(C, name="sam_gpu_dims")
      import :: c_int
      integer(c_int), intent(out) :: out11(11)
    end function
    integer(c_int) function sam_gpu_set_tstep(nrk, dt, time) bind(C, name="sam_gpu_set_tstep")
      import :: c_int, c_double
      integer(c_int), value :: nrk
      real(c_double), value :: dt, time
    end function
    integer(c_int) function sam_gpu_get_stats(st) bind(C, name="sam_gpu_get_stats")
      import :: c_int, sam_gpu_stats
      type(sam_gpu_stats), intent(out) :: st
    end function
    integer(c_int) function sam_gpu_set_stream(cuda_stream) bind(C, name="sam_gpu_set_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: cuda_stream
    end function
    type(c_ptr) function sam_gpu_error_string() bind(C, name="sam_gpu_error_string")
      import :: c_ptr
    end function

    ! ---- per-routine drop-ins (host arrays in the reference layouts)
    ! z_trans_b.f:1
    integer(c_int) function sam_gpu_z_trans_b(u1, u2, n_var, isymm, u_c, u_r, u_i) bind(C, name="sam_gpu_z_trans_b")
      import :: c_int, c_ptr
      type(c_ptr), value :: u1, u2, isymm, u_c, u_r, u_i
      integer(c_int), value :: n_var
    end function
    ! x2z_decomp.f:1
    integer(c_int) function sam_gpu_x2z_decomp(u1, u2, n_var, u3) bind(C, name="sam_gpu_x2z_decomp")
      import :: c_int, c_ptr
      type(c_ptr), value :: u1, u2, u3
      integer(c_int), value :: n_var
    end function
    ! xy_trans_b.f:1
    integer(c_int) function sam_gpu_xy_trans_b(u1, u2, n_var, work) bind(C, name="sam_gpu_xy_trans_b")
      import :: c_int, c_ptr
      type(c_ptr), value :: u1, u2, work
      integer(c_int), value :: n_var
    end function
    ! xy_trans_f.f:1
    integer(c_int) function sam_gpu_xy_trans_f(u1, u2, n_var, work) bind(C, name="sam_gpu_xy_trans_f")
      import :: c_int, c_ptr
      type(c_ptr), value :: u1, u2, work
      integer(c_int), value :: n_var
    end function
    ! z2x_decomp.f:1
    integer(c_int) function sam_gpu_z2x_decomp(u1, u2, n_var, u3) bind(C, name="sam_gpu_z2x_decomp")
      import :: c_int, c_ptr
      type(c_ptr), value :: u1, u2, u3
      integer(c_int), value :: n_var
    end function
    ! z_trans_f.f:1
    integer(c_int) function sam_gpu_z_trans_f(u, n_var, isymm, u_r, u_i) bind(C, name="sam_gpu_z_trans_f")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, isymm, u_r, u_i
      integer(c_int), value :: n_var
    end function
    ! vel_max.f:1
    integer(c_int) function sam_gpu_vel_max(u, work) bind(C, name="sam_gpu_vel_max")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, work
    end function
    ! rhs.f:1
    integer(c_int) function sam_gpu_rhs(u, uu, r, u_sav, work) bind(C, name="sam_gpu_rhs")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, uu, r, u_sav, work
    end function
    ! x_deriv.f:1, y_deriv.f:1
    integer(c_int) function sam_gpu_x_deriv(u, du, work) bind(C, name="sam_gpu_x_deriv")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, du, work
    end function
    integer(c_int) function sam_gpu_y_deriv(u, du, work) bind(C, name="sam_gpu_y_deriv")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, du, work
    end function
    ! filter.f:1
    integer(c_int) function sam_gpu_filter(f_bar, f_hat, n_var) bind(C, name="sam_gpu_filter")
      import :: c_int, c_ptr
      type(c_ptr), value :: f_bar, f_hat
      integer(c_int), value :: n_var
    end function
    ! sm.f:1
    integer(c_int) function sam_gpu_sm(u, u_bar, s_bar, vt) bind(C, name="sam_gpu_sm")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, u_bar, s_bar, vt
    end function
    ! dm.f:1 (c_delta_sq: the volume-averaged coefficient dm.f logs to unit 8)
    integer(c_int) function sam_gpu_dm(u, u_bar, s_bar, s_mag_s, u_bar_u_bar, u_hat, s_hat, el, em, vt, &
                                       c_delta_sq) bind(C, name="sam_gpu_dm")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, u_bar, s_bar, s_mag_s, u_bar_u_bar, u_hat, s_hat, el, em, vt, c_delta_sq
    end function
    ! get_mean.f:1
    integer(c_int) function sam_gpu_get_mean(u, i_symm, i_remove, u_mean, jump, work) bind(C, name="sam_gpu_get_mean")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, u_mean, jump, work
      integer(c_int), value :: i_symm, i_remove
    end function

    ! ---- resident path (u, r and p stay in device memory between steps)
    integer(c_int) function sam_gpu_upload(u) bind(C, name="sam_gpu_upload")
      import :: c_int, c_ptr
      type(c_ptr), value :: u
    end function
    integer(c_int) function sam_gpu_download(u, r) bind(C, name="sam_gpu_download")
      import :: c_int, c_ptr
      type(c_ptr), value :: u, r
    end function
    integer(c_int) function sam_gpu_stage(nrk) bind(C, name="sam_gpu_stage")
      import :: c_int
      integer(c_int), value :: nrk
    end function
    integer(c_int) function sam_gpu_step(nsteps) bind(C, name="sam_gpu_step")
      import :: c_int
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function sam_gpu_profile_stage(nrk, reps, ms5) bind(C, name="sam_gpu_profile_stage")
      import :: c_int, c_float
      integer(c_int), value :: nrk, reps
      real(c_float), intent(out) :: ms5(5)
    end function
    integer(c_int) function sam_gpu_autotune(reps) bind(C, name="sam_gpu_autotune")
      import :: c_int
      integer(c_int), value :: reps
    end function
    integer(c_int) function sam_gpu_tiles(out6) bind(C, name="sam_gpu_tiles")
      import :: c_int
      integer(c_int), intent(out) :: out6(6)
    end function
    integer(c_int) function sam_gpu_set_tiles(in6) bind(C, name="sam_gpu_set_tiles")
      import :: c_int
      integer(c_int), intent(in) :: in6(6)
    end function
    integer(c_int) function sam_gpu_set_fft_schedule(sched5) bind(C, name="sam_gpu_set_fft_schedule")
      import :: c_int
      integer(c_int), intent(in) :: sched5(5)
    end function
    integer(c_int) function sam_gpu_fft_schedule(out5) bind(C, name="sam_gpu_fft_schedule")
      import :: c_int
      integer(c_int), intent(out) :: out5(5)
    end function
    integer(c_int) function sam_gpu_measure_fp64_peak(tflops) bind(C, name="sam_gpu_measure_fp64_peak")
      import :: c_int, c_double
      real(c_double), intent(out) :: tflops
    end function
    ! vel_max on device memory the caller owns, allocating nothing
    integer(c_int) function sam_gpu_vel_max_noalloc(u_dev, nx, ny, nzp, lu, stats_dev, stream) &
        bind(C, name="sam_gpu_vel_max_noalloc")
      import :: c_int, c_ptr
      type(c_ptr), value :: u_dev, stats_dev, stream
      integer(c_int), value :: nx, ny, nzp, lu
    end function

    ! ---- diagnostics on the resident state
    ! spectra.f:1 (out: ek, tk, dk, vt, sample per shell, then energy_w, div_rms, div_max)
    integer(c_int) function sam_gpu_spectra(out) bind(C, name="sam_gpu_spectra")
      import :: c_int, c_ptr
      type(c_ptr), value :: out
    end function
    ! div_check.f:1 (out4: div_avg, div_rms, div_max, n_div)
    integer(c_int) function sam_gpu_div_check(out4) bind(C, name="sam_gpu_div_check")
      import :: c_int, c_double
      real(c_double), intent(out) :: out4(4)
    end function
    ! cl_energy.f:1
    integer(c_int) function sam_gpu_cl_energy(e_cl) bind(C, name="sam_gpu_cl_energy")
      import :: c_int, c_double
      real(c_double), intent(out) :: e_cl
    end function
    ! force.f:1
    integer(c_int) function sam_gpu_force(ek_0, k_force) bind(C, name="sam_gpu_force")
      import :: c_int, c_ptr
      type(c_ptr), value :: ek_0
      integer(c_int), value :: k_force
    end function
    ! write_planes.f:1 and sam.f:145-166 (1-based plane indices)
    integer(c_int) function sam_gpu_planes(k_xy, n_xy, j_xz, n_xz, i_yz, n_yz, xy, xz, yz, mean) &
        bind(C, name="sam_gpu_planes")
      import :: c_int, c_ptr
      type(c_ptr), value :: k_xy, j_xz, i_yz, xy, xz, yz, mean
      integer(c_int), value :: n_xy, n_xz, n_yz
    end function

    ! ---- forcing and subgrid closures (new: the reference has none in the step)
    integer(c_int) function sam_gpu_set_forcing(seed, k_f, sigma, t_l, n_modes) bind(C, name="sam_gpu_set_forcing")
      import :: c_int, c_double, c_long_long
      integer(c_long_long), value :: seed
      real(c_double), value :: k_f, sigma, t_l
      integer(c_int), intent(out) :: n_modes
    end function
    integer(c_int) function sam_gpu_set_les(model, c_smag, pr_t) bind(C, name="sam_gpu_set_les")
      import :: c_int, c_double
      integer(c_int), value :: model
      real(c_double), value :: c_smag, pr_t
    end function
    integer(c_int) function sam_gpu_les_coef(c_delta_sq) bind(C, name="sam_gpu_les_coef")
      import :: c_int, c_double
      real(c_double), intent(out) :: c_delta_sq
    end function
    integer(c_int) function sam_gpu_mlp_set(params, n) bind(C, name="sam_gpu_mlp_set")
      import :: c_int, c_ptr
      type(c_ptr), value :: params
      integer(c_int), value :: n
    end function
    integer(c_int) function sam_gpu_mlp_get(params, n) bind(C, name="sam_gpu_mlp_get")
      import :: c_int, c_ptr
      type(c_ptr), value :: params
      integer(c_int), value :: n
    end function
    integer(c_int) function sam_gpu_mlp_forward(features, n, coef) bind(C, name="sam_gpu_mlp_forward")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: features, coef
      integer(c_long_long), value :: n
    end function
    integer(c_int) function sam_gpu_mlp_grad(features, target, n, grad, loss) bind(C, name="sam_gpu_mlp_grad")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: features, target, grad, loss
      integer(c_long_long), value :: n
    end function
    integer(c_int) function sam_gpu_mlp_set_backward(tensor_cores) bind(C, name="sam_gpu_mlp_set_backward")
      import :: c_int
      integer(c_int), value :: tensor_cores
    end function
    integer(c_int) function sam_gpu_mlp_train(features, target, n, steps, batch, lr, loss_hist) &
        bind(C, name="sam_gpu_mlp_train")
      import :: c_int, c_ptr, c_long_long, c_float
      type(c_ptr), value :: features, target, loss_hist
      integer(c_long_long), value :: n
      integer(c_int), value :: steps, batch
      real(c_float), value :: lr
    end function
    integer(c_int) function sam_gpu_box_filter(f, out) bind(C, name="sam_gpu_box_filter")
      import :: c_int, c_ptr
      integer(c_int), value :: f
      type(c_ptr), value :: out
    end function
    integer(c_int) function sam_gpu_closure_inputs(feat, grads) bind(C, name="sam_gpu_closure_inputs")
      import :: c_int, c_ptr
      type(c_ptr), value :: feat, grads
    end function
    integer(c_int) function sam_gpu_mma_selftest(a, b, d) bind(C, name="sam_gpu_mma_selftest")
      import :: c_int, c_ptr
      type(c_ptr), value :: a, b, d
    end function

    ! ---- ensembles of independent runs (one graph per step over all members)
    integer(c_int) function sam_gpu_ensemble_create(cfgs, n) bind(C, name="sam_gpu_ensemble_create")
      import :: c_int, sam_gpu_config
      integer(c_int), value :: n
      type(sam_gpu_config), intent(in) :: cfgs(n)
    end function
    integer(c_int) function sam_gpu_ensemble_select(m) bind(C, name="sam_gpu_ensemble_select")
      import :: c_int
      integer(c_int), value :: m
    end function
    integer(c_int) function sam_gpu_ensemble_step(nsteps) bind(C, name="sam_gpu_ensemble_step")
      import :: c_int
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function sam_gpu_ensemble_destroy() bind(C, name="sam_gpu_ensemble_destroy")
      import :: c_int
    end function
    integer(c_int) function sam_gpu_ensemble_set_persistent(ctas_per_sm) bind(C, name="sam_gpu_ensemble_set_persistent")
      import :: c_int
      integer(c_int), value :: ctas_per_sm
    end function
    integer(c_int) function sam_gpu_ensemble_persistent_members(n) bind(C, name="sam_gpu_ensemble_persistent_members")
      import :: c_int
      integer(c_int), intent(out) :: n
    end function

    ! ---- restart files: write_field.f:1, read_field.f:1, write_header.f:1, read_header.f:1
    integer(c_int) function sam_gpu_write_field(fname) bind(C, name="sam_gpu_write_field")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: fname(*)
    end function
    integer(c_int) function sam_gpu_read_field(fname) bind(C, name="sam_gpu_read_field")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: fname(*)
    end function
    integer(c_int) function sam_gpu_write_header(fname, nt) bind(C, name="sam_gpu_write_header")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: fname(*)
      integer(c_int), value :: nt
    end function
    integer(c_int) function sam_gpu_read_header(fname, nt) bind(C, name="sam_gpu_read_header")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: fname(*)
      integer(c_int), intent(out) :: nt
    end function

    ! ---- initial fields on the device (initial_field.f:1)
    integer(c_int) function sam_gpu_init_taylor_green() bind(C, name="sam_gpu_init_taylor_green")
      import :: c_int
    end function
    integer(c_int) function sam_gpu_init_random(seed, kind_u, flct_u, kind_t, flct_t) bind(C, name="sam_gpu_init_random")
      import :: c_int, c_double, c_long_long
      integer(c_long_long), value :: seed
      integer(c_int), value :: kind_u, kind_t
      real(c_double), value :: flct_u, flct_t
    end function
    integer(c_int) function sam_gpu_init_packet(seed, kx0, ky0, kz0, sigma, amplitude, noise) &
        bind(C, name="sam_gpu_init_packet")
      import :: c_int, c_double, c_long_long
      integer(c_long_long), value :: seed
      integer(c_int), value :: kx0, ky0, kz0
      real(c_double), value :: sigma, amplitude, noise
    end function
  end interface

contains

  ! The library's last error message as a Fortran string (for stop_on_error).
  function sam_gpu_error_message() result(msg)
    character(len=512) :: msg
    character(kind=c_char), pointer :: s(:)
    integer :: i
    msg = ' '
    call c_f_pointer(sam_gpu_error_string(), s, [512])
    do i = 1, 512
      if (s(i) == c_null_char) exit
      msg(i:i) = s(i)
    end do
  end function

end module sam_gpu
