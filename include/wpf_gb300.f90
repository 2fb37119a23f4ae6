! wpf_gb300.f90 -- Fortran 2003 binding (iso_c_binding) of the C ABI in wpf.h
! and wpf_net.h (libwpf_gb300.so), for the reference's Fortran driver.
!
! The reference runs its time step as argument-less module procedures over
! module-global arrays (wPFAW3D.f90:95-103, called from program main at
! :2249-2280).  A driver that uses this module keeps its arrays and its loop
! and swaps those calls for the functions below; every function returns the
! C status (WPF_OK = 0).  Field arrays are passed exactly as the reference
! declares them -- phase(0:nx+1,0:ny+1,0:nz+1) etc., Fortran order -- so no
! reshaping is needed.  The field arguments of wpf_upload and wpf_download
! are optional: an absent one reaches C as a NULL pointer (TS 29113 /
! Fortran 2018 interoperability), which skips that field.  Device addresses,
! CUDA streams and other opaque C pointers are type(c_ptr), value (pass
! c_null_ptr for "none").
!
! Every derived type is bind(C) and mirrors its C struct field for field
! (tests/test_fortran_binding.py checks names, order, kinds and offsets
! against the C headers and the Python ctypes mirror).
module wpf_gb300
   use, intrinsic :: iso_c_binding
   implicit none

   ! status codes (wpf.h)
   integer(c_int), parameter :: WPF_OK = 0
   integer(c_int), parameter :: WPF_ERR_ARG = 1
   integer(c_int), parameter :: WPF_ERR_CUDA = 2
   integer(c_int), parameter :: WPF_ERR_NOT_CONVERGED = 3
   integer(c_int), parameter :: WPF_ERR_NONFINITE = 4
   integer(c_int), parameter :: WPF_ERR_TIMEOUT = 5
   integer(c_int), parameter :: WPF_ERR_NOMEM = 6
   integer(c_int), parameter :: WPF_ERR_SINGULAR = 7
   integer(c_int), parameter :: WPF_ERR_TOO_LARGE = 8
   ! solver modes and flags
   integer(c_int32_t), parameter :: WPF_SOLVER_FP64 = 0
   integer(c_int32_t), parameter :: WPF_SOLVER_MIXED = 1
   integer(c_int32_t), parameter :: WPF_SOLVER_NO_GRAPHS = 1
   integer(c_int32_t), parameter :: WPF_SOLVER_EXTRAPOLATE = 2
   integer(c_int32_t), parameter :: WPF_SOLVER_NO_TMA = 4
   integer(c_int32_t), parameter :: WPF_SOLVER_STEP_GRAPH = 8
   integer(c_int32_t), parameter :: WPF_SOLVER_NET_ALWAYS = 16
   integer(c_int32_t), parameter :: WPF_SOLVER_FP64_UPDATE = 32
   integer(c_int32_t), parameter :: WPF_SOLVER_NET_COARSE = 64
   integer(c_int32_t), parameter :: WPF_SOLVER_FIXED_START = 128
   integer(c_int32_t), parameter :: WPF_NOALLOC_MAX_PLANES = 4096
   ! learned start (wpf_net.h)
   integer(c_int32_t), parameter :: WPF_NET_IN_CHANNELS = 16
   integer(c_int32_t), parameter :: WPF_NET_FEATURES = 6
   integer(c_int32_t), parameter :: WPF_NET_LAYERS = 7

   ! Param_type scalars the step uses (wPFAW3D.f90:27-76)
   type, bind(C) :: wpf_params
      integer(c_int32_t) :: nx, ny, nz
      integer(c_int32_t) :: ix_ref, iy_ref, iz_ref
      real(c_double) :: dx
      real(c_double) :: epsilon
      real(c_double) :: lambda
      real(c_double) :: porosity
      real(c_double) :: viscosity
      real(c_double) :: diffusion
      real(c_double) :: ral, rat
      real(c_double) :: permeab_hole
      real(c_double) :: alpha
      real(c_double) :: tfac
   end type wpf_params

   ! Well_type (wPFAW3D.f90:82-90)
   type, bind(C) :: wpf_well
      integer(c_int32_t) :: ix, iy, iz, pad
      real(c_double) :: pressure
      real(c_double) :: injection
      real(c_double) :: phase, concent
   end type wpf_well

   type, bind(C) :: wpf_solver_opts
      integer(c_int32_t) :: mode
      integer(c_int32_t) :: max_outer
      integer(c_int32_t) :: max_inner
      integer(c_int32_t) :: smooth_sweeps
      real(c_double) :: rtol
      real(c_double) :: inner_rtol
      integer(c_int64_t) :: sweep_min_cells
      integer(c_int32_t) :: w_from_level
      integer(c_int32_t) :: flags
      integer(c_int32_t) :: sweep_zchunk
      integer(c_int32_t) :: row_blocks_per_sm
   end type wpf_solver_opts

   type, bind(C) :: wpf_step_stats
      integer(c_int32_t) :: outer_iterations
      integer(c_int32_t) :: inner_iterations
      integer(c_int32_t) :: converged
      integer(c_int32_t) :: overshoot_cells
      real(c_double) :: relres
      real(c_double) :: taumin
      real(c_double) :: dtime
      real(c_double) :: max_courant
      real(c_double) :: solve_ms
      real(c_double) :: update_ms
      integer(c_int32_t) :: kernel_launches
      integer(c_int32_t) :: warm_start
      real(c_double) :: relres0
      integer(c_int32_t) :: active_cells
      integer(c_int32_t) :: device_resident
      integer(c_int32_t) :: interface_cells
   end type wpf_step_stats

   ! showProgress reductions (wPFAW3D.f90:1695, 1756-1810) + inlet flux
   type, bind(C) :: wpf_diag
      real(c_double) :: pv
      real(c_double) :: vcal
      real(c_double) :: rwhmax
      real(c_double) :: phase_max, phase_min, concent_max, concent_min
      real(c_double) :: pressure_ref
      real(c_double) :: inlet_flux
      real(c_double) :: phase_max_outlet
   end type wpf_diag

   interface
      ! ---- lifetime (allocate of loadConfig :441-449, freeField :2145-2149)
      integer(c_int) function wpf_create(p, out) bind(C, name="wpf_create")
         import :: c_int, c_ptr, wpf_params
         type(wpf_params), intent(in) :: p
         type(c_ptr), intent(out) :: out
      end function wpf_create
      integer(c_int) function wpf_destroy(h) bind(C, name="wpf_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function wpf_destroy
      type(c_ptr) function wpf_strerror(status) bind(C, name="wpf_strerror")
         import :: c_int, c_ptr
         integer(c_int), value :: status
      end function wpf_strerror
      integer(c_int) function wpf_device_bytes(h, bytes) bind(C, name="wpf_device_bytes")
         import :: c_int, c_ptr, c_int64_t
         type(c_ptr), value :: h
         integer(c_int64_t), intent(out) :: bytes
      end function wpf_device_bytes
      integer(c_int) function wpf_set_wells(h, wells, nwell) bind(C, name="wpf_set_wells")
         import :: c_int, c_ptr, c_int32_t, wpf_well
         type(c_ptr), value :: h
         type(wpf_well), intent(in) :: wells(*)
         integer(c_int32_t), value :: nwell
      end function wpf_set_wells
      ! ---- fields in and out (loadConfig :464-496, loadField :547-554)
      ! absent optional arrays reach C as NULL pointers (skip that field)
      integer(c_int) function wpf_upload(h, permeab_rock, phase, concent, pressure) &
            bind(C, name="wpf_upload")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in), optional :: permeab_rock(*), phase(*), concent(*), pressure(*)
      end function wpf_upload
      integer(c_int) function wpf_download(h, phase, concent, pressure, permeab, velocity, &
            dphasedt, dconcentdt) bind(C, name="wpf_download")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(inout), optional :: phase(*), concent(*), pressure(*)
         real(c_double), intent(inout), optional :: permeab(*), velocity(*)   ! 4*G and 3*G
         real(c_double), intent(inout), optional :: dphasedt(*), dconcentdt(*)
      end function wpf_download
      integer(c_int) function wpf_set_solver(h, o) bind(C, name="wpf_set_solver")
         import :: c_int, c_ptr, wpf_solver_opts
         type(c_ptr), value :: h
         type(wpf_solver_opts), intent(in) :: o
      end function wpf_set_solver
      integer(c_int) function wpf_get_solver(h, o) bind(C, name="wpf_get_solver")
         import :: c_int, c_ptr, wpf_solver_opts
         type(c_ptr), value :: h
         type(wpf_solver_opts), intent(out) :: o
      end function wpf_get_solver
      ! ---- the reference routines, one function each
      integer(c_int) function wpf_calc_permeability(h) bind(C, name="wpf_calc_permeability")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function wpf_calc_permeability
      integer(c_int) function wpf_solve_pressure(h, st) bind(C, name="wpf_solve_pressure")
         import :: c_int, c_ptr, wpf_step_stats
         type(c_ptr), value :: h
         type(wpf_step_stats), intent(out) :: st
      end function wpf_solve_pressure
      integer(c_int) function wpf_calc_velocity(h) bind(C, name="wpf_calc_velocity")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function wpf_calc_velocity
      integer(c_int) function wpf_calc_phase_deriv(h, taumin, overshoot_cells) &
            bind(C, name="wpf_calc_phase_deriv")
         import :: c_int, c_ptr, c_double, c_int32_t
         type(c_ptr), value :: h
         real(c_double), intent(out) :: taumin
         integer(c_int32_t), intent(out) :: overshoot_cells
      end function wpf_calc_phase_deriv
      integer(c_int) function wpf_calc_concent_deriv(h) bind(C, name="wpf_calc_concent_deriv")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function wpf_calc_concent_deriv
      integer(c_int) function wpf_evolve_phase(h, dtime) bind(C, name="wpf_evolve_phase")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), value :: dtime
      end function wpf_evolve_phase
      integer(c_int) function wpf_evolve_concent(h, dtime) bind(C, name="wpf_evolve_concent")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), value :: dtime
      end function wpf_evolve_concent
      ! ---- the fused loop body (:2226-2280) and runs of it
      integer(c_int) function wpf_step(h, itime, dtime_inout, st) bind(C, name="wpf_step")
         import :: c_int, c_ptr, c_int32_t, c_double, wpf_step_stats
         type(c_ptr), value :: h
         integer(c_int32_t), value :: itime
         real(c_double), intent(inout) :: dtime_inout
         type(wpf_step_stats), intent(out) :: st
      end function wpf_step
      integer(c_int) function wpf_run(h, itime0, nsteps, dtime_inout, last) bind(C, name="wpf_run")
         import :: c_int, c_ptr, c_int32_t, c_double, wpf_step_stats
         type(c_ptr), value :: h
         integer(c_int32_t), value :: itime0, nsteps
         real(c_double), intent(inout) :: dtime_inout
         type(wpf_step_stats), intent(out) :: last
      end function wpf_run
      ! ---- diagnostics (showProgress :1665-1836, getPressure :2151-2166)
      integer(c_int) function wpf_reduce(h, d) bind(C, name="wpf_reduce")
         import :: c_int, c_ptr, wpf_diag
         type(c_ptr), value :: h
         type(wpf_diag), intent(out) :: d
      end function wpf_reduce
      integer(c_int) function wpf_reduce_noalloc(p, d_phase, d_concent, out, stream) &
            bind(C, name="wpf_reduce_noalloc")
         import :: c_int, c_ptr, wpf_params, wpf_diag
         type(wpf_params), intent(in) :: p
         type(c_ptr), value :: d_phase, d_concent      ! device addresses
         type(wpf_diag), intent(out) :: out
         type(c_ptr), value :: stream                  ! cudaStream_t or c_null_ptr
      end function wpf_reduce_noalloc
      integer(c_int) function wpf_get_taumin(h, taumin) bind(C, name="wpf_get_taumin")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: taumin
      end function wpf_get_taumin
      integer(c_int) function wpf_set_taumin(h, taumin) bind(C, name="wpf_set_taumin")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), value :: taumin
      end function wpf_set_taumin
      integer(c_int) function wpf_get_stream(h, stream) bind(C, name="wpf_get_stream")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
         type(c_ptr), intent(out) :: stream
      end function wpf_get_stream
      integer(c_int) function wpf_launch_count(h, n) bind(C, name="wpf_launch_count")
         import :: c_int, c_ptr, c_int64_t
         type(c_ptr), value :: h
         integer(c_int64_t), intent(out) :: n
      end function wpf_launch_count
      integer(c_int) function wpf_set_kernel_timing(h, mask) bind(C, name="wpf_set_kernel_timing")
         import :: c_int, c_ptr, c_int32_t
         type(c_ptr), value :: h
         integer(c_int32_t), value :: mask               ! uint32_t bit mask
      end function wpf_set_kernel_timing
      integer(c_int) function wpf_kernel_times(h, ms, counts, n) bind(C, name="wpf_kernel_times")
         import :: c_int, c_ptr, c_double, c_int64_t, c_int32_t
         type(c_ptr), value :: h
         real(c_double), intent(out) :: ms(*)
         integer(c_int64_t), intent(out) :: counts(*)
         integer(c_int32_t), value :: n
      end function wpf_kernel_times
      ! ---- page-locked host buffers and the asynchronous saveResult snapshot
      integer(c_int) function wpf_host_alloc(bytes, ptr) bind(C, name="wpf_host_alloc")
         import :: c_int, c_ptr, c_int64_t
         integer(c_int64_t), value :: bytes
         type(c_ptr), intent(out) :: ptr
      end function wpf_host_alloc
      integer(c_int) function wpf_host_free(ptr) bind(C, name="wpf_host_free")
         import :: c_int, c_ptr
         type(c_ptr), value :: ptr
      end function wpf_host_free
      integer(c_int) function wpf_snapshot(h, out) bind(C, name="wpf_snapshot")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
         type(c_ptr), value :: out                     ! page-locked, 4*nx*ny*nz real(c_float)
      end function wpf_snapshot
      integer(c_int) function wpf_snapshot_wait(h) bind(C, name="wpf_snapshot_wait")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function wpf_snapshot_wait
      ! ---- ensembles of independent domains
      integer(c_int) function wpf_ensemble_run(members, n, itime0, nsteps, nthreads, dtime, stats, &
            status) bind(C, name="wpf_ensemble_run")
         import :: c_int, c_ptr, c_int32_t, c_double, wpf_step_stats
         type(c_ptr), intent(in) :: members(*)
         integer(c_int32_t), value :: n, itime0, nsteps, nthreads
         real(c_double), intent(inout) :: dtime(*)
         type(wpf_step_stats), intent(out) :: stats(*)
         integer(c_int32_t), intent(out) :: status(*)
      end function wpf_ensemble_run
      ! ---- self-checks of the integer-pipe conversions and the reciprocal
      integer(c_int) function wpf_check_conversions(host_values, n, mismatches) &
            bind(C, name="wpf_check_conversions")
         import :: c_int, c_double, c_int64_t
         real(c_double), intent(in) :: host_values(*)
         integer(c_int64_t), value :: n
         integer(c_int64_t), intent(out) :: mismatches
      end function wpf_check_conversions
      integer(c_int) function wpf_check_reciprocal(host_values, n, max_ulp, mismatches) &
            bind(C, name="wpf_check_reciprocal")
         import :: c_int, c_double, c_int64_t
         real(c_double), intent(in) :: host_values(*)
         integer(c_int64_t), value :: n
         integer(c_int64_t), intent(out) :: max_ulp, mismatches
      end function wpf_check_reciprocal
      integer(c_int) function wpf_measure_fp64_rate(tflops) bind(C, name="wpf_measure_fp64_rate")
         import :: c_int, c_double
         real(c_double), intent(out) :: tflops
      end function wpf_measure_fp64_rate
      ! ---- the learned start (wpf_net.h); device arrays as c_ptr
      integer(c_int) function wpf_net_create(nx, ny, nz, net) bind(C, name="wpf_net_create")
         import :: c_int, c_ptr, c_int32_t
         integer(c_int32_t), value :: nx, ny, nz
         type(c_ptr), intent(out) :: net
      end function wpf_net_create
      integer(c_int) function wpf_net_destroy(net) bind(C, name="wpf_net_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: net
      end function wpf_net_destroy
      integer(c_int) function wpf_net_init(net, seed) bind(C, name="wpf_net_init")
         import :: c_int, c_ptr, c_int64_t
         type(c_ptr), value :: net
         integer(c_int64_t), value :: seed               ! uint64_t
      end function wpf_net_init
      integer(c_int) function wpf_net_param_count(net, n) bind(C, name="wpf_net_param_count")
         import :: c_int, c_ptr, c_int64_t
         type(c_ptr), value :: net
         integer(c_int64_t), intent(out) :: n
      end function wpf_net_param_count
      integer(c_int) function wpf_net_get_params(net, host) bind(C, name="wpf_net_get_params")
         import :: c_int, c_ptr, c_float
         type(c_ptr), value :: net
         real(c_float), intent(out) :: host(*)
      end function wpf_net_get_params
      integer(c_int) function wpf_net_set_params(net, host) bind(C, name="wpf_net_set_params")
         import :: c_int, c_ptr, c_float
         type(c_ptr), value :: net
         real(c_float), intent(in) :: host(*)
      end function wpf_net_set_params
      integer(c_int) function wpf_net_forward(net, in, out, stream) bind(C, name="wpf_net_forward")
         import :: c_int, c_ptr
         type(c_ptr), value :: net, in, out, stream
      end function wpf_net_forward
      integer(c_int) function wpf_net_train_step(net, in, target, mask, lr, loss, stream) &
            bind(C, name="wpf_net_train_step")
         import :: c_int, c_ptr, c_float
         type(c_ptr), value :: net, in, target, mask
         real(c_float), value :: lr
         real(c_float), intent(out) :: loss
         type(c_ptr), value :: stream
      end function wpf_net_train_step
      integer(c_int) function wpf_net_get_grads(net, host) bind(C, name="wpf_net_get_grads")
         import :: c_int, c_ptr, c_float
         type(c_ptr), value :: net
         real(c_float), intent(out) :: host(*)
      end function wpf_net_get_grads
      integer(c_int) function wpf_net_get_activation(net, layer, host, n) &
            bind(C, name="wpf_net_get_activation")
         import :: c_int, c_ptr, c_int32_t, c_int64_t
         type(c_ptr), value :: net
         integer(c_int32_t), value :: layer
         type(c_ptr), value :: host                    ! uint16_t (bf16) array
         integer(c_int64_t), value :: n
      end function wpf_net_get_activation
      integer(c_int) function wpf_conv3d(cin, cout, nx, ny, nz, in, w, bias, relu, out16, out32, &
            stream) bind(C, name="wpf_conv3d")
         import :: c_int, c_ptr, c_int32_t
         integer(c_int32_t), value :: cin, cout, nx, ny, nz
         type(c_ptr), value :: in, w, bias
         integer(c_int32_t), value :: relu
         type(c_ptr), value :: out16, out32, stream
      end function wpf_conv3d
      integer(c_int) function wpf_conv3d_wgrad(cin, cout, nx, ny, nz, x, gy, gw, gb, stream) &
            bind(C, name="wpf_conv3d_wgrad")
         import :: c_int, c_ptr, c_int32_t
         integer(c_int32_t), value :: cin, cout, nx, ny, nz
         type(c_ptr), value :: x, gy, gw, gb, stream
      end function wpf_conv3d_wgrad
      integer(c_int) function wpf_set_warm_start_net(h, net) bind(C, name="wpf_set_warm_start_net")
         import :: c_int, c_ptr
         type(c_ptr), value :: h, net
      end function wpf_set_warm_start_net
      integer(c_int) function wpf_ws_features(h, dt_next, in) bind(C, name="wpf_ws_features")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), value :: dt_next
         type(c_ptr), value :: in
      end function wpf_ws_features
      integer(c_int) function wpf_ws_target(h, target) bind(C, name="wpf_ws_target")
         import :: c_int, c_ptr
         type(c_ptr), value :: h, target
      end function wpf_ws_target
   end interface
end module wpf_gb300
