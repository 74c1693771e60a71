! pimdgpu_mod.f90 -- ISO_C_BINDING interface of libpimdgpu (include/pimdgpu.h)
! for the reference's Fortran drivers.  Default INTEGER is 8 bytes and default
! REAL 8 bytes in the reference build (-i8 -r8), which is what integer(c_int64_t)
! and real(c_double) mirror; no CHARACTER or LOGICAL crosses the boundary except
! the NUL-terminated checkpoint path.
!
! Not compiled on the build machines (no Fortran compiler is installed there);
! the C prototypes it binds are exercised by the C++ drivers and the tests.
module pimdgpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: PG_OK = 0, PG_ERR_ARG = 1, PG_ERR_CUDA = 2, PG_ERR_STATE = 3, &
       PG_ERR_UNSUPPORTED = 4, PG_ERR_IO = 5, PG_ERR_NUMERIC = 6
  integer(c_int32_t), parameter :: PG_PES_1D = 1, PG_PES_2DTEST = 2, PG_PES_SYNTH9 = 3, &
       PG_PES_SYNTH18 = 4, PG_PES_HARMONIC = 5, PG_PES_DISTGAUSS = 6
  integer(c_int32_t), parameter :: PG_FP64 = 0, PG_MIXED = 1
  integer(c_int32_t), parameter :: PG_FORM_AUTO = 0, PG_FORM_PLAIN = 1, PG_FORM_FUSED = 2, &
       PG_FORM_TENSOR = 3
  integer(c_int32_t), parameter :: PG_ANDERSEN = 1, PG_LANGEVIN = 2
  integer(c_int32_t), parameter :: PG_TUNE_OFF = 0, PG_TUNE_CACHE = 1, PG_TUNE_ON = 2
  integer(c_int32_t), parameter :: PG_RING_NAN = 1, PG_RING_TIMEOUT = 2   ! per-ring status bits

  type, bind(c) :: pg_ti_config
     integer(c_int64_t) :: nbeads
     real(c_double)     :: beta, dt, tau, gamma
     integer(c_int32_t) :: thermostat, precision, form, cayley
     integer(c_int64_t) :: imin, noutput
     real(c_double)     :: dhdr_limit, init_sigma
  end type pg_ti_config

  type, bind(c) :: pg_lbfgs_opts
     integer(c_int32_t) :: m, max_backtracks
     integer(c_int64_t) :: maxiter
     real(c_double)     :: factr, pgtol
     integer(c_int32_t) :: cluster_ctas = 0, reserved = 0
  end type pg_lbfgs_opts

  interface
     integer(c_int) function pg_create(ctx, device) bind(c, name="pg_create")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), intent(out) :: ctx
       integer(c_int32_t), value :: device
     end function pg_create

     integer(c_int) function pg_destroy(ctx) bind(c, name="pg_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function pg_destroy

     type(c_ptr) function pg_last_error() bind(c, name="pg_last_error")
       import :: c_ptr
     end function pg_last_error

     ! replaces V_init + the mcmod_mass module variables
     integer(c_int) function pg_set_system(ctx, ndim, natom, mass, pes_id, params, nparams, V0) &
          bind(c, name="pg_set_system")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: ndim, natom, nparams
       real(c_double), intent(in) :: mass(*), params(*)
       integer(c_int32_t), value :: pes_id
       real(c_double), value :: V0
     end function pg_set_system

     ! batched V / Vprime (mcmod_*: V, Vprime, potforce)
     integer(c_int) function pg_pes_eval(ctx, nconf, x, V, grad, precision) bind(c, name="pg_pes_eval")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nconf
       real(c_double), intent(in) :: x(*)
       real(c_double), intent(out) :: V(*), grad(*)
       integer(c_int32_t), value :: precision
     end function pg_pes_eval

     ! batched Vdoubleprime
     integer(c_int) function pg_pes_hessian(ctx, nconf, x, hess, quirks) bind(c, name="pg_pes_hessian")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nconf
       real(c_double), intent(in) :: x(*)
       real(c_double), intent(out) :: hess(*)
       integer(c_int32_t), value :: quirks
     end function pg_pes_hessian

     ! a batch of propagate_pimd_pile / propagate_pimd_nm calls
     integer(c_int) function pg_propagate_pimd(ctx, cfg, ntask, nmc, a, b, dbdl, seed, stream, x, p, &
          dHdr, status) bind(c, name="pg_propagate_pimd")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr, pg_ti_config
       type(c_ptr), value :: ctx
       type(pg_ti_config), intent(in) :: cfg
       integer(c_int64_t), value :: ntask, nmc
       real(c_double), intent(in) :: a(*), b(*), dbdl(*)
       integer(c_int64_t), intent(in) :: seed(*)   ! uint64 on the C side
       integer(c_int32_t), intent(in) :: stream(*) ! uint32 on the C side
       real(c_double), intent(inout) :: x(*), p(*)
       real(c_double), intent(out) :: dHdr(*)
       integer(c_int32_t), intent(out) :: status(*)
     end function pg_propagate_pimd

     integer(c_int) function pg_ti_setup(ctx, cfg, nrings, nlambda, ring_lambda, ring_seed, ring_stream, &
          a, b, dbdl, xref, x0, p0) bind(c, name="pg_ti_setup")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr, pg_ti_config
       type(c_ptr), value :: ctx
       type(pg_ti_config), intent(in) :: cfg
       integer(c_int64_t), value :: nrings, nlambda
       integer(c_int32_t), intent(in) :: ring_lambda(*), ring_stream(*)
       integer(c_int64_t), intent(in) :: ring_seed(*)
       real(c_double), intent(in) :: a(*), b(*), dbdl(*), xref(*)
       type(c_ptr), value :: x0, p0      ! c_null_ptr or c_loc(array)
     end function pg_ti_setup

     integer(c_int) function pg_ti_advance(ctx, nsteps) bind(c, name="pg_ti_advance")
       import :: c_int, c_int64_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nsteps
     end function pg_ti_advance

     ! one context per bead number, advanced together on concurrent streams
     integer(c_int) function pg_ti_advance_group(ctxs, nctx, nsteps, device_ms) &
          bind(c, name="pg_ti_advance_group")
       import :: c_int, c_int64_t, c_double, c_ptr
       type(c_ptr), intent(in) :: ctxs(*)
       integer(c_int64_t), value :: nctx, nsteps
       real(c_double), intent(out) :: device_ms
     end function pg_ti_advance_group

     ! restart continuation: dHdr sums, sample counts and the step counter
     integer(c_int) function pg_ti_set_accumulators(ctx, dhdr_sum, nsamples, step) &
          bind(c, name="pg_ti_set_accumulators")
       import :: c_int, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: dhdr_sum(*)
       integer(c_int64_t), intent(in) :: nsamples(*)
       integer(c_int64_t), value :: step
     end function pg_ti_set_accumulators

     integer(c_int) function pg_ti_get_state(ctx, x, p) bind(c, name="pg_ti_get_state")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: x(*), p(*)
     end function pg_ti_get_state

     integer(c_int) function pg_ti_get_results(ctx, dhdr_sum, nsamples, nreinit, status) &
          bind(c, name="pg_ti_get_results")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: dhdr_sum(*)
       integer(c_int64_t), intent(out) :: nsamples(*), nreinit(*)
       integer(c_int32_t), intent(out) :: status(*)
     end function pg_ti_get_results

     integer(c_int) function pg_ti_lambda_reduce(ctx, mean, var, count) bind(c, name="pg_ti_lambda_reduce")
       import :: c_int, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: mean(*), var(*)
       integer(c_int64_t), intent(out) :: count(*)
     end function pg_ti_lambda_reduce

     integer(c_int) function pg_ti_checkpoint_save(ctx, path) bind(c, name="pg_ti_checkpoint_save")
       import :: c_int, c_char, c_ptr
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: path(*)
     end function pg_ti_checkpoint_save

     integer(c_int) function pg_ti_checkpoint_load(ctx, path) bind(c, name="pg_ti_checkpoint_load")
       import :: c_int, c_char, c_ptr
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: path(*)
     end function pg_ti_checkpoint_load

     integer(c_int32_t) function pg_version() bind(c, name="pg_version")
       import :: c_int32_t
     end function pg_version

     integer(c_int) function pg_nm_transform(ctx, P, ncol, xin, xout, precision) bind(c, name="pg_nm_transform")
       import :: c_int, c_ptr, c_int64_t, c_int32_t, c_double
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: P, ncol
       real(c_double), intent(in) :: xin(*)
       real(c_double), intent(out) :: xout(*)
       integer(c_int32_t), value :: precision
     end function pg_nm_transform

     integer(c_int) function pg_nm_transform_noalloc(P, ncol, d_in, d_out, stream) &
          bind(c, name="pg_nm_transform_noalloc")
       import :: c_int, c_ptr, c_int64_t
       integer(c_int64_t), value :: P, ncol
       type(c_ptr), value :: d_in, d_out, stream   ! device pointers, CUDA stream
     end function pg_nm_transform_noalloc

     integer(c_int) function pg_ti_advance_timed(ctx, nsteps, device_ms) bind(c, name="pg_ti_advance_timed")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nsteps
       real(c_double), intent(out) :: device_ms
     end function pg_ti_advance_timed

     integer(c_int) function pg_ti_get_step(ctx, step) bind(c, name="pg_ti_get_step")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int64_t), intent(out) :: step
     end function pg_ti_get_step

     integer(c_int) function pg_ti_get_form(ctx, nsteps, form, launches) bind(c, name="pg_ti_get_form")
       import :: c_int, c_ptr, c_int64_t, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nsteps
       integer(c_int32_t), intent(out) :: form
       integer(c_int64_t), intent(out) :: launches
     end function pg_ti_get_form

     integer(c_int) function pg_ti_kernel_times(ctx, nsteps, nkinds, ms_per_launch, count, bytes_per_launch, &
          names) bind(c, name="pg_ti_kernel_times")
       import :: c_int, c_ptr, c_int64_t, c_int32_t, c_double
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nsteps
       integer(c_int32_t), intent(out) :: nkinds
       real(c_double), intent(out) :: ms_per_launch(*), bytes_per_launch(*)
       integer(c_int64_t), intent(out) :: count(*)
       type(c_ptr), intent(out) :: names(*)   ! C strings (c_f_pointer to read them)
     end function pg_ti_kernel_times

     integer(c_int) function pg_ti_release(ctx) bind(c, name="pg_ti_release")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function pg_ti_release

     integer(c_int) function pg_spline(x, y, n, yp1, ypn, y2) bind(c, name="pg_spline")
       import :: c_int, c_int64_t, c_double
       real(c_double), intent(in) :: x(*), y(*)
       integer(c_int64_t), value :: n
       real(c_double), value :: yp1, ypn
       real(c_double), intent(out) :: y2(*)
     end function pg_spline

     integer(c_int) function pg_splint(xa, ya, y2a, n, x, y, dydx) bind(c, name="pg_splint")
       import :: c_int, c_int64_t, c_double
       real(c_double), intent(in) :: xa(*), ya(*), y2a(*)
       integer(c_int64_t), value :: n
       real(c_double), value :: x
       real(c_double), intent(out) :: y, dydx
     end function pg_splint

     integer(c_int) function pg_splitting_from_ratio(beta, qratio, delta) bind(c, name="pg_splitting_from_ratio")
       import :: c_int, c_double
       real(c_double), value :: beta, qratio
       real(c_double), intent(out) :: delta
     end function pg_splitting_from_ratio

     integer(c_int) function pg_splitting_two_beta(beta1, ratio1, beta2, ratio2, delta, betabar) &
          bind(c, name="pg_splitting_two_beta")
       import :: c_int, c_double
       real(c_double), value :: beta1, ratio1, beta2, ratio2
       real(c_double), intent(out) :: delta, betabar
     end function pg_splitting_two_beta

     integer(c_int) function pg_irrep_ratios(nirrep, nop, chars, rho, ratio) bind(c, name="pg_irrep_ratios")
       import :: c_int, c_int64_t, c_double
       integer(c_int64_t), value :: nirrep, nop
       real(c_double), intent(in) :: chars(*), rho(*)
       real(c_double), intent(out) :: ratio(*)
     end function pg_irrep_ratios

     integer(c_int) function pg_set_tuning(ctx, cache_path, mode) bind(c, name="pg_set_tuning")
       import :: c_int, c_ptr, c_char, c_int32_t
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: cache_path(*)   ! NUL-terminated
       integer(c_int32_t), value :: mode
     end function pg_set_tuning

     integer(c_int) function pg_ti_get_tuning(ctx, form, simt_threads, tc_steps) bind(c, name="pg_ti_get_tuning")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: form, simt_threads, tc_steps
     end function pg_ti_get_tuning

     integer(c_int) function pg_gauleg(x1, x2, x, w, n) bind(c, name="pg_gauleg")
       import :: c_int, c_int64_t, c_double
       real(c_double), value :: x1, x2
       real(c_double), intent(out) :: x(*), w(*)
       integer(c_int64_t), value :: n
     end function pg_gauleg

     integer(c_int) function pg_ti_assemble(nintegral, weights, mean, var, betan, dA, sigmaA, qratio) &
          bind(c, name="pg_ti_assemble")
       import :: c_int, c_int64_t, c_double
       integer(c_int64_t), value :: nintegral
       real(c_double), intent(in) :: weights(*), mean(*), var(*)
       real(c_double), value :: betan
       real(c_double), intent(out) :: dA, sigmaA, qratio
     end function pg_ti_assemble

     integer(c_int) function pg_fp32_peak(ctx, tflops) bind(c, name="pg_fp32_peak")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: tflops
     end function pg_fp32_peak

     integer(c_int) function pg_set_wait_limit(ctx, ns) bind(c, name="pg_set_wait_limit")
       import :: c_int, c_int64_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: ns
     end function pg_set_wait_limit

     ! instanton: fixedends, UMforceenergy, instanton, UMhessian, detJ + log sums
     integer(c_int) function pg_set_fixedends(ctx, fixedends) bind(c, name="pg_set_fixedends")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: fixedends
     end function pg_set_fixedends

     ! a and b are optional (passed as NULL when absent, Fortran 2018) for free ends
     integer(c_int) function pg_instanton_fg(ctx, nbeta, N, x, a, b, betan, UM, grad) &
          bind(c, name="pg_instanton_fg")
       import :: c_int, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nbeta, N
       real(c_double), intent(in) :: x(*), betan(*)
       real(c_double), intent(in), optional :: a(*), b(*)
       real(c_double), intent(out) :: UM(*), grad(*)
     end function pg_instanton_fg

     integer(c_int) function pg_instanton_optimize(ctx, nbeta, N, x, a, b, betan, opts, UM, niter, status) &
          bind(c, name="pg_instanton_optimize")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr, pg_lbfgs_opts
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nbeta, N
       real(c_double), intent(inout) :: x(*)
       real(c_double), intent(in) :: betan(*)
       real(c_double), intent(in), optional :: a(*), b(*)
       type(pg_lbfgs_opts), intent(in) :: opts
       real(c_double), intent(out) :: UM(*)
       integer(c_int64_t), intent(out) :: niter(*)
       integer(c_int32_t), intent(out) :: status(*)
     end function pg_instanton_optimize

     integer(c_int) function pg_um_hessian(ctx, N, betan, x, singlewell, quirks, band) &
          bind(c, name="pg_um_hessian")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: N
       real(c_double), value :: betan
       real(c_double), intent(in) :: x(*)
       integer(c_int32_t), value :: singlewell, quirks
       real(c_double), intent(out) :: band(*)
     end function pg_um_hessian

     integer(c_int) function pg_instanton_logdet(ctx, nbeta, N, x, betan, singlewell, skip_lowest, quirks, &
          lndet, eta2_min, nskipped) bind(c, name="pg_instanton_logdet")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: nbeta, N
       real(c_double), intent(in) :: x(*), betan(*)
       integer(c_int32_t), value :: singlewell, skip_lowest, quirks
       real(c_double), intent(out) :: lndet(*), eta2_min(*)
       integer(c_int64_t), intent(out) :: nskipped(*)
     end function pg_instanton_logdet

     integer(c_int) function pg_rpi_assemble(betan, UM, lndetJ, lndetJ0, S, omega, delta) &
          bind(c, name="pg_rpi_assemble")
       import :: c_int, c_double
       real(c_double), value :: betan, UM, lndetJ, lndetJ0
       real(c_double), intent(out) :: S, omega, delta
     end function pg_rpi_assemble
  end interface
end module pimdgpu
