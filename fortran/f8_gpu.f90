! f8_gpu.f90 -- iso_c_binding interface to the GB300 step library (libf8.so).
!
! A drop-in for the body of the reference's step loop (fenep.f90:2477-2527):
! the main program keeps its own arrays, parameters and output code and calls
!
!   f8_create  once (replaces fft_init + ibm_init, fenep.f90:2459-2462)
!   f8_load    after init / input (fenep.f90:2460-2461)
!   f8_step    for Lstep/Gstep-sized chunks of steps
!   f8_store   before log_progress / get_data_binary / output
!   f8_grad    (optional) gradients of the drag w.r.t. Wi, beta, L^2 and the
!              cylinder centres by the discrete adjoint
!   f8_destroy at the end (fft_finalize)
!
! Array arguments are the reference's own arrays, passed with c_loc():
!   U, V, W, P, Phi : real(8) (0:NX+1, 0:NY+1, 0:NZ+1)
!   C               : real(8) (6, 0:NX+1, 0:NY+1, 0:NZ+1)  (3 components in 2D)
!   Ax0 .. Tz0, Fx..: real(8) (1:NX, 1:NY, 1:NZ)
! so they must be declared with the TARGET attribute.  The layouts are the
! C side's (include/f8.h): column-major, x fastest, component fastest for C.
module f8_gpu
    use, intrinsic :: iso_c_binding
    implicit none

    integer(c_int), parameter :: F8_OK = 0, F8_ERR_ARG = 1, F8_ERR_STATE = 2, F8_ERR_NOMEM = 3, &
                                 F8_ERR_CUDA = 4, F8_ERR_NAN = 5, F8_ERR_UNSUPPORTED = 6, &
                                 F8_ERR_NO_DEVICE = 7, F8_ERR_TOO_LARGE = 8, F8_WARN_NEWTON = 16, &
                                 F8_WARN_SOR = 17
    integer(c_int), parameter :: F8_FP64 = 0, F8_MIXED = 1
    integer(c_int), parameter :: F8_POISSON_FFT = 0, F8_POISSON_SOR = 1
    integer(c_int), parameter :: F8_BC_PERIODIC = 0, F8_BC_WALLS = 1, F8_BC_WALLS_Z = 2
    integer(c_int), parameter :: F8_IBM_CELL_VOLUME = 0, F8_IBM_ARC_VOLUME = 1
    integer(c_int), parameter :: F8_EIGEN_VIETA = 0, F8_EIGEN_CARDANO = 1, F8_EIGEN_SYLVESTER = 2, F8_EIGEN_SYMMETRIC = 3

    type, bind(C) :: f8_grid
        integer(c_int) :: dim, nx, ny, nz
        real(c_double) :: lx, ly, lz
        integer(c_int) :: bc_y
        real(c_double) :: uwall
    end type f8_grid

    type, bind(C) :: f8_phys
        real(c_double) :: re, wi, beta, lp2, dt
        real(c_double) :: newton_dc, newton_eps
        integer(c_int) :: newton_itrmax
        real(c_double) :: sor_omega, sor_eps
        integer(c_int) :: sor_itrmax
        integer(c_int) :: ab2_start
        integer(c_int) :: ibm_volume     ! 0: dX*dY*dZ (fenep), 1: pi*DC/NL*dX*dX (smac.f90:1129)
        integer(c_int) :: ibm_repeats    ! NS of smac.f90:20 (1 in fenep)
        integer(c_int) :: eigen_test     ! F8_EIGEN_*: the reference's eigen_method (fenep.f90:21)
    end type f8_phys

    type, bind(C) :: f8_cyl
        real(c_double) :: xc, yc, r, spin
        integer(c_int) :: filled
    end type f8_cyl

    type, bind(C) :: f8_fields
        type(c_ptr) :: u = c_null_ptr, v = c_null_ptr, w = c_null_ptr, p = c_null_ptr, phi = c_null_ptr
        type(c_ptr) :: c = c_null_ptr
        type(c_ptr) :: ax0 = c_null_ptr, ay0 = c_null_ptr, az0 = c_null_ptr
        type(c_ptr) :: tx0 = c_null_ptr, ty0 = c_null_ptr, tz0 = c_null_ptr
        type(c_ptr) :: fx = c_null_ptr, fy = c_null_ptr, fz = c_null_ptr
    end type f8_fields

    type, bind(C) :: f8_diag
        integer(c_int) :: step
        real(c_double) :: ke, cfl, trc_min, trc_max, trc_mean, div_max
        integer(c_long_long) :: newton_iters, newton_unconverged
        integer(c_int) :: poisson_iters, nan_found
        integer(c_long_long) :: kernel_launches
        real(c_double) :: trc_std
    end type f8_diag

    type, bind(C) :: f8_turb
        real(c_double) :: k_energy, k_staggered, lambda, re_lambda, epsilon
        real(c_double) :: l_kolmogorov, t_kolmogorov, u_kolmogorov, ep_energy, trc_mean, trc_std
    end type f8_turb

    interface
        subroutine f8_default_phys(phys) bind(C, name="f8_default_phys")
            import :: f8_phys
            type(f8_phys), intent(out) :: phys
        end subroutine f8_default_phys

        integer(c_int) function f8_create(ctx, grid, phys, cyls, ncyl, precision, poisson) bind(C, name="f8_create")
            import :: c_ptr, c_int, f8_grid, f8_phys, f8_cyl
            type(c_ptr), intent(out) :: ctx
            type(f8_grid), intent(in) :: grid
            type(f8_phys), intent(in) :: phys
            type(f8_cyl), intent(in) :: cyls(*)
            integer(c_int), value :: ncyl, precision, poisson
        end function f8_create

        integer(c_int) function f8_load(ctx, fields, step0) bind(C, name="f8_load")
            import :: c_ptr, c_int, f8_fields
            type(c_ptr), value :: ctx
            type(f8_fields), intent(in) :: fields
            integer(c_int), value :: step0
        end function f8_load

        ! drag: real(8) (3, ncyl, nsteps), or c_null_ptr
        integer(c_int) function f8_step(ctx, nsteps, drag) bind(C, name="f8_step")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps
            type(c_ptr), value :: drag
        end function f8_step

        integer(c_int) function f8_store(ctx, fields) bind(C, name="f8_store")
            import :: c_ptr, c_int, f8_fields
            type(c_ptr), value :: ctx
            type(f8_fields), intent(in) :: fields
        end function f8_store

        ! Gradient of J = sum(drag_weights * drag) + <seed, final state> by the
        ! discrete adjoint (FP64 2D/3D, mixed 3D).  drag_weights: real(8)
        ! (3, ncyl, nsteps) or c_null_ptr (time-averaged total x drag); seed,
        ! dJ_dstate: c_loc of an f8_fields or c_null_ptr; J: real(8) or
        ! c_null_ptr; dJ_dparams: real(8) (3 + 2*ncyl) = dWi, dbeta, dL^2,
        ! then (dxc, dyc) per cylinder; drag as f8_step's.
        integer(c_int) function f8_grad(ctx, nsteps, checkpoint_every, drag_weights, seed, J, dJ_dparams, &
                                        dJ_dstate, drag) bind(C, name="f8_grad")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps, checkpoint_every
            type(c_ptr), value :: drag_weights, seed, J, dJ_dparams, dJ_dstate, drag
        end function f8_grad

        integer(c_int) function f8_diagnostics(ctx, diag) bind(C, name="f8_diagnostics")
            import :: c_ptr, c_int, f8_diag
            type(c_ptr), value :: ctx
            type(f8_diag), intent(out) :: diag
        end function f8_diagnostics

        integer(c_int) function f8_markers(ctx, n, xy) bind(C, name="f8_markers")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: n
            type(c_ptr), value :: xy
        end function f8_markers

        ! codes: integer(1) (NX, rows, NZ) of the last step's SPD candidate choices
        integer(c_int) function f8_selection_codes(ctx, codes) bind(C, name="f8_selection_codes")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
            type(c_ptr), value :: codes
        end function f8_selection_codes

        ! out: real(8) (18, points) of the mid-plane slice (axis 2: x-y, 1: x-z, 0: y-z);
        ! variant 0: column 7 = KE (fenep.f90), 1: Q (fenep_mpi.f90)
        integer(c_int) function f8_slice(ctx, axis, variant, out) bind(C, name="f8_slice")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
            integer(c_int), value :: axis, variant
            type(c_ptr), value :: out
        end function f8_slice

        ! mean_u/v/w: real(8) (1:NX,1:NY,1:NZ) with the TARGET attribute, or c_null_ptr
        integer(c_int) function f8_turbulence(ctx, mean_u, mean_v, mean_w, out) bind(C, name="f8_turbulence")
            import :: c_ptr, c_int, f8_turb
            type(c_ptr), value :: ctx, mean_u, mean_v, mean_w
            type(f8_turb), intent(out) :: out
        end function f8_turbulence

        ! energy: real(8) (0:NX)
        integer(c_int) function f8_spectrum(ctx, mean_u, mean_v, mean_w, energy) bind(C, name="f8_spectrum")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx, mean_u, mean_v, mean_w, energy
        end function f8_spectrum

        ! mode 1: sums of U, V, W and centre-line probes; mode 2: squared fluctuations
        integer(c_int) function f8_stats_begin(ctx, mode, mean_u, mean_v, mean_w, max_steps) &
                bind(C, name="f8_stats_begin")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx, mean_u, mean_v, mean_w
            integer(c_int), value :: mode, max_steps
        end function f8_stats_begin

        ! probes: real(8) (NZ, steps, 3)
        integer(c_int) function f8_stats_read(ctx, sum_u, sum_v, sum_w, probes, nsteps) bind(C, name="f8_stats_read")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx, sum_u, sum_v, sum_w, probes
            integer(c_int), intent(out) :: nsteps
        end function f8_stats_read

        integer(c_int) function f8_set_timing(ctx, enable) bind(C, name="f8_set_timing")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
            integer(c_int), value :: enable
        end function f8_set_timing

        ! stage_ms: real(8) (7): C+-, Newton, momentum, IBM, Helmholtz, Poisson, projection
        integer(c_int) function f8_timing(ctx, total_ms, stage_ms, steps_timed) bind(C, name="f8_timing")
            import :: c_ptr, c_int, c_double, c_long_long
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: total_ms
            real(c_double), intent(out) :: stage_ms(*)
            integer(c_long_long), intent(out) :: steps_timed
        end function f8_timing

        integer(c_int) function f8_timing_reset(ctx) bind(C, name="f8_timing_reset")
            import :: c_ptr, c_int
            type(c_ptr), value :: ctx
        end function f8_timing_reset

        ! kernel_ms: real(8) (6) of the mixed step's single-launch kernels (enum f8_kernel)
        integer(c_int) function f8_kernel_timing(ctx, kernel_ms, steps_timed) bind(C, name="f8_kernel_timing")
            import :: c_ptr, c_int, c_double, c_long_long
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: kernel_ms(*)
            integer(c_long_long), intent(out) :: steps_timed
        end function f8_kernel_timing

        ! q and phi are device pointers (e.g. from a CUDA Fortran or OpenACC code)
        integer(c_int) function f8_fft_solve(nx, ny, nz, lx, ly, lz, q, phi, lhs0, lhs1) bind(C, name="f8_fft_solve")
            import :: c_int, c_double, c_ptr
            integer(c_int), value :: nx, ny, nz
            real(c_double), value :: lx, ly, lz
            type(c_ptr), value :: q, phi
            real(c_double), value :: lhs0, lhs1
        end function f8_fft_solve

        ! the same solve on a fixed device workspace, for callers that must not
        ! let the library allocate; (nx/2+1)*ny*nz <= 135168, no concurrent calls
        integer(c_int) function f8_fft_solve_noalloc(nx, ny, nz, lx, ly, lz, q, phi, lhs0, lhs1) &
                bind(C, name="f8_fft_solve_noalloc")
            import :: c_int, c_double, c_ptr
            integer(c_int), value :: nx, ny, nz
            real(c_double), value :: lx, ly, lz
            type(c_ptr), value :: q, phi
            real(c_double), value :: lhs0, lhs1
        end function f8_fft_solve_noalloc

        type(c_ptr) function f8_strerror_c(status) bind(C, name="f8_strerror")
            import :: c_ptr, c_int
            integer(c_int), value :: status
        end function f8_strerror_c

        subroutine f8_destroy(ctx) bind(C, name="f8_destroy")
            import :: c_ptr
            type(c_ptr), value :: ctx
        end subroutine f8_destroy
    end interface

contains

    ! Fortran string of a status code
    function f8_strerror(status) result(msg)
        integer(c_int), intent(in) :: status
        character(len=:), allocatable :: msg
        character(kind=c_char), pointer :: chars(:)
        type(c_ptr) :: p
        integer :: n
        interface
            integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
                import :: c_ptr, c_size_t
                type(c_ptr), value :: s
            end function c_strlen
        end interface
        p = f8_strerror_c(status)
        n = int(c_strlen(p))
        call c_f_pointer(p, chars, [n])
        allocate(character(len=n) :: msg)
        msg = transfer(chars(1:n), msg)
    end function f8_strerror

end module f8_gpu
