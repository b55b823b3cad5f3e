! ec2d_gpu_mod.f90 -- Fortran 2003 (iso_c_binding) interface to the C-ABI of
! libec2d_gpu.so, declared in ec2d_gpu.h beside this file.
!
! The reference program (opencfd_ec2d_v1.5.4.f90 and the sub_*.f90 files it
! includes) adds this module and replaces the bodies of its time-marching
! calls with the functions below; reading control.in / bc2d_1.in / Mesh2d.dat
! and writing Residual.dat / flow2d.dat stay in Fortran.  Every function
! returns 0 or an EC2D_ERR_* code.  Arrays are passed in the reference's own
! layout: x(1:nx,1:ny), U(NVAR,-1:nx+1,-1:ny+1), the 9-integer bc_msg rows.
!
! The spliced main loop (opencfd_ec2d_v1.5.4.f90:172-186):
!
!   ierr = ec2d_create(0, ctx)
!   ierr = ec2d_add_case(ctx, params, icase)        ! read_parameter values
!   do m = 1, Mesh(1)%Num_Block                     ! Creat_Mesh1 + read_bcin
!     B => Mesh(1)%Block(m)
!     ierr = ec2d_add_block(ctx, icase, B%nx, B%ny, x_of_block, y_of_block, &
!                           B%subface, bc9_of_block)
!   enddo
!   ierr = ec2d_setup(ctx)
!   ierr = ec2d_init_flow(ctx)
!   do while (tt .lt. t_end)
!     ierr = ec2d_step(ctx, 1)
!     ierr = ec2d_residual(ctx, icase, 1, Mesh(1)%Res_max, Mesh(1)%Res_rms, Mesh(1)%Kstep, tt)
!     if (ierr .eq. EC2D_ERR_STATE) then; print*, "T <1.d-5 !"; stop; endif
!     if (mod(Mesh(1)%Kstep, Kstep_show) .eq. 0) call output_Res(1)
!     if (mod(Mesh(1)%Kstep, Kstep_save) .eq. 0) then
!       do m = 1, Mesh(1)%Num_Block
!         ierr = ec2d_download_U(ctx, icase, 1, m, Mesh(1)%Block(m)%U)
!       enddo
!       call output(1)
!     endif
!   enddo
!   call ec2d_destroy(ctx)
module ec2d_gpu_mod
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: EC2D_OK = 0, EC2D_ERR_ARG = 1, EC2D_ERR_CUDA = 2, &
                               EC2D_ERR_STATE = 3, EC2D_ERR_TIMEOUT = 4, &
                               EC2D_ERR_UNSUPPORTED = 5, EC2D_ERR_NOMEM = 6

  ! the scalars of control.in (Global_Var, opencfd_ec2d_v1.5.4.f90:103-110),
  ! same order and types as struct ec2d_params
  type, bind(C) :: ec2d_params
    real(c_double) :: Ma, Re, gamma, AoA, Pr, t_end
    integer(c_int) :: Kstep_save, If_viscous, Iflag_turbulence_model, Iflag_init
    integer(c_int) :: Iflag_local_dt
    real(c_double) :: dt_global, CFL, dtmax, dtmin
    integer(c_int) :: Time_Method
    real(c_double) :: P_outlet, T_inf, Twall, vt_inf, Kt_inf, Wt_inf
    integer(c_int) :: Iflag_Scheme, Iflag_flux, IFlag_Reconstruction, Kstep_show
    integer(c_int) :: Num_Mesh, Num_Threads, Nstep_Inner_Limit
    real(c_double) :: Res_Inner_Limit
    integer(c_int) :: Pre_Step_Mesh(3)
    real(c_double) :: xaxis, yaxis
    integer(c_int) :: mg_lusgs
  end type ec2d_params

  interface
    ! ---- set-up: read_parameter, Creat_Mesh1, read_bcin, FDM.in, dist_wall.dat
    integer(c_int) function ec2d_version() bind(C)
      import
    end function
    integer(c_int) function ec2d_create(device, ctx) bind(C)
      import
      integer(c_int), value :: device
      type(c_ptr) :: ctx
    end function
    subroutine ec2d_destroy(ctx) bind(C)
      import
      type(c_ptr), value :: ctx
    end subroutine
    integer(c_int) function ec2d_add_case(ctx, p, case_id) bind(C)
      import
      type(c_ptr), value :: ctx
      type(ec2d_params) :: p
      integer(c_int) :: case_id
    end function
    integer(c_int) function ec2d_add_block(ctx, case_id, nx, ny, x, y, nsub, bc9) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, nx, ny, nsub
      real(c_double) :: x(*), y(*)
      integer(c_int) :: bc9(*)
    end function
    integer(c_int) function ec2d_set_fdm_block(ctx, case_id, block) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, block
    end function
    integer(c_int) function ec2d_set_wall_distance(ctx, case_id, block, dw) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, block
      real(c_double) :: dw(*)
    end function
    integer(c_int) function ec2d_setup(ctx) bind(C)
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function ec2d_num_mesh(ctx, num_mesh) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int) :: num_mesh
    end function
    integer(c_int) function ec2d_block_dims(ctx, case_id, mesh, block, nx, ny, nvar) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh, block
      integer(c_int) :: nx, ny, nvar
    end function
    ! ---- state: Init_flow, init_flow_read, output
    integer(c_int) function ec2d_init_flow(ctx) bind(C)
      import
      type(c_ptr), value :: ctx
    end function
    ! dual time stepping after a restart (init_flow_read + ec2d_upload_U):
    ! U(n) = U(n-1) = the restart state, first physical step one-step form
    integer(c_int) function ec2d_dual_time_start(ctx) bind(C)
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function ec2d_upload_U(ctx, case_id, mesh, block, U) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh, block
      real(c_double) :: U(*)
    end function
    integer(c_int) function ec2d_download_U(ctx, case_id, mesh, block, U) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh, block
      real(c_double) :: U(*)
    end function
    ! ---- the main loop body and its outputs
    integer(c_int) function ec2d_step(ctx, nsteps) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function ec2d_residual(ctx, case_id, mesh, res_max, res_rms, kstep, tt) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh
      real(c_double) :: res_max(6), res_rms(6), tt
      integer(c_int) :: kstep
    end function
    integer(c_int) function ec2d_run_to_drop(ctx, drop, r0, max_steps, max_seconds, check_every, &
                                             steps, worst_ratio, seconds) bind(C)
      import
      type(c_ptr), value :: ctx
      real(c_double), value :: drop, max_seconds
      type(c_ptr), value :: r0            ! c_null_ptr: the first step's residual
      integer(c_int), value :: max_steps, check_every
      integer(c_int) :: steps
      real(c_double) :: worst_ratio, seconds
    end function
    integer(c_int) function ec2d_status(ctx, case_id, code, block, i, j) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id
      integer(c_int) :: code, block, i, j
    end function
    integer(c_int) function ec2d_clear_status(ctx, case_id) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id
    end function
    ! output(1) at Kstep_save without stalling the loop: ec2d_snapshot queues
    ! a copy of a case's U and Amu_t to pinned host memory behind the steps;
    ! after later steps, ec2d_snapshot_wait gives its Kstep and tt and
    ! ec2d_snapshot_U / ec2d_snapshot_amut fill the reference's arrays
    ! U(NVAR,-1:nx+1,-1:ny+1) and Amu_t(-1:nx+1,-1:ny+1) of each block
    integer(c_int) function ec2d_snapshot(ctx, case_id) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id
    end function
    integer(c_int) function ec2d_snapshot_wait(ctx, case_id, kstep, tt) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int) :: case_id, kstep
      real(c_double) :: tt
    end function
    integer(c_int) function ec2d_snapshot_U(ctx, block, U) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: block
      real(c_double) :: U(*)
    end function
    integer(c_int) function ec2d_snapshot_amut(ctx, block, amut) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: block
      real(c_double) :: amut(*)
    end function
    integer(c_int) function ec2d_forces(ctx, case_id, cl, cd, cm) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id
      real(c_double) :: cl, cd, cm
    end function
    integer(c_int) function ec2d_wall_cf(ctx, case_id, block, sub, cf, xc, maxn, n) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, block, sub, maxn
      real(c_double) :: cf(*), xc(*)
      integer(c_int) :: n
    end function
    integer(c_int) function ec2d_get_field(ctx, case_id, mesh, block, field, out) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh, block, field
      real(c_double) :: out(*)
    end function
    integer(c_int) function ec2d_field_size(ctx, case_id, mesh, block, field, n) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh, block, field
      integer(c_int) :: n
    end function
    integer(c_int) function ec2d_set_field(ctx, case_id, mesh, block, field, in) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id, mesh, block, field
      real(c_double) :: in(*)
    end function
    ! ---- finer hooks with the reference's routine names
    integer(c_int) function ec2d_comput_residual(ctx, mesh) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: mesh
    end function
    integer(c_int) function ec2d_boundary_condition(ctx, mesh) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: mesh
    end function
    integer(c_int) function ec2d_update_buffer(ctx, mesh) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: mesh
    end function
    integer(c_int) function ec2d_du_lusgs(ctx, mesh, alfa1) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: mesh
      real(c_double), value :: alfa1
    end function
    integer(c_int) function ec2d_time_advance(ctx, mesh) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: mesh
    end function
    integer(c_int) function ec2d_interpolation2h(ctx, m1, m2, flag) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: m1, m2, flag
    end function
    integer(c_int) function ec2d_prolong(ctx, m1, m2, flag) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: m1, m2, flag
    end function
    integer(c_int) function ec2d_force_function(ctx, mesh) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: mesh
    end function
    ! ---- additions with no counterpart in the reference
    integer(c_int) function ec2d_set_graphs(ctx, enable) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: enable
    end function
    integer(c_int) function ec2d_set_lusgs_precision(ctx, bits) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: bits
    end function

    ! turbulent multigrid: coarse levels keep the restricted eddy viscosity
    integer(c_int) function ec2d_mg_eddy_viscosity(ctx, enable, current) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: enable
      integer(c_int) :: current
    end function
    integer(c_int) function ec2d_set_coarse_precision(ctx, bits) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: bits
    end function
    integer(c_int) function ec2d_autotune(ctx, trial_steps, lusgs_cs, rows_per_warp, concurrent, &
                                          ms_per_step) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: trial_steps
      integer(c_int) :: lusgs_cs, rows_per_warp, concurrent
      real(c_double) :: ms_per_step
    end function
    ! the autotuner's choices, read and applied without timing (a host keeps
    ! them per launch signature: buf receives a NUL-terminated line)
    integer(c_int) function ec2d_launch_config(ctx, lusgs_cs, rows, lanes, concurrent, tile_residual) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int) :: lusgs_cs, rows, lanes, concurrent, tile_residual
    end function
    integer(c_int) function ec2d_set_launch_config(ctx, lusgs_cs, rows, lanes, concurrent, tile_residual) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: lusgs_cs, rows, lanes, concurrent, tile_residual
    end function
    integer(c_int) function ec2d_launch_signature(ctx, buf, len, needed) bind(C)
      import
      type(c_ptr), value :: ctx
      character(kind=c_char) :: buf(*)
      integer(c_int), value :: len
      integer(c_int) :: needed
    end function
    integer(c_int) function ec2d_set_case_shape(ctx, case_id, shape) bind(C)
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: case_id
      real(c_double), value :: shape
    end function
    integer(c_int) function ec2d_residual_norms_noalloc(res, nvar, ncell, out, stream) bind(C)
      import
      type(c_ptr), value :: res, out, stream   ! device pointers and a cudaStream_t
      integer(c_int), value :: nvar, ncell
    end function
    integer(c_int) function ec2d_sync(ctx) bind(C)
      import
      type(c_ptr), value :: ctx
    end function
    ! learned warm start
    integer(c_int) function ec2d_mlp_create(device, hidden_layers, width, seed, m) bind(C)
      import
      integer(c_int), value :: device, hidden_layers, width
      integer(c_long_long), value :: seed
      type(c_ptr) :: m
    end function
    subroutine ec2d_mlp_destroy(m) bind(C)
      import
      type(c_ptr), value :: m
    end subroutine
    integer(c_int) function ec2d_mlp_add_samples(m, ctx) bind(C)
      import
      type(c_ptr), value :: m, ctx
    end function
    integer(c_int) function ec2d_mlp_fit_normalization(m) bind(C)
      import
      type(c_ptr), value :: m
    end function
    integer(c_int) function ec2d_mlp_train(m, steps, batch, lr, loss_out) bind(C)
      import
      type(c_ptr), value :: m
      integer(c_int), value :: steps, batch
      real(c_double), value :: lr
      real(c_double) :: loss_out
    end function
    integer(c_int) function ec2d_mlp_warm_start(m, ctx, n_fallback) bind(C)
      import
      type(c_ptr), value :: m, ctx
      integer(c_int) :: n_fallback
    end function
  end interface
end module ec2d_gpu_mod
