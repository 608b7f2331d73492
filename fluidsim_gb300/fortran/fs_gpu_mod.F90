! fs_gpu_mod.F90 -- ISO_C_BINDING interfaces to libfluidsim_gb300.so
! (include/fluidsim_gpu.h) and thin wrappers with the argument lists of the
! reference's module subroutines.  A maintainer replaces the bodies of
! ptcl_step (ptcl_lib.F90:32-97) and lapl_solve (lapl_lib.F90:57-121) and the
! array rotation of main.F90:83-121 with calls to the wrappers below; the
! module arrays ni/ne/nt/nm and ph stay as host mirrors refreshed by
! fs_sync_from_device before writeOut (main.F90:297-303).
module fs_gpu_mod
  use iso_c_binding
  implicit none

  type, bind(C) :: fs_config
    integer(c_int32_t) :: abi_version, nx, ny, nspecies, coef_mode, cyl, rf, &
                          adaptive, precision, lapl_maxit, table_n, mg_smooth
    real(c_double) :: table_emin_ev, table_emax_ev, kir_arrh_a, kir_arrh_e, &
                      p_torr, tg_k, gam, n_init, l, w, ew, gap, vl, res, &
                      abs_tol, rel_tol, dt_min, lapl_rtol
  end type

  type, bind(C) :: fs_mesh
    type(c_ptr) :: dx, dlx, dy, dly, r, type_x, type_y
  end type

  interface
    integer(c_int) function fs_create(cfg, mesh, ctx) bind(C, name="fs_create")
      import :: c_int, c_ptr, fs_config, fs_mesh
      type(fs_config), intent(in) :: cfg
      type(fs_mesh), intent(in) :: mesh
      type(c_ptr), intent(out) :: ctx
    end function
    subroutine fs_destroy(ctx) bind(C, name="fs_destroy")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    integer(c_int) function fs_set_time(ctx, t, dt) bind(C, name="fs_set_time")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: t, dt
    end function
    integer(c_int) function fs_upload_state(ctx, ni, ne, nt, nm, ph, ld, nlev) &
        bind(C, name="fs_upload_state")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: ni(*), ne(*), nt(*), nm(*), ph(*)
      integer(c_int32_t), value :: ld, nlev
    end function
    integer(c_int) function fs_download_state(ctx, ni, ne, nt, nm, ph, ld, nlev) &
        bind(C, name="fs_download_state")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: ni(*), ne(*), nt(*), nm(*), ph(*)
      integer(c_int32_t), value :: ld, nlev
    end function
    integer(c_int) function fs_ptcl_step(ctx, dt, t_m, ida, idc, attempts) &
        bind(C, name="fs_ptcl_step")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: dt
      real(c_double), intent(out) :: t_m, ida, idc
      integer(c_int32_t), intent(out) :: attempts
    end function
    integer(c_int) function fs_lapl_solve(ctx, dt, lerr, iters, relres) &
        bind(C, name="fs_lapl_solve")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), value :: dt
      integer(c_int32_t), intent(out) :: lerr, iters
      real(c_double), intent(out) :: relres
    end function
    integer(c_int) function fs_accept(ctx) bind(C, name="fs_accept")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function fs_reject(ctx) bind(C, name="fs_reject")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function fs_max_ne(ctx, v) bind(C, name="fs_max_ne")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: v
    end function
    ! fs_max_ne with its scratch in a fixed device array of the library, for
    ! callers that may not allocate device memory once set up
    integer(c_int) function fs_max_ne_noalloc(ctx, v) bind(C, name="fs_max_ne_noalloc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: v
    end function
    ! learned Poisson preconditioner of the mixed solver (no reference counterpart)
    integer(c_int) function fs_lpc_init(ctx, crop, max_batch, max_samples, seed) &
        bind(C, name="fs_lpc_init")
      import :: c_ptr, c_int, c_int32_t, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: crop, max_batch, max_samples
      integer(c_int64_t), value :: seed
    end function
    integer(c_int) function fs_lpc_harvest(ctx, per_solve, added) bind(C, name="fs_lpc_harvest")
      import :: c_ptr, c_int, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: per_solve
      integer(c_int32_t), intent(out) :: added
    end function
    integer(c_int) function fs_lpc_train(ctx, iters, batch, lr, seed, loss_hist) bind(C, name="fs_lpc_train")
      import :: c_ptr, c_int, c_int32_t, c_int64_t, c_float
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: iters, batch
      real(c_float), value :: lr
      integer(c_int64_t), value :: seed
      type(c_ptr), value :: loss_hist
    end function
    integer(c_int) function fs_lpc_use(ctx, mode) bind(C, name="fs_lpc_use")
      import :: c_ptr, c_int, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: mode
    end function
    ! the FP64 Poisson solver's warm-start vector, part of the restart state
    integer(c_int) function fs_get_lapl_guess(ctx, d, ld) bind(C, name="fs_get_lapl_guess")
      import :: c_ptr, c_int, c_int32_t, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: d(*)
      integer(c_int32_t), value :: ld
    end function
    integer(c_int) function fs_set_lapl_guess(ctx, d, ld) bind(C, name="fs_set_lapl_guess")
      import :: c_ptr, c_int, c_int32_t, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: d(*)
      integer(c_int32_t), value :: ld
    end function
    ! solver and kernel configuration (no reference counterpart; the Poisson
    ! smoother stands where PETSc's run-time options did, lapl_lib.F90:50-54)
    integer(c_int) function fs_set_line_smoother(ctx, mode) bind(C, name="fs_set_line_smoother")
      import :: c_ptr, c_int, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: mode
    end function
    integer(c_int) function fs_line_smoother(ctx) bind(C, name="fs_line_smoother")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function fs_set_stage_tile(ctx, bx, by) bind(C, name="fs_set_stage_tile")
      import :: c_ptr, c_int, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: bx, by
    end function
    type(c_ptr) function fs_last_error(ctx) bind(C, name="fs_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    ! g_init output set-up (init = 1) and writeOut (init = 0), props.F90:239-320,
    ! main.F90:297-333; dir is a NUL-terminated path
    integer(c_int) function fs_write_output(ctx, dir, init) bind(C, name="fs_write_output")
      import :: c_ptr, c_int, c_int32_t, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: dir(*)
      integer(c_int32_t), value :: init
    end function
    integer(c_int) function fs_output_wait(ctx) bind(C, name="fs_output_wait")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
    end function
    ! circ_lib's Vd_pl, Vd_mi, Vd_or and Vsrc (get), Vd_pl, Vd_mi, Vd_or (set)
    integer(c_int) function fs_get_circuit(ctx, v4) bind(C, name="fs_get_circuit")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: v4(4)
    end function
    integer(c_int) function fs_set_circuit(ctx, v3) bind(C, name="fs_set_circuit")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: v3(3)
    end function
    ! sfc_lib's sig_pl, sig_mi, sig_or (bx+2 each)
    integer(c_int) function fs_get_surface_charge(ctx, sig_pl, sig_mi, sig_or) &
        bind(C, name="fs_get_surface_charge")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: sig_pl(*), sig_mi(*), sig_or(*)
    end function
    integer(c_int) function fs_set_surface_charge(ctx, sig_pl, sig_mi, sig_or) &
        bind(C, name="fs_set_surface_charge")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: sig_pl(*), sig_mi(*), sig_or(*)
    end function
    ! ptcl_step's err_prev and main's ts (restart)
    integer(c_int) function fs_get_controller(ctx, err_prev, ts) bind(C, name="fs_get_controller")
      import :: c_ptr, c_int, c_double, c_int64_t
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: err_prev
      integer(c_int64_t), intent(out) :: ts
    end function
    integer(c_int) function fs_set_controller(ctx, err_prev, ts) bind(C, name="fs_set_controller")
      import :: c_ptr, c_int, c_double, c_int64_t
      type(c_ptr), value :: ctx
      real(c_double), value :: err_prev
      integer(c_int64_t), value :: ts
    end function
  end interface

  type(c_ptr), save :: fs_ctx = c_null_ptr

contains

  ! stop with the library's message on a negative return code (the reference
  ! stops on the same conditions: ptcl_props.F90:174, ptcl_lib.F90:71)
  subroutine fs_check(rc)
    integer(c_int), intent(in) :: rc
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == 0) return
    call c_f_pointer(fs_last_error(fs_ctx), msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n+1) == c_null_char) exit
      n = n + 1
    end do
    write(*,*) 'fluidsim_gb300 error', rc, ': ', msg(1:n)
    stop
  end subroutine

  ! ptcl_step(g, ph, Em) with Em = 0: g%dt in, controller's dt out
  subroutine ptcl_step_gpu(dt, t_m)
    real(8), intent(inout) :: dt, t_m
    real(c_double) :: tm, ida, idc
    integer(c_int32_t) :: att
    call fs_check(fs_ptcl_step(fs_ctx, dt, tm, ida, idc, att))
    t_m = min(t_m, tm)
  end subroutine

  ! writeOut (main.F90:297-333): the record is appended by the library's
  ! writer thread; the g_init set-up passes init = 1 once
  subroutine write_out_gpu(path, init)
    character(len=*), intent(in) :: path
    integer, intent(in) :: init
    call fs_check(fs_write_output(fs_ctx, trim(path)//c_null_char, int(init, c_int32_t)))
  end subroutine

  ! Vd_pl, the electrode voltage main prints and writes (circ_lib.F90:8)
  real(8) function vd_gpu()
    real(c_double) :: v(4)
    call fs_check(fs_get_circuit(fs_ctx, v))
    vd_gpu = v(1)
  end function

  ! lapl_solve(g, ne(:,:,1), ni(:,:,1), nt(:,:,1), sig, lerr)
  subroutine lapl_solve_gpu(dt, lerr)
    real(8), intent(in) :: dt
    integer, intent(out) :: lerr
    integer(c_int32_t) :: l, it
    real(c_double) :: rr
    call fs_check(fs_lapl_solve(fs_ctx, dt, l, it, rr))
    lerr = l
  end subroutine
end module
