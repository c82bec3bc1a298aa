!=====================================================================================
! lbm_gpu_mod.F90 - ISO_C_BINDING interface to liblbmgpu.so (include/lbm_gpu.h).
!
! A Fortran driver shaped like `program main3d` (3DRB.F90:198-330) keeps its loop and
! replaces the module-array subroutines with calls into the GB300 library:
!
!   type(c_ptr) :: h
!   type(lbm_params), target :: p
!   ist = lbm_params_default(3, p)
!   p%nx = nx; p%ny = ny; p%nz = nz; p%Ra = Rayleigh; p%Pr = Prandtl; p%Mach = Mach
!   ist = lbm_create(p, 0, h)
!   ist = lbm_initial(h)                          ! call initial()
!   do while (...)
!     ist = lbm_step(h, 2000_c_int64_t)           ! 2000 x (collision ... macroT)
!     ist = lbm_check(h, errorU, errorT)          ! call check()
!   enddo
!   ist = lbm_RBcalc_Nu_global(h, Nu_global)
!   ist = lbm_calNuRe(h, Nu, Re)
!   ist = lbm_destroy(h)
!
! Shipped as source: no Fortran compiler was available where the library was built, so
! this module is not compiled or tested here.
!=====================================================================================
module lbm_gpu_mod
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: LBM_OK = 0, LBM_ERR_PARAM = 1, LBM_ERR_CUDA = 2, LBM_ERR_OOM = 3
  integer(c_int), parameter :: LBM_ERR_DIVERGED = 4, LBM_ERR_TIMEOUT = 5, LBM_ERR_STATE = 6
  integer(c_int), parameter :: LBM_ERR_TOO_LARGE = 7, LBM_ERR_IO = 8
  integer(c_int), parameter :: LBM_BACKUP_REFERENCE = 0, LBM_BACKUP_CONTINUE = 1
  integer(c_int), parameter :: LBM_RELOAD_REFERENCE = 0, LBM_RELOAD_CONTINUE = 1, LBM_RELOAD_AUTO = 2
  integer(c_int), parameter :: LBM_CELL_RB = 0, LBM_CELL_SIDE = 1
  integer(c_int), parameter :: LBM_BC_NOSLIP = 0, LBM_BC_PERIODIC = 1
  integer(c_int), parameter :: LBM_BCT_CONST = 0, LBM_BCT_ADIABATIC = 1, LBM_BCT_PERIODIC = 2
  integer(c_int), parameter :: LBM_FP64 = 0, LBM_FP32 = 1, LBM_FP16 = 2
  integer(c_int), parameter :: LBM_ARITH_REFERENCE = 0, LBM_ARITH_FIXED = 1  ! FP64: bitwise | integer pipes
  integer(c_int), parameter :: LBM_PATTERN_AB = 0, LBM_PATTERN_AA = 1   ! AA: one in-place array, same values
  integer(c_int), parameter :: LBM_FIELD_F = 0, LBM_FIELD_G = 1, LBM_FIELD_RHO = 2, LBM_FIELD_U = 3
  integer(c_int), parameter :: LBM_FIELD_V = 4, LBM_FIELD_W = 5, LBM_FIELD_T = 6
  integer(c_int), parameter :: LBM_FIELD_BX_PREV = 7, LBM_FIELD_BY_PREV = 8, LBM_FIELD_BZ_PREV = 9
  integer(c_int), parameter :: LBM_FIELD_FX = 10, LBM_FIELD_FY = 11, LBM_FIELD_F_POST = 12, LBM_FIELD_G_POST = 13
  integer(c_int), parameter :: LBM_OPT_SINGLE_KERNEL = 1, LBM_OPT_KCHUNK = 2, LBM_OPT_PAIRS = 3, LBM_OPT_STAGED = 4
  integer(c_int), parameter :: LBM_OPT_FP16_ROUNDING = 5   ! 1 stochastic (default), 0 nearest
  integer(c_int), parameter :: LBM_OPT_HOST_DIRECT = 6     ! state transfer on host arrays directly
  integer(c_int), parameter :: LBM_OPT_ROWS = 7            ! FP32/FP16: interior-row and face-row launches
  integer(c_int), parameter :: LBM_OPT_WIDE_INDEX = 8      ! fixed arithmetic: 64-bit indices in every kernel

  type, bind(C) :: lbm_params
    integer(c_int32_t) :: dim, nx, ny, nz
    real(c_double)     :: Ra, Pr, Mach, Thot, Tcold
    integer(c_int32_t) :: cell
    integer(c_int32_t) :: bc_flow(3), bc_thermal(3)
    integer(c_int32_t) :: use_g, legacy_thermal, precision, pattern
    integer(c_int64_t) :: seed
    real(c_double)     :: noise_amp
    integer(c_int32_t) :: side_heated_ha, arith       ! #define SideHeatedHa (2D); FP64 arithmetic
    real(c_double)     :: Ha, phi_deg
  end type lbm_params

  type, bind(C) :: lbm_nu_wall
    real(c_double) :: Nu_hot, Nu_cold, Nu_middle
    real(c_double) :: Nu_hot_max, Nu_hot_max_position, Nu_hot_min, Nu_hot_min_position
  end type lbm_nu_wall

  ! mid-line / mid-plane velocity maximum (SideHeatedcalc_*mid_max, RBcalc_*mid_max)
  type, bind(C) :: lbm_mid_max
    real(c_double) :: value, pos1, pos2, mid
  end type lbm_mid_max

  ! 2D stream-function summary of calc_psi_vort_and_output
  type, bind(C) :: lbm_psi_summary
    real(c_double) :: psi_center, psi_center_abs, psi_abs_max, x_at_max, y_at_max, psi_center_abs_fine
  end type lbm_psi_summary

  interface
    integer(c_int) function lbm_params_default(dim, p) bind(C, name="lbm_params_default")
      import :: c_int, lbm_params
      integer(c_int), value :: dim
      type(lbm_params) :: p
    end function
    integer(c_int) function lbm_create(p, device, h) bind(C, name="lbm_create")
      import :: c_int, c_ptr, lbm_params
      type(lbm_params), intent(in) :: p
      integer(c_int), value :: device
      type(c_ptr) :: h
    end function
    integer(c_int) function lbm_destroy(h) bind(C, name="lbm_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_initial(h) bind(C, name="lbm_initial")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_collision(h) bind(C, name="lbm_collision")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_streaming(h) bind(C, name="lbm_streaming")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_bounceback(h) bind(C, name="lbm_bounceback")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_macro(h) bind(C, name="lbm_macro")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_collisionT(h) bind(C, name="lbm_collisionT")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_streamingT(h) bind(C, name="lbm_streamingT")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_bouncebackT(h) bind(C, name="lbm_bouncebackT")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_macroT(h) bind(C, name="lbm_macroT")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_step(h, nsteps) bind(C, name="lbm_step")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: h
      integer(c_int64_t), value :: nsteps
    end function
    integer(c_int) function lbm_check(h, errU, errT) bind(C, name="lbm_check")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: errU, errT
    end function
    ! check as the reference's subroutine does it: convergence[3D].plt and
    ! convergence_all[_3D].plt appended in dir (C string; '' = working directory), the line
    ! echoed when echo /= 0
    integer(c_int) function lbm_check_log(h, dir, echo, errU, errT) bind(C, name="lbm_check_log")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: dir(*)
      integer(c_int), value :: echo
      real(c_double) :: errU, errT
    end function
    integer(c_int) function lbm_append_convergence_tecplot(h, filename, itc, errorU, errorT) &
        bind(C, name="lbm_append_convergence_tecplot")
      import :: c_int, c_ptr, c_char, c_int64_t, c_double
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: filename(*)
      integer(c_int64_t), value :: itc
      real(c_double), value :: errorU, errorT
    end function
    integer(c_int) function lbm_append_convergence_master_tecplot(h, filename, zone, itc, errorU, errorT) &
        bind(C, name="lbm_append_convergence_master_tecplot")
      import :: c_int, c_ptr, c_char, c_int64_t, c_double
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: filename(*), zone(*)
      integer(c_int64_t), value :: itc
      real(c_double), value :: errorU, errorT
    end function
    integer(c_int) function lbm_case_tag(h, buf, len) bind(C, name="lbm_case_tag")
      import :: c_int, c_ptr, c_char, c_size_t
      type(c_ptr), value :: h
      character(kind=c_char) :: buf(*)
      integer(c_size_t), value :: len
    end function
    integer(c_int) function lbm_calNuRe(h, Nu, Re) bind(C, name="lbm_calNuRe")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: Nu, Re
    end function
    integer(c_int) function lbm_RBcalc_Nu_global(h, Nu) bind(C, name="lbm_RBcalc_Nu_global")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: Nu
    end function
    integer(c_int) function lbm_RBcalc_Nu_wall_avg(h, w) bind(C, name="lbm_RBcalc_Nu_wall_avg")
      import :: c_int, c_ptr, lbm_nu_wall
      type(c_ptr), value :: h
      type(lbm_nu_wall) :: w
    end function
    ! state arrays in the reference's own layout, e.g. f(0:qf-1,nx,ny,nz)
    integer(c_int) function lbm_get_state(h, field, host, count) bind(C, name="lbm_get_state")
      import :: c_int, c_ptr, c_double, c_size_t
      type(c_ptr), value :: h
      integer(c_int), value :: field
      real(c_double) :: host(*)
      integer(c_size_t), value :: count
    end function
    integer(c_int) function lbm_set_state(h, field, host, count) bind(C, name="lbm_set_state")
      import :: c_int, c_ptr, c_double, c_size_t
      type(c_ptr), value :: h
      integer(c_int), value :: field
      real(c_double), intent(in) :: host(*)
      integer(c_size_t), value :: count
    end function
    ! restart files: call lbm_backupData(h, 'backupFile3D-'//trim(filename)//'.bin'//c_null_char, LBM_BACKUP_CONTINUE)
    ! replaces backupData; lbm_reload replaces the loadInitField = 1 branch of initial
    integer(c_int) function lbm_backupData(h, path, flags) bind(C, name="lbm_backupData")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: flags
    end function
    integer(c_int) function lbm_reload(h, path, mode) bind(C, name="lbm_reload")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: mode
    end function
    integer(c_int) function lbm_reload_form(h) bind(C, name="lbm_reload_form")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    ! side-heated cavity (SideHeatedCell) and mid-line / mid-plane diagnostics
    integer(c_int) function lbm_SideHeatedcalc_Nu_global(h, Nu) bind(C, name="lbm_SideHeatedcalc_Nu_global")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: Nu
    end function
    integer(c_int) function lbm_SideHeatedcalc_Nu_wall_avg(h, w) bind(C, name="lbm_SideHeatedcalc_Nu_wall_avg")
      import :: c_int, c_ptr, lbm_nu_wall
      type(c_ptr), value :: h
      type(lbm_nu_wall) :: w
    end function
    integer(c_int) function lbm_SideHeatedcalc_umid_max(h, m) bind(C, name="lbm_SideHeatedcalc_umid_max")
      import :: c_int, c_ptr, lbm_mid_max
      type(c_ptr), value :: h
      type(lbm_mid_max) :: m
    end function
    integer(c_int) function lbm_SideHeatedcalc_vmid_max(h, m) bind(C, name="lbm_SideHeatedcalc_vmid_max")
      import :: c_int, c_ptr, lbm_mid_max
      type(c_ptr), value :: h
      type(lbm_mid_max) :: m
    end function
    integer(c_int) function lbm_SideHeatedcalc_wmid_max(h, m) bind(C, name="lbm_SideHeatedcalc_wmid_max")
      import :: c_int, c_ptr, lbm_mid_max
      type(c_ptr), value :: h
      type(lbm_mid_max) :: m
    end function
    integer(c_int) function lbm_RBcalc_umid_max(h, m) bind(C, name="lbm_RBcalc_umid_max")
      import :: c_int, c_ptr, lbm_mid_max
      type(c_ptr), value :: h
      type(lbm_mid_max) :: m
    end function
    integer(c_int) function lbm_RBcalc_vmid_max(h, m) bind(C, name="lbm_RBcalc_vmid_max")
      import :: c_int, c_ptr, lbm_mid_max
      type(c_ptr), value :: h
      type(lbm_mid_max) :: m
    end function
    integer(c_int) function lbm_RBcalc_wmid_max(h, m) bind(C, name="lbm_RBcalc_wmid_max")
      import :: c_int, c_ptr, lbm_mid_max
      type(c_ptr), value :: h
      type(lbm_mid_max) :: m
    end function
    ! snapshot writers: output_binary, output_Tecplot(pltFolderPrefix, itc), calc_psi_vort_and_output
    integer(c_int) function lbm_output_binary(h, path) bind(C, name="lbm_output_binary")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: path(*)
    end function
    integer(c_int) function lbm_output_Tecplot(h, prefix, number) bind(C, name="lbm_output_Tecplot")
      import :: c_int, c_ptr, c_char, c_int64_t
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: prefix(*)
      integer(c_int64_t), value :: number
    end function
    ! prefix = c_null_ptr: no file, the summary only
    integer(c_int) function lbm_calc_psi_vort_and_output(h, prefix, number, nFinePerUnit, summary) &
        bind(C, name="lbm_calc_psi_vort_and_output")
      import :: c_int, c_ptr, c_int64_t, lbm_psi_summary
      type(c_ptr), value :: h, prefix
      integer(c_int64_t), value :: number
      integer(c_int), value :: nFinePerUnit
      type(lbm_psi_summary) :: summary
    end function
    ! handle utilities
    integer(c_int) function lbm_sync(h) bind(C, name="lbm_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int64_t) function lbm_itc(h) bind(C, name="lbm_itc")
      import :: c_int64_t, c_ptr
      type(c_ptr), value :: h
    end function
    type(c_ptr) function lbm_last_error(h) bind(C, name="lbm_last_error")   ! C string
      import :: c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function lbm_get_params(h, p) bind(C, name="lbm_get_params")
      import :: c_int, c_ptr, lbm_params
      type(c_ptr), value :: h
      type(lbm_params) :: p
    end function
    integer(c_int) function lbm_set_option(h, option, value) bind(C, name="lbm_set_option")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: option, value
    end function
    integer(c_int) function lbm_footprint(p, bytes) bind(C, name="lbm_footprint")
      import :: c_int, c_size_t, lbm_params
      type(lbm_params), intent(in) :: p
      integer(c_size_t) :: bytes
    end function
  end interface
end module lbm_gpu_mod
