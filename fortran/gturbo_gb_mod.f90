! gturbo_gb_mod.f90 -- Fortran 2003 iso_c_binding interface to libgturbo_gb.so
! (include/gturbo_gb.h), for the driver program in gturbo_driver.f90.
!
! COMPILE-UNVERIFIED: no Fortran compiler exists on the machines this library
! was built and tested on.  The module uses only standard iso_c_binding
! features (bind(C) derived types and interfaces, value arguments, c_ptr).
!
! Layout: the spectral state is complex(c_double_complex) b(NX/2+1, NY, NZ),
! x fastest -- the reference's complex*16 (NX2P1, NY, NZ) (main.f90:14) passed
! as is.  Physical fields are real(c_double) u(NX, NY, NZ).  Every function
! returns GT_OK (0) or a negative GT_E* status.
module gturbo_gb
  use iso_c_binding
  implicit none
  private :: c_int, c_int32_t, c_int64_t, c_double, c_char, c_ptr, c_size_t

  integer(c_int), parameter, public :: GT_OK = 0, GT_EINVAL = -1, GT_ENOMEM = -2, GT_ECUDA = -3
  integer(c_int), parameter, public :: GT_ENFORC = -4, GT_ENONFINITE = -5, GT_EIO = -6
  integer(c_int), parameter, public :: GT_ETIMEOUT = -7
  integer(c_int32_t), parameter, public :: GT_FORCING_NONE = 0, GT_FORCING_3D3C = 1, GT_FORCING_2D2C = 2
  integer(c_int32_t), parameter, public :: GT_DT2_AS_BUILT = 0, GT_DT2_RK2 = 1
  integer(c_int32_t), parameter, public :: GT_PREC_FP64 = 0, GT_PREC_MIXED = 1

  ! struct gt_params (field order and kinds as in the C header)
  type, bind(C), public :: gt_params
    integer(c_int32_t) :: nx, ny, nz
    real(c_double)     :: xlx, xly, xlz
    real(c_double)     :: nu, alpnu, mu, alpmu
    real(c_double)     :: dt, omega
    real(c_double)     :: rtrunc
    integer(c_int32_t) :: truncate
    real(c_double)     :: famp, k1f, k2f
    integer(c_int32_t) :: forcing, dt2_mode, precision, device
  end type gt_params

  ! struct gt_diag: glob's energy and enstrophy terms (diagnostics.f90:114-199)
  type, bind(C), public :: gt_diag
    real(c_double)     :: energy(9), enstrophy(9), helicity, inpe, inpz
    integer(c_int64_t) :: nonfinite
  end type gt_diag

  interface
    ! ---- host only ------------------------------------------------------
    integer(c_int) function gt_params_default(p) bind(C, name="gt_params_default")
      import :: gt_params, c_int
      type(gt_params), intent(out) :: p
    end function
    integer(c_int) function gt_params_read(path, p) bind(C, name="gt_params_read")
      import :: gt_params, c_int, c_char
      character(kind=c_char), intent(in) :: path(*)
      type(gt_params), intent(inout) :: p
    end function
    integer(c_int) function gt_memory_estimate(p, nbytes) bind(C, name="gt_memory_estimate")
      import :: gt_params, c_int, c_size_t
      type(gt_params), intent(in) :: p
      integer(c_size_t), intent(out) :: nbytes
    end function
    integer(c_int) function gt_init_noise(p, seed, ux, uy, uz) bind(C, name="gt_init_noise")
      import :: gt_params, c_int, c_int32_t, c_double
      type(gt_params), intent(in) :: p
      integer(c_int32_t), intent(inout) :: seed
      real(c_double), intent(out) :: ux(*), uy(*), uz(*)
    end function
    integer(c_int) function gt_seed_read(path, seed) bind(C, name="gt_seed_read")
      import :: c_int, c_int32_t, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int32_t), intent(out) :: seed
    end function
    integer(c_int) function gt_seed_write(path, seed) bind(C, name="gt_seed_write")
      import :: c_int, c_int32_t, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int32_t), value :: seed
    end function
    integer(c_int) function gt_frame_read(path, ifr, t) bind(C, name="gt_frame_read")
      import :: c_int, c_int32_t, c_double, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int32_t), intent(out) :: ifr
      real(c_double), intent(out) :: t
    end function
    integer(c_int) function gt_frame_write(path, ifr, t) bind(C, name="gt_frame_write")
      import :: c_int, c_int32_t, c_double, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int32_t), value :: ifr
      real(c_double), value :: t
    end function
    integer(c_int) function gt_field_read_f32(path, nx, ny, nz, u) bind(C, name="gt_field_read_f32")
      import :: c_int, c_int32_t, c_float, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int32_t), value :: nx, ny, nz
      real(c_float), intent(out) :: u(*)
    end function
    integer(c_int) function gt_field_write_f32(path, nx, ny, nz, u) bind(C, name="gt_field_write_f32")
      import :: c_int, c_int32_t, c_float, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int32_t), value :: nx, ny, nz
      real(c_float), intent(in) :: u(*)
    end function
    ! ---- handle ----------------------------------------------------------
    integer(c_int) function gt_create(p, h) bind(C, name="gt_create")
      import :: gt_params, c_int, c_ptr
      type(gt_params), intent(in) :: p
      type(c_ptr), intent(out) :: h
    end function
    integer(c_int) function gt_destroy(h) bind(C, name="gt_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function gt_set_state(h, bx, by, bz) bind(C, name="gt_set_state")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex), intent(in) :: bx(*), by(*), bz(*)
    end function
    integer(c_int) function gt_get_state(h, bx, by, bz) bind(C, name="gt_get_state")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex), intent(out) :: bx(*), by(*), bz(*)
    end function
    integer(c_int) function gt_set_state_physical(h, ux, uy, uz, cc) bind(C, name="gt_set_state_physical")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: ux(*), uy(*), uz(*)
      real(c_double), intent(out) :: cc
    end function
    integer(c_int) function gt_rk2_step(h, nsteps, seed) bind(C, name="gt_rk2_step")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: h
      integer(c_int32_t), value :: nsteps
      integer(c_int32_t), intent(inout) :: seed
    end function
    ! ek, ek2d and flux are c_loc's of NX/2 reals each, or c_null_ptr to skip
    ! (flux = c_null_ptr also skips the extra nonlinear term)
    integer(c_int) function gt_diagnostics(h, d, ek, ek2d, flux) bind(C, name="gt_diagnostics")
      import :: c_int, c_ptr, gt_diag
      type(c_ptr), value :: h
      type(gt_diag), intent(out) :: d
      type(c_ptr), value :: ek, ek2d, flux
    end function
    integer(c_int) function gt_energy(h, e) bind(C, name="gt_energy")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: e(3)
    end function
    integer(c_int) function gt_velocity(h, ux, uy, uz) bind(C, name="gt_velocity")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: ux(*), uy(*), uz(*)
    end function
    integer(c_int) function gt_check_finite(h) bind(C, name="gt_check_finite")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    type(c_ptr) function gt_last_error() bind(C, name="gt_last_error")
      import :: c_ptr
    end function
  end interface

  public :: gt_params_default, gt_params_read, gt_memory_estimate, gt_init_noise
  public :: gt_seed_read, gt_seed_write, gt_frame_read, gt_frame_write
  public :: gt_field_read_f32, gt_field_write_f32, gt_create, gt_destroy, gt_set_state
  public :: gt_get_state, gt_set_state_physical, gt_rk2_step, gt_diagnostics, gt_energy
  public :: gt_velocity, gt_check_finite, gt_last_error, gt_check

contains

  ! Stops the program with the library's message when a call failed.
  subroutine gt_check(ierr, what)
    integer(c_int), intent(in) :: ierr
    character(len=*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (ierr == GT_OK) return
    call c_f_pointer(gt_last_error(), msg, [1024])
    n = 0
    do while (n < 1024)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write(0, '(a, a, i0, a, 1024a)') what, ': status ', ierr, ' ', msg(1:n)
    stop 1
  end subroutine gt_check

end module gturbo_gb
