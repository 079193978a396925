! gturbo_driver.f90 -- the Gturbo3D time loop (main.f90) with the GB300
! library doing the work: the program reads curframe.dat, params.dat and the
! seed file as the reference's driver does, sets up the initial state, runs
! npas RK2 steps with the diagnostics at the reference's times and writes the
! velocity fields, the seed file and curframe.dat at the end.
!
! COMPILE-UNVERIFIED: no Fortran compiler exists on the machines this library
! was built and tested on.  Build sketch:
!   <f90> -O2 gturbo_gb_mod.f90 gturbo_driver.f90 -L<dir of libgturbo_gb.so> -lgturbo_gb
!
! Differences from the reference's driver, by design: the grid is a runtime
! value of gt_params (here set from the parameters below, as modules.f90:4
! sets it at compile time); the forcing variant and precision are fields of
! gt_params instead of link-time choices (Makefile:20-33); the diagnostics are
! returned by the library and written with this program's own list-directed
! statements.
program gturbo_driver
  use iso_c_binding
  use gturbo_gb
  implicit none

  integer(c_int32_t), parameter :: NX = 512, NY = 512, NZ = 512   ! grid (modules.f90:4)
  integer, parameter :: NBIN = NX / 2

  type(gt_params) :: p
  type(gt_diag) :: d
  type(c_ptr) :: h
  integer(c_int32_t) :: ifr, seed, npas, iout, imix, ipas, jfr
  real(c_double) :: t, cc
  real(c_double), allocatable, target :: ux(:,:,:), uy(:,:,:), uz(:,:,:)
  real(c_double), target :: ek(NBIN), ek2d(NBIN), flux(NBIN)
  real(c_float), allocatable :: u32(:,:,:)
  integer :: c0, c1, crate
  character(len=64) :: name

  call system_clock(c0, crate)

  ! curframe.dat: frame and time of the run to continue (main.f90:37-39)
  call gt_check(gt_frame_read('./curframe.dat'//c_null_char, ifr, t), 'curframe.dat')
  ! the seed of that frame (main.f90:41-45)
  write(name, "('./files/seed.',i3.3)") ifr
  call gt_check(gt_seed_read(trim(name)//c_null_char, seed), trim(name))

  ! params.dat (inieuler.f90:14-20): the physics goes into gt_params, the run
  ! control (npas, iout, imix on the fourth line) stays with the driver
  call gt_check(gt_params_default(p), 'gt_params_default')
  p%nx = NX; p%ny = NY; p%nz = NZ
  call gt_check(gt_params_read('./params.dat'//c_null_char, p), 'params.dat')
  call read_run_control('./params.dat', npas, iout, imix)
  p%forcing = GT_FORCING_3D3C      ! Makefile:20-33 links the 3D3C forcing by default
  p%dt2_mode = GT_DT2_AS_BUILT     ! dt2 is never assigned in the reference (rkstep.f90:34)
  p%precision = GT_PREC_FP64
  p%device = 0

  ! cuFFT plans, wavenumbers, emk, forced modes and device arrays
  ! (main.f90:27-34, 48, 71-85; defk.f90; iniforcing_*.f90)
  call gt_check(gt_create(p, h), 'gt_create')

  ! initial velocity: a saved frame (read.f90) or the fresh-start noise
  ! (inieuler.f90:76-82, trunc.f90:75-93)
  allocate(ux(NX, NY, NZ), uy(NX, NY, NZ), uz(NX, NY, NZ), u32(NX, NY, NZ))
  if (ifr > 0) then
    call read_component('ux', ifr, ux)
    call read_component('uy', ifr, uy)
    call read_component('uz', ifr, uz)
  else
    call gt_check(gt_init_noise(p, seed, ux, uy, uz), 'gt_init_noise')
  end if
  ! fft_dir x3, incompr, invcurl, trunc x3 (main.f90:91-106)
  call gt_check(gt_set_state_physical(h, ux, uy, uz, cc), 'gt_set_state_physical')

  open(unit=18, file=frame_name('./files/globalE.', ifr), status='unknown', position='append')
  open(unit=19, file=frame_name('./files/globalZ.', ifr), status='unknown', position='append')
  open(unit=20, file=frame_name('./files/spectra.', ifr), status='unknown', position='append')
  open(unit=30, file=frame_name('./files/fluxes.', ifr), status='unknown', position='append')

  jfr = 1
  do ipas = 1, npas
    ! spectrum and flux of b(t) with N1 = nlt(b(t)), before the step
    ! (main.f90:133-138)
    if (mod(ipas, imix) == 0) then
      call gt_check(gt_diagnostics(h, d, c_loc(ek), c_loc(ek2d), c_loc(flux)), 'gt_diagnostics')
      write(20, *) ipas, ek, ek2d
      write(30, *) ipas, flux
    end if
    ! bnl = b; nlt; step1; nlt; step2; forcing; t = t + dt (main.f90:121-150)
    call gt_check(gt_rk2_step(h, 1_c_int32_t, seed), 'gt_rk2_step')
    t = t + p%dt
    ! glob of b(t + dt) (main.f90:153-160)
    if (mod(ipas, imix) == 0) then
      call gt_check(gt_diagnostics(h, d, c_null_ptr, c_null_ptr, c_null_ptr), 'gt_diagnostics')
      write(18, *) t, d%energy, d%inpe
      write(19, *) t, d%enstrophy, d%inpz
    end if
    ! velocity output every iout steps (main.f90:163-185)
    if (mod(ipas, iout) == 0 .and. ipas /= npas) then
      call gt_check(gt_velocity(h, ux, uy, uz), 'gt_velocity')
      call write_frame_fields(ifr, jfr)
      jfr = jfr + 1
      write(6, *) 'Saved v field, seed and curframe at timestep = ', ipas
    end if
  end do

  ! final frame, seed and curframe.dat (main.f90:188-215)
  ifr = ifr + 1
  call gt_check(gt_velocity(h, ux, uy, uz), 'gt_velocity')
  call write_frame_fields(ifr, -1)
  write(name, "('./files/seed.',i3.3)") ifr
  call gt_check(gt_seed_write(trim(name)//c_null_char, seed), trim(name))
  call gt_check(gt_frame_write('./curframe.dat'//c_null_char, ifr, t), 'curframe.dat')
  close(18); close(19); close(20); close(30)
  call gt_check(gt_destroy(h), 'gt_destroy')

  call system_clock(c1)
  write(6, *) 'Mean time per iteration      = ', real(c1 - c0, c_double) / (real(npas, c_double) * crate)

contains

  function frame_name(prefix, k) result(s)
    character(len=*), intent(in) :: prefix
    integer(c_int32_t), intent(in) :: k
    character(len=64) :: s
    write(s, "(a, i3.3)") prefix, k
  end function frame_name

  ! The fourth line of params.dat: npas, iout, imix (inieuler.f90:17).
  subroutine read_run_control(path, npas, iout, imix)
    character(len=*), intent(in) :: path
    integer(c_int32_t), intent(out) :: npas, iout, imix
    integer :: u, k
    open(newunit=u, file=path, status='old', action='read')
    do k = 1, 3
      read(u, *)
    end do
    read(u, *) npas, iout, imix
    close(u)
  end subroutine read_run_control

  ! One float32 velocity component of frame k (read.f90:12-52), promoted.
  subroutine read_component(c, k, u)
    character(len=2), intent(in) :: c
    integer(c_int32_t), intent(in) :: k
    real(c_double), intent(out) :: u(NX, NY, NZ)
    character(len=64) :: s
    write(s, "('./fields/', a, '.', i3.3)") c, k
    call gt_check(gt_field_read_f32(trim(s)//c_null_char, NX, NY, NZ, u32), trim(s))
    u = real(u32, c_double)
  end subroutine read_component

  ! The three velocity components as float32 records (write.f90:12-22); a
  ! mid-run save (sub >= 1) is frame k, sub-frame sub.
  subroutine write_frame_fields(k, sub)
    integer(c_int32_t), intent(in) :: k, sub
    call write_component('ux', k, sub, ux)
    call write_component('uy', k, sub, uy)
    call write_component('uz', k, sub, uz)
  end subroutine write_frame_fields

  subroutine write_component(c, k, sub, u)
    character(len=2), intent(in) :: c
    integer(c_int32_t), intent(in) :: k, sub
    real(c_double), intent(in) :: u(NX, NY, NZ)
    character(len=64) :: s
    if (sub >= 1) then
      write(s, "('./fields/', a, '.', i3.3, '.', i3.3)") c, k, sub
    else
      write(s, "('./fields/', a, '.', i3.3)") c, k
    end if
    u32 = real(u, c_float)
    call gt_check(gt_field_write_f32(trim(s)//c_null_char, NX, NY, NZ, u32), trim(s))
  end subroutine write_component

end program gturbo_driver
