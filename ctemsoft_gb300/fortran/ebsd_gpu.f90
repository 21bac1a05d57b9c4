! ebsd_gpu.f90 -- ISO_C_BINDING interface to libebsdgpu.so for Fortran hosts.
!
! A Fortran program such as CTEMsoft's CTEMEBSD calls the GPU pattern loop
! through these interfaces; every argument maps one for one onto the C
! prototypes in include/ebsd_gpu.h.  Arrays are passed as the Fortran arrays
! themselves (column-major, no transposition); pointers are borrowed for the
! call only.  Build with any Fortran 2003 compiler and link -lebsdgpu.
module ebsd_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: EBSD_OK = 0, EBSD_EINVAL = -1, EBSD_ECUDA = -2, &
                               EBSD_ENOMEM = -3, EBSD_ESTATE = -4, EBSD_EIO = -5, &
                               EBSD_EFORMAT = -6, EBSD_EUNSUPPORTED = -7, EBSD_ETIMEOUT = -8
  integer(c_int32_t), parameter :: EBSD_SCALING_NOT = 0, EBSD_SCALING_LIN = 1, &
                                   EBSD_SCALING_GAM = 2
  integer(c_int32_t), parameter :: EBSD_VJP_COTANGENT = 0, EBSD_VJP_NDP = 1

  type, bind(C) :: ebsd_geometry
    real(c_float)     :: L, thetac, delta
    integer(c_int32_t):: numsx, numsy
    real(c_float)     :: xpc, ypc
    real(c_double)    :: sig
  end type ebsd_geometry

  type, bind(C) :: ebsd_epilogue
    real(c_double)    :: prefactor
    integer(c_int32_t):: binning, scalingmode
    real(c_float)     :: gammavalue
    integer(c_int32_t):: poisson
    integer(c_int64_t):: seed
  end type ebsd_epilogue

  type, bind(C) :: ebsd_gn_options
    integer(c_int32_t):: max_iterations, refine_pc
    real(c_double)    :: damping, tol_rad, tol_pc
  end type ebsd_gn_options

  interface
    integer(c_int) function ebsd_create(h, device) bind(C, name="ebsd_create")
      import :: c_int, c_ptr
      type(c_ptr), intent(out) :: h
      integer(c_int), value :: device
    end function

    subroutine ebsd_destroy(h) bind(C, name="ebsd_destroy")
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine

    type(c_ptr) function ebsd_last_error(h) bind(C, name="ebsd_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function ebsd_set_master(h, sr, npx, npy, nE, numset) &
        bind(C, name="ebsd_set_master")
      import :: c_int, c_ptr, c_float, c_int32_t
      type(c_ptr), value :: h
      real(c_float), intent(in) :: sr(*)          ! srtmp(-npx:npx,-npy:npy,nE,numset)
      integer(c_int32_t), value :: npx, npy, nE, numset
    end function

    integer(c_int) function ebsd_energy_window(energymin, energymax, Ehistmin, Ebinsize, &
        numEbins, Emin, Emax) bind(C, name="ebsd_energy_window")
      import :: c_int, c_float, c_double, c_int32_t
      real(c_float), value :: energymin, energymax
      real(c_double), value :: Ehistmin, Ebinsize
      integer(c_int32_t), value :: numEbins
      integer(c_int32_t), intent(out) :: Emin, Emax
    end function

    integer(c_int) function ebsd_set_detector(h, g, accum_e, nsx, nsy, numEbins, Emin, Emax, &
        num_el) bind(C, name="ebsd_set_detector")
      import :: c_int, c_ptr, c_int32_t, ebsd_geometry
      type(c_ptr), value :: h
      type(ebsd_geometry), intent(in) :: g
      integer(c_int32_t), intent(in) :: accum_e(*)  ! accum_e(numEbins,-nsx:nsx,-nsy:nsy)
      integer(c_int32_t), value :: nsx, nsy, numEbins, Emin, Emax
      integer(c_int32_t), intent(out) :: num_el
    end function

    real(c_double) function ebsd_prefactor(beamcurrent, dwelltime, num_el) &
        bind(C, name="ebsd_prefactor")
      import :: c_double, c_int32_t
      real(c_double), value :: beamcurrent, dwelltime
      integer(c_int32_t), value :: num_el
    end function

    integer(c_int) function ebsd_output_dims(h, e, nx, ny) bind(C, name="ebsd_output_dims")
      import :: c_int, c_ptr, c_int32_t, ebsd_epilogue
      type(c_ptr), value :: h
      type(ebsd_epilogue), intent(in) :: e
      integer(c_int32_t), intent(out) :: nx, ny
    end function

    integer(c_int) function ebsd_forward(h, quats, n, e, out) bind(C, name="ebsd_forward")
      import :: c_int, c_ptr, c_float, c_int64_t, ebsd_epilogue
      type(c_ptr), value :: h
      real(c_float), intent(in) :: quats(*)        ! quatang(4,numeuler)
      integer(c_int64_t), value :: n
      type(ebsd_epilogue), intent(in) :: e
      real(c_float), intent(out) :: out(*)         ! n records of (nx,ny)
    end function

    ! Replaces SampleRFZ (so3.f90:267-371): rods(3,count) and quats(4,count)
    ! of the fundamental zone of point group pgnum.  Call first with
    ! c_null_ptr for both arrays and capacity 0 to get count.
    integer(c_int) function ebsd_sample_rfz(h, nsteps, pgnum, rods, quats, capacity, count) &
        bind(C, name="ebsd_sample_rfz")
      import :: c_int, c_ptr, c_int32_t, c_int64_t
      type(c_ptr), value :: h
      integer(c_int32_t), value :: nsteps, pgnum
      type(c_ptr), value :: rods, quats              ! c_loc(rods(1,1)), c_loc(quats(1,1))
      integer(c_int64_t), value :: capacity
      integer(c_int64_t), intent(out) :: count
    end function

    integer(c_int) function ebsd_run_namelist(nmlfile, device, quiet) &
        bind(C, name="ebsd_run_namelist")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: nmlfile(*)  ! NUL-terminated
      integer(c_int), value :: device, quiet
    end function

    ! The program with the orientations split over several devices.
    integer(c_int) function ebsd_run_namelist_devices(nmlfile, devices, ndev, quiet) &
        bind(C, name="ebsd_run_namelist_devices")
      import :: c_int, c_int32_t, c_char
      character(kind=c_char), intent(in) :: nmlfile(*)  ! NUL-terminated
      integer(c_int32_t), intent(in) :: devices(*)
      integer(c_int32_t), value :: ndev
      integer(c_int), value :: quiet
    end function

    ! Another handle's master and detector set-up, shared without a copy.
    integer(c_int) function ebsd_share_detector(dst, src) bind(C, name="ebsd_share_detector")
      import :: c_int, c_ptr
      type(c_ptr), value :: dst, src
    end function

    ! The CTEMMC program (&MCdata namelist in, MC file out).
    integer(c_int) function ebsd_run_mc_namelist(nmlfile, device, quiet) &
        bind(C, name="ebsd_run_mc_namelist")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: nmlfile(*)  ! NUL-terminated
      integer(c_int), value :: device, quiet
    end function

    ! The CTEMMC program with the electrons split over several devices.
    integer(c_int) function ebsd_run_mc_namelist_devices(nmlfile, devices, ndev, quiet) &
        bind(C, name="ebsd_run_mc_namelist_devices")
      import :: c_int, c_int32_t, c_char
      character(kind=c_char), intent(in) :: nmlfile(*)  ! NUL-terminated
      integer(c_int32_t), intent(in) :: devices(*)
      integer(c_int32_t), value :: ndev
      integer(c_int), value :: quiet
    end function

    ! Tuning and precision options by name, e.g. "strict_order"//c_null_char.
    integer(c_int) function ebsd_set_option(h, key, val) bind(C, name="ebsd_set_option")
      import :: c_int, c_ptr, c_char, c_int64_t
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: key(*)      ! NUL-terminated
      integer(c_int64_t), value :: val
    end function

    ! Adjoint: gradient of the records (or of the loss against target records,
    ! mode EBSD_VJP_NDP) with respect to the 3 rotation tangents and (xpc, ypc, L).
    integer(c_int) function ebsd_vjp(h, quats, n, e, mode, data, loss, grad) &
        bind(C, name="ebsd_vjp")
      import :: c_int, c_ptr, c_float, c_int32_t, c_int64_t, ebsd_epilogue
      type(c_ptr), value :: h
      real(c_float), intent(in) :: quats(*)        ! quatang(4,n)
      integer(c_int64_t), value :: n
      type(ebsd_epilogue), intent(in) :: e
      integer(c_int32_t), value :: mode
      real(c_float), intent(in) :: data(*)         ! n records of (nx,ny)
      real(c_float), intent(out) :: loss(*)        ! loss(n), mode EBSD_VJP_NDP
      real(c_float), intent(out) :: grad(*)        ! grad(6,n)
    end function

    ! Gauss-Newton refinement; quats, targets and loss are device pointers.
    integer(c_int) function ebsd_refine(h, quats, n, e, targets, opt, loss, geom, iterations) &
        bind(C, name="ebsd_refine")
      import :: c_int, c_ptr, c_int32_t, c_int64_t, ebsd_epilogue, ebsd_gn_options, &
                ebsd_geometry
      type(c_ptr), value :: h
      type(c_ptr), value :: quats                   ! device float(4,n), updated in place
      integer(c_int64_t), value :: n
      type(ebsd_epilogue), intent(in) :: e
      type(c_ptr), value :: targets                 ! device, n records
      type(ebsd_gn_options), intent(in) :: opt
      type(c_ptr), value :: loss                    ! device float(n) or c_null_ptr
      type(ebsd_geometry), intent(inout) :: geom
      integer(c_int32_t), intent(out) :: iterations
    end function
  end interface

contains

  ! Message of the last error as a Fortran string.
  function ebsd_error_message(h) result(msg)
    type(c_ptr), intent(in) :: h
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: p(:)
    type(c_ptr) :: cp
    integer :: n
    cp = ebsd_last_error(h)
    call c_f_pointer(cp, p, [4096])
    n = 0
    do while (n < 4096)
      if (p(n + 1) == c_null_char) exit
      n = n + 1
    end do
    allocate(character(len=n) :: msg)
    msg = transfer(p(1:n), msg)
  end function ebsd_error_message

end module ebsd_gpu
