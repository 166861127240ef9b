! ISO_C_BINDING interface of libacumen_gpu.so for the reference's Fortran
! driver programs, and a drop-in module `Tomography_gpu` that keeps the
! reference module's interface (tomography/tv_hpc.F90:1-390: module globals
! nimage, ntheta, ncg, ninnner, nouter, wpu, lambda, mu, theta and the
! subroutines int_radon, radon, iradon, tvopt, get_slice, fin_radon) while
! the compute runs in the C ABI.  A driver switches by replacing
! `use Tomography` with `use Tomography_gpu`; arrays keep the reference's
! shapes: img(nimage,nimage), sinogram(nimage,ntheta).
!
! Build (with a Fortran compiler, which this image does not have):
!   gfortran -c acumen_gpu.f90
!   mpif90 tv_hpc.F90 acumen_gpu.o -L<pkg> -lacumen_gpu -Wl,-rpath,<pkg>
module acumen_gpu
  use iso_c_binding
  implicit none
  integer(c_int), parameter :: ACU_OK = 0, ACU_ERR_INVALID = -1, ACU_ERR_CUDA = -2, ACU_ERR_NOMEM = -3
  integer(c_int), parameter :: ACU_ERR_TIMEOUT = -4, ACU_ERR_UNSUPPORTED = -5
  integer(c_int), parameter :: ACU_OPT_FILTER = 1, ACU_OPT_LANES = 2, ACU_OPT_GRAPH = 3
  integer(c_int), parameter :: ACU_OPT_VERBOSE = 4, ACU_OPT_PRINT_EVERY = 5, ACU_OPT_SLICE_BASE = 6
  integer(c_int), parameter :: ACU_OPT_PROJECTOR = 7, ACU_OPT_POSITIONS = 8, ACU_OPT_RESIDUAL = 9
  integer(c_int), parameter :: ACU_OPT_BP_GROUPS = 10, ACU_OPT_RADON_REFRESH = 11
  integer(c_int), parameter :: ACU_OPT_BP_PARAM_TABLE = 12, ACU_OPT_MAX_BATCH = 13, ACU_OPT_BP_STAGED = 14

  interface
    integer(c_int) function acu_ctx_create(ctx, nimage, ntheta, theta_deg, wpu) bind(C, name="acu_ctx_create")
      import :: c_int, c_ptr, c_float
      type(c_ptr), intent(out) :: ctx
      integer(c_int), value :: nimage, ntheta, wpu
      real(c_float), intent(in) :: theta_deg(*)
    end function acu_ctx_create

    integer(c_int) function acu_ctx_destroy(ctx) bind(C, name="acu_ctx_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function acu_ctx_destroy

    type(c_ptr) function acu_last_error(ctx) bind(C, name="acu_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function acu_last_error

    integer(c_int) function acu_set_option(ctx, option, val) bind(C, name="acu_set_option")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: option, val
    end function acu_set_option

    integer(c_int) function acu_iradon(ctx, nslices, sino, img) bind(C, name="acu_iradon")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      integer(c_int), value :: nslices
      real(c_float), intent(in) :: sino(*)
      real(c_float), intent(out) :: img(*)
    end function acu_iradon

    integer(c_int) function acu_radon(ctx, nslices, img, sino) bind(C, name="acu_radon")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      integer(c_int), value :: nslices
      real(c_float), intent(in) :: img(*)
      real(c_float), intent(out) :: sino(*)
    end function acu_radon

    integer(c_int) function acu_radon_adjoint(ctx, nslices, sino, img) bind(C, name="acu_radon_adjoint")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      integer(c_int), value :: nslices
      real(c_float), intent(in) :: sino(*)
      real(c_float), intent(out) :: img(*)
    end function acu_radon_adjoint

    integer(c_int) function acu_tvopt(ctx, nslices, f, ninner, nouter, ncg, lambda, mu, tv_out, fbp_out) &
        bind(C, name="acu_tvopt")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      integer(c_int), value :: nslices, ninner, nouter, ncg
      real(c_float), value :: lambda, mu
      real(c_float), intent(in) :: f(*)
      real(c_float), intent(out) :: tv_out(*), fbp_out(*)
    end function acu_tvopt

    integer(c_int) function acu_normalize_stack_u16(ctx, mode, nproj, npix, raw, nflat, flats, ndark, darks, out) &
        bind(C, name="acu_normalize_stack_u16")
      import :: c_int, c_long, c_ptr, c_float, c_int16_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: mode, nproj, nflat, ndark
      integer(c_long), value :: npix
      integer(c_int16_t), intent(in) :: raw(*), flats(*), darks(*)   ! unsigned 16-bit counts
      real(c_float), intent(out) :: out(*)
    end function acu_normalize_stack_u16

    integer(c_int) function acu_proj_to_sino(ctx, nproj, ndet, nrows, proj, theta_deg, reg_method, sino_out, &
        theta_out, shift_out) bind(C, name="acu_proj_to_sino")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      integer(c_int), value :: nproj, ndet, nrows, reg_method
      real(c_float), intent(in) :: proj(*), theta_deg(*)
      real(c_float), intent(out) :: sino_out(*)
      real(c_float), intent(out) :: theta_out, shift_out
    end function acu_proj_to_sino
  end interface

contains

  ! Stops with the library's message when a call fails (the reference has no
  ! error returns; its MPI drivers would otherwise continue on garbage).
  subroutine acu_check(rc, ctx)
    integer(c_int), intent(in) :: rc
    type(c_ptr), intent(in) :: ctx
    character(kind=c_char), pointer :: msg(:)
    type(c_ptr) :: p
    integer :: n
    if (rc == ACU_OK) return
    p = acu_last_error(ctx)
    call c_f_pointer(p, msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write (*, *) "acumen_gpu error ", rc, ": ", msg(1:n)
    stop 1
  end subroutine acu_check
end module acumen_gpu


! Drop-in for `module Tomography` (tomography/tv_hpc.F90:1-390).
module Tomography_gpu
  use iso_c_binding
  use acumen_gpu
  implicit none
  integer, public :: ncg, ninnner, nouter, nimage, ntheta, nfilt, nstart, wpu, add_Nx
  real, public :: pi, midpoint, lambda, mu
  real, public, dimension(:), allocatable :: theta
  real, public, dimension(:,:), allocatable :: f
  type(c_ptr), private :: ctx = c_null_ptr
  ! the geometry the library context was created with
  integer, private :: ctx_nimage = -1, ctx_ntheta = -1, ctx_wpu = -1
  real, private, dimension(:), allocatable :: ctx_theta

contains

  ! tv_hpc.F90:11-78.  The drivers fill theta after this call (:560-562), so
  ! the library context is created lazily on first use.
  subroutine int_radon()
    midpoint = (nimage + 1) / 2
    pi = 4.0 * atan(1.0)
    nfilt = 2 * nimage + 1
    nstart = nimage
    if (.not. allocated(theta)) allocate(theta(ntheta))
    if (.not. allocated(f)) allocate(f(nimage, ntheta))
  end subroutine int_radon

  ! (Re)creates the library context when the grid, the angles or the mask
  ! taper differ from the ones it was created with: a driver may change
  ! theta, nimage or wpu between slices at the same ntheta.
  subroutine ensure_ctx()
    logical :: same
    same = .false.
    if (c_associated(ctx)) then
      if (ctx_nimage == nimage .and. ctx_ntheta == ntheta .and. ctx_wpu == wpu) then
        same = all(ctx_theta == theta(1:ntheta))
      end if
      if (same) return
      call acu_check(acu_ctx_destroy(ctx), c_null_ptr)
      ctx = c_null_ptr
    end if
    call acu_check(acu_ctx_create(ctx, int(nimage, c_int), int(ntheta, c_int), theta, int(wpu, c_int)), c_null_ptr)
    ctx_nimage = nimage
    ctx_ntheta = ntheta
    ctx_wpu = wpu
    if (allocated(ctx_theta)) deallocate(ctx_theta)
    allocate(ctx_theta(ntheta))
    ctx_theta = theta(1:ntheta)
  end subroutine ensure_ctx

  subroutine fin_radon()
    if (c_associated(ctx)) call acu_check(acu_ctx_destroy(ctx), c_null_ptr)
    ctx = c_null_ptr
    ctx_nimage = -1
    ctx_ntheta = -1
    ctx_wpu = -1
  end subroutine fin_radon

  ! tv_hpc.F90:84-126
  subroutine iradon(img_rec, sinogram)
    real, intent(in) :: sinogram(nimage, ntheta)
    real, intent(out) :: img_rec(nimage, nimage)
    call ensure_ctx()
    call acu_check(acu_iradon(ctx, 1_c_int, sinogram, img_rec), ctx)
  end subroutine iradon

  ! tv_hpc.F90:129-159
  subroutine radon(sinogram, img)
    real, intent(in) :: img(nimage, nimage)
    real, intent(out) :: sinogram(nimage, ntheta)
    call ensure_ctx()
    call acu_check(acu_radon(ctx, 1_c_int, img, sinogram), ctx)
  end subroutine radon

  ! tv_hpc.F90:162-363: f (module global) in, TV and FBP images out
  subroutine tvopt(img_rec_tv, img_rec_fbp, jslice)
    real, intent(out) :: img_rec_tv(nimage, nimage), img_rec_fbp(nimage, nimage)
    integer, intent(in) :: jslice
    call ensure_ctx()
    call acu_check(acu_set_option(ctx, ACU_OPT_VERBOSE, 1_c_int), ctx)
    call acu_check(acu_set_option(ctx, ACU_OPT_SLICE_BASE, int(jslice, c_int)), ctx)
    call acu_check(acu_tvopt(ctx, 1_c_int, f, int(ninnner, c_int), int(nouter, c_int), int(ncg, c_int), &
                             real(lambda, c_float), real(mu, c_float), img_rec_tv, img_rec_fbp), ctx)
  end subroutine tvopt

  ! tv_hpc.F90:365-386
  subroutine get_slice(img_rec_fbp)
    real, intent(out) :: img_rec_fbp(nimage, nimage)
    call iradon(img_rec_fbp, f)
  end subroutine get_slice
end module Tomography_gpu
