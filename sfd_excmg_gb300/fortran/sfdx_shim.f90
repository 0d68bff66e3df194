! sfdx_shim.f90 -- ISO_C_BINDING interface of the GB300 forward solver for the
! SFD_EXCMG Fortran host.  Replaces the body of fwd_solver
! (sfd_excmg/src/fdfe_main.f90:1565-1594) with one call into libsfdx.so; the
! caller's arrays are passed without copies (Fortran sigma(ncell,6) and
! ex(2*nl,nf) are exactly the C layouts [6][ncell] and [nf][2][nl]).
!
! Build (needs a Fortran 2003 compiler, not present in the build image), after
! global_para.f90, whose module global_parameter supplies fwd_acc:
!   gfortran -c global_para.f90 sfdx_shim.f90 && gfortran ... sfdx_shim.o -L<lib dir> -lsfdx
module sfdx
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SFDX_OK = 0
  integer(c_int), parameter :: SFDX_FP64 = 0, SFDX_MIXED = 1

  type, bind(c) :: sfdx_opts
    integer(c_int) :: level
    real(c_double) :: eps
    integer(c_int) :: solver
    integer(c_int) :: excmg
    integer(c_int) :: precond
    integer(c_int) :: div_cor
    integer(c_int) :: corr_intv
    real(c_double) :: corr_tol
    real(c_double) :: ssor_omega
    real(c_double) :: sigma_air
    integer(c_int) :: maxit_plain
    integer(c_int) :: maxit_level
    integer(c_int) :: precision
    integer(c_int) :: quirks
    real(c_double) :: coarse_tol
    integer(c_int) :: coarse_maxit
    integer(c_int) :: reliable_every
    integer(c_int) :: batch
    integer(c_int) :: verbose
    integer(c_int) :: use_graphs
  end type

  interface
    subroutine sfdx_default_opts(o) bind(c, name="sfdx_default_opts")
      import :: sfdx_opts
      type(sfdx_opts), intent(out) :: o
    end subroutine

    function sfdx_fwd_solve(o, nx, ny, nz, nair, a, b, c, sigma, nf, freq, ex, iters, relres) &
        bind(c, name="sfdx_fwd_solve") result(rc)
      import :: sfdx_opts, c_int, c_double, c_double_complex, c_ptr
      type(sfdx_opts), intent(in) :: o
      integer(c_int), value :: nx, ny, nz, nair, nf
      real(c_double), intent(in) :: a(*), b(*), c(*), sigma(*), freq(*)
      complex(c_double_complex), intent(out) :: ex(*)
      type(c_ptr), value :: iters, relres
      integer(c_int) :: rc
    end function

    function sfdx_impedance(nx, ny, nz, nair, a, b, c, nf, freq, ex, nrec, recv, out_type, quirks, res, tipper) &
        bind(c, name="sfdx_impedance") result(rc)
      import :: c_int, c_double, c_double_complex, c_ptr
      integer(c_int), value :: nx, ny, nz, nair, nf, nrec, out_type, quirks
      real(c_double), intent(in) :: a(*), b(*), c(*), freq(*), recv(*)
      complex(c_double_complex), intent(in) :: ex(*)
      real(c_double), intent(out) :: res(*)
      type(c_ptr), value :: tipper
      integer(c_int) :: rc
    end function

    function sfdx_strerror(code) bind(c, name="sfdx_strerror") result(p)
      import :: c_int, c_ptr
      integer(c_int), value :: code
      type(c_ptr) :: p
    end function
  end interface

contains

  ! Drop-in for fwd_solver (fdfe_main.f90:1565): same arguments, same
  ! allocation of ex(nl*2, nf); level/slv/eps come from the .fwd file or argv
  ! exactly as before.  fwd_acc (global_para.f90:19) maps to o%excmg.
  subroutine fwd_solver(modelname, a, b, c, nair, level, slv, eps, sigma, freq, ex)
    use global_parameter, only: fwd_acc   ! the reference's switch (global_para.f90:19)
    character(len=30) :: modelname
    real(c_double), allocatable :: a(:), b(:), c(:), sigma(:,:), freq(:)
    integer :: nair, level, slv
    real(c_double) :: eps
    complex(c_double_complex), allocatable :: ex(:,:)
    type(sfdx_opts) :: o
    integer :: nx, ny, nz, nf, nl
    integer(c_int) :: rc

    nx = size(a); ny = size(b); nz = size(c); nf = size(freq)
    nl = nx*(ny+1)*(nz+1) + (nx+1)*ny*(nz+1) + (nx+1)*(ny+1)*nz
    allocate(ex(nl*2, nf))
    call sfdx_default_opts(o)
    o%level = level
    o%eps = eps
    o%solver = slv
    o%excmg = 0
    if (fwd_acc /= 0) o%excmg = 1         ! doublemode_acc instead of doublemode_nor
    rc = sfdx_fwd_solve(o, nx, ny, nz, nair, a, b, c, sigma, nf, freq, ex, c_null_ptr, c_null_ptr)
    if (rc /= SFDX_OK) then
      write(*,*) 'sfdx_fwd_solve failed, status ', rc
      if (rc /= 4) stop
    endif
  end subroutine

end module
