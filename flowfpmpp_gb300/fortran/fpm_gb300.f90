! Fortran 2018 drop-in modules over the C ABI of libfpm_gb300.so
! (include/fpm_capi.h): the reference's module and procedure names with
! identical dummy arguments, so a Fortran caller swaps the reference sources
! for this file and links -lfpm_gb300 -lcudart.
!
! Scope: one MPI rank on one GPU.  Every neighbour argument must be
! MPI_PROC_NULL (physical boundary); a real decomposition stops with an
! error, as the reference stops on its own unsupported inputs.  use_openacc
! is accepted and ignored: the GPU path always runs.  A nonzero status from
! the library stops with the library's message (the reference's error stop).
!
! Build (needs a Fortran compiler and an MPI module providing MPI_PROC_NULL;
! without MPI, compile fpm_gb300_mpi_stub first):
!   mpif90 -c fpm_gb300.f90 && mpif90 app.f90 fpm_gb300.o -L. -lfpm_gb300 -lcudart

module fpm_gb300_capi
  use, intrinsic :: iso_c_binding
  implicit none
  private
  public :: fpm_check
  interface
    function c_last_error() bind(C, name='fpm_last_error') result(p)
      import :: c_ptr
      type(c_ptr) :: p
    end function
    function c_strlen(s) bind(C, name='strlen') result(n)
      import :: c_ptr, c_size_t
      type(c_ptr), value :: s
      integer(c_size_t) :: n
    end function
  end interface
contains
  ! Stops with the library's message when status /= 0.
  subroutine fpm_check(status, where)
    integer(c_int), intent(in) :: status
    character(*), intent(in) :: where
    type(c_ptr) :: p
    character(kind=c_char), pointer :: s(:)
    character(len=:), allocatable :: msg
    integer :: i, n
    if (status == 0) return
    p = c_last_error()
    n = int(c_strlen(p))
    call c_f_pointer(p, s, [n])
    allocate(character(len=n) :: msg)
    do i = 1, n
      msg(i:i) = s(i)
    end do
    write(*, '(a,a,i0,a,a)') where, ': status ', status, ': ', msg
    error stop 'fpm_gb300: library call failed'
  end subroutine fpm_check
end module fpm_gb300_capi

module fpm_stairstep_mpi_3d
  use, intrinsic :: iso_fortran_env, only: real64
  use, intrinsic :: iso_c_binding
  use mpi, only: MPI_PROC_NULL
  use fpm_gb300_capi
  implicit none
  private
  public :: exchange_solid_halo_3d, enforce_stairstep_compatibility_3d, solve_stairstep_poisson_3d
  public :: stairstep_residual_3d, compute_stairstep_fpm_terms_3d
  interface
    integer(c_int) function c_halo(solid, nx, ny, nz) bind(C, name='fpm_exchange_solid_halo_3d')
      import :: c_int
      integer(c_int), intent(inout) :: solid(*)
      integer(c_int), value :: nx, ny, nz
    end function
    integer(c_int) function c_compat(rhs, solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz, &
         correction, imbalance) bind(C, name='fpm_enforce_stairstep_compatibility_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: rhs(*), bg(3), dx(*), dy(*), dz(*)
      integer(c_int), intent(in) :: solid(*)
      real(c_double), intent(inout) :: xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      integer(c_int), value :: nx, ny, nz
      real(c_double), intent(out) :: correction, imbalance
    end function
    integer(c_int) function c_solve(phi, rhs, solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, &
         nx, ny, nz, tolerance, max_sweeps, check_interval, method, sweeps, residual) &
         bind(C, name='fpm_solve_stairstep_poisson_3d')
      import :: c_int, c_double
      real(c_double), intent(inout) :: phi(*)
      real(c_double), intent(in) :: rhs(*), bg(3), xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      real(c_double), intent(in) :: xc(*), yc(*), zc(*), dx(*), dy(*), dz(*)
      integer(c_int), intent(in) :: solid(*)
      integer(c_int), value :: nx, ny, nz, max_sweeps, check_interval, method
      real(c_double), value :: tolerance
      integer(c_int), intent(out) :: sweeps
      real(c_double), intent(out) :: residual
    end function
    integer(c_int) function c_check(phi, rhs, solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, &
         nx, ny, nz, value) bind(C, name='fpm_stairstep_residual_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: phi(*), rhs(*), bg(3), xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      real(c_double), intent(in) :: xc(*), yc(*), zc(*), dx(*), dy(*), dz(*)
      integer(c_int), intent(in) :: solid(*)
      integer(c_int), value :: nx, ny, nz
      real(c_double), intent(out) :: value
    end function
    integer(c_int) function c_terms(phi, u, v, w, ox, oy, oz, ax, ay, az, solid, bg, xc, yc, zc, dx, dy, dz, &
         xlo, xhi, ylo, yhi, zlo, zhi, bounds, gx, gy, gz, vortex, advection, totals, nx, ny, nz) &
         bind(C, name='fpm_compute_stairstep_fpm_terms_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: phi(*), u(*), v(*), w(*), ox(*), oy(*), oz(*), ax(*), ay(*), az(*)
      real(c_double), intent(in) :: bg(3), xc(*), yc(*), zc(*), dx(*), dy(*), dz(*)
      real(c_double), intent(in) :: xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*), bounds(6)
      integer(c_int), intent(in) :: solid(*)
      real(c_double), intent(out) :: gx(*), gy(*), gz(*), vortex(*), advection(*), totals(2)
      integer(c_int), value :: nx, ny, nz
    end function
  end interface
contains
  subroutine one_rank(west, east, south, north)
    integer, intent(in) :: west, east, south, north
    if (any([west, east, south, north] /= MPI_PROC_NULL)) &
         error stop 'fpm_gb300: domain decomposition is not supported; run one rank per grid'
  end subroutine one_rank

  subroutine exchange_solid_halo_3d(solid, nx, ny, nz, west, east, south, north, comm)
    integer, intent(in) :: nx, ny, nz, west, east, south, north, comm
    integer(c_int), intent(inout) :: solid(0:nx+1, 0:ny+1, nz)
    call one_rank(west, east, south, north)
    call fpm_check(c_halo(solid, nx, ny, nz), 'exchange_solid_halo_3d')
  end subroutine exchange_solid_halo_3d

  subroutine enforce_stairstep_compatibility_3d(rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, &
       nx, ny, nz, west, east, south, north, comm, correction, imbalance)
    integer, intent(in) :: nx, ny, nz, west, east, south, north, comm
    integer(c_int), intent(in) :: solid(0:nx+1, 0:ny+1, nz)
    real(real64), intent(in) :: rhs(nx, ny, nz), body_grad(3), dx(nx), dy(ny), dz(nz)
    real(real64), intent(inout) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny)
    real(real64), intent(out) :: correction, imbalance
    call one_rank(west, east, south, north)
    call fpm_check(c_compat(rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz, &
         correction, imbalance), 'enforce_stairstep_compatibility_3d')
  end subroutine enforce_stairstep_compatibility_3d

  subroutine solve_stairstep_poisson_3d(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, &
       dx, dy, dz, nx, ny, nz, west, east, south, north, comm, tolerance, max_sweeps, check_interval, sweeps, &
       residual, use_openacc, method)
    integer, intent(in) :: nx, ny, nz, west, east, south, north, comm, max_sweeps, check_interval
    integer(c_int), intent(in) :: solid(0:nx+1, 0:ny+1, nz)
    real(real64), intent(inout) :: phi(0:nx+1, 0:ny+1, nz)
    real(real64), intent(in) :: rhs(nx, ny, nz), body_grad(3)
    real(real64), intent(in) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny)
    real(real64), intent(in) :: xc(0:nx+1), yc(0:ny+1), zc(nz), dx(nx), dy(ny), dz(nz), tolerance
    integer, intent(out) :: sweeps
    real(real64), intent(out) :: residual
    logical, intent(in), optional :: use_openacc
    character(*), intent(in), optional :: method
    integer(c_int) :: m, sw
    call one_rank(west, east, south, north)
    m = 0
    if (present(method)) then
      select case (method)
      case ('pcg'); m = 0
      case ('jacobi'); m = 1
      case ('jacobi_df'); m = 2
      case ('pcg_mixed'); m = 3
      case ('pcg_mg'); m = 4
      case ('jacobi_fma'); m = 6
      case ('jacobi_tf'); m = 7
      case default; error stop 'stair-step method must be pcg or jacobi'
      end select
    end if
    call fpm_check(c_solve(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, &
         nx, ny, nz, tolerance, max_sweeps, check_interval, m, sw, residual), 'solve_stairstep_poisson_3d')
    sweeps = sw
  end subroutine solve_stairstep_poisson_3d

  function stairstep_residual_3d(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, &
       nx, ny, nz, west, east, south, north, comm) result(value)
    integer, intent(in) :: nx, ny, nz, west, east, south, north, comm
    integer(c_int), intent(in) :: solid(0:nx+1, 0:ny+1, nz)
    real(real64), intent(in) :: phi(0:nx+1, 0:ny+1, nz), rhs(nx, ny, nz), body_grad(3)
    real(real64), intent(in) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny)
    real(real64), intent(in) :: xc(0:nx+1), yc(0:ny+1), zc(nz), dx(nx), dy(ny), dz(nz)
    real(real64) :: value
    call one_rank(west, east, south, north)
    call fpm_check(c_check(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, &
         nx, ny, nz, value), 'stairstep_residual_3d')
  end function stairstep_residual_3d

  subroutine compute_stairstep_fpm_terms_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, solid, body_grad, &
       xc, yc, zc, dx, dy, dz, xlo, xhi, ylo, yhi, zlo, zhi, bounds, gx, gy, gz, vortex, advection, totals, &
       nx, ny, nz, west, east, south, north, comm, use_openacc)
    integer, intent(in) :: nx, ny, nz, west, east, south, north, comm
    integer(c_int), intent(in) :: solid(0:nx+1, 0:ny+1, nz)
    real(real64), intent(in) :: phi(0:nx+1, 0:ny+1, nz), u(nx, ny, nz), v(nx, ny, nz), w(nx, ny, nz)
    real(real64), intent(in) :: ox(nx, ny, nz), oy(nx, ny, nz), oz(nx, ny, nz), ax(nx, ny, nz), ay(nx, ny, nz)
    real(real64), intent(in) :: az(nx, ny, nz), body_grad(3), xc(0:nx+1), yc(0:ny+1), zc(nz), dx(nx), dy(ny), dz(nz)
    real(real64), intent(in) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny), bounds(6)
    real(real64), intent(out) :: gx(nx, ny, nz), gy(nx, ny, nz), gz(nx, ny, nz), vortex(nx, ny, nz)
    real(real64), intent(out) :: advection(nx, ny, nz), totals(2)
    logical, intent(in), optional :: use_openacc
    call one_rank(west, east, south, north)
    call fpm_check(c_terms(phi, u, v, w, ox, oy, oz, ax, ay, az, solid, body_grad, xc, yc, zc, dx, dy, dz, &
         xlo, xhi, ylo, yhi, zlo, zhi, bounds, gx, gy, gz, vortex, advection, totals, nx, ny, nz), &
         'compute_stairstep_fpm_terms_3d')
  end subroutine compute_stairstep_fpm_terms_3d
end module fpm_stairstep_mpi_3d

module fpm_laplace_3d
  use, intrinsic :: iso_fortran_env, only: real64
  use, intrinsic :: iso_c_binding
  use fpm_gb300_capi
  implicit none
  private
  public :: enforce_neumann_compatibility_3d, solve_neumann_poisson_3d
  public :: enforce_neumann_compatibility_nonuniform_3d, solve_neumann_poisson_nonuniform_3d
  interface
    integer(c_int) function c_ucompat(rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, correction, &
         imbalance) bind(C, name='fpm_enforce_neumann_compatibility_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: rhs(*)
      real(c_double), intent(inout) :: xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dx, dy, dz
      real(c_double), intent(out) :: correction, imbalance
    end function
    integer(c_int) function c_usolve(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, tolerance, &
         max_iterations, check_interval, iterations, final_residual) bind(C, name='fpm_solve_neumann_poisson_3d')
      import :: c_int, c_double
      real(c_double), intent(inout) :: phi(*)
      real(c_double), intent(in) :: rhs(*), xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      integer(c_int), value :: nx, ny, nz, max_iterations, check_interval
      real(c_double), value :: dx, dy, dz, tolerance
      integer(c_int), intent(out) :: iterations
      real(c_double), intent(out) :: final_residual
    end function
    integer(c_int) function c_ncompat(rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz, correction, &
         imbalance) bind(C, name='fpm_enforce_neumann_compatibility_nonuniform_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: rhs(*), dx(*), dy(*), dz(*)
      real(c_double), intent(inout) :: xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      integer(c_int), value :: nx, ny, nz
      real(c_double), intent(out) :: correction, imbalance
    end function
    integer(c_int) function c_nsolve(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, nx, ny, nz, &
         tolerance, max_iterations, check_interval, iterations, final_residual) &
         bind(C, name='fpm_solve_neumann_poisson_nonuniform_3d')
      import :: c_int, c_double
      real(c_double), intent(inout) :: phi(*)
      real(c_double), intent(in) :: rhs(*), xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*)
      real(c_double), intent(in) :: xc(*), yc(*), zc(*), dx(*), dy(*), dz(*)
      integer(c_int), value :: nx, ny, nz, max_iterations, check_interval
      real(c_double), value :: tolerance
      integer(c_int), intent(out) :: iterations
      real(c_double), intent(out) :: final_residual
    end function
  end interface
contains
  subroutine enforce_neumann_compatibility_3d(rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, &
       correction, imbalance)
    integer, intent(in) :: nx, ny, nz
    real(real64), intent(in) :: rhs(nx, ny, nz), dx, dy, dz
    real(real64), intent(inout) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny)
    real(real64), intent(out) :: correction, imbalance
    call fpm_check(c_ucompat(rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, correction, imbalance), &
         'enforce_neumann_compatibility_3d')
  end subroutine enforce_neumann_compatibility_3d

  subroutine solve_neumann_poisson_3d(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, tolerance, &
       max_iterations, check_interval, iterations, final_residual)
    integer, intent(in) :: nx, ny, nz, max_iterations, check_interval
    real(real64), intent(inout) :: phi(0:nx+1, 0:ny+1, 0:nz+1)
    real(real64), intent(in) :: rhs(nx, ny, nz), xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz)
    real(real64), intent(in) :: zlo(nx, ny), zhi(nx, ny), dx, dy, dz, tolerance
    integer, intent(out) :: iterations
    real(real64), intent(out) :: final_residual
    integer(c_int) :: it
    call fpm_check(c_usolve(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, tolerance, &
         max_iterations, check_interval, it, final_residual), 'solve_neumann_poisson_3d')
    iterations = it
  end subroutine solve_neumann_poisson_3d

  subroutine enforce_neumann_compatibility_nonuniform_3d(rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, &
       nx, ny, nz, correction, imbalance)
    integer, intent(in) :: nx, ny, nz
    real(real64), intent(in) :: rhs(nx, ny, nz), dx(nx), dy(ny), dz(nz)
    real(real64), intent(inout) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny)
    real(real64), intent(out) :: correction, imbalance
    call fpm_check(c_ncompat(rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz, correction, imbalance), &
         'enforce_neumann_compatibility_nonuniform_3d')
  end subroutine enforce_neumann_compatibility_nonuniform_3d

  subroutine solve_neumann_poisson_nonuniform_3d(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, &
       nx, ny, nz, tolerance, max_iterations, check_interval, iterations, final_residual)
    integer, intent(in) :: nx, ny, nz, max_iterations, check_interval
    real(real64), intent(inout) :: phi(nx, ny, nz)
    real(real64), intent(in) :: rhs(nx, ny, nz), xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz)
    real(real64), intent(in) :: zlo(nx, ny), zhi(nx, ny), xc(nx), yc(ny), zc(nz), dx(nx), dy(ny), dz(nz), tolerance
    integer, intent(out) :: iterations
    real(real64), intent(out) :: final_residual
    integer(c_int) :: it
    call fpm_check(c_nsolve(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, nx, ny, nz, tolerance, &
         max_iterations, check_interval, it, final_residual), 'solve_neumann_poisson_nonuniform_3d')
    iterations = it
  end subroutine solve_neumann_poisson_nonuniform_3d
end module fpm_laplace_3d

module fpm_terms_3d
  use, intrinsic :: iso_fortran_env, only: real64
  use, intrinsic :: iso_c_binding
  use fpm_gb300_capi
  implicit none
  private
  public :: compute_fpm_terms_uniform_3d, compute_fpm_terms_nonuniform_3d
  interface
    integer(c_int) function c_uterms(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, gx, gy, gz, vortex, advection, &
         totals, nx, ny, nz, dx, dy, dz) bind(C, name='fpm_compute_fpm_terms_uniform_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: phi(*), u(*), v(*), w(*), ox(*), oy(*), oz(*), ax(*), ay(*), az(*)
      integer(c_int), intent(in) :: fluid(*)
      real(c_double), intent(out) :: gx(*), gy(*), gz(*), vortex(*), advection(*), totals(2)
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dx, dy, dz
    end function
    integer(c_int) function c_nterms(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, xc, yc, zc, dx, dy, dz, &
         xlo, xhi, ylo, yhi, zlo, zhi, bounds, gx, gy, gz, vortex, advection, totals, nx, ny, nz) &
         bind(C, name='fpm_compute_fpm_terms_nonuniform_3d')
      import :: c_int, c_double
      real(c_double), intent(in) :: phi(*), u(*), v(*), w(*), ox(*), oy(*), oz(*), ax(*), ay(*), az(*)
      real(c_double), intent(in) :: xc(*), yc(*), zc(*), dx(*), dy(*), dz(*)
      real(c_double), intent(in) :: xlo(*), xhi(*), ylo(*), yhi(*), zlo(*), zhi(*), bounds(6)
      integer(c_int), intent(in) :: fluid(*)
      real(c_double), intent(out) :: gx(*), gy(*), gz(*), vortex(*), advection(*), totals(2)
      integer(c_int), value :: nx, ny, nz
    end function
  end interface
contains
  subroutine compute_fpm_terms_uniform_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, gx, gy, gz, vortex, &
       advection, totals, nx, ny, nz, dx, dy, dz)
    integer, intent(in) :: nx, ny, nz
    integer(c_int), intent(in) :: fluid(nx, ny, nz)
    real(real64), intent(in) :: phi(0:nx+1, 0:ny+1, 0:nz+1), u(nx, ny, nz), v(nx, ny, nz), w(nx, ny, nz)
    real(real64), intent(in) :: ox(nx, ny, nz), oy(nx, ny, nz), oz(nx, ny, nz), ax(nx, ny, nz), ay(nx, ny, nz)
    real(real64), intent(in) :: az(nx, ny, nz), dx, dy, dz
    real(real64), intent(out) :: gx(nx, ny, nz), gy(nx, ny, nz), gz(nx, ny, nz), vortex(nx, ny, nz)
    real(real64), intent(out) :: advection(nx, ny, nz), totals(2)
    call fpm_check(c_uterms(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, gx, gy, gz, vortex, advection, totals, &
         nx, ny, nz, dx, dy, dz), 'compute_fpm_terms_uniform_3d')
  end subroutine compute_fpm_terms_uniform_3d

  subroutine compute_fpm_terms_nonuniform_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, xc, yc, zc, dx, dy, dz, &
       xlo, xhi, ylo, yhi, zlo, zhi, bounds, gx, gy, gz, vortex, advection, totals, nx, ny, nz)
    integer, intent(in) :: nx, ny, nz
    integer(c_int), intent(in) :: fluid(nx, ny, nz)
    real(real64), intent(in) :: phi(nx, ny, nz), u(nx, ny, nz), v(nx, ny, nz), w(nx, ny, nz)
    real(real64), intent(in) :: ox(nx, ny, nz), oy(nx, ny, nz), oz(nx, ny, nz), ax(nx, ny, nz), ay(nx, ny, nz)
    real(real64), intent(in) :: az(nx, ny, nz), xc(nx), yc(ny), zc(nz), dx(nx), dy(ny), dz(nz)
    real(real64), intent(in) :: xlo(ny, nz), xhi(ny, nz), ylo(nx, nz), yhi(nx, nz), zlo(nx, ny), zhi(nx, ny), bounds(6)
    real(real64), intent(out) :: gx(nx, ny, nz), gy(nx, ny, nz), gz(nx, ny, nz), vortex(nx, ny, nz)
    real(real64), intent(out) :: advection(nx, ny, nz), totals(2)
    call fpm_check(c_nterms(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, xc, yc, zc, dx, dy, dz, &
         xlo, xhi, ylo, yhi, zlo, zhi, bounds, gx, gy, gz, vortex, advection, totals, nx, ny, nz), &
         'compute_fpm_terms_nonuniform_3d')
  end subroutine compute_fpm_terms_nonuniform_3d
end module fpm_terms_3d

module fpm_partition_2d
  use, intrinsic :: iso_fortran_env, only: real64, int8
  use, intrinsic :: iso_c_binding
  use fpm_gb300_capi
  implicit none
  private
  public :: fpm_partition_terms_2d
  interface
    integer(c_int) function c_part(phi, g, u, v, solid, xf, yf, kin, ring, dt, nu, nx, ny, terms, vif_density, &
         omega, slip_body) bind(C, name='fpm_partition_terms_2d')
      import :: c_int, c_double, c_int8_t
      real(c_double), intent(in) :: phi(*), g(2), u(*), v(*), xf(*), yf(*), kin(6), ring(*)
      integer(c_int8_t), intent(in) :: solid(*)
      real(c_double), value :: dt, nu
      integer(c_int), value :: nx, ny, slip_body
      real(c_double), intent(out) :: terms(4), vif_density(*), omega(*)
    end function
  end interface
contains
  subroutine fpm_partition_terms_2d(phi, g, u, v, solid, xf, yf, kin, ring, dt, nu, nx, ny, terms, vif_density, &
       omega, slip_body)
    integer, intent(in) :: nx, ny
    real(real64), intent(in) :: phi(nx, ny), g(2), u(nx, ny), v(nx, ny), xf(0:nx), yf(0:ny), kin(6)
    real(real64), intent(in) :: ring(2*nx+2*ny, 2, 2), dt, nu
    logical, intent(in) :: solid(nx, ny)
    real(real64), intent(out) :: terms(4), vif_density(nx, ny), omega(nx, ny)
    logical, intent(in), optional :: slip_body
    integer(c_int8_t), allocatable :: s8(:,:)
    integer(c_int) :: slip
    allocate(s8(nx, ny))
    s8 = merge(1_c_int8_t, 0_c_int8_t, solid)
    slip = 0
    if (present(slip_body)) then
      if (slip_body) slip = 1
    end if
    call fpm_check(c_part(phi, g, u, v, s8, xf, yf, kin, ring, dt, nu, nx, ny, terms, vif_density, omega, slip), &
         'fpm_partition_terms_2d')
  end subroutine fpm_partition_terms_2d
end module fpm_partition_2d
