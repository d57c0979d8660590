!------------------------------------------------------------------------------
! ads_gpu — ISO_C_BINDING interface of the GB300 ADS library (include/ads_gpu.h)
! and drop-in style wrappers with the reference ADSS module's names.
!
! The reference drives the time step with
!   call Initialize(n, p, ads, ads_data, mierr)            (src/ADS.F90:11)
!   call Step(iter, ComputePointForRHS, ads, ads_data, l2norm, mierr)   (:437)
!   call Cleanup(ads, ads_data, mierr)                      (:802)
! Here the two derived types are replaced by an opaque handle, and the
! per-point callback by an integrand form plus arrays sampled at the
! quadrature points (GpuQpPoints gives their coordinates), because a GPU
! kernel cannot call a Fortran procedure.  Layouts match the reference:
! coefficients F(x, y+z*Ny) (x fastest), per-point arrays (kx,ky,kz,ex,ey,ez).
!------------------------------------------------------------------------------
module ads_gpu
   use iso_c_binding
   implicit none

   integer(c_int), parameter :: ADS_OK = 0
   integer(c_int), parameter :: ADS_PREC_FP64 = 0, ADS_PREC_MIXED = 1, ADS_PREC_MIXED_FAST = 2
   integer(c_int), parameter :: ADS_FORM_PROJECT = 0, ADS_FORM_HEAT = 1, ADS_FORM_OIL = 2

   type, bind(c) :: ads_opts
      integer(c_int) :: precision
      real(c_double) :: refine_tol
      integer(c_int) :: max_refine
      integer(c_int) :: device
   end type ads_opts

   type, bind(c) :: ads_stats
      real(c_double) :: l2norm
      real(c_double) :: rel_residual
      integer(c_int) :: refinements
      integer(c_int) :: converged
      integer(c_int) :: fp64_residuals
      integer(c_int) :: host_path
   end type ads_stats

   type :: ads_gpu_handle
      type(c_ptr) :: h = c_null_ptr
      integer(c_int) :: nelem(3), ndof(3), nq(3)
   end type ads_gpu_handle

   interface
      integer(c_int) function ads_default_opts(opts) bind(c, name="ads_default_opts")
         import :: c_int, ads_opts
         type(ads_opts), intent(out) :: opts
      end function
      integer(c_int) function ads_create(n, p, opts, h) bind(c, name="ads_create")
         import :: c_int, c_ptr, ads_opts
         integer(c_int), intent(in) :: n(3), p(3)
         type(ads_opts), intent(in) :: opts
         type(c_ptr), intent(out) :: h
      end function
      integer(c_int) function ads_destroy(h) bind(c, name="ads_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function
      integer(c_int) function ads_dims(h, nelem, ndof, nq) bind(c, name="ads_dims")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
         integer(c_int), intent(out) :: nelem(3), ndof(3), nq(3)
      end function
      integer(c_int) function ads_qp_points(h, axis, x) bind(c, name="ads_qp_points")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: axis
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function ads_set_form(h, form, f_qp, kappa_qp, kappa, dt) bind(c, name="ads_set_form")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: form
         type(c_ptr), value :: f_qp, kappa_qp
         real(c_double), value :: kappa, dt
      end function
      integer(c_int) function ads_set_oil(h, drain_qp, mu) bind(c, name="ads_set_oil")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in) :: drain_qp(*)
         real(c_double), value :: mu
      end function
      integer(c_int) function ads_get_drained(h, drained) bind(c, name="ads_get_drained")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: drained
      end function
      integer(c_int) function ads_save_spline_plot(h, name, range, res, vals) bind(c, name="ads_save_spline_plot")
         import :: c_int, c_ptr, c_double, c_char
         type(c_ptr), value :: h
         character(kind=c_char), intent(in) :: name(*)
         real(c_double), intent(in) :: range(6)
         integer(c_int), intent(in) :: res(3)
         type(c_ptr), value :: vals
      end function
      integer(c_int) function ads_multistep(h, mix, l2norm) bind(c, name="ads_multistep")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in) :: mix(4, 3)
         real(c_double), intent(out) :: l2norm
      end function
      integer(c_int) function ads_set_coeffs(h, u) bind(c, name="ads_set_coeffs")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in) :: u(*)
      end function
      integer(c_int) function ads_get_coeffs(h, u) bind(c, name="ads_get_coeffs")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: u(*)
      end function
      integer(c_int) function ads_step(h, l2norm) bind(c, name="ads_step")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: l2norm
      end function
      ! u_out may be u_in: both are passed as c_loc of the state array
      integer(c_int) function ads_step_host(h, u_in, u_out, l2norm) bind(c, name="ads_step_host")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         type(c_ptr), value :: u_in
         type(c_ptr), value :: u_out
         real(c_double), intent(out) :: l2norm
      end function
      integer(c_int) function ads_steps(h, k, l2norms) bind(c, name="ads_steps")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k
         real(c_double), intent(out) :: l2norms(*)
      end function
      integer(c_int) function ads_get_stats(h, st) bind(c, name="ads_get_stats")
         import :: c_int, c_ptr, ads_stats
         type(c_ptr), value :: h
         type(ads_stats), intent(out) :: st
      end function
      integer(c_int) function ads_assemble(h, F, l2norm) bind(c, name="ads_assemble")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: F(*)
         real(c_double), intent(out) :: l2norm
      end function
      integer(c_int) function ads_solve(h, F, u) bind(c, name="ads_solve")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in) :: F(*)
         real(c_double), intent(out) :: u(*)
      end function
      integer(c_int) function ads_apply_mass(h, u, out) bind(c, name="ads_apply_mass")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in) :: u(*)
         real(c_double), intent(out) :: out(*)
      end function
      integer(c_int) function ads_heat_adjoint(h, k, checkpoint_every, u0, u_target, loss, grad_u0, &
                                               grad_kappa_qp) bind(c, name="ads_heat_adjoint")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k, checkpoint_every
         real(c_double), intent(in) :: u0(*), u_target(*)
         real(c_double), intent(out) :: loss
         type(c_ptr), value :: grad_u0, grad_kappa_qp
      end function
      integer(c_int) function ads_heat_jvp(h, k, u0, du0, dkappa_qp, uk, duk) bind(c, name="ads_heat_jvp")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: k
         real(c_double), intent(in) :: u0(*)
         type(c_ptr), value :: du0, dkappa_qp, uk, duk
      end function
      type(c_ptr) function ads_status_string(status) bind(c, name="ads_status_string")
         import :: c_int, c_ptr
         integer(c_int), value :: status
      end function
   end interface

contains

   ! Initialize (src/ADS.F90:11): n = functions minus one, p = degrees per axis.
   subroutine GpuInitialize(n, p, precision, g, mierr)
      integer(kind=4), intent(in) :: n(3), p(3)
      integer(c_int), intent(in) :: precision
      type(ads_gpu_handle), intent(out) :: g
      integer(kind=4), intent(out) :: mierr
      type(ads_opts) :: o
      mierr = ads_default_opts(o)
      o % precision = precision
      mierr = ads_create(int(n, c_int), int(p, c_int), o, g % h)
      if (mierr /= ADS_OK) return
      mierr = ads_dims(g % h, g % nelem, g % ndof, g % nq)
   end subroutine GpuInitialize

   ! Gauss points of one axis, X(q, nelem) as the reference's ads % Xx.
   subroutine GpuQpPoints(g, axis, X, mierr)
      type(ads_gpu_handle), intent(in) :: g
      integer(kind=4), intent(in) :: axis
      real(c_double), intent(out) :: X(:,:)
      integer(kind=4), intent(out) :: mierr
      mierr = ads_qp_points(g % h, int(axis - 1, c_int), X)
   end subroutine GpuQpPoints

   ! Select the integrand; fqp/kqp are per-point arrays (kx,ky,kz,ex,ey,ez).
   subroutine GpuSetForm(g, form, fqp, kqp, kappa, dt, mierr)
      type(ads_gpu_handle), intent(in) :: g
      integer(c_int), intent(in) :: form
      real(c_double), intent(in), target, optional :: fqp(:), kqp(:)
      real(c_double), intent(in) :: kappa, dt
      integer(kind=4), intent(out) :: mierr
      type(c_ptr) :: pf, pk
      pf = c_null_ptr
      pk = c_null_ptr
      if (present(fqp)) pf = c_loc(fqp)
      if (present(kqp)) pk = c_loc(kqp)
      mierr = ads_set_form(g % h, form, pf, pk, kappa, dt)
   end subroutine GpuSetForm

   ! The oil problem's draining weight at the points (draining(u, X) = w u,
   ! problems/oil/input_data.F90:265-283) and mi; pumping and Kqvals go to
   ! GpuSetForm(g, ADS_FORM_OIL, pump_qp, kq_qp, 1d0, Dt, mierr).
   subroutine GpuSetOil(g, drain_qp, mi, mierr)
      type(ads_gpu_handle), intent(in) :: g
      real(c_double), intent(in) :: drain_qp(:)
      real(c_double), intent(in) :: mi
      integer(kind=4), intent(out) :: mierr
      mierr = ads_set_oil(g % h, drain_qp, mi)
   end subroutine GpuSetOil

   ! The drained total since GpuSetOil (what ComputeResults reduces and prints).
   subroutine GpuDrained(g, drained, mierr)
      type(ads_gpu_handle), intent(in) :: g
      real(c_double), intent(out) :: drained
      integer(kind=4), intent(out) :: mierr
      mierr = ads_get_drained(g % h, drained)
   end subroutine GpuDrained

   ! PrintSolution (src/ADS.F90:955-989): the solution on 31^3 points of
   ! [0,1]^3 written to step<iter>.vti by the library's VtkOutput.
   subroutine GpuPrintSolution(iter, g, mierr)
      integer(kind=4), intent(in) :: iter
      type(ads_gpu_handle), intent(in) :: g
      integer(kind=4), intent(out) :: mierr
      character(len=20) :: filename
      real(c_double) :: range(6) = (/ 0d0, 1d0, 0d0, 1d0, 0d0, 1d0 /)
      integer(c_int) :: res(3) = (/ 31, 31, 31 /)
      write(filename, '(I10)') iter
      filename = 'step' // adjustl(filename)
      mierr = ads_save_spline_plot(g % h, trim(filename) // c_null_char, range, res, c_null_ptr)
   end subroutine GpuPrintSolution

   ! Step (src/ADS.F90:437); F receives the solution (ads_data % F after Step).
   subroutine GpuStep(iter, g, F, l2norm, mierr)
      integer(kind=4), intent(in) :: iter
      type(ads_gpu_handle), intent(in) :: g
      real(c_double), intent(out) :: F(:)
      real(c_double), intent(out) :: l2norm
      integer(kind=4), intent(out) :: mierr
      mierr = ads_step(g % h, l2norm)
      if (mierr /= ADS_OK) return
      mierr = ads_get_coeffs(g % h, F)
   end subroutine GpuStep

   ! Step (src/ADS.F90:437) on the state array itself: u holds the coefficients
   ! before the call and the new ones after it (ads_step_host with u_out = u_in).
   subroutine GpuStepInPlace(g, u, l2norm, mierr)
      type(ads_gpu_handle), intent(in) :: g
      real(c_double), intent(inout), target, contiguous :: u(:)
      real(c_double), intent(out) :: l2norm
      integer(kind=4), intent(out) :: mierr
      mierr = ads_step_host(g % h, c_loc(u), c_loc(u), l2norm)
   end subroutine GpuStepInPlace

   ! MultiStep (src/ADS.F90:391): mix(4,3) as the reference's; F receives the solution.
   subroutine GpuMultiStep(iter, mix, g, F, l2norm, mierr)
      integer(kind=4), intent(in) :: iter
      real(c_double), intent(in) :: mix(4, 3)
      type(ads_gpu_handle), intent(in) :: g
      real(c_double), intent(out) :: F(:)
      real(c_double), intent(out) :: l2norm
      integer(kind=4), intent(out) :: mierr
      mierr = ads_multistep(g % h, mix, l2norm)
      if (mierr /= ADS_OK) return
      mierr = ads_get_coeffs(g % h, F)
   end subroutine GpuMultiStep

   ! Cleanup (src/ADS.F90:802).
   subroutine GpuCleanup(g, mierr)
      type(ads_gpu_handle), intent(inout) :: g
      integer(kind=4), intent(out) :: mierr
      mierr = ads_destroy(g % h)
      g % h = c_null_ptr
   end subroutine GpuCleanup

end module ads_gpu
