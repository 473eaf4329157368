module sht_gpu_radial
   !
   ! The radial-loop pieces around the transforms on the GB300 library:
   ! Courant steps (courant.f90:54-278) and the boundary routines of
   ! nonlinear_bcs.f90 and the Lorentz torques of outRot.f90, with the
   ! reference's argument lists plus the radial
   ! quantities the reference takes from its modules.  rIter.f90 calls these
   ! in place of `courant`, `v_rigid_boundary`, `v_center_sphere`,
   ! `get_br_v_bcs`, `get_b_nl_bcs` and `get_lorentz_torque`; a non-zero status becomes abortRun
   ! through module sht.  Host arrays are staged by the library.
   !
   use iso_c_binding
   use precision_mod, only: cp
   use sht, only: sht_handle, sht_check

   implicit none

   private

   type, bind(C) :: magic_sht_courant_args
      type(c_ptr) :: vr, vt, vp, br, bt, bp
      integer(c_long_long) :: grid_ld
      type(c_ptr) :: orho1, orho2, or2, or4, delxr2, delxh2
      real(c_double) :: courfac, alffac, LFfac, opm
      integer(c_int) :: l_cour_alf_damp
   end type magic_sht_courant_args

   type, bind(C) :: magic_sht_rigid_args
      type(c_ptr) :: vr, vt, vp, cvr, dvrdt, dvrdp, dvtdp, dvpdp
   end type magic_sht_rigid_args

   interface
      integer(c_int) function c_courant(h, n, a, dtrkc, dthkc) bind(C, name='magic_sht_courant')
         import :: c_int, c_ptr, c_double, magic_sht_courant_args
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(magic_sht_courant_args), intent(in) :: a
         real(c_double), intent(inout) :: dtrkc(*), dthkc(*)
      end function
      integer(c_int) function c_rigid(h, r2_rho0, omega, keep_vr, a) bind(C, name='magic_sht_v_rigid_boundary')
         import :: c_int, c_ptr, c_double, magic_sht_rigid_args
         type(c_ptr), value :: h
         real(c_double), value :: r2_rho0, omega
         integer(c_int), value :: keep_vr
         type(magic_sht_rigid_args), intent(in) :: a
      end function
      integer(c_int) function c_center(h, ddw, vr, vt, vp) bind(C, name='magic_sht_v_center_sphere')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: ddw(*)
         real(c_double), intent(out) :: vr(*), vt(*), vp(*)
      end function
      integer(c_int) function c_br_v(h, br, vt, vp, omega, or2, orho1, bvt, bvp) bind(C, name='magic_sht_get_br_v_bcs')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), intent(in) :: br(*), vt(*), vp(*)
         real(c_double), value :: omega, or2, orho1
         complex(c_double_complex), intent(out) :: bvt(*), bvp(*)
      end function
      integer(c_int) function c_torque(h, br, bp, LFfac, b0, torque) bind(C, name='magic_sht_lorentz_torque')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), intent(in) :: br(*), bp(*)
         real(c_double), value :: LFfac, b0
         real(c_double), intent(out) :: torque
      end function
      integer(c_int) function c_b_nl(h, fac, bvt, bvp, b_nl, aj_nl) bind(C, name='magic_sht_get_b_nl_bcs')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: h
         real(c_double), value :: fac
         type(c_ptr), value :: bvt, bvp, b_nl, aj_nl
      end function
   end interface

   public :: courant_gpu, v_rigid_boundary_gpu, v_center_sphere_gpu, get_br_v_bcs_gpu, get_b_nl_bcs_gpu, &
        &    get_lorentz_torque_gpu

contains

   subroutine courant_gpu(dtrkc, dthkc, vr, vt, vp, br, bt, bp, courfac, alffac, l_lorentz, &
              &           orho1, orho2, or2, or4, delxr2, delxh2, LFfac, opm, l_cour_alf_damp)
      ! courant() of one radial level; l_lorentz = l_mag .and. l_mag_LF .and. .not. l_mag_kin
      real(cp), intent(inout) :: dtrkc, dthkc
      real(cp), target, intent(in) :: vr(:,:), vt(:,:), vp(:,:), br(:,:), bt(:,:), bp(:,:)
      real(cp), intent(in) :: courfac, alffac, LFfac, opm
      real(cp), target, intent(in) :: orho1, orho2, or2, or4, delxr2, delxh2
      logical,  intent(in) :: l_lorentz, l_cour_alf_damp
      type(magic_sht_courant_args) :: a
      real(c_double) :: r(1), h(1)
      a%vr = c_loc(vr); a%vt = c_loc(vt); a%vp = c_loc(vp)
      a%br = c_null_ptr; a%bt = c_null_ptr; a%bp = c_null_ptr
      if ( l_lorentz ) then
         a%br = c_loc(br); a%bt = c_loc(bt); a%bp = c_loc(bp)
      end if
      a%grid_ld = size(vr, kind=c_long_long)
      a%orho1 = c_loc(orho1); a%orho2 = c_loc(orho2); a%or2 = c_loc(or2); a%or4 = c_loc(or4)
      a%delxr2 = c_loc(delxr2); a%delxh2 = c_loc(delxh2)
      a%courfac = courfac; a%alffac = alffac; a%LFfac = LFfac; a%opm = opm
      a%l_cour_alf_damp = merge(1, 0, l_cour_alf_damp)
      r(1) = dtrkc; h(1) = dthkc
      call sht_check(c_courant(sht_handle(), 1, a, r, h))
      dtrkc = r(1); dthkc = h(1)
   end subroutine courant_gpu

   subroutine v_rigid_boundary_gpu(r2_rho0, omega, lDeriv, l_vr, vrr, vtr, vpr, cvrr, dvrdtr, &
              &                    dvrdpr, dvtdpr, dvpdpr)
      ! v_rigid_boundary with r2_rho0 = r(nR)**2 * rho0(nR) and l_vr = l_vr_cmb / l_vr_icb
      real(cp), intent(in) :: r2_rho0, omega
      logical,  intent(in) :: lDeriv, l_vr
      real(cp), target, intent(inout) :: vrr(:,:), vtr(:,:), vpr(:,:)
      real(cp), target, intent(inout) :: cvrr(:,:), dvrdtr(:,:), dvrdpr(:,:), dvtdpr(:,:), dvpdpr(:,:)
      type(magic_sht_rigid_args) :: a
      a%vr = c_loc(vrr); a%vt = c_loc(vtr); a%vp = c_loc(vpr)
      a%cvr = c_null_ptr; a%dvrdt = c_null_ptr; a%dvrdp = c_null_ptr; a%dvtdp = c_null_ptr
      a%dvpdp = c_null_ptr
      if ( lDeriv ) then
         a%cvr = c_loc(cvrr); a%dvrdt = c_loc(dvrdtr); a%dvrdp = c_loc(dvrdpr)
         a%dvtdp = c_loc(dvtdpr); a%dvpdp = c_loc(dvpdpr)
      end if
      call sht_check(c_rigid(sht_handle(), r2_rho0, omega, merge(1, 0, l_vr), a))
   end subroutine v_rigid_boundary_gpu

   subroutine v_center_sphere_gpu(ddw, vrr, vtr, vpr)
      complex(cp), intent(in) :: ddw(:)
      real(cp), intent(out) :: vrr(:,:), vtr(:,:), vpr(:,:)
      call sht_check(c_center(sht_handle(), ddw, vrr, vtr, vpr))
   end subroutine v_center_sphere_gpu

   subroutine get_br_v_bcs_gpu(br, vt, vp, omega, O_r_E_2, O_rho, br_vt_lm, br_vp_lm)
      real(cp), intent(in) :: br(:,:), vt(:,:), vp(:,:)
      real(cp), intent(in) :: omega, O_r_E_2, O_rho
      complex(cp), intent(out) :: br_vt_lm(:), br_vp_lm(:)
      call sht_check(c_br_v(sht_handle(), br, vt, vp, omega, O_r_E_2, O_rho, br_vt_lm, br_vp_lm))
   end subroutine get_br_v_bcs_gpu

   subroutine get_lorentz_torque_gpu(lorentz_torque, br, bp, LFfac, b0)
      ! get_lorentz_torque of one boundary level; b0 = 2*BIC*r_icb**2 (times
      ! r_icb/r_cmb at the CMB) with lGrenoble, else 0.  The radial loop
      ! negates the mantle's value (rIter.f90:462).
      real(cp), intent(out) :: lorentz_torque
      real(cp), intent(in) :: br(:,:), bp(:,:)
      real(cp), intent(in) :: LFfac, b0
      real(c_double) :: t
      call sht_check(c_torque(sht_handle(), br, bp, LFfac, b0, t))
      lorentz_torque = t
   end subroutine get_lorentz_torque_gpu

   subroutine get_b_nl_bcs_gpu(bc, fac, br_vt_lm, br_vp_lm, b_nl_bc, aj_nl_bc)
      ! get_b_nl_bcs with fac = conductance_ma*prmag ('CMB') or sigma_ratio*prmag ('ICB')
      character(len=3), intent(in) :: bc
      real(cp), intent(in) :: fac
      complex(cp), target, intent(in) :: br_vt_lm(:), br_vp_lm(:)
      complex(cp), target, intent(out) :: b_nl_bc(:), aj_nl_bc(:)
      if ( bc == 'CMB' ) then
         call sht_check(c_b_nl(sht_handle(), fac, c_loc(br_vt_lm), c_loc(br_vp_lm), c_loc(b_nl_bc), &
              &                c_loc(aj_nl_bc)))
      else
         call sht_check(c_b_nl(sht_handle(), fac, c_null_ptr, c_loc(br_vp_lm), c_null_ptr, c_loc(aj_nl_bc)))
      end if
   end subroutine get_b_nl_bcs_gpu

end module sht_gpu_radial
