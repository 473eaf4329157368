module sht
   !
   ! Drop-in replacement of MagIC's native `module sht` (src/sht_native.f90)
   ! that forwards every public routine to the GB300 CUDA library
   ! libmagic_sht.so through its C ABI (include/magic_sht.h).  The public
   ! names and argument lists are those of src/sht_native.f90:16-20, so the
   ! callers (rIter.f90 and the diagnostics) compile unchanged.  A non-zero
   ! status from the library is turned into abortRun, as the reference does
   ! on bad sizes (truncation.f90:126-160, fft.f90:55-65).
   !
   ! Host arrays are passed as they are: the library stages them through the
   ! GPU and returns once the results are back on the host.
   !
   use iso_c_binding
   use precision_mod, only: cp
   use truncation, only: l_max, m_max, minc, n_theta_max, n_phi_max, nlat_padded, lm_max
   use useful, only: abortRun

   implicit none

   private

   type, bind(C) :: magic_sht_desc
      integer(c_int) :: l_max, m_max, minc, n_theta_max, n_phi_max, nlat_padded
      integer(c_int) :: precision, device
   end type magic_sht_desc

   type(c_ptr), save :: handle = c_null_ptr

   interface
      integer(c_int) function c_init(desc, h) bind(C, name='magic_sht_init')
         import :: c_int, c_ptr, magic_sht_desc
         type(magic_sht_desc), intent(in) :: desc
         type(c_ptr), intent(out) :: h
      end function
      integer(c_int) function c_finalize(h) bind(C, name='magic_sht_finalize')
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function
      type(c_ptr) function c_last_error() bind(C, name='magic_sht_last_error')
         import :: c_ptr
      end function
      integer(c_int) function c_scal_to_spat(h, S, f, lcut) bind(C, name='magic_sht_scal_to_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: S(*)
         real(c_double), intent(out) :: f(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_scal_to_grad_spat(h, S, gt, gp, lcut) bind(C, name='magic_sht_scal_to_grad_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: S(*)
         real(c_double), intent(out) :: gt(*), gp(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_pol_to_grad_spat(h, S, gt, gp, lcut) bind(C, name='magic_sht_pol_to_grad_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: S(*)
         real(c_double), intent(out) :: gt(*), gp(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_torpol_to_spat(h, W, dW, Z, vr, vt, vp, lcut) bind(C, name='magic_sht_torpol_to_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: W(*), dW(*), Z(*)
         real(c_double), intent(out) :: vr(*), vt(*), vp(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_sphtor_to_spat(h, dW, Z, vt, vp, lcut) bind(C, name='magic_sht_sphtor_to_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: dW(*), Z(*)
         real(c_double), intent(out) :: vt(*), vp(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_torpol_to_curl_spat_IC(h, r, r_ICB, dB, ddB, J, dJ, cbr, cbt, cbp) &
            bind(C, name='magic_sht_torpol_to_curl_spat_IC')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), value :: r, r_ICB
         complex(c_double_complex), intent(in) :: dB(*), ddB(*), J(*), dJ(*)
         real(c_double), intent(out) :: cbr(*), cbt(*), cbp(*)
      end function
      integer(c_int) function c_torpol_to_spat_IC(h, r, r_ICB, W, dW, Z, Br, Bt, Bp) &
            bind(C, name='magic_sht_torpol_to_spat_IC')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), value :: r, r_ICB
         complex(c_double_complex), intent(in) :: W(*), dW(*), Z(*)
         real(c_double), intent(out) :: Br(*), Bt(*), Bp(*)
      end function
      integer(c_int) function c_torpol_to_dphspat(h, dW, Z, a, b, lcut) bind(C, name='magic_sht_torpol_to_dphspat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: dW(*), Z(*)
         real(c_double), intent(out) :: a(*), b(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_pol_to_curlr_spat(h, Q, f, lcut) bind(C, name='magic_sht_pol_to_curlr_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: Q(*)
         real(c_double), intent(out) :: f(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_torpol_to_curl_spat(h, or2, B, ddB, J, dJ, a, b, c, lcut) &
            bind(C, name='magic_sht_torpol_to_curl_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), value :: or2
         complex(c_double_complex), intent(in) :: B(*), ddB(*), J(*), dJ(*)
         real(c_double), intent(out) :: a(*), b(*), c(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_axi_to_spat(h, fl, f) bind(C, name='magic_sht_axi_to_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: fl(*)
         real(c_double), intent(out) :: f(*)
      end function
      integer(c_int) function c_toraxi_to_spat(h, fl, ft, fp, lcut) bind(C, name='magic_sht_toraxi_to_spat')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in) :: fl(*)
         real(c_double), intent(out) :: ft(*), fp(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_scal_to_SH(h, f, fLM, lcut) bind(C, name='magic_sht_scal_to_SH')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), intent(in) :: f(*)
         complex(c_double_complex), intent(out) :: fLM(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_spat_to_qst(h, f, g, hh, q, s, t, lcut) bind(C, name='magic_sht_spat_to_qst')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), intent(in) :: f(*), g(*), hh(*)
         complex(c_double_complex), intent(out) :: q(*), s(*), t(*)
         integer(c_int), value :: lcut
      end function
      integer(c_int) function c_spat_to_sphertor(h, f, g, fLM, gLM, lcut) bind(C, name='magic_sht_spat_to_sphertor')
         import :: c_int, c_ptr, c_double, c_double_complex
         type(c_ptr), value :: h
         real(c_double), intent(in) :: f(*), g(*)
         complex(c_double_complex), intent(out) :: fLM(*), gLM(*)
         integer(c_int), value :: lcut
      end function
   end interface

   public :: sht_handle, sht_check
   public :: initialize_sht, scal_to_spat, scal_to_grad_spat, pol_to_grad_spat, &
   &         torpol_to_spat, pol_to_curlr_spat, torpol_to_curl_spat,            &
   &         torpol_to_dphspat, scal_to_SH, spat_to_sphertor,                   &
   &         torpol_to_spat_IC, torpol_to_curl_spat_IC, axi_to_spat,            &
   &         spat_to_qst, sphtor_to_spat, toraxi_to_spat, finalize_sht

contains

   subroutine check(rc)
      integer(c_int), intent(in) :: rc
      character(kind=c_char), pointer :: msg(:)
      character(len=256) :: text
      integer :: i
      if ( rc /= 0 ) then
         call c_f_pointer(c_last_error(), msg, [256])
         text = ' '
         do i=1,256
            if ( msg(i) == c_null_char ) exit
            text(i:i) = msg(i)
         end do
         call abortRun('magic_sht: '//trim(text))
      end if
   end subroutine check

   type(c_ptr) function sht_handle()
      ! the library handle, for the radial-loop pieces (module sht_gpu_radial)
      sht_handle = handle
   end function sht_handle

   subroutine sht_check(rc)
      integer(c_int), intent(in) :: rc
      call check(rc)
   end subroutine sht_check

   subroutine initialize_sht(l_scrambled_theta)
      ! The plain FP64 form (the drop-in's arithmetic) unless the environment
      ! variable MAGIC_SHT_PRECISION selects another form of the library:
      ! fp64tc (FP64-accurate on the tensor cores, the same 1e-12 parity with
      ! the native transforms), bf16x5, bf16x3, tf32x2 or fp32.
      logical, intent(out) :: l_scrambled_theta
      type(magic_sht_desc) :: d
      character(len=16) :: form
      integer :: length, status
      d%l_max = l_max; d%m_max = m_max; d%minc = minc
      d%n_theta_max = n_theta_max; d%n_phi_max = n_phi_max
      d%nlat_padded = nlat_padded; d%precision = 0; d%device = -1
      call get_environment_variable('MAGIC_SHT_PRECISION', form, length, status)
      if ( status == 0 .and. length > 0 ) then
         select case ( trim(form) )
         case ( 'fp64' )
            d%precision = 0
         case ( 'fp32' )
            d%precision = 1
         case ( 'bf16x3' )
            d%precision = 2
         case ( 'tf32x2' )
            d%precision = 3
         case ( 'fp64tc' )
            d%precision = 4
         case ( 'bf16x5' )
            d%precision = 5
         case default
            call abortRun('magic_sht: MAGIC_SHT_PRECISION='//trim(form)// &
                 &        ' is not one of fp64, fp64tc, bf16x5, bf16x3, tf32x2, fp32')
         end select
      end if
      call check(c_init(d, handle))
      l_scrambled_theta = .true.
   end subroutine initialize_sht

   subroutine finalize_sht()
      call check(c_finalize(handle))
      handle = c_null_ptr
   end subroutine finalize_sht

   subroutine scal_to_spat(Slm, fieldc, lcut)
      complex(cp), intent(in) :: Slm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: fieldc(:,:)
      call check(c_scal_to_spat(handle, Slm, fieldc, lcut))
   end subroutine scal_to_spat

   subroutine scal_to_grad_spat(Slm, gradtc, gradpc, lcut)
      complex(cp), intent(in) :: Slm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: gradtc(:,:), gradpc(:,:)
      call check(c_scal_to_grad_spat(handle, Slm, gradtc, gradpc, lcut))
   end subroutine scal_to_grad_spat

   subroutine pol_to_grad_spat(Slm, gradtc, gradpc, lcut)
      complex(cp), intent(in) :: Slm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: gradtc(:,:), gradpc(:,:)
      call check(c_pol_to_grad_spat(handle, Slm, gradtc, gradpc, lcut))
   end subroutine pol_to_grad_spat

   subroutine torpol_to_spat(Wlm, dWlm, Zlm, vrc, vtc, vpc, lcut)
      complex(cp), intent(in) :: Wlm(:), dWlm(:), Zlm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: vrc(:,:), vtc(:,:), vpc(:,:)
      call check(c_torpol_to_spat(handle, Wlm, dWlm, Zlm, vrc, vtc, vpc, lcut))
   end subroutine torpol_to_spat

   subroutine sphtor_to_spat(dWlm, Zlm, vtc, vpc, lcut)
      complex(cp), intent(in) :: dWlm(:), Zlm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: vtc(:,:), vpc(:,:)
      call check(c_sphtor_to_spat(handle, dWlm, Zlm, vtc, vpc, lcut))
   end subroutine sphtor_to_spat

   subroutine torpol_to_curl_spat_IC(r, r_ICB, dBlm, ddBlm, Jlm, dJlm, cbr, cbt, cbp)
      real(cp),    intent(in) :: r, r_ICB
      complex(cp), intent(in) :: dBlm(:), ddBlm(:), Jlm(:), dJlm(:)
      real(cp),    intent(out) :: cbr(:,:), cbt(:,:), cbp(:,:)
      call check(c_torpol_to_curl_spat_IC(handle, r, r_ICB, dBlm, ddBlm, Jlm, dJlm, cbr, cbt, cbp))
   end subroutine torpol_to_curl_spat_IC

   subroutine torpol_to_spat_IC(r, r_ICB, Wlm, dWlm, Zlm, Br, Bt, Bp)
      real(cp),    intent(in) :: r, r_ICB
      complex(cp), intent(in) :: Wlm(:), dWlm(:), Zlm(:)
      real(cp),    intent(out) :: Br(:,:), Bt(:,:), Bp(:,:)
      call check(c_torpol_to_spat_IC(handle, r, r_ICB, Wlm, dWlm, Zlm, Br, Bt, Bp))
   end subroutine torpol_to_spat_IC

   subroutine torpol_to_dphspat(dWlm, Zlm, dvtdp, dvpdp, lcut)
      complex(cp), intent(in) :: dWlm(:), Zlm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: dvtdp(:,:), dvpdp(:,:)
      call check(c_torpol_to_dphspat(handle, dWlm, Zlm, dvtdp, dvpdp, lcut))
   end subroutine torpol_to_dphspat

   subroutine pol_to_curlr_spat(Qlm, cvrc, lcut)
      complex(cp), intent(in) :: Qlm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: cvrc(:,:)
      call check(c_pol_to_curlr_spat(handle, Qlm, cvrc, lcut))
   end subroutine pol_to_curlr_spat

   subroutine torpol_to_curl_spat(or2, Blm, ddBlm, Jlm, dJlm, cvrc, cvtc, cvpc, lcut)
      real(cp),    intent(in) :: or2
      complex(cp), intent(in) :: Blm(:), ddBlm(:), Jlm(:), dJlm(:)
      integer,     intent(in) :: lcut
      real(cp),    intent(out) :: cvrc(:,:), cvtc(:,:), cvpc(:,:)
      call check(c_torpol_to_curl_spat(handle, or2, Blm, ddBlm, Jlm, dJlm, cvrc, cvtc, cvpc, lcut))
   end subroutine torpol_to_curl_spat

   subroutine scal_to_SH(f, fLM, lcut)
      real(cp),    intent(inout) :: f(:,:)
      integer,     intent(in) :: lcut
      complex(cp), intent(out) :: fLM(:)
      call check(c_scal_to_SH(handle, f, fLM, lcut))
   end subroutine scal_to_SH

   subroutine spat_to_qst(f, g, h, qLM, sLM, tLM, lcut)
      real(cp),    intent(inout) :: f(:,:), g(:,:), h(:,:)
      integer,     intent(in) :: lcut
      complex(cp), intent(out) :: qLM(:), sLM(:), tLM(:)
      call check(c_spat_to_qst(handle, f, g, h, qLM, sLM, tLM, lcut))
   end subroutine spat_to_qst

   subroutine spat_to_sphertor(f, g, fLM, gLM, lcut)
      real(cp),    intent(inout) :: f(:,:), g(:,:)
      integer,     intent(in) :: lcut
      complex(cp), intent(out) :: fLM(:), gLM(:)
      call check(c_spat_to_sphertor(handle, f, g, fLM, gLM, lcut))
   end subroutine spat_to_sphertor

   subroutine axi_to_spat(fl_ax, f)
      complex(cp), intent(in) :: fl_ax(l_max+1)
      real(cp),    intent(out) :: f(:)
      call check(c_axi_to_spat(handle, fl_ax, f))
   end subroutine axi_to_spat

   subroutine toraxi_to_spat(fl_ax, ft, fp, lcut)
      integer,     intent(in) :: lcut
      complex(cp), intent(in) :: fl_ax(l_max+1)
      real(cp),    intent(out) :: ft(:), fp(:)
      call check(c_toraxi_to_spat(handle, fl_ax, ft, fp, lcut))
   end subroutine toraxi_to_spat

end module sht
