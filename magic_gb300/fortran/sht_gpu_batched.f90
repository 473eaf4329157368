module sht_gpu_batched
   !
   ! The batched entry points of the GB300 library, for a radial loop that
   ! keeps its levels on the GPU: the radial loop's transform set for all of a
   ! rank's levels in one call each (transform_to_grid_space,
   ! rIter.f90:466-622; transform_to_lm_space, rIter.f90:624-712), the
   ! grid-space products (get_nl.f90:213-441), the spectral assembly with the
   ! boundary flags (get_td.f90:133-619) and the new time step
   ! (dt_courant, courant.f90:280-346).
   !
   ! Spectral arrays are the reference's R-distributed fields
   ! f_Rloc(lm_max, nRstart:nRstop) (one column per level); grids are
   ! (nlat_padded, n_phi_max, levels), i.e. the per-level grids of
   ! grid_space_arrays stacked over the levels.  Host arrays are staged by the
   ! library and the call returns with its results; device arrays (CUDA
   ! Fortran `device` arrays, or OpenACC `host_data use_device`) are used in
   ! place and the call is asynchronous on the library's stream.  A non-zero
   ! status becomes abortRun through module sht.
   !
   use iso_c_binding
   use precision_mod, only: cp
   use sht, only: sht_handle, sht_check

   implicit none

   private

   type, bind(C) :: magic_sht_grid_space_args
      type(c_ptr) :: s, p, xi, w, dw, ddw, z, dz, b, db, ddb, aj, dj
      integer(c_long_long) :: spec_ld
      type(c_ptr) :: sc, pc, xic, vrc, vtc, vpc, cvrc, cvtc, cvpc, brc, btc, bpc, cbrc, cbtc, cbpc
      integer(c_long_long) :: grid_ld
      type(c_ptr) :: dvrdrc, dvtdrc, dvpdrc, dvrdtc, dvrdpc, dvtdpc, dvpdpc
   end type magic_sht_grid_space_args

   type, bind(C) :: magic_sht_lm_space_args
      type(c_ptr) :: Advr, Advt, Advp, VSr, VSt, VSp, VxBr, VxBt, VxBp, heatTerms
      integer(c_long_long) :: grid_ld
      type(c_ptr) :: AdvrLM, AdvtLM, AdvpLM, VSrLM, VStLM, VSpLM, VxBrLM, VxBtLM, VxBpLM, heatTermsLM
      integer(c_long_long) :: spec_ld
      type(c_ptr) :: VXir, VXit, VXip
      type(c_ptr) :: VXirLM, VXitLM, VXipLM
   end type magic_sht_lm_space_args

   type, bind(C) :: magic_sht_td_args
      type(c_ptr) :: w, dw, z, AdvrLM, AdvtLM, AdvpLM, VStLM, VxBrLM, VxBtLM, VxBpLM
      type(c_ptr) :: dwdt, dzdt, dpdt, dsdt, dbdt, djdt, dVxBhLM
      integer(c_long_long) :: spec_ld
   end type magic_sht_td_args

   ! one facade routine over many levels (magic_sht_inv_batch / _fwd_batch):
   ! in(:) its array inputs, out(:) its outputs in the routine's argument
   ! order (c_loc of the first level), unused slots c_null_ptr
   type, bind(C) :: magic_sht_job
      integer(c_int) :: routine, pad_
      type(c_ptr) :: in(4)
      type(c_ptr) :: out(3)
   end type magic_sht_job

   integer(c_int), parameter, public :: MAGIC_SHT_JOB_SCAL_TO_SPAT = 1, MAGIC_SHT_JOB_SCAL_TO_GRAD_SPAT = 2, &
        &    MAGIC_SHT_JOB_POL_TO_GRAD_SPAT = 3, MAGIC_SHT_JOB_TORPOL_TO_SPAT = 4,                         &
        &    MAGIC_SHT_JOB_SPHTOR_TO_SPAT = 5, MAGIC_SHT_JOB_TORPOL_TO_CURL_SPAT = 6,                      &
        &    MAGIC_SHT_JOB_POL_TO_CURLR_SPAT = 7, MAGIC_SHT_JOB_TORPOL_TO_DPHSPAT = 8,                     &
        &    MAGIC_SHT_JOB_SCAL_TO_SH = 101, MAGIC_SHT_JOB_SPAT_TO_QST = 102,                               &
        &    MAGIC_SHT_JOB_SPAT_TO_SPHERTOR = 103

   interface
      integer(c_int) function c_to_grid(h, n, or2, lcut, a) bind(C, name='magic_sht_transform_to_grid_space')
         import :: c_int, c_ptr, magic_sht_grid_space_args
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(c_ptr), value :: or2, lcut
         type(magic_sht_grid_space_args), intent(in) :: a
      end function
      integer(c_int) function c_to_lm(h, n, lcut, a) bind(C, name='magic_sht_transform_to_lm_space')
         import :: c_int, c_ptr, magic_sht_lm_space_args
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(c_ptr), value :: lcut
         type(magic_sht_lm_space_args), intent(in) :: a
      end function
      integer(c_int) function c_get_nl(h, n, or2, g, nl) bind(C, name='magic_sht_get_nl')
         import :: c_int, c_ptr, magic_sht_grid_space_args, magic_sht_lm_space_args
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(c_ptr), value :: or2
         type(magic_sht_grid_space_args), intent(in) :: g
         type(magic_sht_lm_space_args), intent(in) :: nl
      end function
      integer(c_int) function c_get_td_nbc(h, n, r, lcut, cor_fac, epsc, nbc, a) &
            &        bind(C, name='magic_sht_get_td_nbc')
         import :: c_int, c_ptr, c_double, magic_sht_td_args
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(c_ptr), value :: r, lcut
         real(c_double), value :: cor_fac
         type(c_ptr), value :: epsc, nbc
         type(magic_sht_td_args), intent(in) :: a
      end function
      integer(c_int) function c_dt_courant(n, dtrkc, dthkc, dt, dtMax, l_new_dt, dt_new) &
            &        bind(C, name='magic_sht_dt_courant')
         import :: c_int, c_double
         integer(c_int), value :: n
         real(c_double), intent(in) :: dtrkc(*), dthkc(*)
         real(c_double), value :: dt, dtMax
         integer(c_int), intent(out) :: l_new_dt
         real(c_double), intent(out) :: dt_new
      end function
      integer(c_int) function c_reserve(h, n) bind(C, name='magic_sht_reserve')
         import :: c_int, c_ptr
         type(c_ptr), value :: h
         integer(c_int), value :: n
      end function
      integer(c_int) function c_inv_batch(h, n, or2, lcut, spec_ld, grid_ld, jobs, n_jobs) &
            &        bind(C, name='magic_sht_inv_batch')
         import :: c_int, c_ptr, c_long_long, magic_sht_job
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(c_ptr), value :: or2, lcut
         integer(c_long_long), value :: spec_ld, grid_ld
         type(magic_sht_job), intent(in) :: jobs(*)
         integer(c_int), value :: n_jobs
      end function
      integer(c_int) function c_fwd_batch(h, n, lcut, grid_ld, spec_ld, jobs, n_jobs) &
            &        bind(C, name='magic_sht_fwd_batch')
         import :: c_int, c_ptr, c_long_long, magic_sht_job
         type(c_ptr), value :: h
         integer(c_int), value :: n
         type(c_ptr), value :: lcut
         integer(c_long_long), value :: grid_ld, spec_ld
         type(magic_sht_job), intent(in) :: jobs(*)
         integer(c_int), value :: n_jobs
      end function
   end interface

   public :: transform_to_grid_space_gpu, transform_to_lm_space_gpu, get_nl_gpu, get_td_gpu, &
        &    dt_courant_gpu, reserve_levels_gpu, magic_sht_job, inv_batch_gpu, fwd_batch_gpu

contains

   subroutine transform_to_grid_space_gpu(or2, lcut, w, dw, ddw, z, dz, vrc, vtc, vpc, cvrc, cvtc, cvpc, &
              &                           s, p, xi, b, db, ddb, aj, dj, sc, pc, xic, brc, btc, bpc,    &
              &                           cbrc, cbtc, cbpc, dvrdrc, dvtdrc, dvpdrc, dvrdtc, dvrdpc,    &
              &                           dvtdpc, dvpdpc)
      ! transform_to_grid_space of every level (column) of the spectra at
      ! once: or2(nR) = 1/r^2, lcut(nR) = l_R.  The velocity set is always
      ! transformed; s, p, xi (scalars) and b, db, ddb, aj, dj (magnetic
      ! field) with their grids only when present.  Without cvtc and cvpc,
      ! cvrc is pol_to_curlr_spat(z) (the u.grad u set, rIter.f90:540);
      ! dvrdrc .. dvpdpc, when present, are the velocity derivatives
      ! (rIter.f90:527-545).
      real(cp),       target, contiguous, intent(in) :: or2(:)
      integer(c_int), target, contiguous, intent(in) :: lcut(:)
      complex(cp), target, contiguous, intent(in) :: w(:,:), dw(:,:), ddw(:,:), z(:,:), dz(:,:)
      real(cp), target, contiguous, intent(out) :: vrc(:,:,:), vtc(:,:,:), vpc(:,:,:)
      real(cp), target, contiguous, intent(out) :: cvrc(:,:,:)
      real(cp), target, contiguous, optional, intent(out) :: cvtc(:,:,:), cvpc(:,:,:)
      complex(cp), target, contiguous, optional, intent(in) :: s(:,:), p(:,:), xi(:,:)
      complex(cp), target, contiguous, optional, intent(in) :: b(:,:), db(:,:), ddb(:,:), aj(:,:), dj(:,:)
      real(cp), target, contiguous, optional, intent(out) :: sc(:,:,:), pc(:,:,:), xic(:,:,:)
      real(cp), target, contiguous, optional, intent(out) :: brc(:,:,:), btc(:,:,:), bpc(:,:,:)
      real(cp), target, contiguous, optional, intent(out) :: cbrc(:,:,:), cbtc(:,:,:), cbpc(:,:,:)
      real(cp), target, contiguous, optional, intent(out) :: dvrdrc(:,:,:), dvtdrc(:,:,:), dvpdrc(:,:,:)
      real(cp), target, contiguous, optional, intent(out) :: dvrdtc(:,:,:), dvrdpc(:,:,:)
      real(cp), target, contiguous, optional, intent(out) :: dvtdpc(:,:,:), dvpdpc(:,:,:)
      type(magic_sht_grid_space_args) :: a

      call null_grid_args(a)
      a%w = c_loc(w); a%dw = c_loc(dw); a%ddw = c_loc(ddw); a%z = c_loc(z); a%dz = c_loc(dz)
      a%vrc = c_loc(vrc); a%vtc = c_loc(vtc); a%vpc = c_loc(vpc)
      a%cvrc = c_loc(cvrc)
      if ( present(cvtc) .and. present(cvpc) ) then
         a%cvtc = c_loc(cvtc); a%cvpc = c_loc(cvpc)
      end if
      if ( present(dvrdrc) .and. present(dvtdrc) .and. present(dvpdrc) ) then
         a%dvrdrc = c_loc(dvrdrc); a%dvtdrc = c_loc(dvtdrc); a%dvpdrc = c_loc(dvpdrc)
      end if
      if ( present(dvrdtc) .and. present(dvrdpc) ) then
         a%dvrdtc = c_loc(dvrdtc); a%dvrdpc = c_loc(dvrdpc)
      end if
      if ( present(dvtdpc) .and. present(dvpdpc) ) then
         a%dvtdpc = c_loc(dvtdpc); a%dvpdpc = c_loc(dvpdpc)
      end if
      if ( present(s) .and. present(sc) ) then
         a%s = c_loc(s); a%sc = c_loc(sc)
      end if
      if ( present(p) .and. present(pc) ) then
         a%p = c_loc(p); a%pc = c_loc(pc)
      end if
      if ( present(xi) .and. present(xic) ) then
         a%xi = c_loc(xi); a%xic = c_loc(xic)
      end if
      ! B from b, db, aj (rIter.f90:606); curl B from b, ddb, aj, dj (:610)
      if ( present(b) .and. present(db) .and. present(aj) .and. present(brc) .and. &
           present(btc) .and. present(bpc) ) then
         a%b = c_loc(b); a%db = c_loc(db); a%aj = c_loc(aj)
         a%brc = c_loc(brc); a%btc = c_loc(btc); a%bpc = c_loc(bpc)
      end if
      if ( present(b) .and. present(ddb) .and. present(aj) .and. present(dj) .and. present(cbrc) .and. &
           present(cbtc) .and. present(cbpc) ) then
         a%b = c_loc(b); a%ddb = c_loc(ddb); a%aj = c_loc(aj); a%dj = c_loc(dj)
         a%cbrc = c_loc(cbrc); a%cbtc = c_loc(cbtc); a%cbpc = c_loc(cbpc)
      end if
      a%spec_ld = size(w, 1, kind=c_long_long)
      a%grid_ld = size(vrc, 1, kind=c_long_long) * size(vrc, 2, kind=c_long_long)
      call sht_check(c_to_grid(sht_handle(), int(size(w, 2), c_int), c_loc(or2), c_loc(lcut), a))
   end subroutine transform_to_grid_space_gpu

   subroutine transform_to_lm_space_gpu(lcut, Advr, Advt, Advp, VSr, VSt, VSp, VxBr, VxBt, VxBp, heatTerms, &
              &                         AdvrLM, AdvtLM, AdvpLM, VSrLM, VStLM, VSpLM, VxBrLM, VxBtLM,      &
              &                         VxBpLM, heatTermsLM)
      ! transform_to_lm_space of every level (third dimension of the grids)
      ! at once; lcut(nR) = l_R.
      integer(c_int), target, contiguous, intent(in) :: lcut(:)
      real(cp), target, contiguous, intent(in) :: Advr(:,:,:), Advt(:,:,:), Advp(:,:,:)
      real(cp), target, contiguous, intent(in) :: VSr(:,:,:), VSt(:,:,:), VSp(:,:,:)
      real(cp), target, contiguous, intent(in) :: VxBr(:,:,:), VxBt(:,:,:), VxBp(:,:,:), heatTerms(:,:,:)
      complex(cp), target, contiguous, intent(out) :: AdvrLM(:,:), AdvtLM(:,:), AdvpLM(:,:)
      complex(cp), target, contiguous, intent(out) :: VSrLM(:,:), VStLM(:,:), VSpLM(:,:)
      complex(cp), target, contiguous, intent(out) :: VxBrLM(:,:), VxBtLM(:,:), VxBpLM(:,:), heatTermsLM(:,:)
      type(magic_sht_lm_space_args) :: a

      a%Advr = c_loc(Advr); a%Advt = c_loc(Advt); a%Advp = c_loc(Advp)
      a%VSr = c_loc(VSr); a%VSt = c_loc(VSt); a%VSp = c_loc(VSp)
      a%VxBr = c_loc(VxBr); a%VxBt = c_loc(VxBt); a%VxBp = c_loc(VxBp); a%heatTerms = c_loc(heatTerms)
      a%grid_ld = size(Advr, 1, kind=c_long_long) * size(Advr, 2, kind=c_long_long)
      a%AdvrLM = c_loc(AdvrLM); a%AdvtLM = c_loc(AdvtLM); a%AdvpLM = c_loc(AdvpLM)
      a%VSrLM = c_loc(VSrLM); a%VStLM = c_loc(VStLM); a%VSpLM = c_loc(VSpLM)
      a%VxBrLM = c_loc(VxBrLM); a%VxBtLM = c_loc(VxBtLM); a%VxBpLM = c_loc(VxBpLM)
      a%heatTermsLM = c_loc(heatTermsLM)
      a%spec_ld = size(AdvrLM, 1, kind=c_long_long)
      a%VXir = c_null_ptr; a%VXit = c_null_ptr; a%VXip = c_null_ptr
      a%VXirLM = c_null_ptr; a%VXitLM = c_null_ptr; a%VXipLM = c_null_ptr
      call sht_check(c_to_lm(sht_handle(), int(size(Advr, 3), c_int), c_loc(lcut), a))
   end subroutine transform_to_lm_space_gpu

   subroutine get_nl_gpu(or2, vrc, vtc, vpc, cvrc, cvtc, cvpc, brc, btc, bpc, cbrc, cbtc, cbpc, sc, &
              &          Advr, Advt, Advp, VSr, VSt, VSp, VxBr, VxBt, VxBp, heatTerms)
      ! get_nl of every level (third dimension) at once: Boussinesq, curl-form
      ! advection, magnetic field and heat equation, unit physical constants;
      ! heatTerms receives the ohmic losses.  Device arrays only (16-byte
      ! aligned, even nlat_padded); or2(nR) = 1/r^2 (host or device).
      real(cp), target, contiguous, intent(in) :: or2(:)
      real(cp), target, contiguous, intent(in) :: vrc(:,:,:), vtc(:,:,:), vpc(:,:,:)
      real(cp), target, contiguous, intent(in) :: cvrc(:,:,:), cvtc(:,:,:), cvpc(:,:,:)
      real(cp), target, contiguous, intent(in) :: brc(:,:,:), btc(:,:,:), bpc(:,:,:)
      real(cp), target, contiguous, intent(in) :: cbrc(:,:,:), cbtc(:,:,:), cbpc(:,:,:), sc(:,:,:)
      real(cp), target, contiguous, intent(out) :: Advr(:,:,:), Advt(:,:,:), Advp(:,:,:)
      real(cp), target, contiguous, intent(out) :: VSr(:,:,:), VSt(:,:,:), VSp(:,:,:)
      real(cp), target, contiguous, intent(out) :: VxBr(:,:,:), VxBt(:,:,:), VxBp(:,:,:), heatTerms(:,:,:)
      type(magic_sht_grid_space_args) :: g
      type(magic_sht_lm_space_args) :: nl

      call null_grid_args(g)
      g%vrc = c_loc(vrc); g%vtc = c_loc(vtc); g%vpc = c_loc(vpc)
      g%cvrc = c_loc(cvrc); g%cvtc = c_loc(cvtc); g%cvpc = c_loc(cvpc)
      g%brc = c_loc(brc); g%btc = c_loc(btc); g%bpc = c_loc(bpc)
      g%cbrc = c_loc(cbrc); g%cbtc = c_loc(cbtc); g%cbpc = c_loc(cbpc); g%sc = c_loc(sc)
      g%grid_ld = size(vrc, 1, kind=c_long_long) * size(vrc, 2, kind=c_long_long)
      ! the analysis inputs are this call's outputs
      nl%Advr = c_loc(Advr); nl%Advt = c_loc(Advt); nl%Advp = c_loc(Advp)
      nl%VSr = c_loc(VSr); nl%VSt = c_loc(VSt); nl%VSp = c_loc(VSp)
      nl%VxBr = c_loc(VxBr); nl%VxBt = c_loc(VxBt); nl%VxBp = c_loc(VxBp); nl%heatTerms = c_loc(heatTerms)
      nl%grid_ld = size(Advr, 1, kind=c_long_long) * size(Advr, 2, kind=c_long_long)
      nl%AdvrLM = c_null_ptr; nl%AdvtLM = c_null_ptr; nl%AdvpLM = c_null_ptr
      nl%VSrLM = c_null_ptr; nl%VStLM = c_null_ptr; nl%VSpLM = c_null_ptr
      nl%VxBrLM = c_null_ptr; nl%VxBtLM = c_null_ptr; nl%VxBpLM = c_null_ptr; nl%heatTermsLM = c_null_ptr
      nl%spec_ld = 0
      nl%VXir = c_null_ptr; nl%VXit = c_null_ptr; nl%VXip = c_null_ptr
      nl%VXirLM = c_null_ptr; nl%VXitLM = c_null_ptr; nl%VXipLM = c_null_ptr
      call sht_check(c_get_nl(sht_handle(), int(size(vrc, 3), c_int), c_loc(or2), g, nl))
   end subroutine get_nl_gpu

   subroutine get_td_gpu(r, lcut, cor_fac, epsc, nbc, w, dw, z, AdvrLM, AdvtLM, AdvpLM, VStLM, VxBrLM, VxBtLM, &
              &          VxBpLM, dwdt, dzdt, dpdt, dsdt, dbdt, djdt, dVxBhLM)
      ! get_dwdt, get_dzdt, get_dpdt, get_dsdt and get_dbdt of every level
      ! (column) at once: Boussinesq, Coriolis force (cor_fac = CorFac),
      ! magnetic field and heat equation, no double-curl form.  nbc(nR) is the
      ! radial loop's nBc: at a level with nbc /= 0 only dVxBhLM is written.
      ! epsc(nR): internal heating added to dsdt at l = 0.  Device spectra.
      real(cp),       target, contiguous, intent(in) :: r(:), epsc(:)
      integer(c_int), target, contiguous, intent(in) :: lcut(:), nbc(:)
      real(cp), intent(in) :: cor_fac
      complex(cp), target, contiguous, intent(in) :: w(:,:), dw(:,:), z(:,:)
      complex(cp), target, contiguous, intent(in) :: AdvrLM(:,:), AdvtLM(:,:), AdvpLM(:,:), VStLM(:,:)
      complex(cp), target, contiguous, intent(in) :: VxBrLM(:,:), VxBtLM(:,:), VxBpLM(:,:)
      complex(cp), target, contiguous, intent(inout) :: dwdt(:,:), dzdt(:,:), dpdt(:,:), dsdt(:,:)
      complex(cp), target, contiguous, intent(inout) :: dbdt(:,:), djdt(:,:), dVxBhLM(:,:)
      type(magic_sht_td_args) :: a

      a%w = c_loc(w); a%dw = c_loc(dw); a%z = c_loc(z)
      a%AdvrLM = c_loc(AdvrLM); a%AdvtLM = c_loc(AdvtLM); a%AdvpLM = c_loc(AdvpLM); a%VStLM = c_loc(VStLM)
      a%VxBrLM = c_loc(VxBrLM); a%VxBtLM = c_loc(VxBtLM); a%VxBpLM = c_loc(VxBpLM)
      a%dwdt = c_loc(dwdt); a%dzdt = c_loc(dzdt); a%dpdt = c_loc(dpdt); a%dsdt = c_loc(dsdt)
      a%dbdt = c_loc(dbdt); a%djdt = c_loc(djdt); a%dVxBhLM = c_loc(dVxBhLM)
      a%spec_ld = size(w, 1, kind=c_long_long)
      call sht_check(c_get_td_nbc(sht_handle(), int(size(w, 2), c_int), c_loc(r), c_loc(lcut), &
           &                      real(cor_fac, c_double), c_loc(epsc), c_loc(nbc), a))
   end subroutine get_td_gpu

   subroutine inv_batch_gpu(n_levels, spec_ld, grid_ld, jobs, or2, lcut)
      ! synthesis jobs (MAGIC_SHT_JOB_SCAL_TO_SPAT .. _TORPOL_TO_DPHSPAT) over
      ! n_levels levels in one call: spectra spec_ld complex apart per level,
      ! grids grid_ld reals apart; or2(nR) for torpol_to_curl_spat jobs,
      ! lcut(nR) = l_R for all jobs.
      integer, intent(in) :: n_levels
      integer(c_long_long), intent(in) :: spec_ld, grid_ld
      type(magic_sht_job), intent(in) :: jobs(:)
      real(cp),       target, contiguous, optional, intent(in) :: or2(:)
      integer(c_int), target, contiguous, optional, intent(in) :: lcut(:)
      type(c_ptr) :: por2, plc

      por2 = c_null_ptr
      plc = c_null_ptr
      if ( present(or2) ) por2 = c_loc(or2)
      if ( present(lcut) ) plc = c_loc(lcut)
      call sht_check(c_inv_batch(sht_handle(), int(n_levels, c_int), por2, plc, spec_ld, grid_ld, jobs, &
           &                     int(size(jobs), c_int)))
   end subroutine inv_batch_gpu

   subroutine fwd_batch_gpu(n_levels, grid_ld, spec_ld, jobs, lcut)
      ! analysis jobs (MAGIC_SHT_JOB_SCAL_TO_SH, _SPAT_TO_QST,
      ! _SPAT_TO_SPHERTOR) over n_levels levels in one call.
      integer, intent(in) :: n_levels
      integer(c_long_long), intent(in) :: grid_ld, spec_ld
      type(magic_sht_job), intent(in) :: jobs(:)
      integer(c_int), target, contiguous, optional, intent(in) :: lcut(:)
      type(c_ptr) :: plc

      plc = c_null_ptr
      if ( present(lcut) ) plc = c_loc(lcut)
      call sht_check(c_fwd_batch(sht_handle(), int(n_levels, c_int), plc, grid_ld, spec_ld, jobs, &
           &                     int(size(jobs), c_int)))
   end subroutine fwd_batch_gpu

   subroutine dt_courant_gpu(dtrkc, dthkc, dt, dtMax, l_new_dt, dt_new)
      ! dt_courant without its log lines (host arrays of all levels)
      real(cp), intent(in) :: dtrkc(:), dthkc(:), dt, dtMax
      logical,  intent(out) :: l_new_dt
      real(cp), intent(out) :: dt_new
      integer(c_int) :: flag
      real(c_double) :: dnew
      call sht_check(c_dt_courant(int(size(dtrkc), c_int), dtrkc, dthkc, real(dt, c_double), &
           &                      real(dtMax, c_double), flag, dnew))
      l_new_dt = flag /= 0
      dt_new = dnew
   end subroutine dt_courant_gpu

   subroutine reserve_levels_gpu(n_levels)
      ! size the library's workspace and tensor-core data images for batches
      ! of n_levels levels ahead of the first call (and of graph capture)
      integer, intent(in) :: n_levels
      call sht_check(c_reserve(sht_handle(), int(n_levels, c_int)))
   end subroutine reserve_levels_gpu

   subroutine null_grid_args(a)
      type(magic_sht_grid_space_args), intent(out) :: a
      a%s = c_null_ptr; a%p = c_null_ptr; a%xi = c_null_ptr; a%w = c_null_ptr; a%dw = c_null_ptr
      a%ddw = c_null_ptr; a%z = c_null_ptr; a%dz = c_null_ptr; a%b = c_null_ptr; a%db = c_null_ptr
      a%ddb = c_null_ptr; a%aj = c_null_ptr; a%dj = c_null_ptr
      a%sc = c_null_ptr; a%pc = c_null_ptr; a%xic = c_null_ptr; a%vrc = c_null_ptr; a%vtc = c_null_ptr
      a%vpc = c_null_ptr; a%cvrc = c_null_ptr; a%cvtc = c_null_ptr; a%cvpc = c_null_ptr
      a%brc = c_null_ptr; a%btc = c_null_ptr; a%bpc = c_null_ptr; a%cbrc = c_null_ptr
      a%cbtc = c_null_ptr; a%cbpc = c_null_ptr
      a%dvrdrc = c_null_ptr; a%dvtdrc = c_null_ptr; a%dvpdrc = c_null_ptr; a%dvrdtc = c_null_ptr
      a%dvrdpc = c_null_ptr; a%dvtdpc = c_null_ptr; a%dvpdpc = c_null_ptr
      a%spec_ld = 0; a%grid_ld = 0
   end subroutine null_grid_args

end module sht_gpu_batched
