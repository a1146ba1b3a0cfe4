!#######################################################################
! adcgpu_iface: ISO_C_BINDING interface to libadcgpu.so (include/adcgpu.h)
! and drop-in wrappers for the ADC(2)-s hot path of ADC_ottawa.
!
! The wrappers keep the reference's argument lists and read the same
! module globals (parameters.f90), so the calling routines change only the name
! they call:
!
!   write_fspace_adc2_1  -> write_fspace_adc2_1_gpu   (fspacetrial.f90:533)
!   davdiag_block        -> davdiag_block_gpu         (block_davidson.f90:33)
!   davdir_block         -> davdir_block_gpu          (dmatvec_davidson.f90:41)
!   lancdiag_block       -> lancdiag_block_gpu        (block_lanczos.f90:28)
!   propagate_fvec       -> propagate_fvec_gpu        (fvecprop.f90:27)
!   chebyshev_auto_order_domain
!                        -> chebyshev_auto_order_domain_gpu (chebyspec.f90:25)
!   write_fspace_adc2_1_cvs
!                        -> write_fspace_adc2_1_cvs_gpu (fspacetrial.f90:566)
!   get_modifiedtm_adc2  -> get_modifiedtm_adc2_gpu   (get_moment.f90:153)
!   fill_stvc            -> fill_stvc_gpu             (fspacetrial.f90:1255)
!   hxvec_incore         -> hxvec_gpu                 (block_davidson.f90:844)
!
! A non-zero status from the library is turned into errmsg +
! error_control, as the reference does for its own failures.
!#######################################################################
module adcgpu_iface

  use iso_c_binding
  implicit none

  type, bind(C) :: adcgpu_dav_params
     integer(c_int) :: davstates, dmain, maxsubdim, maxiter, precon, ldfl, &
                       lsubdiag, guessdim
     real(c_double) :: davtol
     integer(c_int) :: precision, refine
     real(c_double) :: tol_bf16, tol_fp32
     integer(c_int) :: refine_block
  end type adcgpu_dav_params

  type, bind(C) :: adcgpu_dav_info
     integer(c_int)     :: iterations
     integer(c_int64_t) :: nmult
     integer(c_int)     :: nconv
     real(c_double)     :: seconds, sigma_seconds, max_residual
     integer(c_int)     :: iters_bf16, iters_fp32, iters_fp64
     integer(c_int64_t) :: nmult_reference
  end type adcgpu_dav_info

  interface
     integer(c_int) function adcgpu_ctx_create(device, ctx) bind(C, name="adcgpu_ctx_create")
       import :: c_int, c_ptr
       integer(c_int), value :: device
       type(c_ptr)           :: ctx
     end function adcgpu_ctx_create

     integer(c_int) function adcgpu_ctx_destroy(ctx) bind(C, name="adcgpu_ctx_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function adcgpu_ctx_destroy

     integer(c_int) function adcgpu_set_orbitals(ctx, nocc, nvirt, e) bind(C, name="adcgpu_set_orbitals")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: nocc, nvirt
       real(c_double)        :: e(*)
     end function adcgpu_set_orbitals

     integer(c_int) function adcgpu_set_eri_mo_complex(ctx, buf) bind(C, name="adcgpu_set_eri_mo_complex")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       type(c_ptr), value :: buf      ! c_loc(moIntegrals%buffer_real)
     end function adcgpu_set_eri_mo_complex

     integer(c_int) function adcgpu_build_adc2s(ctx, ndim, kpq, noffd, flag, precision) &
          bind(C, name="adcgpu_build_adc2s")
       import :: c_int, c_ptr, c_int32_t, c_int64_t, c_char
       type(c_ptr), value          :: ctx
       integer(c_int), value       :: ndim, precision
       integer(c_int32_t)          :: kpq(*)
       integer(c_int64_t)          :: noffd
       character(kind=c_char), value :: flag
     end function adcgpu_build_adc2s

     integer(c_int) function adcgpu_write_hmlt_files(ctx, dir, flag) bind(C, name="adcgpu_write_hmlt_files")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value            :: ctx
       character(kind=c_char)        :: dir(*)
       character(kind=c_char), value :: flag
     end function adcgpu_write_hmlt_files

     integer(c_int) function adcgpu_davidson(ctx, p, evals, evecs, info) bind(C, name="adcgpu_davidson")
       import :: c_int, c_ptr, c_double, adcgpu_dav_params, adcgpu_dav_info
       type(c_ptr), value      :: ctx
       type(adcgpu_dav_params) :: p
       real(c_double)          :: evals(*), evecs(*)
       type(adcgpu_dav_info)   :: info
     end function adcgpu_davidson

     integer(c_int) function adcgpu_write_davidson_file(path, ndim, nstates, evals, evecs) &
          bind(C, name="adcgpu_write_davidson_file")
       import :: c_int, c_double, c_char
       character(kind=c_char)   :: path(*)
       integer(c_int), value    :: ndim, nstates
       real(c_double)           :: evals(*), evecs(*)
     end function adcgpu_write_davidson_file

     integer(c_int) function adcgpu_block_lanczos(ctx, lmain, ncycles, orthotype, q0, tmat, evals, ritz) &
          bind(C, name="adcgpu_block_lanczos")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: lmain, ncycles, orthotype
       real(c_double)        :: q0(*)
       type(c_ptr), value    :: tmat, evals, ritz
     end function adcgpu_block_lanczos

     integer(c_int) function adcgpu_autocorr(ctx, nwp, f, tout, tfinal, kdim, tol, auto, ntimes, nmult) &
          bind(C, name="adcgpu_autocorr")
       import :: c_int, c_ptr, c_double, c_int64_t
       type(c_ptr), value    :: ctx
       integer(c_int), value :: nwp, kdim
       real(c_double)        :: f(*)
       real(c_double), value :: tout, tfinal, tol
       complex(c_double)     :: auto(*)
       integer(c_int)        :: ntimes
       integer(c_int64_t)    :: nmult
     end function adcgpu_autocorr

     integer(c_int) function adcgpu_spectral_bounds(ctx, p, bounds) bind(C, name="adcgpu_spectral_bounds")
       import :: c_int, c_ptr, c_double, adcgpu_dav_params
       type(c_ptr), value      :: ctx
       type(adcgpu_dav_params) :: p
       real(c_double)          :: bounds(2)
     end function adcgpu_spectral_bounds

     integer(c_int) function adcgpu_chebyshev_auto(ctx, nvec, q0, bounds, chebyord, df, auto, q1h1p, order) &
          bind(C, name="adcgpu_chebyshev_auto")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: nvec, chebyord, df
       real(c_double)        :: q0(*), bounds(2), auto(*)
       type(c_ptr), value    :: q1h1p
       integer(c_int)        :: order
     end function adcgpu_chebyshev_auto

     integer(c_int) function adcgpu_chebyshev_project(ctx, nvec, q0, bounds, chebyord, projen, df) &
          bind(C, name="adcgpu_chebyshev_project")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: nvec, chebyord, df
       real(c_double)        :: q0(*), bounds(2)
       real(c_double), value :: projen
     end function adcgpu_chebyshev_project

     integer(c_int) function adcgpu_set_fp64_arith(ctx, mode) bind(C, name="adcgpu_set_fp64_arith")
       import :: c_int, c_ptr
       type(c_ptr), value    :: ctx
       integer(c_int), value :: mode
     end function adcgpu_set_fp64_arith

     integer(c_int) function adcgpu_build_adc2s_cvs(ctx, ndim, kpq, ncore, core, noffd, flag) &
          bind(C, name="adcgpu_build_adc2s_cvs")
       import :: c_int, c_ptr, c_int32_t, c_int64_t, c_char
       type(c_ptr), value            :: ctx
       integer(c_int), value         :: ndim, ncore
       integer(c_int32_t)            :: kpq(*), core(*)
       integer(c_int64_t)            :: noffd
       character(kind=c_char), value :: flag
     end function adcgpu_build_adc2s_cvs

     integer(c_int) function adcgpu_set_dipole(ctx, dpl) bind(C, name="adcgpu_set_dipole")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double)     :: dpl(*)
     end function adcgpu_set_dipole

     integer(c_int) function adcgpu_modified_tm_adc2(ctx, ndim, kpq, mtm) bind(C, name="adcgpu_modified_tm_adc2")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: ndim
       integer(c_int32_t)    :: kpq(*)
       real(c_double)        :: mtm(*)
     end function adcgpu_modified_tm_adc2

     integer(c_int) function adcgpu_fill_stvc(ndim, vctr, lmain, stvc_lbl) bind(C, name="adcgpu_fill_stvc")
       import :: c_int, c_int32_t, c_double
       integer(c_int), value :: ndim, lmain
       real(c_double)        :: vctr(*)
       integer(c_int32_t)    :: stvc_lbl(*)
     end function adcgpu_fill_stvc

     integer(c_int) function adcgpu_sigma(ctx, m, v, w) bind(C, name="adcgpu_sigma")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value    :: ctx
       integer(c_int), value :: m
       real(c_double)        :: v(*), w(*)
     end function adcgpu_sigma

     type(c_ptr) function adcgpu_last_error(ctx) bind(C, name="adcgpu_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function adcgpu_last_error
  end interface

  type(c_ptr), save :: gpu_ctx = c_null_ptr

contains

!#######################################################################

  subroutine adcgpu_check(st, where)
    use iomod, only: error_control, errmsg
    integer(c_int), intent(in)   :: st
    character(len=*), intent(in) :: where
    if (st.ne.0) then
       write(errmsg,'(a,a,i3)') trim(where),': libadcgpu status ',st
       call error_control
    endif
  end subroutine adcgpu_check

!#######################################################################
! Creates the context and uploads the orbital energies and the MO ERIs
! (moIntegrals%buffer_real, read through vpqrs in the reference).

  subroutine adcgpu_init
    use parameters, only: e, nocc, nvirt, moIntegrals
    integer(c_int) :: st
    if (c_associated(gpu_ctx)) return
    st = adcgpu_ctx_create(0_c_int, gpu_ctx)
    call adcgpu_check(st, 'adcgpu_ctx_create')
    st = adcgpu_set_orbitals(gpu_ctx, int(nocc,c_int), int(nvirt,c_int), e)
    call adcgpu_check(st, 'adcgpu_set_orbitals')
    st = adcgpu_set_eri_mo_complex(gpu_ctx, c_loc(moIntegrals%buffer_real))
    call adcgpu_check(st, 'adcgpu_set_eri_mo_complex')
  end subroutine adcgpu_init

!#######################################################################
! write_fspace_adc2_1 (fspacetrial.f90:533-564): the matrix stays on the
! device; the SCRATCH files are also written so that unmodified consumers
! of hmlt.dia/hmlt.off keep working.

  subroutine write_fspace_adc2_1_gpu(ndim, kpq, noffdel, chr)
    use parameters, only: nbas, nocc
    integer, intent(in)                                 :: ndim
    integer, dimension(7,0:nBas**2*nOcc**2), intent(in) :: kpq
    integer*8, intent(out)                              :: noffdel
    character(1), intent(in)                            :: chr
    integer(c_int)     :: st
    integer(c_int64_t) :: n
    call adcgpu_init
    st = adcgpu_build_adc2s(gpu_ctx, int(ndim,c_int), kpq, n, chr, 0_c_int)
    call adcgpu_check(st, 'write_fspace_adc2_1')
    noffdel = n
    st = adcgpu_write_hmlt_files(gpu_ctx, 'SCRATCH'//c_null_char, chr)
    call adcgpu_check(st, 'write_hmlt_files')
  end subroutine write_fspace_adc2_1_gpu

!#######################################################################
! The matvec (direct) path: get_interm_adc2_save (get_matrix.f90:625-701)
! and davdir_block (dmatvec_davidson.f90:41-149).  The ph-ph block and the
! diagonal are built from Ca1/Cb1/Cc1/Cc2 and kept on the device; the
! coupling block is recomputed from the integrals in every sigma product,
! as get_matvec_adc2s_omp (:1031-1230) does, so nothing is written to
! SCRATCH.  The Davidson settings are those of davdiag_block_gpu.

  subroutine davdir_block_gpu(matdim, kpq)
    use parameters, only: nbas, nocc, hamflag
    integer, intent(in)                                 :: matdim
    integer, dimension(7,0:nBas**2*nOcc**2), intent(in) :: kpq
    integer(c_int)     :: st
    integer(c_int64_t) :: n
    integer*8          :: noffd
    call adcgpu_init
    st = adcgpu_build_adc2s(gpu_ctx, int(matdim,c_int), kpq, n, hamflag, 2_c_int)
    call adcgpu_check(st, 'get_interm_adc2_save')
    noffd = n
    call davdiag_block_gpu(matdim, noffd)
  end subroutine davdir_block_gpu

!#######################################################################
! davdiag_block (block_davidson.f90:33-145), initial space ('i') or final
! space ('f') parameters as selected by hamflag.

  subroutine davdiag_block_gpu(matdim, noffd)
    use parameters
    integer, intent(in)   :: matdim
    integer*8, intent(in) :: noffd
    type(adcgpu_dav_params) :: p
    type(adcgpu_dav_info)   :: info
    real(dp), allocatable   :: ev(:), vec(:,:)
    integer(c_int)          :: st
    if (hamflag.eq.'i') then
       p%davstates=davstates; p%dmain=dmain; p%maxsubdim=maxsubdim; p%maxiter=maxiter
       p%precon=precon; p%ldfl=merge(1,0,ldfl); p%lsubdiag=merge(1,0,lsubdiag)
       if (ladc1guess) p%lsubdiag=2     ! initvec_adc1 ahead of initvec_subdiag (:107-117)
       p%guessdim=guessdim; p%davtol=davtol
    else
       p%davstates=davstates_f; p%dmain=dmain_f; p%maxsubdim=maxsubdim_f; p%maxiter=maxiter_f
       p%precon=precon_f; p%ldfl=merge(1,0,ldfl_f); p%lsubdiag=merge(1,0,lsubdiag_f)
       if (ladc1guess_f) p%lsubdiag=2
       p%guessdim=guessdim_f; p%davtol=davtol_f
    endif
    p%precision=0; p%refine=0; p%tol_bf16=0.0_dp; p%tol_fp32=0.0_dp
    allocate(ev(p%davstates), vec(matdim,p%davstates))
    st = adcgpu_davidson(gpu_ctx, p, ev, vec, info)
    call adcgpu_check(st, 'davdiag_block')
    if (hamflag.eq.'i') then
       st = adcgpu_write_davidson_file(trim(davname)//c_null_char, int(matdim,c_int), p%davstates, ev, vec)
    else
       st = adcgpu_write_davidson_file(trim(davname_f)//c_null_char, int(matdim,c_int), p%davstates, ev, vec)
    endif
    call adcgpu_check(st, 'wreigenpairs')
    deallocate(ev, vec)
  end subroutine davdiag_block_gpu

!#######################################################################
! lancdiag_block (block_lanczos.f90:28-81) from a random start block
! (init_vecs_random, lancguess = 7).  The pseudospectrum is returned in
! lanc_evals (lancstates = lmain*ncycles, :1234).

  subroutine lancdiag_block_gpu(dimf, noff, flag, lanc_evals)
    use parameters
    integer, intent(in)     :: dimf
    integer*8, intent(in)   :: noff
    character(1),intent(in) :: flag
    real(dp), dimension(:), allocatable, intent(out) :: lanc_evals
    real(dp), allocatable, target :: q0(:,:), ev(:)
    integer(c_int) :: st
    allocate(q0(dimf,lmain), ev(lmain*ncycles))
    call random_number(q0)
    st = adcgpu_block_lanczos(gpu_ctx, int(lmain,c_int), int(ncycles,c_int), int(orthotype,c_int), q0, &
         c_null_ptr, c_loc(ev), c_null_ptr)
    call adcgpu_check(st, 'lancdiag_block')
    lancstates = lmain*ncycles
    call move_alloc(ev, lanc_evals)
    deallocate(q0)
  end subroutine lancdiag_block_gpu

!#######################################################################
! propagate_fvec (fvecprop.f90:27-105) for autoord = 0: the zeroth-order
! autocorrelation a(t) for t = 0, tout, ..., written by the caller.

  subroutine propagate_fvec_gpu(fvec, ndimf, auto, ntimes)
    use parameters
    integer, intent(in)                       :: ndimf
    real(dp), dimension(ndimf), intent(in)    :: fvec
    complex(dp), dimension(:), intent(out)    :: auto
    integer, intent(out)                      :: ntimes
    integer(c_int)     :: st, nt
    integer(c_int64_t) :: nm
    st = adcgpu_autocorr(gpu_ctx, 1_c_int, fvec, tout, tfinal, int(kdim,c_int), autotol, auto, nt, nm)
    call adcgpu_check(st, 'propagate_fvec')
    ntimes = nt
  end subroutine propagate_fvec_gpu

!#######################################################################
! chebyshev_auto_order_domain (chebyspec.f90:25-116): the 'davlanc'
! spectral bounds (specbounds.f90:121-205) widened to [0.9 Ea, 1.1 Eb],
! the optional energy-window projection of q0 (lprojpsi0, projen), the
! order-domain autocorrelation C_0..C_2*chebyord, and the files chebyauto
! and (save1h1p) cheby1h1p in the layouts of write_chebyshev_auto and
! write_1h1p (:334-394).  ndimsf is the 1h1p dimension, nocc*nvirt here.

  subroutine chebyshev_auto_order_domain_gpu(q0, ndimf, noffdf, ndimsf)
    use parameters
    use iomod, only: freeunit
    integer, intent(in)                       :: ndimf, ndimsf
    integer*8, intent(in)                     :: noffdf
    real(dp), dimension(ndimf), intent(inout) :: q0
    type(adcgpu_dav_params)               :: p
    real(dp)                              :: bounds(2)
    real(dp), allocatable                 :: auto(:)
    real(dp), allocatable, target         :: q1h1p(:,:)
    integer(c_int)                        :: st, ord
    integer                               :: unit, k
    p%davstates=1; p%dmain=5; p%maxsubdim=20; p%maxiter=maxiter_f
    p%precon=precon_f; p%ldfl=merge(1,0,ldfl_f); p%lsubdiag=1
    p%guessdim=guessdim_f; p%davtol=1e-8_dp
    p%precision=0; p%refine=0; p%tol_bf16=0.0_dp; p%tol_fp32=0.0_dp; p%refine_block=0
    st = adcgpu_spectral_bounds(gpu_ctx, p, bounds)
    call adcgpu_check(st, 'spectral_bounds')
    bounds(1)=0.9d0*bounds(1)
    bounds(2)=1.1d0*bounds(2)
    if (mod(chebyord,2).ne.0) chebyord=chebyord-1
    if (lprojpsi0) then
       st = adcgpu_chebyshev_project(gpu_ctx, 1_c_int, q0, bounds, int(chebyord,c_int), projen, 0_c_int)
       call adcgpu_check(st, 'project_psi0')
    endif
    allocate(auto(0:2*chebyord))
    if (save1h1p) then
       allocate(q1h1p(ndimsf,0:chebyord))
       st = adcgpu_chebyshev_auto(gpu_ctx, 1_c_int, q0, bounds, int(chebyord,c_int), 0_c_int, auto, &
            c_loc(q1h1p), ord)
    else
       st = adcgpu_chebyshev_auto(gpu_ctx, 1_c_int, q0, bounds, int(chebyord,c_int), 0_c_int, auto, &
            c_null_ptr, ord)
    endif
    call adcgpu_check(st, 'chebyshev_auto')
    call freeunit(unit)
    open(unit,file='chebyauto',form='formatted',status='unknown')
    write(unit,'(a,2(2x,E21.14),/)') '#    Spectral bounds:',bounds(1),bounds(2)
    write(unit,'(a)') '#    Order [k]    C_k'
    do k=0,chebyord*2
       write(unit,'(i6,11x,E21.14)') k,auto(k)
    enddo
    close(unit)
    if (save1h1p) then
       call freeunit(unit)
       open(unit=unit,file='cheby1h1p',status='unknown',access='sequential',form='unformatted')
       do k=0,chebyord
          write(unit) q1h1p(:,k)
       enddo
       close(unit)
       deallocate(q1h1p)
    endif
    deallocate(auto)
  end subroutine chebyshev_auto_order_domain_gpu

!#######################################################################
! write_fspace_adc2_1_cvs (fspacetrial.f90:566-596): the CVS matrix of the
! core-hole list icore(1:ncore) (parameters.f90), kept on the device, with
! the SCRATCH files as for write_fspace_adc2_1_gpu.  The library checks that
! kpq is the list select_atom_is_cvs / select_atom_d_cvs produce.

  subroutine write_fspace_adc2_1_cvs_gpu(ndim, kpq, noffdel, chr)
    use parameters, only: nbas, nocc, icore, ncore
    integer, intent(in)                                 :: ndim
    integer, dimension(7,0:nBas**2*nOcc**2), intent(in) :: kpq
    integer*8, intent(out)                              :: noffdel
    character(1), intent(in)                            :: chr
    integer(c_int)     :: st
    integer(c_int64_t) :: n
    call adcgpu_init
    st = adcgpu_build_adc2s_cvs(gpu_ctx, int(ndim,c_int), kpq, int(ncore,c_int), icore, n, chr)
    call adcgpu_check(st, 'write_fspace_adc2_1_cvs')
    noffdel = n
    st = adcgpu_write_hmlt_files(gpu_ctx, 'SCRATCH'//c_null_char, chr)
    call adcgpu_check(st, 'write_hmlt_files')
  end subroutine write_fspace_adc2_1_cvs_gpu

!#######################################################################
! get_modifiedtm_adc2 (get_moment.f90:153-442): the f-vector of the dipole
! component held in dpl (parameters.f90, as the reference's caller sets it),
! for an ADC(2)-s or CVS kpq.  ista is accepted for the reference's
! argument list; the f-vector is that of the ground state, as there.

  subroutine get_modifiedtm_adc2_gpu(ndim, kpq, mtm, ista)
    use parameters, only: dp, dpl
    integer, intent(in)                      :: ndim, ista
    integer, dimension(7,0:*), intent(in)    :: kpq
    real(dp), dimension(ndim), intent(out)   :: mtm
    integer(c_int) :: st
    call adcgpu_init
    st = adcgpu_set_dipole(gpu_ctx, dpl)
    call adcgpu_check(st, 'set_dipole')
    st = adcgpu_modified_tm_adc2(gpu_ctx, int(ndim,c_int), kpq, mtm)
    call adcgpu_check(st, 'get_modifiedtm_adc2')
  end subroutine get_modifiedtm_adc2_gpu

!#######################################################################
! fill_stvc (fspacetrial.f90:1255-1270): stvc_lbl(1:lmain) = the indices of
! the lmain largest vctr(i)**2 in the order of dsortindxa1('D').

  subroutine fill_stvc_gpu(ndim, vctr)
    use parameters, only: dp, lmain, stvc_lbl
    integer, intent(in)                  :: ndim
    real(dp), dimension(ndim), intent(in) :: vctr
    integer(c_int) :: st
    st = adcgpu_fill_stvc(int(ndim,c_int), vctr, int(lmain,c_int), stvc_lbl)
    call adcgpu_check(st, 'fill_stvc')
  end subroutine fill_stvc_gpu

!#######################################################################
! hxvec_incore (block_davidson.f90:844-883): W = H V for m columns of the
! matrix the context holds (host arrays, ndim x m).

  subroutine hxvec_gpu(ndim, m, v, w)
    use parameters, only: dp
    integer, intent(in)                     :: ndim, m
    real(dp), dimension(ndim,m), intent(in)  :: v
    real(dp), dimension(ndim,m), intent(out) :: w
    integer(c_int) :: st
    st = adcgpu_sigma(gpu_ctx, int(m,c_int), v, w)
    call adcgpu_check(st, 'hxvec_incore')
  end subroutine hxvec_gpu

end module adcgpu_iface
