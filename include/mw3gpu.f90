! iso_c_binding interface to libmw3gpu (include/mw3gpu.h) for the Fortran
! host of madwave3: the derived types mirror the C structs field by field
! (pointer members as type(c_ptr), filled with c_loc of the host arrays) and
! every entry point is an interface with the C signature.  Status codes are
! integer(c_int), 0 = success; mw3_check turns a non-zero status into the
! reference's convention (write(6,*) the message, then stop).
!
! Array arguments pass Fortran arrays unchanged: VVV(npuntot,nangu,nelec,nelec)
! is the C vvv[nelec][nelec][nangu][npuntot], Djmmp(nangu,0:nangu2,nelec,0:Jtot)
! the C djmmp[Jtot+1][nelec][nangu2+1][nangu], and so on (include/mw3gpu.h
! gives each layout).
module mw3gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: MW3_OK = 0, MW3_ERR_ARG = 1, MW3_ERR_CUDA = 2, &
       MW3_ERR_UNSUPPORTED = 3, MW3_ERR_STATE = 4, MW3_ERR_NOMEM = 5, MW3_ERR_NUMERIC = 6
  integer(c_int32_t), parameter :: MW3_PREC_FP64 = 0, MW3_PREC_MIXED = 1

  type, bind(c) :: mw3_grid
     integer(c_int32_t) :: npun1, npun2, nangu, nelec
     integer(c_int32_t) :: npun1min, npuntot
     real(c_double) :: rmis1, rfin1, rmis2, rfin2
     real(c_double) :: hbr
     real(c_double) :: xm1red, xm2red
     real(c_double) :: radcutmax, rotcutmax
     real(c_double) :: emindlt, delta2
     integer(c_int32_t) :: precision
  end type mw3_grid

  type, bind(c) :: mw3_wave
     integer(c_int32_t) :: Jtot, iparity, inc, j0, iommin, iommax
     integer(c_int32_t) :: ncan
     type(c_ptr) :: iombas, nelebas
     type(c_ptr) :: nojbas, j00
     type(c_ptr) :: jbas
     type(c_ptr) :: iomdiat, iomatom
     type(c_ptr) :: sigdiat, sigatom
     integer(c_int32_t) :: nangu2
     type(c_ptr) :: djmmp
     integer(c_int32_t) :: proj_j2_up
     real(c_double) :: absr1, absalp1, absr2, absalp2
     integer(c_int32_t) :: n1expo, ninterv1, n2expo, ninterv2
     real(c_double) :: r1flux_ang, ekinmin, ekinmax
     integer(c_int32_t) :: netot, kminelastic, iphoto, iprod
     integer(c_int32_t) :: nvini, nvmax, jini, jmax, nvref, jref, iomref, ielecref
     type(c_ptr) :: nobc
     type(c_ptr) :: ediat
     type(c_ptr) :: fd
     real(c_double) :: xm1reac, xm2reac
     real(c_double) :: rcolini, alpha0, xk0, factor0, xmasa0
     integer(c_int32_t) :: il0
     integer(c_int32_t) :: nofe
     type(c_ptr) :: efe
  end type mw3_wave

  type, bind(c) :: mw3_prodproj
     integer(c_int32_t) :: n2prod0, n2prod1, nangproj0, nangproj1
     integer(c_int32_t) :: iomminprod, iommaxprod, jiniprod, jmaxprod
     integer(c_int32_t) :: nviniprod, nvmaxprod
     type(c_ptr) :: nobcprod, transrgjac, dtrans, prodwf
  end type mw3_prodproj

  interface
     integer(c_int) function mw3_create(ctx, grid, npunreal, indr1, indr2, vvv) bind(c)
       import
       type(c_ptr) :: ctx
       type(mw3_grid), intent(in) :: grid
       integer(c_int32_t), intent(in) :: npunreal(*), indr1(*), indr2(*)
       real(c_double), intent(in) :: vvv(*)
     end function
     integer(c_int) function mw3_add_wave(ctx, wave, wave_id) bind(c)
       import
       type(c_ptr), value :: ctx
       type(mw3_wave), intent(in) :: wave
       integer(c_int32_t) :: wave_id
     end function
     integer(c_int) function mw3_wave_size(ctx, wave_id, ntot) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       integer(c_int64_t) :: ntot
     end function
     integer(c_int) function mw3_hphi(ctx, wave_id, psi, hpsi) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double), intent(in) :: psi(*)
       real(c_double) :: hpsi(*)
     end function
     integer(c_int) function mw3_start(ctx, psi0s) bind(c)
       import
       type(c_ptr), value :: ctx
       type(c_ptr), intent(in) :: psi0s(*)
     end function
     integer(c_int) function mw3_upload_state(ctx, wave_id, psi_km1, psi_k, it) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double), intent(in) :: psi_km1(*), psi_k(*)
       integer(c_int64_t), value :: it
     end function
     integer(c_int) function mw3_run(ctx, n_iter) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: n_iter
     end function
     integer(c_int) function mw3_sync(ctx) bind(c)
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function mw3_download_state(ctx, wave_id, psi_km1, psi_k, it) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double) :: psi_km1(*), psi_k(*)
       integer(c_int64_t) :: it
     end function
     integer(c_int) function mw3_norms(ctx, wave_id, norms, n) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double) :: norms(*)
       integer(c_int64_t) :: n
     end function
     integer(c_int) function mw3_autocorrelation(ctx, wave_id, autos, n) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double) :: autos(*)
       integer(c_int64_t) :: n
     end function
     integer(c_int) function mw3_totalflux(ctx, wave_id, s2prodtot, s2prodelec) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double) :: s2prodtot(*), s2prodelec(*)
     end function
     integer(c_int) function mw3_flux_count(ctx, wave_id, nflux) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       integer(c_int32_t) :: nflux
     end function
     integer(c_int) function mw3_download_accumulators(ctx, wave_id, zcr, zcdr, zs2, cvj, zfe) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       complex(c_double_complex) :: zcr(*), zcdr(*), zs2(*)
       real(c_double) :: cvj(*)
       type(c_ptr), value :: zfe
     end function
     integer(c_int) function mw3_upload_accumulators(ctx, wave_id, zcr, zcdr, zs2) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       complex(c_double_complex), intent(in) :: zcr(*), zcdr(*), zs2(*)
     end function
     integer(c_int) function mw3_cvj_history(ctx, capacity) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int64_t), value :: capacity
     end function
     integer(c_int) function mw3_download_cvj_history(ctx, wave_id, n, cvj, cvjprod, it_last) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       integer(c_int64_t), value :: n
       type(c_ptr), value :: cvj, cvjprod
       integer(c_int64_t) :: it_last
     end function
     integer(c_int) function mw3_set_flux_gate(ctx, wave_id, on) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id, on
     end function
     integer(c_int) function mw3_set_ecoriolis(ctx, wave_id, on) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id, on
     end function
     integer(c_int) function mw3_set_choices(ctx, choice) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(in) :: choice(4)
     end function
     integer(c_int) function mw3_get_choices(ctx, choice) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: choice(4)
     end function
     integer(c_int) function mw3_autotune(ctx, iterations, scope, choice, ms_best) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: iterations, scope
       integer(c_int32_t), intent(out) :: choice(4)
       real(c_double), intent(out) :: ms_best
     end function
     integer(c_int) function mw3_packet_energy_norm(ctx, wave_id, apaqini) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       real(c_double) :: apaqini(*)
     end function
     integer(c_int) function mw3_set_product_projection(ctx, wave_id, proj) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       type(mw3_prodproj), intent(in) :: proj
     end function
     integer(c_int) function mw3_download_product(ctx, wave_id, zs2prod, cvjprod) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       complex(c_double_complex) :: zs2prod(*)
       real(c_double) :: cvjprod(*)
     end function
     integer(c_int) function mw3_upload_product(ctx, wave_id, zs2prod) bind(c)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: wave_id
       complex(c_double_complex), intent(in) :: zs2prod(*)
     end function
     type(c_ptr) function mw3_last_error(ctx) bind(c)
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function mw3_destroy(ctx) bind(c)
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_size_t) function c_strlen(s) bind(c, name="strlen")
       import
       type(c_ptr), value :: s
     end function
  end interface

contains

  ! a non-zero status ends the run the way the reference does on bad input
  subroutine mw3_check(ctx, rc)
    type(c_ptr), intent(in) :: ctx
    integer(c_int), intent(in) :: rc
    character(kind=c_char), pointer :: msg(:)
    character(len=:), allocatable :: text
    type(c_ptr) :: p
    integer :: n, i
    if (rc == MW3_OK) return
    p = mw3_last_error(ctx)
    n = int(c_strlen(p))
    call c_f_pointer(p, msg, [n])
    allocate(character(len=n) :: text)
    do i = 1, n
       text(i:i) = msg(i)
    end do
    write(6,*) ' libmw3gpu error ', rc, ': ', text
    call flush(6)
    stop
  end subroutine mw3_check

end module mw3gpu
