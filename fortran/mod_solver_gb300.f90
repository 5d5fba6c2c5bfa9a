!
! mod_solver_gb300 -- the GB300 pressure-projection path for the FluTAS apps.
!
! Every public routine keeps the name-free argument list of the FluTAS routine
! it replaces, so an app swaps modules with one `use` line per routine:
!
!   use mod_solver_gb300, only: initsolver => gb300_initsolver, solver_cpu => gb300_solver_cpu, &
!                               solver_gpu => gb300_solver_gpu, fillps => gb300_fillps,         &
!                               correc => gb300_correc, boundp => gb300_boundp,                 &
!                               bounduvw => gb300_bounduvw, updt_rhs_b => gb300_updt_rhs_b,     &
!                               chkdiv => gb300_chkdiv, pres_tw_src => gb300_pres_tw_src,       &
!                               fftend => gb300_fftend, initgrid => gb300_initgrid,             &
!                               rk => gb300_rk, cmpt_time_factors => gb300_cmpt_time_factors
!
! (gb300_rk follows the app's build: the two-phase right-hand sides with _USE_VOF,
! momad_xyz_sp with mu_sp/rho_sp of mod_param otherwise; the file is preprocessed
! like the reference's own sources.)
!
! Each wrapper calls the C ABI of libflutas_gb300.so (include/flutas_gb300.h)
! through iso_c_binding and hands a non-zero status to the app's usual abort
! path, flutas_error (src/sanity.f90:332-353), with the library's message.
!
! Arrays may be host arrays (copied to the device and back inside each call),
! or device / managed arrays (`!@cuf attributes(managed)`, as the reference's
! GPU build declares them, or `!$acc host_data use_device(...)`): those are
! used in place.  Array dummies are declared `contiguous` so the compiler
! passes the caller's array itself, without a copy-in/copy-out temporary.
!
! Requires rp == c_double (FluTAS built without _SINGLE_PRECISION) and the
! default integer kind == c_int.
!
module mod_solver_gb300
  use, intrinsic :: iso_c_binding
  use mod_types, only: rp
  use mod_sanity, only: flutas_error
  implicit none
  private
  public :: gb300_initsolver, gb300_solver_cpu, gb300_solver_gpu, gb300_fillps, gb300_correc, &
            gb300_boundp, gb300_bounduvw, gb300_updt_rhs_b, gb300_chkdiv, gb300_pres_tw_src, &
            gb300_fftend, gb300_update_property, gb300_load, gb300_chkdiv_noalloc, gb300_initgrid, &
            gb300_rk, gb300_cmpt_time_factors
  !
  interface
    ! src/initsolver.f90:21
    integer(c_int) function c_initsolver(n, dli, nh_d, dzci, dzfi, cbc, bc, c_or_f, lambdaxy, a, b, c, &
                                         arrplan, normfft, rhsbx, rhsby, rhsbz) &
                   bind(C, name='flutas_gb300_initsolver')
      import
      integer(c_int), intent(in) :: n(3)
      real(c_double), intent(in) :: dli(3)
      integer(c_int), value      :: nh_d
      real(c_double), intent(in) :: dzci(*), dzfi(*)
      character(kind=c_char), intent(in) :: cbc(6)
      real(c_double), intent(in) :: bc(6)
      character(kind=c_char), intent(in) :: c_or_f(3)
      real(c_double) :: lambdaxy(*), a(*), b(*), c(*)
      type(c_ptr)    :: arrplan(4)
      real(c_double) :: normfft
      real(c_double) :: rhsbx(*), rhsby(*), rhsbz(*)
    end function
    ! src/solver_cpu.f90:20 and src/solver_gpu.f90:31
    integer(c_int) function c_solver(n, arrplan, normfft, lambdaxy, a, b, c, bcz, c_or_f, p) &
                   bind(C, name='flutas_gb300_solver')
      import
      integer(c_int), intent(in) :: n(3)
      type(c_ptr), intent(in)    :: arrplan(4)
      real(c_double), value      :: normfft
      real(c_double), intent(in) :: lambdaxy(*), a(*), b(*), c(*)
      character(kind=c_char), intent(in) :: bcz(2), c_or_f(3)
      real(c_double) :: p(*)
    end function
    ! src/fillps.f90:16
    integer(c_int) function c_fillps(nx, ny, nz, nh_d, nh_u, dxi, dyi, dzi, dzfi, dti, rho0, u, v, w, p) &
                   bind(C, name='flutas_gb300_fillps')
      import
      integer(c_int), value :: nx, ny, nz, nh_d, nh_u
      real(c_double), value :: dxi, dyi, dzi
      real(c_double), intent(in) :: dzfi(*)
      real(c_double), value :: dti, rho0
      real(c_double), intent(in) :: u(*), v(*), w(*)
      real(c_double) :: p(*)
    end function
    ! src/correc.f90:16
    integer(c_int) function c_correc(nx, ny, nz, nh_d, nh_u, dxi, dyi, dzi, dzci, dt, rho0, p, u, v, w, rho) &
                   bind(C, name='flutas_gb300_correc')
      import
      integer(c_int), value :: nx, ny, nz, nh_d, nh_u
      real(c_double), value :: dxi, dyi, dzi
      real(c_double), intent(in) :: dzci(*)
      real(c_double), value :: dt, rho0
      real(c_double), intent(in) :: p(*)
      real(c_double) :: u(*), v(*), w(*)
      real(c_double), intent(in) :: rho(*)
    end function
    ! src/bound.f90:146
    integer(c_int) function c_boundp(cbc, n, bc, nh_d, nh_p, halo, dl, dzc, dzf, p) &
                   bind(C, name='flutas_gb300_boundp')
      import
      character(kind=c_char), intent(in) :: cbc(6)
      integer(c_int), intent(in) :: n(3)
      real(c_double), intent(in) :: bc(6)
      integer(c_int), value :: nh_d, nh_p
      integer(c_int), intent(in) :: halo(3)
      real(c_double), intent(in) :: dl(3), dzc(*), dzf(*)
      real(c_double) :: p(*)
    end function
    ! src/bound.f90:17
    integer(c_int) function c_bounduvw(cbcvel, n, bcvel, nh_d, nh_u, halo, isoutflow, dl, dzc, dzf, u, v, w) &
                   bind(C, name='flutas_gb300_bounduvw')
      import
      character(kind=c_char), intent(in) :: cbcvel(18)
      integer(c_int), intent(in) :: n(3)
      real(c_double), intent(in) :: bcvel(18)
      integer(c_int), value :: nh_d, nh_u
      integer(c_int), intent(in) :: halo(3), isoutflow(6)
      real(c_double), intent(in) :: dl(3), dzc(*), dzf(*)
      real(c_double) :: u(*), v(*), w(*)
    end function
    ! src/bound.f90:829
    integer(c_int) function c_updt_rhs_b(nx, ny, nz, c_or_f, cbc, nh_p, rhsbx, rhsby, rhsbz, p) &
                   bind(C, name='flutas_gb300_updt_rhs_b')
      import
      integer(c_int), value :: nx, ny, nz
      character(kind=c_char), intent(in) :: c_or_f(3), cbc(6)
      integer(c_int), value :: nh_p
      real(c_double), intent(in) :: rhsbx(*), rhsby(*), rhsbz(*)
      real(c_double) :: p(*)
    end function
    ! src/chkdiv.f90:18
    integer(c_int) function c_chkdiv(nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w, divtot, divmax) &
                   bind(C, name='flutas_gb300_chkdiv')
      import
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dxi, dyi, dzi
      integer(c_int), value :: nh_d, nh_u
      real(c_double), intent(in) :: dzfi(*), u(*), v(*), w(*)
      real(c_double) :: divtot, divmax
    end function
    ! no counterpart in the reference: chkdiv with no device allocation
    integer(c_int) function c_chkdiv_noalloc(nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w, divtot, divmax) &
                   bind(C, name='flutas_gb300_chkdiv_noalloc')
      import
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dxi, dyi, dzi
      integer(c_int), value :: nh_d, nh_u
      real(c_double), intent(in) :: dzfi(*), u(*), v(*), w(*)
      real(c_double) :: divtot, divmax
    end function
    ! src/source.f90:247
    integer(c_int) function c_pres_tw_src(nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, rho0i, f_t12, f_t12_o, &
                                          p, pold, rho, u, v, w) bind(C, name='flutas_gb300_pres_tw_src')
      import
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dxi, dyi, dzi
      integer(c_int), value :: nh_d, nh_u
      real(c_double), intent(in) :: dzci(*)
      real(c_double), value :: rho0i, f_t12, f_t12_o
      real(c_double), intent(in) :: p(*), pold(*), rho(*)
      real(c_double) :: u(*), v(*), w(*)
    end function
    ! src/fft.f90:159
    integer(c_int) function c_fftend(arrplan) bind(C, name='flutas_gb300_fftend')
      import
      type(c_ptr) :: arrplan(4)
    end function
    ! src/vof.f90:240
    integer(c_int) function c_update_property(n, prop12, vof, prop) bind(C, name='flutas_gb300_update_property')
      import
      integer(c_int), intent(in) :: n(3)
      real(c_double), intent(in) :: prop12(2), vof(*)
      real(c_double) :: prop(*)
    end function
    ! src/load.f90:21
    integer(c_int) function c_load(io, filename, n, nh, fld) bind(C, name='flutas_gb300_load')
      import
      character(kind=c_char), value :: io
      character(kind=c_char), intent(in) :: filename(*)
      integer(c_int), intent(in) :: n(3)
      integer(c_int), value :: nh
      real(c_double) :: fld(*)
    end function
    ! src/initgrid.f90:17
    integer(c_int) function c_initgrid(inivel, n, gr, lz, nh_d, dzc, dzf, zc, zf) bind(C, name='flutas_gb300_initgrid')
      import
      character(kind=c_char), intent(in) :: inivel(3)
      integer(c_int), value :: n
      real(c_double), value :: gr, lz
      integer(c_int), value :: nh_d
      real(c_double) :: dzc(*), dzf(*), zc(*), zf(*)
    end function
    ! src/rk.f90:26 (two-phase right-hand sides)
    integer(c_int) function c_rk(space_scheme_mom, f_t1, f_t2, nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, &
                                 u, v, w, mu, rho, dudtrko, dvdtrko, dwdtrko) bind(C, name='flutas_gb300_rk')
      import
      character(kind=c_char), intent(in) :: space_scheme_mom(3)
      real(c_double), value :: f_t1, f_t2
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dxi, dyi, dzi
      integer(c_int), value :: nh_d, nh_u
      real(c_double), intent(in) :: dzci(*), dzfi(*)
      real(c_double) :: u(*), v(*), w(*)
      real(c_double), intent(in) :: mu(*), rho(*)
      real(c_double) :: dudtrko(*), dvdtrko(*), dwdtrko(*)
    end function
    ! src/rk.f90:26 (single-phase right-hand sides)
    integer(c_int) function c_rk_sp(f_t1, f_t2, nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, visc_sp, &
                                    u, v, w, dudtrko, dvdtrko, dwdtrko) bind(C, name='flutas_gb300_rk_sp')
      import
      real(c_double), value :: f_t1, f_t2
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: dxi, dyi, dzi
      integer(c_int), value :: nh_d, nh_u
      real(c_double), intent(in) :: dzci(*), dzfi(*)
      real(c_double), value :: visc_sp
      real(c_double) :: u(*), v(*), w(*)
      real(c_double) :: dudtrko(*), dvdtrko(*), dwdtrko(*)
    end function
    ! src/rk.f90:104
    integer(c_int) function c_cmpt_time_factors(time_scheme, restart, istep, irk_ss, rkcoeff, dt, dto, &
                                                 f_t1, f_t2, f_t12) bind(C, name='flutas_gb300_cmpt_time_factors')
      import
      character(kind=c_char), intent(in) :: time_scheme(3)
      integer(c_int), value :: restart, istep, irk_ss
      real(c_double), intent(in) :: rkcoeff(6)
      real(c_double), value :: dt, dto
      real(c_double) :: f_t1, f_t2, f_t12
    end function
    integer(c_int) function c_last_error(buf, len) bind(C, name='flutas_gb300_last_error')
      import
      character(kind=c_char) :: buf(*)
      integer(c_int), value :: len
    end function
  end interface
  !
contains
  !
  ! a non-zero status stops the run through the app's abort path, with the library's message
  subroutine check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    character(kind=c_char) :: buf(512)
    character(len=512) :: msg
    integer :: i, ierr
    if (rc == 0) return
    ierr = c_last_error(buf, 512_c_int)
    msg = ''
    do i = 1, 512
      if (buf(i) == c_null_char) exit
      msg(i:i) = buf(i)
    end do
    call flutas_error('GB300 '//what//': '//trim(msg))
  end subroutine check
  !
  subroutine gb300_initsolver(n, dims, dims_z, dli, nh_d, dzci, dzfi, cbc, bc, c_or_f, lambdaxy, a, b, c, &
                              arrplan, normfft, rhsbx, rhsby, rhsbz)
    ! one GPU: dims and dims_z are 1 (no pencil decomposition)
    integer         , intent(in ), dimension(3)       :: n, dims, dims_z
    real(rp)        , intent(in ), dimension(3)       :: dli
    integer         , intent(in )                     :: nh_d
    real(rp)        , intent(in ), dimension(1-nh_d:) :: dzci, dzfi
    character(len=1), intent(in ), dimension(0:1,3)   :: cbc
    real(rp)        , intent(in ), dimension(0:1,3)   :: bc
    character(len=1), intent(in ), dimension(3)       :: c_or_f
    real(rp)        , intent(out), dimension(:,:), contiguous   :: lambdaxy
    real(rp)        , intent(out), dimension(:), contiguous     :: a, b, c
    type(c_ptr)     , intent(out), dimension(2,2)     :: arrplan
    real(rp)        , intent(out)                     :: normfft
    real(rp)        , intent(out), dimension(:,:,0:), contiguous :: rhsbx, rhsby, rhsbz
    if (any(dims /= 1) .or. any(dims_z /= 1)) call flutas_error('GB300 initsolver: one GPU, dims must be 1')
    call check(c_initsolver(int(n, c_int), dli, int(nh_d, c_int), dzci, dzfi, cbc, bc, c_or_f, lambdaxy, &
                            a, b, c, arrplan, normfft, rhsbx, rhsby, rhsbz), 'initsolver')
  end subroutine gb300_initsolver
  !
  ! the CPU form: solver_cpu(n,arrplan,normfft,lambdaxy,a,b,c,bcz,c_or_f,p)
  subroutine gb300_solver_cpu(n, arrplan, normfft, lambdaxy, a, b, c, bcz, c_or_f, p)
    integer         , intent(in   ), dimension(3)   :: n
    type(c_ptr)     , intent(in   ), dimension(2,2) :: arrplan
    real(rp)        , intent(in   )                 :: normfft
    real(rp)        , intent(in   ), dimension(:,:), contiguous :: lambdaxy
    real(rp)        , intent(in   ), dimension(:), contiguous   :: a, b, c
    character(len=1), intent(in   ), dimension(0:1) :: bcz
    character(len=1), intent(in   ), dimension(3)   :: c_or_f
    real(rp)        , intent(inout), dimension(0:,0:,0:), contiguous :: p
    call check(c_solver(int(n, c_int), arrplan, normfft, lambdaxy, a, b, c, bcz, c_or_f, p), 'solver')
  end subroutine gb300_solver_cpu
  !
  ! the OpenACC form: solver_gpu(n_z,dims,arrplan,normfft,lambdaxy,a,b,c,bc,c_or_f,p), where bc is
  ! cbcpre(0:1,1:3) and n is the z-pencil size, i.e. the whole grid on one GPU
  subroutine gb300_solver_gpu(n, dims, arrplan, normfft, lambdaxy, a, b, c, bc, c_or_f, p)
    integer         , intent(in   ), dimension(3)     :: n, dims
    type(c_ptr)     , intent(in   ), dimension(2,2)   :: arrplan
    real(rp)        , intent(in   )                   :: normfft
    real(rp)        , intent(in   ), dimension(:,:), contiguous :: lambdaxy
    real(rp)        , intent(in   ), dimension(:), contiguous   :: a, b, c
    character(len=1), intent(in   ), dimension(0:1,3) :: bc
    character(len=1), intent(in   ), dimension(3)     :: c_or_f
    real(rp)        , intent(inout), dimension(0:,0:,0:), contiguous :: p
    if (any(dims /= 1)) call flutas_error('GB300 solver: one GPU, dims must be 1')
    call check(c_solver(int(n, c_int), arrplan, normfft, lambdaxy, a, b, c, bc(0:1,3), c_or_f, p), 'solver')
  end subroutine gb300_solver_gpu
  !
  subroutine gb300_fillps(nx, ny, nz, nh_d, nh_u, dxi, dyi, dzi, dzfi, dti, rho0, u, v, w, p)
    integer , intent(in )                        :: nx, ny, nz, nh_d, nh_u
    real(rp), intent(in )                        :: dxi, dyi, dzi
    real(rp), intent(in ), dimension(1-nh_d:)    :: dzfi
    real(rp), intent(in )                        :: dti, rho0
    real(rp), intent(in ), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    real(rp), intent(out), dimension(0:,0:,0:), contiguous                :: p
    call check(c_fillps(int(nx, c_int), int(ny, c_int), int(nz, c_int), int(nh_d, c_int), int(nh_u, c_int), &
                        dxi, dyi, dzi, dzfi, dti, rho0, u, v, w, p), 'fillps')
  end subroutine gb300_fillps
  !
  subroutine gb300_correc(nx, ny, nz, nh_d, nh_u, dxi, dyi, dzi, dzci, dt, rho0, p, u, v, w, rho)
    integer , intent(in   )                      :: nx, ny, nz, nh_d, nh_u
    real(rp), intent(in   )                      :: dxi, dyi, dzi
    real(rp), intent(in   ), dimension(1-nh_d:)  :: dzci
    real(rp), intent(in   )                      :: dt, rho0
    real(rp), intent(in   ), dimension(0:,0:,0:), contiguous                :: p
    real(rp), intent(inout), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    real(rp), intent(in   ), dimension(0:,0:,0:), contiguous                :: rho
    call check(c_correc(int(nx, c_int), int(ny, c_int), int(nz, c_int), int(nh_d, c_int), int(nh_u, c_int), &
                        dxi, dyi, dzi, dzci, dt, rho0, p, u, v, w, rho), 'correc')
  end subroutine gb300_correc
  !
  subroutine gb300_boundp(cbc, n, bc, nh_d, nh_p, halo, dl, dzc, dzf, p)
    character(len=1), intent(in   ), dimension(0:1,3) :: cbc
    integer         , intent(in   ), dimension(3)     :: n
    real(rp)        , intent(in   ), dimension(0:1,3) :: bc
    integer         , intent(in   )                   :: nh_d, nh_p
    integer         , intent(in   ), dimension(3)     :: halo
    real(rp)        , intent(in   ), dimension(3)     :: dl
    real(rp)        , intent(in   ), dimension(1-nh_d:) :: dzc, dzf
    real(rp)        , intent(inout), dimension(1-nh_p:,1-nh_p:,1-nh_p:), contiguous :: p
    call check(c_boundp(cbc, int(n, c_int), bc, int(nh_d, c_int), int(nh_p, c_int), int(halo, c_int), dl, &
                        dzc, dzf, p), 'boundp')
  end subroutine gb300_boundp
  !
  subroutine gb300_bounduvw(cbc, n, bc, nh_d, nh_u, halo, isoutflow, dl, dzc, dzf, u, v, w)
    character(len=1), intent(in   ), dimension(0:1,3,3) :: cbc
    integer         , intent(in   ), dimension(3)       :: n
    real(rp)        , intent(in   ), dimension(0:1,3,3) :: bc
    integer         , intent(in   )                     :: nh_d, nh_u
    integer         , intent(in   ), dimension(3)       :: halo
    logical         , intent(in   ), dimension(0:1,3)   :: isoutflow
    real(rp)        , intent(in   ), dimension(3)       :: dl
    real(rp)        , intent(in   ), dimension(1-nh_d:) :: dzc, dzf
    real(rp)        , intent(inout), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    integer(c_int) :: iout(6)
    iout = reshape(merge(1_c_int, 0_c_int, isoutflow), [6])  ! logical kinds differ between compilers
    call check(c_bounduvw(cbc, int(n, c_int), bc, int(nh_d, c_int), int(nh_u, c_int), int(halo, c_int), iout, &
                          dl, dzc, dzf, u, v, w), 'bounduvw')
  end subroutine gb300_bounduvw
  !
  subroutine gb300_updt_rhs_b(nx, ny, nz, c_or_f, cbc, nh_p, rhsbx, rhsby, rhsbz, p)
    integer         , intent(in   )                   :: nx, ny, nz
    character       , intent(in   ), dimension(3)     :: c_or_f
    character(len=1), intent(in   ), dimension(0:1,3) :: cbc
    integer         , intent(in   )                   :: nh_p
    real(rp)        , intent(in   ), dimension(:,:,0:), contiguous :: rhsbx, rhsby, rhsbz
    real(rp)        , intent(inout), dimension(1-nh_p:,1-nh_p:,1-nh_p:), contiguous :: p
    call check(c_updt_rhs_b(int(nx, c_int), int(ny, c_int), int(nz, c_int), c_or_f, cbc, int(nh_p, c_int), &
                            rhsbx, rhsby, rhsbz, p), 'updt_rhs_b')
  end subroutine gb300_updt_rhs_b
  !
  subroutine gb300_chkdiv(nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w, divtot, divmax)
    integer , intent(in )                        :: nx, ny, nz
    real(rp), intent(in )                        :: dxi, dyi, dzi
    integer , intent(in )                        :: nh_d, nh_u
    real(rp), intent(in ), dimension(1-nh_d:)    :: dzfi
    real(rp), intent(in ), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    real(rp), intent(out)                        :: divtot, divmax
    call check(c_chkdiv(int(nx, c_int), int(ny, c_int), int(nz, c_int), dxi, dyi, dzi, int(nh_d, c_int), &
                        int(nh_u, c_int), dzfi, u, v, w, divtot, divmax), 'chkdiv')
  end subroutine gb300_chkdiv
  !
  ! chkdiv for a caller that must not allocate device memory (its own pool owns the GPU, or it
  ! checks after an out-of-memory error): device or managed arrays only, ny*nz <= 65536
  subroutine gb300_chkdiv_noalloc(nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w, divtot, divmax)
    integer , intent(in )                        :: nx, ny, nz
    real(rp), intent(in )                        :: dxi, dyi, dzi
    integer , intent(in )                        :: nh_d, nh_u
    real(rp), intent(in ), dimension(1-nh_d:)    :: dzfi
    real(rp), intent(in ), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    real(rp), intent(out)                        :: divtot, divmax
    call check(c_chkdiv_noalloc(int(nx, c_int), int(ny, c_int), int(nz, c_int), dxi, dyi, dzi, int(nh_d, c_int), &
                                int(nh_u, c_int), dzfi, u, v, w, divtot, divmax), 'chkdiv_noalloc')
  end subroutine gb300_chkdiv_noalloc
  !
  subroutine gb300_pres_tw_src(nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, rho0i, f_t12, f_t12_o, p, pold, rho, &
                               u, v, w)
    integer , intent(in   )                      :: nx, ny, nz
    real(rp), intent(in   )                      :: dxi, dyi, dzi
    integer , intent(in   )                      :: nh_d, nh_u
    real(rp), intent(in   ), dimension(1-nh_d:)  :: dzci
    real(rp), intent(in   )                      :: rho0i, f_t12, f_t12_o
    real(rp), intent(in   ), dimension(0:,0:,0:), contiguous :: p, pold, rho
    real(rp), intent(inout), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    call check(c_pres_tw_src(int(nx, c_int), int(ny, c_int), int(nz, c_int), dxi, dyi, dzi, int(nh_d, c_int), &
                             int(nh_u, c_int), dzci, rho0i, f_t12, f_t12_o, p, pold, rho, u, v, w), 'pres_tw_src')
  end subroutine gb300_pres_tw_src
  !
  subroutine gb300_fftend(arrplan)
    type(c_ptr), intent(inout), dimension(2,2) :: arrplan
    call check(c_fftend(arrplan), 'fftend')
  end subroutine gb300_fftend
  !
  subroutine gb300_update_property(n, prop12, vof, prop)
    integer , intent(in ), dimension(3)        :: n
    real(rp), intent(in ), dimension(2)        :: prop12
    real(rp), intent(in ), dimension(0:,0:,0:), contiguous :: vof
    real(rp), intent(out), dimension(0:,0:,0:), contiguous :: prop
    call check(c_update_property(int(n, c_int), prop12, vof, prop), 'update_property')
  end subroutine gb300_update_property
  !
  ! load(io,filename,n,fld) with fld(n(1),n(2),n(3)): the interior (no halo, nh = 0)
  subroutine gb300_load(io, filename, n, fld)
    character(len=1), intent(in   )               :: io
    character(len=*), intent(in   )               :: filename
    integer         , intent(in   ), dimension(3) :: n
    real(rp)        , intent(inout), dimension(n(1),n(2),n(3)) :: fld
    call check(c_load(io, trim(filename)//c_null_char, int(n, c_int), 0_c_int, fld), 'load')
  end subroutine gb300_load
  !
  subroutine gb300_rk(space_scheme_mom, f_t1, f_t2, nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w, &
                      mu, rho, dudtrko, dvdtrko, dwdtrko)
#if !defined(_USE_VOF)
    use mod_param, only: mu_sp, rho_sp
#endif
    character(len=3), intent(in   )                        :: space_scheme_mom
    real(rp)        , intent(in   )                        :: f_t1, f_t2
    integer         , intent(in   )                        :: nx, ny, nz
    real(rp)        , intent(in   )                        :: dxi, dyi, dzi
    integer         , intent(in   )                        :: nh_d, nh_u
    real(rp)        , intent(in   ), dimension(1-nh_d:)    :: dzci, dzfi
    real(rp)        , intent(inout), dimension(1-nh_u:,1-nh_u:,1-nh_u:), contiguous :: u, v, w
    real(rp)        , intent(in   ), dimension(0:,0:,0:), contiguous                :: mu, rho
    real(rp)        , intent(inout), dimension(:,:,:), contiguous                   :: dudtrko, dvdtrko, dwdtrko
#if defined(_USE_VOF)
    call check(c_rk(space_scheme_mom, f_t1, f_t2, int(nx, c_int), int(ny, c_int), int(nz, c_int), dxi, dyi, dzi, &
                    int(nh_d, c_int), int(nh_u, c_int), dzci, dzfi, u, v, w, mu, rho, dudtrko, dvdtrko, dwdtrko), 'rk')
#else
    call check(c_rk_sp(f_t1, f_t2, int(nx, c_int), int(ny, c_int), int(nz, c_int), dxi, dyi, dzi, int(nh_d, c_int), &
                       int(nh_u, c_int), dzci, dzfi, mu_sp/rho_sp, u, v, w, dudtrko, dvdtrko, dwdtrko), 'rk')
#endif
  end subroutine gb300_rk
  !
  subroutine gb300_cmpt_time_factors(time_scheme, restart, istep, irk_ss, rkcoeff, dt, dto, f_t1, f_t2, f_t12)
    character(len=3), intent(in )                 :: time_scheme
    logical         , intent(in )                 :: restart
    integer         , intent(in )                 :: istep, irk_ss
    real(rp)        , intent(in ), dimension(2,3) :: rkcoeff
    real(rp)        , intent(in )                 :: dt, dto
    real(rp)        , intent(out)                 :: f_t1, f_t2, f_t12
    call check(c_cmpt_time_factors(time_scheme, merge(1_c_int, 0_c_int, restart), int(istep, c_int), &
                                   int(irk_ss, c_int), rkcoeff, dt, dto, f_t1, f_t2, f_t12), 'cmpt_time_factors')
  end subroutine gb300_cmpt_time_factors
  !
  subroutine gb300_initgrid(inivel, n, gr, lz, nh_d, dzc, dzf, zc, zf)
    character(len=3), intent(in )                           :: inivel
    integer         , intent(in )                           :: n
    real(rp)        , intent(in )                           :: gr, lz
    integer         , intent(in )                           :: nh_d
    real(rp)        , intent(out), dimension(1-nh_d:n+nh_d) :: dzc, dzf, zc, zf
    call check(c_initgrid(inivel, int(n, c_int), gr, lz, int(nh_d, c_int), dzc, dzf, zc, zf), 'initgrid')
  end subroutine gb300_initgrid
  !
end module mod_solver_gb300
