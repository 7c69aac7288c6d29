!=============================================================================
! hh_dmrg_f.f90 -- ISO_C_BINDING shim between the Fortran DMRG of
! cfengno1/Hofstadter_Hubbard_TSC and libhh_dmrg.so (C ABI: hh_dmrg.h).
!
! What it replaces (paths inside that project):
!   lanczos_memo_new            code/lanczos.f90:4          drop-in, same name and arguments
!   Get_density_matrix_sys_new  code/get_den.f90:103        drop-in (levels = 1)
!   Get_density_matrix_env_new  code/get_den.f90:143        drop-in (levels = 1)
!   Get_truncation_operator     code/get_den.f90:184        drop-in
!   model_wave                  code/mat_vec.f90:3476       hh_model_wave, same arguments
!   update_trun_dia / _ndia     code/update.f90:1387,1457   hh_update_trun_dia / _ndia
!   wave_trans_LR / _RL         code/warm_up.f90:1855,2016  hh_wave_trans_LR / _RL
!
! Build: compile this file after pubdata.f90 and link with -lhh_dmrg -lcudart.
! For the drop-ins, leave lanczos.f90 out of the build and delete the three
! routines named above from get_den.f90; their callers (code/warm_up.f90:1413,
! 1416, 1431, 1552, 1563, ...) are unchanged.  The other wrappers carry an hh_
! prefix so that the reference's own routines stay available next to them.
!
! Once, before the first call:  call hh_f_init(device)
! Precision of the superblock matvec (module variable, FP64 by default):
!   hh_precision = HH_PREC_BF16X3   ! split precision on the tensor cores;
! lanczos_memo_new then returns FP64-accurate energies (one FP64 product per
! call, see hh_lanczos in hh_dmrg.h).  At the end:  call hh_f_finalize()
!
! Every wrapper stops the program when the library returns an error status,
! printing hh_last_error, as the reference stops on a quantum-number
! mismatch.  Side channels of the replaced routines are kept: Energys(1) and
! Energy0, the Energy_All.dat line of lanczos_memo_new, Entropys, Entropy0 and
! the Entropy.dat line of Get_truncation_operator.
!
! Data are copied to the device at each call and the device copies freed on
! return, so every wrapper is stateless except for the density-matrix wave
! (set by Get_density_matrix_*_new, used by the next Get_truncation_operator).
! Keeping the blocks resident across a whole sweep is what the library's own
! sweep driver does; this shim trades that for an unchanged Fortran program.
!
! This file is not compiled in the repository that ships it (its machines
! have no Fortran compiler); it follows the Fortran 2003 standard.
!=============================================================================
module hh_dmrg_f
  use iso_c_binding
  use pubdata
  implicit none

  integer(c_int), parameter :: HH_PREC_FP64 = 0, HH_PREC_BF16X6 = 1, HH_PREC_BF16X3 = 2, &
       HH_PREC_FP32 = 3, HH_PREC_FP32X2 = 4
  integer(c_int), parameter :: HH_BLOCK_VEC_DIA = 1, HH_VEC_BLOCK_DIA = 2, HH_SITE_VEC_SITE_DIA = 3, &
       HH_SITE_VEC_SITE_NDIA = 4, HH_BLOCK_SITE_VEC_NDIA = 5, HH_VEC_BLOCK_SITE_NDIA = 6, &
       HH_BLOCK_VEC_SITE_NDIA = 7, HH_SITE_VEC_BLOCK_NDIA = 8, HH_BLOCK_VEC_BLOCK_NDIA = 9, &
       HH_BLOCK_SITE_VEC_DIA = 10, HH_VEC_BLOCK_SITE_DIA = 11, HH_BLOCK_VEC_SITE_DIA = 12, &
       HH_SITE_VEC_BLOCK_DIA = 13, HH_BLOCK_VEC_BLOCK_DIA = 14
  integer(c_int), parameter :: HH_F = iachar('F'), HH_B = iachar('B')
  integer, parameter :: HH_MAX_TERMS = 16 * nxx + 64

  ! one term of model_wave (hh_term_t of hh_dmrg.h)
  type, bind(C) :: hh_term_t
    integer(c_int) :: kind, flag0, flag1, trans0, trans1
    type(c_ptr) :: op0, op1
    real(c_double) :: coef_re, coef_im
  end type hh_term_t

  type(c_ptr), save :: hh_ctx = c_null_ptr
  integer(c_int), save :: hh_precision = HH_PREC_FP64
  ! wave of the density matrix set by Get_density_matrix_*_new (side 0 sys, 1 env)
  type(c_ptr), save :: hh_den_wave = c_null_ptr
  integer(c_int), save :: hh_den_side = -1

  ! device copies made for one call, freed together by hh_f_release
  type(c_ptr), save :: hh_held(4 * HH_MAX_TERMS)
  integer, save :: hh_nheld = 0

  interface
    integer(c_int) function hh_init(device, ctx) bind(C, name="hh_init")
      import :: c_int, c_ptr
      integer(c_int), value :: device
      type(c_ptr) :: ctx
    end function hh_init
    integer(c_int) function hh_finalize(ctx) bind(C, name="hh_finalize")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function hh_finalize
    type(c_ptr) function hh_last_error(ctx) bind(C, name="hh_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function hh_last_error
    integer(c_int) function hh_block_create(ctx, len, up_dif, down_dif, nsub, sub_qn, data, blk) &
         bind(C, name="hh_block_create")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: len, up_dif, down_dif, nsub
      integer(c_int) :: sub_qn(5, *)
      complex(c_double_complex) :: data(*)
      type(c_ptr) :: blk
    end function hh_block_create
    integer(c_int) function hh_block_info(b, len, up_dif, down_dif, nsub, nelem) bind(C, name="hh_block_info")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: b
      integer(c_int) :: len, up_dif, down_dif, nsub
      integer(c_long_long) :: nelem
    end function hh_block_info
    integer(c_int) function hh_block_qn(b, sub_qn) bind(C, name="hh_block_qn")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int) :: sub_qn(5, *)
    end function hh_block_qn
    integer(c_int) function hh_block_download(b, data) bind(C, name="hh_block_download")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: b
      complex(c_double_complex) :: data(*)
    end function hh_block_download
    integer(c_int) function hh_block_free(b) bind(C, name="hh_block_free")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
    end function hh_block_free
    integer(c_int) function hh_basis_create(ctx, len, nsec, sec, subs, bs) bind(C, name="hh_basis_create")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: len, nsec
      integer(c_int) :: sec(3, *), subs(6, *)
      type(c_ptr) :: bs
    end function hh_basis_create
    integer(c_int) function hh_basis_free(bs) bind(C, name="hh_basis_free")
      import :: c_int, c_ptr
      type(c_ptr), value :: bs
    end function hh_basis_free
    integer(c_int) function hh_wave_create(ctx, sys_len, env_len, nsec, sec, nbatch, w) &
         bind(C, name="hh_wave_create")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: sys_len, env_len, nsec, nbatch
      integer(c_int) :: sec(6, *)
      type(c_ptr) :: w
    end function hh_wave_create
    integer(c_int) function hh_wave_upload(w, data) bind(C, name="hh_wave_upload")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: w
      complex(c_double_complex) :: data(*)
    end function hh_wave_upload
    integer(c_int) function hh_wave_download(w, data) bind(C, name="hh_wave_download")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: w
      complex(c_double_complex) :: data(*)
    end function hh_wave_download
    integer(c_int) function hh_wave_normalize(w) bind(C, name="hh_wave_normalize")
      import :: c_int, c_ptr
      type(c_ptr), value :: w
    end function hh_wave_normalize
    integer(c_int) function hh_wave_free(w) bind(C, name="hh_wave_free")
      import :: c_int, c_ptr
      type(c_ptr), value :: w
    end function hh_wave_free
    integer(c_int) function hh_plan_create(ctx, sys_bs, env_bs, layout, nterm, terms, plan) &
         bind(C, name="hh_plan_create")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, sys_bs, env_bs, layout
      integer(c_int), value :: nterm
      type(c_ptr), value :: terms
      type(c_ptr) :: plan
    end function hh_plan_create
    integer(c_int) function hh_plan_free(plan) bind(C, name="hh_plan_free")
      import :: c_int, c_ptr
      type(c_ptr), value :: plan
    end function hh_plan_free
    integer(c_int) function hh_matvec(plan, vin, vout, precision) bind(C, name="hh_matvec")
      import :: c_int, c_ptr
      type(c_ptr), value :: plan, vin, vout
      integer(c_int), value :: precision
    end function hh_matvec
    integer(c_int) function hh_lanczos(plan, psi, lanzero, maxit, precision, energy, iters) &
         bind(C, name="hh_lanczos")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: plan, psi
      real(c_double), value :: lanzero
      integer(c_int), value :: maxit, precision
      real(c_double) :: energy
      integer(c_int) :: iters
    end function hh_lanczos
    integer(c_int) function hh_density_truncate(ctx, psi, side, kept_min, kept_max, trun_err, trun, &
         num_state, discarded, entropy, spectrum) bind(C, name="hh_density_truncate")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, psi
      integer(c_int), value :: side, kept_min, kept_max
      real(c_double), value :: trun_err
      type(c_ptr) :: trun
      integer(c_int) :: num_state
      real(c_double) :: discarded, entropy
      type(c_ptr), value :: spectrum
    end function hh_density_truncate
    integer(c_int) function hh_renormalize(ctx, op, trun, dia, out) bind(C, name="hh_renormalize")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, op, trun
      integer(c_int), value :: dia
      type(c_ptr) :: out
    end function hh_renormalize
    integer(c_int) function hh_wave_transform(ctx, dir, sys_bs, env_bs, sys_trun, env_trun, old_wave, &
         new_wave) bind(C, name="hh_wave_transform")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave
      integer(c_int), value :: dir
    end function hh_wave_transform
    ! arithmetic of the split hh_lanczos's restart product and of hh_renormalize
    ! (HH_PREC_FP32X2: double-float, FP64-class, on the FP32 pipe)
    integer(c_int) function hh_ctx_set_restart_precision(ctx, precision) &
         bind(C, name="hh_ctx_set_restart_precision")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: precision
    end function hh_ctx_set_restart_precision
    integer(c_int) function hh_ctx_set_renormalize_precision(ctx, precision) &
         bind(C, name="hh_ctx_set_renormalize_precision")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: precision
    end function hh_ctx_set_renormalize_precision
    integer(c_long) function c_strlen(s) bind(C, name="strlen")
      import :: c_long, c_ptr
      type(c_ptr), value :: s
    end function c_strlen
  end interface

contains

  !--------------------------------------------------------------- set-up
  subroutine hh_f_init(device)
    integer, intent(in) :: device
    if (c_associated(hh_ctx)) return
    if (hh_init(int(device, c_int), hh_ctx) /= 0) then
      write(*, *) 'hh_init failed: no usable CUDA device ', device
      stop
    end if
  end subroutine hh_f_init

  subroutine hh_f_finalize()
    integer(c_int) :: st
    if (c_associated(hh_den_wave)) st = hh_wave_free(hh_den_wave)
    hh_den_wave = c_null_ptr
    if (c_associated(hh_ctx)) st = hh_finalize(hh_ctx)
    hh_ctx = c_null_ptr
  end subroutine hh_f_finalize

  ! stops with the library's message on an error status (the reference's
  ! convention: write(*,*) and stop)
  subroutine hh_f_check(st, what)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    character(len=512) :: text
    type(c_ptr) :: p
    integer :: n, i
    if (st == 0) return
    text = ' '
    p = hh_last_error(hh_ctx)
    n = min(512, int(c_strlen(p)))
    if (n > 0) then
      call c_f_pointer(p, msg, [n])
      do i = 1, n
        text(i:i) = msg(i)
      end do
    end if
    write(*, *) 'libhh_dmrg: ', what, ' failed, status ', st, ': ', trim(text)
    stop
  end subroutine hh_f_check

  subroutine hh_f_hold(h)
    type(c_ptr), intent(in) :: h
    if (hh_nheld >= size(hh_held)) then
      write(*, *) 'hh_dmrg_f: too many device copies in one call'
      stop
    end if
    hh_nheld = hh_nheld + 1
    hh_held(hh_nheld) = h
  end subroutine hh_f_hold

  subroutine hh_f_release()
    integer :: i
    integer(c_int) :: st
    do i = 1, hh_nheld
      st = hh_block_free(hh_held(i))
    end do
    hh_nheld = 0
  end subroutine hh_f_release

  !------------------------------------------------------ flattening
  ! Total_Block (code/pubdata.f90:141-149) -> device block; sub matrices back
  ! to back in their own column-major order.  Held until hh_f_release.
  function hh_f_block(blk) result(h)
    type(Total_Block), intent(in) :: blk
    type(c_ptr) :: h
    integer(c_int), allocatable :: qn(:, :)
    complex(c_double_complex), allocatable :: data(:)
    integer :: i, n, nel
    allocate(qn(5, max(1, blk%num)))
    nel = 0
    do i = 1, blk%num
      qn(:, i) = [blk%sub(i)%num_up, blk%sub(i)%num_down, blk%sub(i)%down_dif, &
                  blk%sub(i)%row_dim, blk%sub(i)%sdim]
      nel = nel + blk%sub(i)%row_dim * blk%sub(i)%sdim
    end do
    allocate(data(max(1, nel)))
    nel = 0
    do i = 1, blk%num
      n = blk%sub(i)%row_dim * blk%sub(i)%sdim
      if (n > 0) data(nel + 1:nel + n) = reshape(blk%sub(i)%mat, [n])
      nel = nel + n
    end do
    h = c_null_ptr
    call hh_f_check(hh_block_create(hh_ctx, blk%len, blk%up_dif, blk%down_dif, blk%num, qn, data, h), &
                    'hh_block_create')
    call hh_f_hold(h)
  end function hh_f_block

  ! device block -> Total_Block (allocates blk%sub and every mat)
  subroutine hh_f_block_get(h, blk)
    type(c_ptr), intent(in) :: h
    type(Total_Block), intent(inout) :: blk
    integer(c_int) :: len, up_dif, down_dif, nsub
    integer(c_long_long) :: nelem
    integer(c_int), allocatable :: qn(:, :)
    complex(c_double_complex), allocatable :: data(:)
    integer :: i, n, nel
    call hh_f_check(hh_block_info(h, len, up_dif, down_dif, nsub, nelem), 'hh_block_info')
    allocate(qn(5, max(1, nsub)), data(max(1_c_long_long, nelem)))
    if (nsub > 0) call hh_f_check(hh_block_qn(h, qn), 'hh_block_qn')
    if (nelem > 0) call hh_f_check(hh_block_download(h, data), 'hh_block_download')
    if (allocated(blk%sub)) call deallocate_block(blk)
    blk%len = len
    blk%up_dif = up_dif
    blk%down_dif = down_dif
    blk%num = nsub
    blk%dim = 0
    allocate(blk%sub(nsub))
    nel = 0
    do i = 1, nsub
      blk%sub(i)%num_up = qn(1, i)
      blk%sub(i)%num_down = qn(2, i)
      blk%sub(i)%down_dif = qn(3, i)
      blk%sub(i)%row_dim = qn(4, i)
      blk%sub(i)%sdim = qn(5, i)
      blk%dim = blk%dim + qn(5, i)
      n = qn(4, i) * qn(5, i)
      allocate(blk%sub(i)%mat(qn(4, i), qn(5, i)))
      if (n > 0) blk%sub(i)%mat = reshape(data(nel + 1:nel + n), [qn(4, i), qn(5, i)])
      nel = nel + n
    end do
  end subroutine hh_f_block_get

  ! Total_Basis (code/pubdata.f90:91-108) -> device basis
  function hh_f_basis(bs) result(h)
    type(Total_Basis), intent(in) :: bs
    type(c_ptr) :: h
    integer(c_int), allocatable :: sec(:, :), subs(:, :)
    integer :: x, y, k, nsub
    nsub = 0
    do x = 1, bs%num
      nsub = nsub + bs%sub(x)%num
    end do
    allocate(sec(3, max(1, bs%num)), subs(6, max(1, nsub)))
    k = 0
    do x = 1, bs%num
      sec(:, x) = [bs%sub(x)%new_num_up, bs%sub(x)%new_num_down, bs%sub(x)%num]
      do y = 1, bs%sub(x)%num
        k = k + 1
        subs(:, k) = [bs%sub(x)%sub(y)%spos, bs%sub(x)%sub(y)%sdim, bs%sub(x)%sub(y)%bl_num_up, &
                      bs%sub(x)%sub(y)%bl_num_down, bs%sub(x)%sub(y)%st_num_up, bs%sub(x)%sub(y)%st_num_down]
      end do
    end do
    h = c_null_ptr
    call hh_f_check(hh_basis_create(hh_ctx, bs%len, bs%num, sec, subs, h), 'hh_basis_create')
  end function hh_f_basis

  ! device wave with the layout of a Wavefunction (code/pubdata.f90:126-136),
  ! its vectors uploaded when load is true
  function hh_f_wave(w, load) result(h)
    type(Wavefunction), intent(in) :: w
    logical, intent(in) :: load
    type(c_ptr) :: h
    integer(c_int), allocatable :: sec(:, :)
    complex(c_double_complex), allocatable :: data(:)
    integer :: i, n, nel
    allocate(sec(6, max(1, w%num)))
    nel = 0
    do i = 1, w%num
      sec(:, i) = [w%sub(i)%sys_num_up, w%sub(i)%sys_num_down, w%sub(i)%env_num_up, &
                   w%sub(i)%env_num_down, w%sub(i)%sys_dim, w%sub(i)%env_dim]
      nel = nel + w%sub(i)%sys_dim * w%sub(i)%env_dim
    end do
    h = c_null_ptr
    call hh_f_check(hh_wave_create(hh_ctx, w%sys_len, w%env_len, w%num, sec, 1, h), 'hh_wave_create')
    if (.not. load) return
    allocate(data(max(1, nel)))
    nel = 0
    do i = 1, w%num
      n = w%sub(i)%sys_dim * w%sub(i)%env_dim
      if (n > 0) data(nel + 1:nel + n) = reshape(w%sub(i)%vec, [n])
      nel = nel + n
    end do
    call hh_f_check(hh_wave_upload(h, data), 'hh_wave_upload')
  end function hh_f_wave

  ! device wave -> the vec arrays of an allocated Wavefunction of that layout
  subroutine hh_f_wave_get(h, w)
    type(c_ptr), intent(in) :: h
    type(Wavefunction), intent(inout) :: w
    complex(c_double_complex), allocatable :: data(:)
    integer :: i, n, nel
    nel = 0
    do i = 1, w%num
      nel = nel + w%sub(i)%sys_dim * w%sub(i)%env_dim
    end do
    allocate(data(max(1, nel)))
    call hh_f_check(hh_wave_download(h, data), 'hh_wave_download')
    nel = 0
    do i = 1, w%num
      n = w%sub(i)%sys_dim * w%sub(i)%env_dim
      if (n > 0) w%sub(i)%vec = reshape(data(nel + 1:nel + n), [w%sub(i)%sys_dim, w%sub(i)%env_dim])
      nel = nel + n
    end do
  end subroutine hh_f_wave_get

  !---------------------------------------------------------- model_wave
  subroutine hh_f_add(terms, nt, kind, op0, op1, flag0, flag1, trans0, trans1, coef)
    type(hh_term_t), intent(inout) :: terms(:)
    integer, intent(inout) :: nt
    integer(c_int), intent(in) :: kind, flag0, flag1, trans0, trans1
    type(c_ptr), intent(in) :: op0, op1
    double complex, intent(in) :: coef
    if (nt >= size(terms)) then
      write(*, *) 'hh_dmrg_f: more model_wave terms than HH_MAX_TERMS'
      stop
    end if
    nt = nt + 1
    terms(nt) = hh_term_t(kind, flag0, flag1, trans0, trans1, op0, op1, dble(coef), dimag(coef))
  end subroutine hh_f_add

  ! The term list of model_wave (code/mat_vec.f90:3502-3615), in its order,
  ! with the merged boundary operators hmerge left in sys%snc, env%snc,
  ! sys%sub_s, env%sub_s and the counts in coup_bs, coup_bb and inb.
  ! block_transfer_trans(X) becomes trans = 1 on the untransposed X.
  subroutine hh_f_terms(sys, env, terms, nt)
    type(Total_Model), intent(in) :: sys, env
    type(hh_term_t), intent(inout) :: terms(:)
    integer, intent(out) :: nt
    integer :: is, js, ii, i, jc, jc1, i1
    double complex :: coefx
    type(c_ptr) :: dbl, si, eup, edn, sd, nel, a, b
    nt = 0
    dbl = hh_f_block(st_double)
    si = hh_f_block(st_si)
    eup = hh_f_block(st_elec_up)
    edn = hh_f_block(st_elec_down)
    sd = c_null_ptr
    nel = c_null_ptr
    if (tjmodel == 1) sd = hh_f_block(st_sd)
    if (v123 == 1 .or. tjmodel == 1) nel = hh_f_block(num_elec)
    call hh_f_add(terms, nt, HH_BLOCK_VEC_DIA, hh_f_block(sys%ham), c_null_ptr, HH_B, HH_B, 0, 0, cone)
    call hh_f_add(terms, nt, HH_VEC_BLOCK_DIA, hh_f_block(env%ham), c_null_ptr, HH_B, HH_B, 0, 0, cone)
    is = nposi_lat(sys%len + 1)
    js = nposi_lat(sys%len + env%len + 2)
    ii = neiba(is, js)
    if (hubbard(is) /= 0.0d0) &
      call hh_f_add(terms, nt, HH_SITE_VEC_SITE_DIA, dbl, si, HH_B, HH_B, 0, 0, dcmplx(hubbard(is), 0.0d0))
    if (hubbard(js) /= 0.0d0) &
      call hh_f_add(terms, nt, HH_SITE_VEC_SITE_DIA, si, dbl, HH_B, HH_B, 0, 0, dcmplx(hubbard(js), 0.0d0))
    if (ii /= 0) then
      coefx = jt(ii, is) * pint(is, js)
      if (coefx /= czero) call hh_f_add(terms, nt, HH_SITE_VEC_SITE_NDIA, eup, edn, HH_F, HH_F, 0, 1, coefx)
      if (jd(ii, is) /= czero) call hh_f_add(terms, nt, HH_SITE_VEC_SITE_NDIA, sd, sd, HH_B, HH_B, 0, 0, jd(ii, is))
      if (jn(ii, is) /= czero) call hh_f_add(terms, nt, HH_SITE_VEC_SITE_DIA, nel, nel, HH_B, HH_B, 0, 0, jn(ii, is))
    end if
    if (coup_bs(1, 1) == 1) then
      call hh_f_add(terms, nt, HH_BLOCK_SITE_VEC_NDIA, hh_f_block(sys%snc(1)%elec_up), edn, HH_F, HH_F, 0, 1, cone)
      if (tjmodel == 1) &
        call hh_f_add(terms, nt, HH_BLOCK_SITE_VEC_NDIA, hh_f_block(sys%snc(1)%spin_sd), sd, HH_B, HH_B, 0, 0, cone)
      if (v123 == 1) &
        call hh_f_add(terms, nt, HH_BLOCK_SITE_VEC_DIA, hh_f_block(sys%snc(1)%num_sn), nel, HH_B, HH_B, 0, 0, cone)
    end if
    if (coup_bs(1, 2) == 1) then
      call hh_f_add(terms, nt, HH_BLOCK_VEC_SITE_NDIA, hh_f_block(sys%snc(2)%elec_up), edn, HH_F, HH_F, 0, 1, cone)
      if (tjmodel == 1) &
        call hh_f_add(terms, nt, HH_BLOCK_VEC_SITE_NDIA, hh_f_block(sys%snc(2)%spin_sd), sd, HH_B, HH_B, 0, 0, cone)
      if (v123 == 1) &
        call hh_f_add(terms, nt, HH_BLOCK_VEC_SITE_DIA, hh_f_block(sys%snc(2)%num_sn), nel, HH_B, HH_B, 0, 0, cone)
    end if
    if (coup_bs(2, 1) == 1) then
      call hh_f_add(terms, nt, HH_SITE_VEC_BLOCK_NDIA, eup, hh_f_block(env%snc(1)%elec_down), HH_F, HH_F, 0, 1, cone)
      if (tjmodel == 1) &
        call hh_f_add(terms, nt, HH_SITE_VEC_BLOCK_NDIA, sd, hh_f_block(env%snc(1)%spin_sd), HH_B, HH_B, 0, 1, cone)
      if (v123 == 1) &
        call hh_f_add(terms, nt, HH_SITE_VEC_BLOCK_DIA, nel, hh_f_block(env%snc(1)%num_sn), HH_B, HH_B, 0, 0, cone)
    end if
    if (coup_bs(2, 2) == 1) then
      call hh_f_add(terms, nt, HH_VEC_BLOCK_SITE_NDIA, hh_f_block(env%snc(2)%elec_up), edn, HH_F, HH_F, 0, 1, cone)
      if (tjmodel == 1) &
        call hh_f_add(terms, nt, HH_VEC_BLOCK_SITE_NDIA, hh_f_block(env%snc(2)%spin_sd), sd, HH_B, HH_B, 0, 0, cone)
      if (v123 == 1) &
        call hh_f_add(terms, nt, HH_VEC_BLOCK_SITE_DIA, hh_f_block(env%snc(2)%num_sn), nel, HH_B, HH_B, 0, 0, cone)
    end if
    ! block-block terms: every boundary-coupled block site (inb) with its
    ! merged partner on the other side
    jc = 0
    do i = 1, sys%len + 1 + env%len
      if (inb(i) == 0) cycle
      jc = jc + 1
      if (i <= sys%len) then
        i1 = inb1(i, sys%len)
        a = hh_f_block(sys%sub(i1)%elec_up)
        b = hh_f_block(env%sub_s(jc)%elec_down)
        call hh_f_add(terms, nt, HH_BLOCK_VEC_BLOCK_NDIA, a, b, HH_F, HH_F, 0, 1, cone)
        if (tjmodel == 1) call hh_f_add(terms, nt, HH_BLOCK_VEC_BLOCK_NDIA, hh_f_block(sys%sub(i1)%spin_sd), &
                                        hh_f_block(env%sub_s(jc)%spin_sd), HH_B, HH_B, 0, 1, cone)
        if (v123 == 1) call hh_f_add(terms, nt, HH_BLOCK_VEC_BLOCK_DIA, hh_f_block(sys%sub(i1)%num_sn), &
                                     hh_f_block(env%sub_s(jc)%num_sn), HH_B, HH_B, 0, 0, cone)
      else
        i1 = inb1(i - sys%len - 1, env%len)
        jc1 = jc - coup_bb(1)
        a = hh_f_block(sys%sub_s(jc1)%elec_up)
        b = hh_f_block(env%sub(i1)%elec_down)
        call hh_f_add(terms, nt, HH_BLOCK_VEC_BLOCK_NDIA, a, b, HH_F, HH_F, 0, 1, cone)
        if (tjmodel == 1) call hh_f_add(terms, nt, HH_BLOCK_VEC_BLOCK_NDIA, hh_f_block(sys%sub_s(jc1)%spin_sd), &
                                        hh_f_block(env%sub(i1)%spin_sd), HH_B, HH_B, 0, 1, cone)
        if (v123 == 1) call hh_f_add(terms, nt, HH_BLOCK_VEC_BLOCK_DIA, hh_f_block(sys%sub_s(jc1)%num_sn), &
                                     hh_f_block(env%sub(i1)%num_sn), HH_B, HH_B, 0, 0, cone)
      end if
    end do
  end subroutine hh_f_terms

  ! hmerge (the reference's, on the host blocks) + the plan of one superblock
  subroutine hh_f_plan(sys, env, sys_bs, env_bs, layout, plan, dsys_bs, denv_bs)
    type(Total_Model), intent(inout) :: sys, env
    type(Total_Basis), intent(in) :: sys_bs, env_bs
    type(c_ptr), intent(in) :: layout
    type(c_ptr), intent(out) :: plan, dsys_bs, denv_bs
    type(hh_term_t), target :: terms(HH_MAX_TERMS)
    integer :: nt
    if (add_op == 1) call hmerge(sys, env, sys_bs, env_bs)
    call hh_f_terms(sys, env, terms, nt)
    dsys_bs = hh_f_basis(sys_bs)
    denv_bs = hh_f_basis(env_bs)
    plan = c_null_ptr
    call hh_f_check(hh_plan_create(hh_ctx, dsys_bs, denv_bs, layout, int(nt, c_int), c_loc(terms), plan), &
                    'hh_plan_create')
  end subroutine hh_f_plan

  ! model_wave(sys,env,sys_bs,env_bs,invec,outvec) on the GPU at hh_precision
  subroutine hh_model_wave(sys, env, sys_bs, env_bs, invec, outvec)
    type(Total_Model), intent(inout) :: sys, env
    type(Total_Basis), intent(in) :: sys_bs, env_bs
    type(Wavefunction), intent(in) :: invec
    type(Wavefunction), intent(inout) :: outvec
    type(c_ptr) :: win, wout, plan, dsb, deb
    integer(c_int) :: st
    win = hh_f_wave(invec, .true.)
    wout = hh_f_wave(outvec, .false.)
    call hh_f_plan(sys, env, sys_bs, env_bs, win, plan, dsb, deb)
    call hh_f_check(hh_matvec(plan, win, wout, hh_precision), 'hh_matvec')
    call hh_f_wave_get(wout, outvec)
    st = hh_plan_free(plan)
    st = hh_basis_free(dsb)
    st = hh_basis_free(deb)
    st = hh_wave_free(win)
    st = hh_wave_free(wout)
    call hh_f_release()
  end subroutine hh_model_wave

  !------------------------------------------- renormalisation, transforms
  subroutine hh_f_renorm(ori, eff, trun, dia)
    type(Total_Block), intent(in) :: ori, trun
    type(Total_Block), intent(inout) :: eff
    integer(c_int), intent(in) :: dia
    type(c_ptr) :: o, t, e
    integer(c_int) :: st
    o = hh_f_block(ori)
    t = hh_f_block(trun)
    e = c_null_ptr
    call hh_f_check(hh_renormalize(hh_ctx, o, t, dia, e), 'hh_renormalize')
    call hh_f_block_get(e, eff)
    st = hh_block_free(e)
    call hh_f_release()
  end subroutine hh_f_renorm

  ! update_trun_dia(ori,eff,trun), code/update.f90:1387
  subroutine hh_update_trun_dia(ori, eff, trun)
    type(Total_Block), intent(in) :: ori, trun
    type(Total_Block), intent(inout) :: eff
    call hh_f_renorm(ori, eff, trun, 1)
  end subroutine hh_update_trun_dia

  ! update_trun_ndia(ori,eff,trun), code/update.f90:1457
  subroutine hh_update_trun_ndia(ori, eff, trun)
    type(Total_Block), intent(in) :: ori, trun
    type(Total_Block), intent(inout) :: eff
    call hh_f_renorm(ori, eff, trun, 0)
  end subroutine hh_update_trun_ndia

  subroutine hh_f_trans(dir, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave)
    integer(c_int), intent(in) :: dir
    type(Total_Basis), intent(in) :: sys_bs, env_bs
    type(Total_Block), intent(in) :: sys_trun, env_trun
    type(Wavefunction), intent(in) :: old_wave
    type(Wavefunction), intent(inout) :: new_wave
    type(c_ptr) :: sb, eb, wo, wn
    integer(c_int) :: st
    sb = hh_f_basis(sys_bs)
    eb = hh_f_basis(env_bs)
    wo = hh_f_wave(old_wave, .true.)
    wn = hh_f_wave(new_wave, .false.)
    call hh_f_check(hh_wave_transform(hh_ctx, dir, sb, eb, hh_f_block(sys_trun), hh_f_block(env_trun), wo, wn), &
                    'hh_wave_transform')
    call hh_f_wave_get(wn, new_wave)
    st = hh_wave_free(wo)
    st = hh_wave_free(wn)
    st = hh_basis_free(sb)
    st = hh_basis_free(eb)
    call hh_f_release()
  end subroutine hh_f_trans

  ! wave_trans_LR(sys_bs,env_bs,sys_trun,env_trun,old_wave,new_wave), code/warm_up.f90:1855;
  ! new_wave allocated by the caller (allocate_wave) as for the reference's routine
  subroutine hh_wave_trans_LR(sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave)
    type(Total_Basis), intent(in) :: sys_bs, env_bs
    type(Total_Block), intent(in) :: sys_trun, env_trun
    type(Wavefunction), intent(in) :: old_wave
    type(Wavefunction), intent(inout) :: new_wave
    call hh_f_trans(0, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave)
  end subroutine hh_wave_trans_LR

  ! wave_trans_RL, code/warm_up.f90:2016
  subroutine hh_wave_trans_RL(sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave)
    type(Total_Basis), intent(in) :: sys_bs, env_bs
    type(Total_Block), intent(in) :: sys_trun, env_trun
    type(Wavefunction), intent(in) :: old_wave
    type(Wavefunction), intent(inout) :: new_wave
    call hh_f_trans(1, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave)
  end subroutine hh_wave_trans_RL

  !------------------------------------------------------- density matrix
  ! Get_density_matrix_*_new with levels = 1: the wave is normalised on the
  ! device and kept for the next Get_truncation_operator; den receives the
  ! sector headers (one per wave sector, as the reference's density has) with
  ! empty matrices, which deallocate_block frees as usual.
  subroutine hh_f_density(den, wave, levels, side)
    type(Total_Block), intent(inout) :: den
    integer, intent(in) :: levels, side
    type(Wavefunction), intent(in) :: wave(levels)
    integer :: i, d
    integer(c_int) :: st
    if (levels /= 1) then
      write(*, *) 'hh_dmrg_f: the GPU density matrix takes levels = 1'
      stop
    end if
    if (c_associated(hh_den_wave)) st = hh_wave_free(hh_den_wave)
    hh_den_wave = hh_f_wave(wave(1), .true.)
    call hh_f_check(hh_wave_normalize(hh_den_wave), 'hh_wave_normalize')
    hh_den_side = side
    if (allocated(den%sub)) call deallocate_block(den)
    den%up_dif = 0
    den%down_dif = 0
    den%num = wave(1)%num
    den%dim = 0
    if (side == 0) then
      den%len = wave(1)%sys_len
    else
      den%len = wave(1)%env_len
    end if
    allocate(den%sub(den%num))
    do i = 1, den%num
      if (side == 0) then
        den%sub(i)%num_up = wave(1)%sub(i)%sys_num_up
        den%sub(i)%num_down = wave(1)%sub(i)%sys_num_down
        d = wave(1)%sub(i)%sys_dim
      else
        den%sub(i)%num_up = wave(1)%sub(i)%env_num_up
        den%sub(i)%num_down = wave(1)%sub(i)%env_num_down
        d = wave(1)%sub(i)%env_dim
      end if
      den%sub(i)%down_dif = 0
      den%sub(i)%row_dim = d
      den%sub(i)%sdim = d
      den%dim = den%dim + d
      allocate(den%sub(i)%mat(0, 0))
    end do
  end subroutine hh_f_density

end module hh_dmrg_f


!=============================================================================
! Drop-ins (external procedures with the reference's names and arguments)
!=============================================================================

! lanczos_memo_new, code/lanczos.f90:4-177 (levels = 1, the reference's only
! use in the sweep): hmerge on the host, then the whole Lanczos run on the GPU.
subroutine lanczos_memo_new(sys, env, sys_bs, env_bs, super, eigvec, levels, num_idx)
  use hh_dmrg_f
  implicit none
  integer, intent(in) :: levels, num_idx
  type(Super_Basis), intent(in) :: super
  type(Total_Basis), intent(in) :: sys_bs, env_bs
  type(Total_Model), intent(inout) :: sys, env
  type(Wavefunction), intent(inout) :: eigvec(levels)
  type(c_ptr) :: w, plan, dsb, deb
  real(c_double) :: e0
  integer(c_int) :: iters, st
  real(8) :: bg_time, end_time
  if (levels /= 1) then
    write(*, *) 'hh_dmrg_f: the GPU lanczos_memo_new takes levels = 1'
    stop
  end if
  call cpu_time(bg_time)
  w = hh_f_wave(eigvec(1), .true.)
  call hh_f_plan(sys, env, sys_bs, env_bs, w, plan, dsb, deb)
  call hh_f_check(hh_lanczos(plan, w, lanzero, 100, hh_precision, e0, iters), 'hh_lanczos')
  call hh_f_wave_get(w, eigvec(1))
  Energys(1) = e0
  Energy0 = e0
  st = hh_plan_free(plan)
  st = hh_basis_free(dsb)
  st = hh_basis_free(deb)
  st = hh_wave_free(w)
  call hh_f_release()
  call cpu_time(end_time)
  open(11, file="Energy_All.dat", position='append')
  write(11, *) "Sys_len=", eigvec(1)%sys_len, "E0=", Energys(1), "Iter=", iters, "time=", end_time - bg_time
  close(11)
end subroutine lanczos_memo_new

! Get_density_matrix_sys_new, code/get_den.f90:103
subroutine Get_density_matrix_sys_new(sys_den, wave, levels)
  use hh_dmrg_f
  implicit none
  integer, intent(in) :: levels
  type(Wavefunction), intent(in) :: wave(levels)
  type(Total_Block), intent(inout) :: sys_den
  call hh_f_density(sys_den, wave, levels, 0)
end subroutine Get_density_matrix_sys_new

! Get_density_matrix_env_new, code/get_den.f90:143
subroutine Get_density_matrix_env_new(env_den, wave, levels)
  use hh_dmrg_f
  implicit none
  integer, intent(in) :: levels
  type(Wavefunction), intent(in) :: wave(levels)
  type(Total_Block), intent(inout) :: env_den
  call hh_f_density(env_den, wave, levels, 1)
end subroutine Get_density_matrix_env_new

! Get_truncation_operator(den_mat,trun_op,trun_err,num_state), code/get_den.f90:184:
! density matrix, per-sector eigensolve, global sort, selection between
! kept_min and kept_max, entropy, and the truncation operator, on the GPU,
! for the wave of the last Get_density_matrix_*_new.
subroutine Get_truncation_operator(den_mat, trun_op, trun_err, num_state)
  use hh_dmrg_f
  implicit none
  real(8), intent(in) :: trun_err
  type(Total_Block), intent(in) :: den_mat
  type(Total_Block), intent(inout) :: trun_op
  integer, intent(inout) :: num_state
  type(c_ptr) :: t
  integer(c_int) :: ns, st
  real(c_double) :: err, ent
  integer :: sys_len
  if (.not. c_associated(hh_den_wave)) then
    write(*, *) 'hh_dmrg_f: Get_truncation_operator without a density matrix'
    stop
  end if
  t = c_null_ptr
  call hh_f_check(hh_density_truncate(hh_ctx, hh_den_wave, hh_den_side, kept_min, kept_max, trun_err, t, ns, &
                                      err, ent, c_null_ptr), 'hh_density_truncate')
  call hh_f_block_get(t, trun_op)
  trun_op%len = den_mat%len
  st = hh_block_free(t)
  st = hh_wave_free(hh_den_wave)
  hh_den_wave = c_null_ptr
  num_state = ns
  Entropys = ent
  if (system_block) then
    sys_len = den_mat%len
  else
    sys_len = Num_site - den_mat%len
  end if
  if (sys_len == Num_site / 2) Entropy0 = Entropys
  open(60, file="Entropy.dat", position='append')
  write(60, *) "N=", Num_site, "N_up=", tot_num_up, "N_down=", tot_num_down, "Err=", err, &
               "Sys_len=", sys_len, "S=", Entropys
  close(60)
end subroutine Get_truncation_operator
