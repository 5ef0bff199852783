! ISO_C_BINDING interface of libpsmma_gb300 for Fortran callers (the C declarations are in
! psmma.h next to this file).
!
! The reference's routines PSMMA_CAUCHY / PSMMA_TOEPLITZ / PSMMA_HANKEL
! (psmma_cauchy.f90:2-3, psmma_toeplitz.f90:2-3, psmma_hankel.f90:2-3), PSMMA_CAUCHYEIG
! (psmma_cauchyeig.f90:2-3) and PZMDFTL / PZMDFTL1 (pzmdftL.f90:1-2, pzmdftL1.f90:1-2) keep
! their argument meaning; the ScaLAPACK descriptors become leading dimensions, WORK becomes
! opts%work, REDIST is the caller's (plan / pack / MPI_Alltoallv / unpack, below).
!   * the *_host functions take ordinary host arrays (copy in, compute, copy out);
!   * the device entry points take device addresses (type(c_ptr): CUDA Fortran device
!     arrays through c_loc, OpenACC host_data use_device, or cudaMalloc'ed memory) and a
!     cudaStream_t (c_null_ptr for the legacy default stream); they return without waiting,
!     psmma_stream_status(stream) waits and reports device-side failures.
! Every function returns 0 or a negative status: the reference's PXERBLA INFO number,
! negated, for argument errors, PSMMA_E* otherwise (psmma_status_string gives the text).
!
! Unchanged reference call sites need no module: the library also exports psmma_cauchy_,
! psmma_toeplitz_, psmma_hankel_, pzmdftl_, pzmdftl1_ and psmma_cauchyeig_ with the
! reference's by-reference argument lists (1 x 1 process grid, host arrays).
!
! Not compiled in this tree: neither the build host nor the GPU host has a Fortran compiler.
! tests/test_capi.py checks that every bind(c) name here is declared in psmma.h and exported
! by the library.
module psmma_gb300
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter, public :: PSMMA_PREC_FP64 = 0, PSMMA_PREC_SPLIT = 1
  integer(c_int), parameter, public :: PSMMA_KIND_CAUCHY = 0, PSMMA_KIND_TOEPLITZ = 1, &
                                       PSMMA_KIND_HANKEL = 2, PSMMA_KIND_DFT = 3, &
                                       PSMMA_KIND_CAUCHY_EIG = 5
  integer(c_int), parameter, public :: PSMMA_COMPRESS_RRQR = 0, PSMMA_COMPRESS_RRLU = 1

  ! psmma_opts: precision, moduli count of the split path (0 = default), optional caller
  ! workspace (device address and bytes), Toeplitz / Hankel block levels of the split path
  ! (0 = automatic, -1 = none), reserved words that must stay zero
  type, bind(c), public :: psmma_opts
     integer(c_int)    :: precision = PSMMA_PREC_FP64
     integer(c_int)    :: n_moduli = 0
     type(c_ptr)       :: work = c_null_ptr
     integer(c_size_t) :: lwork = 0
     integer(c_int)    :: block_levels = 0
     integer(c_int)    :: reserved(7) = 0
  end type psmma_opts

  ! one multiply of a merge level: A (n x n, lda), generators gen (ldgen), Q (ldq), device
  type, bind(c), public :: psmma_batch_item
     integer(c_int) :: n
     type(c_ptr)    :: A
     integer(c_int) :: lda
     type(c_ptr)    :: gen
     integer(c_int) :: ldgen
     type(c_ptr)    :: Q
     integer(c_int) :: ldq
  end type psmma_batch_item

  type, bind(c), public :: psmma_batch_stats
     real(c_double) :: effective_flops, executed_flops, compress_flops
     integer(c_int) :: n_blocks, max_rank, full_rank_blocks, graph_reused
  end type psmma_batch_stats

  type, bind(c), public :: psmma_tune_result
     integer(c_int) :: narrow_max, mid_max, group_m, candidates
     real(c_float)  :: ms_best, ms_default
  end type psmma_tune_result

  ! process grid of a block-cyclic layout: order 0 = BLACS 'R' (row-major ranks), 1 = 'C'
  type, bind(c), public :: psmma_grid
     integer(c_int) :: nprow, npcol, order
  end type psmma_grid

  public :: psmma_cauchy, psmma_toeplitz, psmma_hankel, psmma_cauchyeig, pzmdftl, pzmdftl1, &
            psmma_cauchy_host, psmma_toeplitz_host, psmma_hankel_host, pzmdftl_host, &
            psmma_cauchyeig_host, psmma_cauchy_split_noalloc, psmma_cauchy_batch_lowrank, &
            psmma_cauchyeig_batch_lowrank, psmma_toeplitz_batch_lowrank, psmma_batch_workspace_size, &
            psmma_tune_batch, psmma_workspace_size, psmma_release_workspace, psmma_stream_status, &
            psmma_stream_release, psmma_status_string, psmma_last_status, psmma_numroc, &
            psmma_redist_plan_create, psmma_redist_counts, psmma_redist_pack, psmma_redist_unpack, &
            psmma_redist_plan_destroy

  interface
     ! ---- device-pointer entry points (asynchronous on `stream`) ----------------------
     ! Q := alpha*A*H + beta*Q, H(i,j) = U(i)*V(j)/(D(i)-F(j)), gen = [D|F|U|V] (ldgen x 4)
     integer(c_int) function psmma_cauchy(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts, stream) &
          bind(c, name="psmma_cauchy")
       import :: c_int, c_double, c_ptr, psmma_opts
       integer(c_int), value :: n, k, lda, ldgen, ldq
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: A, gen, Q, stream
       type(psmma_opts), intent(in) :: opts
     end function psmma_cauchy

     ! H(i,j) = G(K+j-i), gen = G (2k-1 entries)
     integer(c_int) function psmma_toeplitz(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts, stream) &
          bind(c, name="psmma_toeplitz")
       import :: c_int, c_double, c_ptr, psmma_opts
       integer(c_int), value :: n, k, lda, ldgen, ldq
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: A, gen, Q, stream
       type(psmma_opts), intent(in) :: opts
     end function psmma_toeplitz

     ! H(i,j) = G(i+j-1), gen = G (2k-1 entries)
     integer(c_int) function psmma_hankel(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts, stream) &
          bind(c, name="psmma_hankel")
       import :: c_int, c_double, c_ptr, psmma_opts
       integer(c_int), value :: n, k, lda, ldgen, ldq
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: A, gen, Q, stream
       type(psmma_opts), intent(in) :: opts
     end function psmma_hankel

     ! the eigensolver's multiply with accurate denominators from DIFL / DIFR (D not read)
     integer(c_int) function psmma_cauchyeig(n, k, alpha, A, lda, F, D, U, V, difl, difr, beta, Q, ldq, &
          opts, stream) bind(c, name="psmma_cauchyeig")
       import :: c_int, c_double, c_ptr, psmma_opts
       integer(c_int), value :: n, k, lda, ldq
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: A, F, D, U, V, difl, difr, Q, stream
       type(psmma_opts), intent(in) :: opts
     end function psmma_cauchyeig

     ! C := alpha*F*B + beta*C, F the N x N DFT matrix on the left, B and C complex*16
     integer(c_int) function pzmdftl(n, k, alpha, B, ldb, beta, C, ldc, opts, stream) &
          bind(c, name="pzmdftl")
       import :: c_int, c_double, c_ptr, psmma_opts
       integer(c_int), value :: n, k, ldb, ldc
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: B, C, stream
       type(psmma_opts), intent(in) :: opts
     end function pzmdftl

     integer(c_int) function pzmdftl1(n, k, alpha, B, ldb, beta, C, ldc, opts, stream) &
          bind(c, name="pzmdftl1")
       import :: c_int, c_double, c_ptr, psmma_opts
       integer(c_int), value :: n, k, ldb, ldc
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: B, C, stream
       type(psmma_opts), intent(in) :: opts
     end function pzmdftl1

     ! ---- host-array entry points (copy in, compute, copy out, synchronise) -----------
     integer(c_int) function psmma_cauchy_host(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts) &
          bind(c, name="psmma_cauchy_host")
       import :: c_int, c_double, psmma_opts
       integer(c_int), value :: n, k, lda, ldgen, ldq
       real(c_double), value :: alpha, beta
       real(c_double), intent(in)    :: A(lda, *), gen(ldgen, 4)
       real(c_double), intent(inout) :: Q(ldq, *)
       type(psmma_opts), intent(in)  :: opts
     end function psmma_cauchy_host

     integer(c_int) function psmma_toeplitz_host(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts) &
          bind(c, name="psmma_toeplitz_host")
       import :: c_int, c_double, psmma_opts
       integer(c_int), value :: n, k, lda, ldgen, ldq
       real(c_double), value :: alpha, beta
       real(c_double), intent(in)    :: A(lda, *), gen(ldgen)
       real(c_double), intent(inout) :: Q(ldq, *)
       type(psmma_opts), intent(in)  :: opts
     end function psmma_toeplitz_host

     integer(c_int) function psmma_hankel_host(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts) &
          bind(c, name="psmma_hankel_host")
       import :: c_int, c_double, psmma_opts
       integer(c_int), value :: n, k, lda, ldgen, ldq
       real(c_double), value :: alpha, beta
       real(c_double), intent(in)    :: A(lda, *), gen(ldgen)
       real(c_double), intent(inout) :: Q(ldq, *)
       type(psmma_opts), intent(in)  :: opts
     end function psmma_hankel_host

     integer(c_int) function pzmdftl_host(n, k, alpha, B, ldb, beta, C, ldc, opts) &
          bind(c, name="pzmdftl_host")
       import :: c_int, c_double, c_double_complex, psmma_opts
       integer(c_int), value :: n, k, ldb, ldc
       real(c_double), value :: alpha, beta
       complex(c_double_complex), intent(in)    :: B(ldb, *)
       complex(c_double_complex), intent(inout) :: C(ldc, *)
       type(psmma_opts), intent(in) :: opts
     end function pzmdftl_host

     integer(c_int) function psmma_cauchyeig_host(n, k, alpha, A, lda, F, D, U, V, difl, difr, beta, Q, &
          ldq, opts) bind(c, name="psmma_cauchyeig_host")
       import :: c_int, c_double, psmma_opts
       integer(c_int), value :: n, k, lda, ldq
       real(c_double), value :: alpha, beta
       real(c_double), intent(in)    :: A(lda, *), F(k), D(k), U(k), V(k), difl(k), difr(k)
       real(c_double), intent(inout) :: Q(ldq, *)
       type(psmma_opts), intent(in)  :: opts
     end function psmma_cauchyeig_host

     ! split-path Cauchy multiply that allocates no device memory (fixed library scratch);
     ! blocks until done; PSMMA_ESCRATCH when the request does not fit the scratch
     integer(c_int) function psmma_cauchy_split_noalloc(n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, &
          n_moduli, stream) bind(c, name="psmma_cauchy_split_noalloc")
       import :: c_int, c_double, c_ptr
       integer(c_int), value :: n, k, lda, ldgen, ldq, n_moduli
       real(c_double), value :: alpha, beta
       type(c_ptr), value    :: A, gen, Q, stream
     end function psmma_cauchy_split_noalloc

     ! ---- batched merge level ------------------------------------------------------------
     integer(c_int) function psmma_cauchy_batch_lowrank(count, items, alpha, beta, compressor, tol, &
          opts, ranks, stats, stream) bind(c, name="psmma_cauchy_batch_lowrank")
       import :: c_int, c_double, c_ptr, psmma_batch_item, psmma_opts, psmma_batch_stats
       integer(c_int), value :: count, compressor
       real(c_double), value :: alpha, beta, tol
       type(psmma_batch_item), intent(in) :: items(*)
       type(psmma_opts), intent(in) :: opts
       integer(c_int), intent(out) :: ranks(*)
       type(psmma_batch_stats), intent(out) :: stats
       type(c_ptr), value :: stream
     end function psmma_cauchy_batch_lowrank

     integer(c_int) function psmma_cauchyeig_batch_lowrank(count, items, alpha, beta, compressor, tol, &
          opts, ranks, stats, stream) bind(c, name="psmma_cauchyeig_batch_lowrank")
       import :: c_int, c_double, c_ptr, psmma_batch_item, psmma_opts, psmma_batch_stats
       integer(c_int), value :: count, compressor
       real(c_double), value :: alpha, beta, tol
       type(psmma_batch_item), intent(in) :: items(*)
       type(psmma_opts), intent(in) :: opts
       integer(c_int), intent(out) :: ranks(*)
       type(psmma_batch_stats), intent(out) :: stats
       type(c_ptr), value :: stream
     end function psmma_cauchyeig_batch_lowrank

     integer(c_int) function psmma_toeplitz_batch_lowrank(count, items, alpha, beta, tol, opts, ranks, &
          stats, stream) bind(c, name="psmma_toeplitz_batch_lowrank")
       import :: c_int, c_double, c_ptr, psmma_batch_item, psmma_opts, psmma_batch_stats
       integer(c_int), value :: count
       real(c_double), value :: alpha, beta, tol
       type(psmma_batch_item), intent(in) :: items(*)
       type(psmma_opts), intent(in) :: opts
       integer(c_int), intent(out) :: ranks(*)
       type(psmma_batch_stats), intent(out) :: stats
       type(c_ptr), value :: stream
     end function psmma_toeplitz_batch_lowrank

     integer(c_size_t) function psmma_batch_workspace_size(count, items, compressor, opts) &
          bind(c, name="psmma_batch_workspace_size")
       import :: c_int, c_size_t, psmma_batch_item, psmma_opts
       integer(c_int), value :: count, compressor
       type(psmma_batch_item), intent(in) :: items(*)
       type(psmma_opts), intent(in) :: opts
     end function psmma_batch_workspace_size

     integer(c_int) function psmma_tune_batch(count, items, alpha, beta, compressor, tol, opts, res, stream) &
          bind(c, name="psmma_tune_batch")
       import :: c_int, c_double, c_ptr, psmma_batch_item, psmma_opts, psmma_tune_result
       integer(c_int), value :: count, compressor
       real(c_double), value :: alpha, beta, tol
       type(psmma_batch_item), intent(in) :: items(*)
       type(psmma_opts), intent(in) :: opts
       type(psmma_tune_result), intent(out) :: res
       type(c_ptr), value :: stream
     end function psmma_tune_batch

     ! ---- workspace, status, housekeeping ------------------------------------------------
     integer(c_size_t) function psmma_workspace_size(kind, n, k, opts) bind(c, name="psmma_workspace_size")
       import :: c_int, c_size_t, psmma_opts
       integer(c_int), value :: kind, n, k
       type(psmma_opts), intent(in) :: opts
     end function psmma_workspace_size

     subroutine psmma_release_workspace() bind(c, name="psmma_release_workspace")
     end subroutine psmma_release_workspace

     integer(c_int) function psmma_stream_status(stream) bind(c, name="psmma_stream_status")
       import :: c_int, c_ptr
       type(c_ptr), value :: stream
     end function psmma_stream_status

     integer(c_int) function psmma_stream_release(stream) bind(c, name="psmma_stream_release")
       import :: c_int, c_ptr
       type(c_ptr), value :: stream
     end function psmma_stream_release

     ! a C string (NUL-terminated); c_f_pointer it to a character array to print
     type(c_ptr) function psmma_status_string(status) bind(c, name="psmma_status_string")
       import :: c_int, c_ptr
       integer(c_int), value :: status
     end function psmma_status_string

     ! status of the last Fortran-ABI call (psmma_cauchy_ ...) on the calling thread
     integer(c_int) function psmma_last_status() bind(c, name="psmma_last_status")
       import :: c_int
     end function psmma_last_status

     ! ---- block-cyclic redistribution (the REDIST branch's PDGEMR2D) ---------------------
     integer(c_int) function psmma_numroc(n, nb, iproc, isrcproc, nprocs) bind(c, name="psmma_numroc")
       import :: c_int
       integer(c_int), value :: n, nb, iproc, isrcproc, nprocs
     end function psmma_numroc

     integer(c_int) function psmma_redist_plan_create(m, n, desca, ia, ja, ga, descb, ib, jb, gb, rank, plan) &
          bind(c, name="psmma_redist_plan_create")
       import :: c_int, c_ptr, psmma_grid
       integer(c_int), value :: m, n, ia, ja, ib, jb, rank
       integer(c_int), intent(in) :: desca(9), descb(9)
       type(psmma_grid), value :: ga, gb
       type(c_ptr), intent(out) :: plan
     end function psmma_redist_plan_create

     integer(c_int) function psmma_redist_counts(plan, send_counts, recv_counts) &
          bind(c, name="psmma_redist_counts")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: plan
       integer(c_long_long), intent(out) :: send_counts(*), recv_counts(*)
     end function psmma_redist_counts

     integer(c_int) function psmma_redist_pack(plan, A, sendbuf, elem_bytes, stream) &
          bind(c, name="psmma_redist_pack")
       import :: c_int, c_ptr
       type(c_ptr), value :: plan, A, sendbuf, stream
       integer(c_int), value :: elem_bytes
     end function psmma_redist_pack

     integer(c_int) function psmma_redist_unpack(plan, recvbuf, B, elem_bytes, stream) &
          bind(c, name="psmma_redist_unpack")
       import :: c_int, c_ptr
       type(c_ptr), value :: plan, recvbuf, B, stream
       integer(c_int), value :: elem_bytes
     end function psmma_redist_unpack

     integer(c_int) function psmma_redist_plan_destroy(plan) bind(c, name="psmma_redist_plan_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: plan
     end function psmma_redist_plan_destroy
  end interface
end module psmma_gb300
