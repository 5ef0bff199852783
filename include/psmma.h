/*
 * psmma.h -- C ABI of the GB300 structured multiply library (libpsmma_gb300.so).
 *
 * The library computes the PSMMA structured products on one GPU:
 *
 *   psmma_cauchy   Q := alpha * A * H + beta * Q,  H(i,j) = U(i)*V(j) / (D(i) - F(j))
 *   psmma_toeplitz Q := alpha * A * H + beta * Q,  H(i,j) = G(K + j - i)          (1-based)
 *   psmma_hankel   Q := alpha * A * H + beta * Q,  H(i,j) = G(i + j - 1)          (1-based)
 *   pzmdftl        C := alpha * F * B + beta * C,  F(j,k) = w^((j-1)(k-1)), w = exp(-2*pi*i/N)
 *
 * A and Q are N-by-K, H is K-by-K, F is N-by-N, B and C are N-by-K.  All matrices are
 * column-major (Fortran order) with an explicit leading dimension, exactly as the
 * reference's local arrays are.  H and F are never stored: every thread block rebuilds
 * the tile it needs from the O(K) generators.
 *
 * Generators keep the reference's storage conventions:
 *   Cauchy   gen is a (ldgen x 4) column-major array [D | F | U | V], ldgen >= K
 *            (PSMMA_CAUCHY's B(LDB,4); psmma_cauchy.f90:22, Auxil_2p5D.f90:138-141).
 *   Toeplitz gen has 2K-1 entries: gen[0..K-1] is the first column from bottom to top,
 *            gen[K-1] the diagonal, gen[K..2K-2] the first row after the diagonal
 *            (psmma_toeplitz.f90:27-32).
 *   Hankel   gen has 2K-1 entries: gen[0..K-1] is the first row, gen[K..2K-2] the last
 *            column below the anti-diagonal (psmma_hankel.f90:27-32).
 *   DFT      the root of unity is implied by N, as in PZMDFTL (pzmdftL.f90:325-326).
 *
 * Entry points taking device pointers enqueue on `stream` (a cudaStream_t, NULL for the
 * legacy default stream) and return without synchronising.  Device-side failures of those
 * calls (a bounded wait that gave up) are recorded per stream and returned by
 * psmma_stream_status(stream).  The *_host entry points take
 * host pointers, copy to the device, run and copy back before returning; they are the
 * drop-in for the reference's host-array calls.
 *
 * Return value: PSMMA_OK (0) or a negative status.  Argument errors return -INFO with the
 * INFO numbering of the reference routine that performs the same check (PXERBLA codes of
 * PSCAUCHY_COMPUTE, pscauchy_compute.f90:234-255, and PZMDFTL, pzmdftL.f90:182-205);
 * the reference prints these and returns nothing, this library returns them.
 */
#ifndef PSMMA_GB300_H
#define PSMMA_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define PSMMA_OK              0
/* -2 (N<0), -3 (K<0), -9 (LDA), -14 (LDQ): PSCAUCHY_COMPUTE INFO numbering.            */
/* -1 (N<0), -2 (K<0), -7 (LDB), -10 (LDC): PZMDFTL INFO numbering.                     */
#define PSMMA_EGEN          -108  /* generator pointer NULL or ldgen too small            */
#define PSMMA_ENULL         -109  /* matrix pointer NULL for a non-empty operand           */
#define PSMMA_ENOMEM        -110  /* device or pinned-host allocation failed              */
#define PSMMA_EDEVICE       -111  /* CUDA launch/runtime error                            */
#define PSMMA_ETIMEDOUT     -112  /* a bounded device-side wait expired                   */
#define PSMMA_ESINGULAR     -113  /* split path: a Cauchy denominator D(i)-F(j) is zero   */
#define PSMMA_EUNSUPPORTED  -114  /* option combination not supported                     */
#define PSMMA_EWORKSPACE    -115  /* caller workspace smaller than psmma_workspace_size   */
#define PSMMA_ERANGE        -116  /* split path: non-finite input or exponent out of range */
#define PSMMA_ESCRATCH      -117  /* request exceeds the fixed scratch of psmma_cauchy_split_noalloc */

/* ---- options ------------------------------------------------------------------------ */
#define PSMMA_PREC_FP64   0   /* plain path: FP64 tensor-core MMA, H tile generated in smem  */
#define PSMMA_PREC_SPLIT  1   /* split path: exact modular slices on BF16 tensor cores (tcgen05),
                                 FP64 scaling and recombination (all four kinds)              */

typedef struct psmma_opts {
  int    precision;   /* PSMMA_PREC_FP64 (default) or PSMMA_PREC_SPLIT                        */
  int    n_moduli;    /* split path: number of moduli, 0 = default (14); 8..16                 */
  void*  work;        /* optional caller-owned device workspace (NULL: library-owned pool)      */
  size_t lwork;       /* size of `work` in bytes                                               */
  int    block_levels; /* split path: Toeplitz / Hankel: levels of the block step (see
                          psmma_split_block_levels): 0 = automatic, -1 = none (one product),
                          1..3 = that many (k padded to a multiple of 64 * 2^L);
                          Cauchy / CAUCHYEIG: 1 = Strassen's step on the residue planes
                          (n even, k divisible by 128; the same result bit for bit, seven
                          half-size modular products instead of eight), else none        */
  int    reserved[7]; /* must be zero                                                          */
} psmma_opts;

/* Interleaved complex double, layout-compatible with cuDoubleComplex and COMPLEX*16. */
typedef struct psmma_complex {
  double re, im;
} psmma_complex;

/* Kinds for psmma_workspace_size. */
#define PSMMA_KIND_CAUCHY   0
#define PSMMA_KIND_TOEPLITZ 1
#define PSMMA_KIND_HANKEL   2
#define PSMMA_KIND_DFT      3
#define PSMMA_KIND_CAUCHY_EIG 5

/* ---- device-pointer entry points --------------------------------------------------- */

/* Replaces PSMMA_CAUCHY(N,K,ALPHA,A,IA,JA,DESCA,B,LDB,BETA,Q,IQ,JQ,DESCQ,WORK,REDIST)
 * (psmma_cauchy.f90:2-3) and its ring kernel PSCAUCHY_COMPUTE (pscauchy_compute.f90:2-3).
 * DESCA/DESCQ become lda/ldq, B/LDB become gen/ldgen, WORK becomes opts->work. */
int psmma_cauchy(int n, int k, double alpha, const double* A, int lda,
                 const double* gen, int ldgen, double beta, double* Q, int ldq,
                 const psmma_opts* opts, void* stream);

/* Replaces PSMMA_TOEPLITZ(...) (psmma_toeplitz.f90:2-3) / PSTOEPLITZ_COMPUTE
 * (pstoeplitz_compute.f90:2-3); gen has ldgen >= 2k-1 entries. */
int psmma_toeplitz(int n, int k, double alpha, const double* A, int lda,
                   const double* gen, int ldgen, double beta, double* Q, int ldq,
                   const psmma_opts* opts, void* stream);

/* Replaces PSMMA_HANKEL(...) (psmma_hankel.f90:2-3) / PSHANKEL_COMPUTE
 * (pshankel_compute.f90:2-3); gen has ldgen >= 2k-1 entries. */
int psmma_hankel(int n, int k, double alpha, const double* A, int lda,
                 const double* gen, int ldgen, double beta, double* Q, int ldq,
                 const psmma_opts* opts, void* stream);

/* Replaces PSMMA_CAUCHYEIG(N,K,ID,ALPHA,A,IA,JA,DESCA,F,D,U,V,DIFL,DIFR,BETA,Q,IQ,JQ,DESCQ,
 * WORK,REDIST) (psmma_cauchyeig.f90:2-3) and PSCAUCHYEIG_COMPUTE (pscauchyeig_compute.f90:2-3),
 * the divide-and-conquer eigensolver's multiply: Q := alpha*A*H + beta*Q with
 * H(i,j) = U(i)*V(j) / (F(i) - D(j)), F the old eigenvalues (sorted) and D(j) in
 * (F(j), F(j+1)) the new ones, given by their distances DIFL(j) = D(j) - F(j) and
 * DIFR(j) = D(j) - F(j+1).  The denominators are formed as (F(i) - F(j)) - DIFL(j) for i <= j
 * and (F(i) - F(j+1)) - DIFR(j) for i > j (CauchylikeEig, CauchyHssEig.f90:1693-1774), so
 * they keep full relative accuracy however close D(j) is to a pole.  F, U, V, DIFL, DIFR have
 * k entries (DIFR(k) is not read); D is accepted for the reference's argument list and not
 * read.  INFO numbers of PSCAUCHYEIG_COMPUTE (pscauchyeig_compute.f90:231-250): N -> -1,
 * K -> -2, LDA -> -7, LDQ -> -17.  Both precisions. */
int psmma_cauchyeig(int n, int k, double alpha, const double* A, int lda, const double* F,
                    const double* D, const double* U, const double* V, const double* difl,
                    const double* difr, double beta, double* Q, int ldq, const psmma_opts* opts,
                    void* stream);

/* Replaces PZMDFTL(N,K,NB,KB,ALPHA,B,LDB,BETA,C,LDC,IMROW,IMCOL,WORK,RWORK)
 * (pzmdftL.f90:1-2): C := alpha*F*B + beta*C with F the N-by-N DFT matrix on the left.
 * The reference's ALPHA and BETA are real (DOUBLE PRECISION); so are these. */
int pzmdftl(int n, int k, double alpha, const psmma_complex* B, int ldb,
            double beta, psmma_complex* C, int ldc, const psmma_opts* opts, void* stream);

/* Replaces PZMDFTL1 (pzmdftL1.f90:1-2), the RRQR variant of PZMDFTL.  Both reference
 * routines compute the same product up to their 1e-13 truncation; on the GPU the DFT
 * tile is generated exactly, so this is the same computation as pzmdftl. */
int pzmdftl1(int n, int k, double alpha, const psmma_complex* B, int ldb,
             double beta, psmma_complex* C, int ldc, const psmma_opts* opts, void* stream);

/* No counterpart in the reference.  The radix R (1, 2, 4 or 8) of the split path's first DFT
 * step for size n: with R > 1, pzmdftl / pzmdftl1 on the split path multiply F_(n/R) by the R k
 * columns B(r::R, :) (n^2 k / R complex multiply-adds on the tensor cores) and combine the R
 * partial transforms with the twiddles w^(j r) and R-point butterflies in FP64; R is the
 * largest of 8, 4, 2 that divides n with n / R >= 1024, else 1.  0 for n <= 0. */
int psmma_split_dft_radix(int n);

/* No counterpart in the reference.  The levels L (0 to 3) of the block step that
 * psmma_toeplitz / psmma_hankel take on the split path (kind PSMMA_KIND_TOEPLITZ or
 * PSMMA_KIND_HANKEL; 0 for the other kinds): H (k x k) is cut into 2 x 2 blocks, and the
 * structure (Toeplitz: Y11 = Y00; Hankel: Y10 = Y01) turns the four block products into three,
 * (X1 + X2) Y00, X2 (Y10 - Y00) and X1 (Y01 - Y00) for Toeplitz; L levels give 3^L products of
 * width w = k / 2^L, (3/4)^L of the modular GEMM work, in exact modular arithmetic.  Columns j
 * and j + c w share one scaling exponent.  Where 64 * 2^L does not divide k, the product runs
 * on an order k' padded up to a multiple of it: H extended with the generator read as zero
 * beyond its 2k - 1 entries (still Toeplitz / Hankel), A with zero columns, and only the first
 * k columns of Q written.  This returns the automatic choice (opts->block_levels = 0): the L
 * in {1, 2} with w = k' / 2^L >= 4096 that minimises the modular GEMM work (k'/k)^2 (3/4)^L,
 * if that is at most 0.85, else 0 (smaller leaves make the modular GEMMs' per-tile epilogue
 * outweigh their MMAs).  The
 * device-pointer calls, the host-pointer calls (in their overlapped row panels) and the server
 * take the step.  On the device, without a synchronisation, the call takes the single product
 * instead when an entry of H is not finite (NaN then appears in exactly the columns it does
 * there) or when a nonzero column's maximum is more than 2^4 below the largest of its group
 * j + c w (the shared exponent would cost that column's entries more than 4 bits).  Cauchy and
 * CAUCHYEIG: 0 (Strassen's step runs only when opts->block_levels asks for it: its operands
 * take 7/4 of the residue planes' HBM traffic, which costs about what it saves). */
int psmma_split_block_levels(int kind, int n, int k);

/* No counterpart in the reference.  The split-path Cauchy multiply (same arguments and
 * result as psmma_cauchy with opts->precision = PSMMA_PREC_SPLIT) for callers that cannot
 * let a library allocate device memory -- they own all of it through their own pool, or
 * run a latency-critical loop where cudaMalloc/cudaFree's device-wide synchronisation is
 * not acceptable.  It allocates nothing: its workspace is a fixed 96 MiB device array of
 * the library (held by every GPU that loads it until exit), so it accepts requests whose
 * split workspace fits in it (n = k = 1024 with the default 14 moduli does) and returns
 * PSMMA_ESCRATCH otherwise.  All calls share that array: calls that overlap on the GPU
 * (other streams or threads) race and must be serialised by the caller.  The first call
 * on a device looks up the array's address and keeps it until the process exits (a
 * cudaDeviceReset afterwards is not supported); make that first call before any stream
 * capture.  Unlike psmma_cauchy, the call blocks: it waits for its work on `stream` and
 * returns the device status, so Q is written when it returns.  alpha = 0 only scales Q by
 * beta (A and gen are not read), as in psmma_cauchy. */
int psmma_cauchy_split_noalloc(int n, int k, double alpha, const double* A, int lda,
                               const double* gen, int ldgen, double beta, double* Q, int ldq,
                               int n_moduli, void* stream);

/* ---- batched merge level with low-rank off-diagonal blocks ------------------------ */
/* Replaces the low-rank branch of PSCAUCHY_COMPUTE (pscauchy_compute.f90:371-391) for a
 * batch of independent Cauchy multiplies, the products of one level of a divide-and-conquer
 * tree.  Each item is Q := alpha*A*H + beta*Q with H (n x n) the Cauchy-like matrix of the
 * item's generators [D|F|U|V] (the psmma_cauchy layout, ldgen >= n).  H is split 2 x 2 at
 * h = n/2; the diagonal blocks are multiplied as generated tiles, and each off-diagonal
 * block H(R,C) is compressed to X*Y and multiplied as (A(:,R)*X)*Y:
 *   PSMMA_COMPRESS_RRQR: the explicit tile is factorised by column-pivoted QR, rank = first
 *     i with |R_ii| <= tol*|R_11| (Compress_RRQR, Auxil_2p5D.f90:1063-1189), X = Q(:,1:Rk),
 *     Y = R(1:Rk,:)*P^T;
 *   PSMMA_COMPRESS_RRLU: the structured rank-revealing LU in generator space (rrluCauchy and
 *     compress_cauchy, Cauchylowrank.f90:7-134, 387-491), X = P^-1 [I; Z], Y = H(PL(1:Rk),:),
 *     both Cauchy-like.
 * A block compressed to full rank is multiplied as a generated tile (the reference reuses a
 * stale buffer there, Cauchylowrank.f90:455-464).  The product phase runs as one CUDA graph.
 * ranks_out (optional) receives 2 ranks per item with n >= 2, in item order: H(1:h, h+1:n)
 * then H(h+1:n, 1:h).  stats (optional) reports the dense-equivalent flops sum(2 n^3), the
 * flops actually executed, the compression flops and the largest rank.  Synchronises
 * `stream` once after the compression (the ranks size the products). */
#define PSMMA_COMPRESS_RRQR 0
#define PSMMA_COMPRESS_RRLU 1

typedef struct psmma_batch_item {
  int n;
  const double* A;    /* n x n, lda */
  int lda;
  const double* gen;  /* [D|F|U|V], ldgen >= n */
  int ldgen;
  double* Q;          /* n x n, ldq */
  int ldq;
} psmma_batch_item;

typedef struct psmma_batch_stats {
  double effective_flops;  /* sum of 2 n^3 */
  double executed_flops;   /* tensor-core products actually run */
  double compress_flops;   /* factorisations (QR: 4 m n r per block; RRLU: O(r (m + n))) */
  int n_blocks;            /* off-diagonal blocks */
  int max_rank;
  int full_rank_blocks;    /* blocks multiplied as generated tiles */
  int graph_reused;        /* 1: the product rounds relaunched the stream's cached CUDA graph,
                              updated in place (cudaGraphExecUpdate); 0: it was instantiated */
} psmma_batch_stats;

int psmma_cauchy_batch_lowrank(int count, const psmma_batch_item* items, double alpha, double beta,
                               int compressor, double tol, const psmma_opts* opts, int* ranks_out,
                               psmma_batch_stats* stats, void* stream);
/* The same merge level for the eigensolver's matrices (PSCAUCHYEIG_COMPUTE's low-rank
 * branch, pscauchyeig_compute.f90:371-391 with ConstCauchyEiglowrank, Auxil_2p5D.f90:642-748):
 * each item's gen is [F|U|V|DIFL|DIFR] (ldgen >= n, the arguments of psmma_cauchyeig) and H
 * has the accurate denominators of CauchylikeEig.  Compressors: PSMMA_COMPRESS_RRLU is the
 * reference's structured rrluCauchyEigrow with Compress_cauchyEig2's factors
 * (CauchyHssEig.f90:7-212, 2640-2829: every F(i) - D(j) and D(j) - D(k) formed from DIFL/DIFR);
 * PSMMA_COMPRESS_RRQR factorises the explicit tiles. */
int psmma_cauchyeig_batch_lowrank(int count, const psmma_batch_item* items, double alpha, double beta,
                                  int compressor, double tol, const psmma_opts* opts, int* ranks_out,
                                  psmma_batch_stats* stats, void* stream);
size_t psmma_cauchyeig_batch_workspace_size(int count, const psmma_batch_item* items, int compressor,
                                            const psmma_opts* opts);

/* The merge level of Toeplitz multiplies (PSTOEPLITZ_COMPUTE's low-rank branch,
 * pstoeplitz_compute.f90:262-294 with ConstToeplitzlowrank, Auxil_2p5D.f90:968-1060): each
 * item's gen is the generator G of psmma_toeplitz (2n - 1 entries; ldgen holds its length), the
 * off-diagonal blocks of H are explicit tiles compressed by the column-pivoted QR of
 * Compress_RRQR (the reference has no structured RRLU for Toeplitz), and a block that does not
 * compress is multiplied as the tile. */
int psmma_toeplitz_batch_lowrank(int count, const psmma_batch_item* items, double alpha, double beta, double tol,
                                 const psmma_opts* opts, int* ranks_out, psmma_batch_stats* stats, void* stream);
size_t psmma_toeplitz_batch_workspace_size(int count, const psmma_batch_item* items, const psmma_opts* opts);

/* No counterpart in the reference.  Autotuner of the split path's grouped GEMM (output-tile
 * widths 64/128/256 by product width, raster group): times psmma_cauchy_batch_lowrank on
 * this batch for each candidate configuration and keeps the fastest for batches of the same
 * signature (count, precision, moduli, compressor and the sizes in 1/8-octave bins), if it
 * beats the default configuration by more than 2 % (else the default is kept); later
 * calls with that signature use it.  With the environment variable PSMMA_TUNE_CACHE naming a
 * file, results are appended there and read back by later processes.  Runs the batch about
 * 40 times: the Q_i are overwritten (meaningless afterwards when beta != 0).  The FP64 path
 * has one tile shape: returns at once. */
typedef struct psmma_tune_result {
  int narrow_max, mid_max, group_m;  /* chosen: width 64 for N <= narrow_max, 128 for N <= mid_max */
  int candidates;                    /* configurations timed */
  float ms_best, ms_default;          /* batch time of the chosen and of the default configuration */
} psmma_tune_result;

int psmma_tune_batch(int count, const psmma_batch_item* items, double alpha, double beta,
                     int compressor, double tol, const psmma_opts* opts, psmma_tune_result* out,
                     void* stream);

/* Bytes of workspace psmma_cauchy_batch_lowrank needs for this batch (for opts->work). */
size_t psmma_batch_workspace_size(int count, const psmma_batch_item* items, int compressor,
                                  const psmma_opts* opts);

/* ---- block-cyclic redistribution (REDIST / PDGEMR2D) -------------------------------- */

/* With REDIST = .TRUE. the reference copies A from its block-cyclic layout to a blocked one
 * and Q back with PDGEMR2D (psmma_cauchy.f90:113-162; the same in psmma_toeplitz.f90,
 * psmma_hankel.f90, psmma_cauchyeig.f90).  Here that copy is: a plan (host, built once per
 * pair of layouts), a pack kernel that gathers this rank's elements into one contiguous
 * segment per destination rank, ONE all-to-all exchange run by the caller (MPI_Alltoallv,
 * NCCL, torch.distributed all_to_all_single) with the plan's counts, and an unpack kernel
 * that scatters the received segments into the destination's local array.
 *
 * A layout is a ScaLAPACK descriptor desc[9] = {DTYPE_=1, CTXT_ (unused), M_, N_, MB_, NB_,
 * RSRC_, CSRC_, LLD_} on a process grid.  The sub-matrix A(ia:ia+m-1, ja:ja+n-1) (1-based)
 * of layout a goes to B(ib:ib+m-1, jb:jb+n-1) of layout b; both grids span the same nprocs
 * processes, `rank` is this process (its grid coordinates follow from the grid's order).
 * Descriptor errors return -(100 * argument position + entry) as ScaLAPACK's CHK1MAT. */
typedef struct psmma_grid {
  int nprow, npcol;
  int order;           /* 0: rank = prow * npcol + pcol (BLACS_GRIDINIT 'R'), 1: column-major ('C') */
} psmma_grid;

typedef struct psmma_redist_plan psmma_redist_plan;

/* ScaLAPACK's NUMROC (0-based process numbers): the local count of an n-vector in blocks of
 * nb on process iproc when block 0 is on isrcproc. */
int psmma_numroc(int n, int nb, int iproc, int isrcproc, int nprocs);
int psmma_redist_plan_create(int m, int n, const int* desca, int ia, int ja, psmma_grid ga,
                             const int* descb, int ib, int jb, psmma_grid gb, int rank,
                             psmma_redist_plan** out);
/* Elements this rank sends to / receives from each rank (nprocs entries each, rank order);
 * segments are packed in rank order, so the displacements are the prefix sums. */
int psmma_redist_counts(const psmma_redist_plan* p, long long* send_counts, long long* recv_counts);
/* This rank's local array shapes (rows x cols) in layout a and layout b. */
int psmma_redist_local_shape(const psmma_redist_plan* p, int* a_rows, int* a_cols, int* b_rows,
                             int* b_cols);
/* The plan's index maps: which = 0/1 rows/cols of the a-local array (the b-grid process row /
 * column that receives each local index, -1 outside the sub-matrix, and its place in that
 * segment), 2/3 rows/cols of the b-local array (the a-grid sender).  Returns the entry count;
 * part/pos may be NULL to query it. */
int psmma_redist_maps(const psmma_redist_plan* p, int which, int* part, int* pos);
/* Device pointers; elem_bytes 8 (double) or 16 (double complex).  The A-local array has
 * leading dimension desca[8], the B-local array descb[8]; the buffers hold the sums of the
 * send / receive counts.  The first call uploads the plan's maps to the current device. */
int psmma_redist_pack(psmma_redist_plan* p, const void* A, void* sendbuf, int elem_bytes, void* stream);
int psmma_redist_unpack(psmma_redist_plan* p, const void* recvbuf, void* B, int elem_bytes, void* stream);
int psmma_redist_plan_destroy(psmma_redist_plan* p);

/* 2.5D helpers (Auxil_2p5D.f90:315-419).  psmma_redist2p5_index is Redist2P5a: the 1-based
 * indices 1..k ordered by process column, columns visited as I + J*(npcol/npzc) with I outer,
 * J < npzc inner, each column's block-cyclic slice in order (npzc must divide npcol).
 * psmma_redist2p5 is Redist2P5 on the device: TB(i,:) = B(pindex(i),:) for the ncb generator
 * columns.  psmma_const_index1 is ConstIndex1: process column mycol's full block segments of a
 * permuted list (cindex = pindex(mycol*nb + s*npcol*nb + 1 .. +nb)); it returns the count
 * written and stops at n where the reference would read past it. */
int psmma_redist2p5_index(int k, int nb, int npzc, int npcol, int* pindex);
int psmma_redist2p5(int k, int nb, int npzc, int npcol, const double* B, int ldb, int ncb, double* TB,
                    int ldtb, void* stream);
int psmma_const_index1(int n, int nb, int mycol, int npcol, const int* pindex, int* cindex);

/* ---- host-pointer entry points (copy in, compute, copy out, synchronise) ------------ */
int psmma_cauchy_host(int n, int k, double alpha, const double* A, int lda,
                      const double* gen, int ldgen, double beta, double* Q, int ldq,
                      const psmma_opts* opts);
int psmma_toeplitz_host(int n, int k, double alpha, const double* A, int lda,
                        const double* gen, int ldgen, double beta, double* Q, int ldq,
                        const psmma_opts* opts);
int psmma_hankel_host(int n, int k, double alpha, const double* A, int lda,
                      const double* gen, int ldgen, double beta, double* Q, int ldq,
                      const psmma_opts* opts);
int pzmdftl_host(int n, int k, double alpha, const psmma_complex* B, int ldb,
                 double beta, psmma_complex* C, int ldc, const psmma_opts* opts);
int psmma_cauchyeig_host(int n, int k, double alpha, const double* A, int lda, const double* F,
                         const double* D, const double* U, const double* V, const double* difl,
                         const double* difr, double beta, double* Q, int ldq, const psmma_opts* opts);

/* ---- Fortran-ABI entry points ------------------------------------------------------ */
/* Same argument lists as the reference's Fortran subroutines, passed by reference with
 * gfortran's trailing-underscore names, on host arrays.  The descriptors must describe a
 * 1x1 process grid (the whole matrix is local): only DESC(9) (LLD) is read.  IA, JA, IQ,
 * JQ must be 1, WORK is not touched and REDIST is ignored (there is nothing to
 * redistribute on one device).  The INFO-style status of the last call is returned by
 * psmma_last_status(). */
void psmma_cauchy_(const int* n, const int* k, const double* alpha, const double* A,
                   const int* ia, const int* ja, const int* desca, const double* B,
                   const int* ldb, const double* beta, double* Q, const int* iq,
                   const int* jq, const int* descq, double* work, const int* redist);
void psmma_toeplitz_(const int* n, const int* k, const double* alpha, const double* A,
                     const int* ia, const int* ja, const int* desca, const double* B,
                     const int* ldb, const double* beta, double* Q, const int* iq,
                     const int* jq, const int* descq, double* work, const int* redist);
void psmma_hankel_(const int* n, const int* k, const double* alpha, const double* A,
                   const int* ia, const int* ja, const int* desca, const double* B,
                   const int* ldb, const double* beta, double* Q, const int* iq,
                   const int* jq, const int* descq, double* work, const int* redist);
void pzmdftl_(const int* n, const int* k, const int* nb, const int* kb, const double* alpha,
              const psmma_complex* B, const int* ldb, const double* beta, psmma_complex* C,
              const int* ldc, const int* imrow, const int* imcol, psmma_complex* work,
              double* rwork);
void pzmdftl1_(const int* n, const int* k, const int* nb, const int* kb, const double* alpha,
               const psmma_complex* B, const int* ldb, const double* beta, psmma_complex* C,
               const int* ldc, const int* imrow, const int* imcol, psmma_complex* work,
               double* rwork);
void psmma_cauchyeig_(const int* n, const int* k, const int* id, const double* alpha,
                      const double* A, const int* ia, const int* ja, const int* desca,
                      const double* F, const double* D, const double* U, const double* V,
                      const double* difl, const double* difr, const double* beta, double* Q,
                      const int* iq, const int* jq, const int* descq, double* work,
                      const int* redist);
int psmma_last_status(void);

/* ---- serving loop (continuous batching) -------------------------------------------- */
/* No counterpart in the reference, whose callers make one blocking call at a time.  A
 * server admits queued requests in arrival order as soon as a stream slot is free and the
 * request's workspace fits in the remaining part of an HBM budget allocated once at
 * creation; admitted requests run concurrently on their own streams, whose priorities follow
 * admission order (the oldest request in flight has the highest).  Operands stay on the
 * device: A/B, generators and Q/C are device pointers owned by the caller, who must keep
 * them alive (and not touch Q/C) until the request completes. */
typedef struct psmma_request {
  int kind;            /* PSMMA_KIND_CAUCHY / _TOEPLITZ / _HANKEL / _DFT / _CAUCHY_EIG           */
  int precision;       /* PSMMA_PREC_FP64 or PSMMA_PREC_SPLIT                                     */
  int n_moduli;        /* split path: 0 = default                                                 */
  int n, k;            /* sizes as in the matching entry point                                    */
  double alpha, beta;
  const void* A;       /* A (double) or, for the DFT, B (psmma_complex)                           */
  int lda;
  const double* gen;   /* generators (unused for the DFT; CAUCHY_EIG: ldgen x 5 [F|U|V|DIFL|DIFR]) */
  int ldgen;
  void* Q;             /* Q (double) or, for the DFT, C (psmma_complex)                           */
  int ldq;
  unsigned long long user_tag;
} psmma_request;

typedef struct psmma_completion {
  unsigned long long ticket, user_tag;
  int status;                    /* status of the request (0 = ok)                              */
  double submit_s, start_s, end_s; /* host monotonic clock: submitted, admitted, completed      */
  float gpu_ms;                  /* CUDA-event time of the request's work on its stream          */
} psmma_completion;

typedef struct psmma_server psmma_server;

/* Creates a server on the current device with an HBM budget (bytes, allocated now) for
 * request workspaces and at most max_inflight concurrent requests (1..64). */
int psmma_server_create(size_t hbm_budget_bytes, int max_inflight, psmma_server** out);
/* Queues a request (argument checks as the direct entry points; PSMMA_ENOMEM if its
 * workspace exceeds the whole budget).  Returns at once with a ticket. */
int psmma_server_submit(psmma_server* s, const psmma_request* r, unsigned long long* ticket);
/* Waits up to timeout_s seconds for a ticket; fills *out and returns the request's status
 * (PSMMA_ETIMEDOUT if the wait itself timed out; the ticket stays valid then). */
int psmma_server_wait(psmma_server* s, unsigned long long ticket, double timeout_s, psmma_completion* out);
/* Number of queued (not yet admitted) and in-flight requests. */
int psmma_server_pending(psmma_server* s, int* queued, int* inflight);
/* Completes in-flight requests, drops queued ones, frees the budget and the streams. */
int psmma_server_destroy(psmma_server* s);

/* ---- workspace and housekeeping ----------------------------------------------------- */

/* Bytes of device workspace a call with these sizes and options needs.  The FP64 path needs
 * none, except for products with too few 128 x 128 output tiles to fill the SMs, which it
 * splits along K into partial sums when workspace is available (0 otherwise).  Pass a buffer
 * at least this large in opts->work to avoid library allocation. */
size_t psmma_workspace_size(int kind, int n, int k, const psmma_opts* opts);

/* Frees the library-owned workspace pools of the current device. */
void psmma_release_workspace(void);

/* Waits for `stream` and returns PSMMA_ETIMEDOUT if a split-path call enqueued on it since the
 * last check recorded a device-side timeout (then clears the record), else PSMMA_OK.  The
 * record is kept per (device, stream handle) in a small device word created by the stream's
 * first split-path call; a stream destroyed before its status was read leaves its record
 * behind, and a new stream that gets the same handle value would inherit it: read the
 * status, or call psmma_stream_release, before destroying a stream. */
int psmma_stream_status(void* stream);

/* Waits for `stream`, frees the status record of (current device, stream) and returns what
 * psmma_stream_status would have returned.  Call it before cudaStreamDestroy on streams that
 * ran split-path calls; a later call on the stream creates a fresh record. */
int psmma_stream_release(void* stream);

/* Per-phase tracing.  While enabled, each call records a CUDA event on its stream after
 * every phase (split path: row scales, H generation, parameters, A residues, H residues,
 * modular GEMMs, CRT recombination; FP64 path: the structured GEMM).  psmma_profile_read
 * waits for the last recorded call and returns its phase times in milliseconds and the
 * phase names (static strings); the return value is the number of phases. */
void psmma_set_profiling(int on);
int psmma_profile_read(float* ms, const char** names, int max_phases);
/* The same marks as a timeline: each mark's time in milliseconds since the call began, in the
 * order they were recorded, waiting for every one of them.  Host-pointer split calls also mark
 * their copy stream (a_panel_up: a row panel of A has landed; q_panel_down: a panel of Q is
 * back on the host), which psmma_profile_read's consecutive differences do not separate. */
int psmma_profile_read_timeline(float* ms, const char** names, int max_phases);

/* No counterpart in the reference.  Self-test of the failure detection: launches a kernel
 * that waits on a device barrier nothing ever releases, with a limit of limit_ns
 * nanoseconds (at most 10 s), and returns PSMMA_ETIMEDOUT when the bounded wait gave up as
 * designed (PSMMA_OK would mean the wait was released, which cannot happen).  The library's
 * pipelined kernels use the same bounded waits with a 2 s limit. */
int psmma_selftest_wait_timeout(unsigned long long limit_ns);

/* No counterpart in the reference.  Self-check of the split path's fast FP64 division
 * (Newton-Raphson refinement of the hardware reciprocal, used for the Cauchy entries
 * U(i)V(j)/(D(i)-F(j))) against the IEEE division on `count` seeded operand pairs:
 * returns the number of results that differ and the largest difference in ulp. */
int psmma_selftest_division(long long count, unsigned long long seed, unsigned long long* mismatches,
                            int* max_ulp);
/* The same check for the split path's H entries u*v/(d-w) (double-float arithmetic on the FP32
 * pipe, with an FP32-seeded FP64 Newton division for operands outside its range): max_ulp
 * bounds the error against the IEEE quotient of the rounded product (the split path is
 * designed for about 2^-45 relative; the test allows 2^-44, 256 ulp). */
int psmma_selftest_division_split(long long count, unsigned long long seed, unsigned long long* mismatches,
                                  int* max_ulp);

/* Text for a status code (static storage). */
const char* psmma_status_string(int status);

/* Library version string. */
const char* psmma_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PSMMA_GB300_H */
