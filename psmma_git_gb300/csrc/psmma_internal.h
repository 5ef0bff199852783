// Internal declarations shared by the CUDA translation units of libpsmma_gb300.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <cstddef>
#include <cstdint>

#include "../../include/psmma.h"

namespace psmma {

enum Kind { KIND_CAUCHY = 0, KIND_TOEPLITZ = 1, KIND_HANKEL = 2, KIND_DFT = 3, KIND_DENSE = 4, KIND_CAUCHY_EIG = 5 };

// Generators of the structured operand H (K x N) of one product.
//   Cauchy    H(i,j) = Ur[i]*Vc[j] / (Dr[i] - Fc[j])   (row and column generators independent)
//   Toeplitz  H(i,j) = g[(order-1) + j - i]           (sub-blocks: g offset by c0 - r0)
//   Hankel    H(i,j) = g[i + j]                        (sub-blocks: g offset by r0 + c0)
//   DFT       embedding of F = (w^(r c mod n_dft)), table wtab (t < n_dft)
//   Dense     H(i,j) = B[i + j*ldb]                   (explicit factors of the low-rank path)
//   CauchyEig H(i,j) = Ur[i]*Vc[j] / den(i,j), the accurate denominators of CauchylikeEig
//             (CauchyHssEig.f90:1693-1774): with Dr = F(rows), Fc = F(cols), Fc1 = F(cols + 1),
//             dl = DIFL(cols), dr = DIFR(cols) and global row <= global column (i - j <= diag_off):
//             den = (Dr[i] - Fc[j]) - dl[j], else (Dr[i] - Fc1[j]) - dr[j]  (Fc1, dr: j < fc1_len)
// Split path only: an H with k1 > 0 has a tail of rows i >= k1, either dense
// (B[(i-k1) + j*ldb]; any kind) or, for Cauchy kinds, Cauchy with its own row generators
// (Dr2, Ur2 at i - k1) and the same column generators.
struct GenSpec {
  int kind = KIND_CAUCHY;
  const double *Dr = nullptr, *Ur = nullptr, *Fc = nullptr, *Vc = nullptr;
  const double* g = nullptr;
  long order = 0;
  // glen > 0: Toeplitz / Hankel indices outside [0, glen) read zero (an H padded beyond the
  // generator's k x k, still Toeplitz / Hankel: the split path's padded block step)
  long glen = 0;
  // srows > 0: only rows [0, srows) count in the column statistics (the rows of a padded H past
  // the real ones multiply zero columns of A)
  long srows = 0;
  const double2* wtab = nullptr;
  int n_dft = 0;
  const double* B = nullptr;
  long ldb = 0;
  int k1 = 0;
  const double *Dr2 = nullptr, *Ur2 = nullptr;
  const double *Fc1 = nullptr, *dl = nullptr, *dr = nullptr;
  int fc1_len = 0, diag_off = 0;
  // CauchyEig rows in a permuted order (the RRLU's Y factor): rglob[i] is the 1-based global
  // index of row i and cg0 the 0-based global index of column 0, so the branch is taken by
  // rglob[i] - 1 <= cg0 + j; rglob2 likewise for Cauchy tail rows (Dr2, Ur2).
  const int *rglob = nullptr, *rglob2 = nullptr;
  int cg0 = 0;
};

#ifdef __CUDACC__
// The denominator F(i) - D(j) of CauchylikeEig with D(j) in (F(j), F(j+1)) given by its
// distances DIFL(j) = D(j) - F(j) and DIFR(j) = D(j) - F(j+1): for i <= j it is
// (F(i) - F(j)) - DIFL(j), else (F(i) - F(j+1)) - DIFR(j) (CauchyHssEig.f90:1759-1763).
__device__ __forceinline__ double eig_den(double fi, double fj, double fj1, double dlj, double drj, bool upper) {
  return upper ? (fi - fj) - dlj : (fi - fj1) - drj;
}
#endif

// The generators of the reference's square H (k x k) from its storage conventions: Cauchy
// [D|F|U|V] with leading dimension ldgen, Toeplitz/Hankel vector of 2k-1.
inline GenSpec reference_gens(int kind, const double* gen, long ldgen, int k) {
  GenSpec g;
  g.kind = kind;
  if (kind == KIND_CAUCHY) {
    g.Dr = gen;
    g.Fc = gen + ldgen;
    g.Ur = gen + 2 * ldgen;
    g.Vc = gen + 3 * ldgen;
  } else {
    g.g = gen;
    g.order = k;
  }
  return g;
}

// The generators of PSMMA_CAUCHYEIG's k x k matrix from a packed (ldgen x 5) array
// [F|U|V|DIFL|DIFR] (the layout of the batch and serving calls).
inline GenSpec eig_gens_packed(const double* gen, long ldgen, int k) {
  GenSpec g;
  g.kind = KIND_CAUCHY_EIG;
  g.Dr = gen;
  g.Fc = gen;
  g.Fc1 = gen + 1;
  g.Ur = gen + ldgen;
  g.Vc = gen + 2 * ldgen;
  g.dl = gen + 3 * ldgen;
  g.dr = gen + 4 * ldgen;
  g.fc1_len = k - 1;
  g.diag_off = 0;
  return g;
}

// cudaFuncSetAttribute(fn, MaxDynamicSharedMemorySize, bytes), after reading any launch error
// still pending from an earlier <<<>>> launch on this thread: the attribute call succeeds and
// clears that error, so without the read a launch the device refused would go unreported.
template <class F>
inline cudaError_t set_smem_attr(F* fn, int bytes) {
  const cudaError_t pending = cudaGetLastError();
  if (pending != cudaSuccess) return pending;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// FP64 plain path (fp64_structured.cu).  Real GEMM C(MxN) = alpha*X*G + beta*C where one
// operand is streamed (X, column-major, ldx) and the other generated.
int launch_struct_f64(int M, int N, int K, double alpha, const double* X, long ldx, const GenSpec& gs,
                      double beta, double* C, long ldc, cudaStream_t stream);
// The same with a workspace for split K (used when the output has too few tiles to fill the
// SMs and lwork >= f64_splitk_bytes); work may be NULL.
int launch_struct_f64_ws(int M, int N, int K, double alpha, const double* X, long ldx, const GenSpec& gs,
                         double beta, double* C, long ldc, void* work, size_t lwork, cudaStream_t stream);
size_t f64_splitk_bytes(int M, int N, int K, int sms);
int launch_dft_table(double2* w, int n, cudaStream_t stream);
// C (n x k complex, ldc) = alpha F_n B + beta C on the FP64 path (plain embedding, or the
// radix-R first step of dft_radix_for(n)); workspace dft_f64_workspace(n, k) bytes.
size_t dft_f64_workspace(int n, int k);
int launch_dft_f64(int n, int k, double alpha, const double* B, long ldb, double beta, double* C, long ldc,
                   void* work, size_t lwork, cudaStream_t stream);
// The DFT's radix step (split_crt.cu): the radix for size n (1, 2, 4 or 8); B' (n/R x R k
// complex) = [B(0::R,:) | ... | B(R-1::R,:)]; C(j + (n/R) s, c) = sum_r w_R^(s r) w_n^(j r)
// P(j, r k + c) + beta C.
int dft_radix_for(int n);
int launch_dft_deinterleave(const double2* B, long ldb, int n, int k, int R, double2* Bp, cudaStream_t stream);
int launch_dft_radix_combine(const double2* P, int nq, int k, const double2* wn, double beta, double2* C, long ldc,
                             int R, cudaStream_t stream);

// Argument checks of PSCAUCHY_COMPUTE / PSTOEPLITZ_COMPUTE / PSHANKEL_COMPUTE on a 1x1 grid
// (psmma_capi.cu): 0 = run, 1 = quick return (nothing to do), else the status to return.
int check_real_args(int kind, int n, int k, double alpha, const double* A, int lda, const double* gen,
                    int ldgen, double beta, const double* Q, int ldq);

// Split path (split_crt.cu).
// block_levels: psmma_opts::block_levels (Toeplitz / Hankel block step; 0 = automatic).
size_t split_workspace_bytes(int kind, int n, int k, int n_moduli, int block_levels = 0);
// wait_status: wait for the call and return its device status (for callers that must not
// allocate); otherwise the status is ORed into the stream's status word (psmma_stream_status).
int launch_split(int kind, int n, int k, double alpha, const double* A, long lda,
                 const double* gen, long ldgen, double beta, double* Q, long ldq, int n_moduli,
                 void* work, size_t lwork, cudaStream_t stream, bool wait_status = false,
                 int block_levels = 0);
// The per-(device, stream) status word the asynchronous calls OR their device status into
// (psmma_capi.cu; created on first use, NULL if that fails).
unsigned* stream_status_word(cudaStream_t stream);
// status_dev_out value asking the split path to wait for the call and return its status.
static unsigned* const kStatusWait = reinterpret_cast<unsigned*>(1);
// As launch_split, also for KIND_DFT (A = B and Q = C as interleaved complex, lda/ldq in
// complex elements).  status_dev_out: nullptr -> ORed into the stream's status word (no
// synchronisation); kStatusWait -> wait and return it; any other pointer receives a copy of
// the device timeout flag at the end of the stream's work (no synchronisation).
int launch_split_any(int kind, int n, int k, double alpha, const double* A, long lda,
                     const double* gen, long ldgen, double beta, double* Q, long ldq, int n_moduli,
                     void* work, size_t lwork, cudaStream_t stream, unsigned* status_dev_out,
                     int block_levels = 0);
// General real product on the split path: Q (M x N) = alpha * A (M x K) * H (K x N) + beta * Q
// with H given by gs (Cauchy, Toeplitz or Hankel).
size_t split_workspace_general(int M, int N, int K, int n_moduli, int block_levels = 0);
// Host-pointer split multiply with the host<->device copies overlapped (split_crt.cu): A
// and Q on the host, dA / dQ device buffers (leading dimension M), the copies on stream cs,
// nev >= 15 events.
int launch_split_host(int kind, int n, int k, double alpha, const double* A_h, long lda_h, double* dA,
                      const double* dgen, long ldgen, double beta, double* Q_h, long ldq_h, double* dQ,
                      int n_moduli, void* work, size_t lwork, cudaStream_t s, cudaStream_t cs, cudaEvent_t* ev,
                      int nev, int block_levels = 0);
int launch_split_host_general(int M, int N, int K, double alpha, const double* A_h, long lda_h, double* dA,
                              const GenSpec& gs, double beta, double* Q_h, long ldq_h, double* dQ, int n_moduli,
                              void* work, size_t lwork, cudaStream_t s, cudaStream_t cs, cudaEvent_t* ev, int nev);
int launch_split_general(int M, int N, int K, double alpha, const double* A, long lda, const GenSpec& gs,
                         double beta, double* Q, long ldq, int n_moduli, void* work, size_t lwork,
                         cudaStream_t stream, unsigned* status_dev_out, int block_levels = 0);

// Grouped split path (split_crt.cu): independent real products of uneven sizes, each
// Q = alpha * A * H + beta * Q (M, N, K >= 1; H from gs, not the DFT), run as one launch
// per phase with one persistent modular GEMM per output-tile width (256, 128, 64).  prepare lays out the workspace and copies the descriptors (not
// capturable: it copies from host memory); enqueue only launches kernels.
struct SplitProblem {
  int M, N, K;
  double alpha, beta;
  const double* A;
  long lda;
  GenSpec gs;
  double* Q;
  long ldq;
  const double* A2 = nullptr;  // columns k >= ka of A come from A2 (ld lda2) at k - ka
  long lda2 = 0;
  int ka = 0;                  // 0: A alone
};
// Tunables of the grouped GEMM: output-tile width 64 for products with N <= narrow_max, 128
// for N <= mid_max, else 256; raster group of group_m row tiles.
struct SplitTune {
  int narrow_max = 64, mid_max = 128, group_m = 12;
};
struct SplitGroup {
  int count = 0, nmod = 0, group_m = 12;
  void* d_probs = nullptr;
  void* d_gemm[3] = {nullptr, nullptr, nullptr};  // tile widths 256, 64, 128
  int n_gemm[3] = {0, 0, 0}, tiles[3] = {0, 0, 0};
  int blocks_row = 0, blocks_h = 0, blocks_ra = 0, blocks_rh = 0, blocks_crt = 0;
  void* small = nullptr;
  size_t small_bytes = 0;
  unsigned* status = nullptr;
};
size_t split_group_bytes(const SplitProblem* P, int count, int n_moduli);
int split_group_prepare(const SplitProblem* P, int count, int n_moduli, const SplitTune& tune, void* work,
                        size_t lwork, cudaStream_t stream, SplitGroup* g);
int split_group_enqueue(const SplitGroup& g, cudaStream_t stream, unsigned* status_out);

// Grouped FP64 path (fp64_structured.cu): products of one kind (Cauchy or dense H) in one
// launch, blocks mapped to (product, tile).
struct F64Prob {
  int M, N, K;
  double alpha, beta;
  const double* X;
  long ldx;
  GenSpec gs;
  double* C;
  long ldc;
};
struct F64Group {
  int count = 0, kind = 0, blocks = 0;
  void* d_args = nullptr;
  int* d_t0 = nullptr;
};
size_t f64_group_bytes(int count);
int f64_group_prepare(const F64Prob* P, int count, void* dev, cudaStream_t stream, F64Group* g);
int f64_group_enqueue(const F64Group& g, cudaStream_t stream);

// Library-owned device workspace (psmma_capi.cu): grow-only, one pool per (device, stream,
// slot); a call that needs two independent regions takes them from two slots.
void* pool_get(size_t bytes, cudaStream_t stream, int* status, int slot = 0);

// Per-phase tracing (psmma_capi.cu): when enabled, launchers record a CUDA event on the
// launch stream after each phase; psmma_profile_read turns them into milliseconds.
constexpr int PROF_MAX_PHASES = 64;
bool prof_enabled();
void prof_begin(cudaStream_t stream);
void prof_mark(cudaStream_t stream, const char* name);

}  // namespace psmma
