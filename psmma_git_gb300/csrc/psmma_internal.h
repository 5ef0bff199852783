// Internal declarations shared by the CUDA translation units of libpsmma_gb300.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <cstddef>
#include <cstdint>

#include "../../include/psmma.h"

namespace psmma {

enum Kind { KIND_CAUCHY = 0, KIND_TOEPLITZ = 1, KIND_HANKEL = 2, KIND_DFT = 3 };

// FP64 plain path (fp64_structured.cu).  Real GEMM C(MxN) = alpha*X*G + beta*C where one
// operand is streamed (X, column-major, ldx) and the other generated.
int launch_struct_f64(int kind, int M, int N, int K, double alpha, const double* X, long ldx,
                      const double* gen, long ldgen, int korder, const double2* wtab, double beta,
                      double* C, long ldc, cudaStream_t stream);
int launch_dft_table(double2* w, int n, cudaStream_t stream);

// Split path (split_crt.cu).
size_t split_workspace_bytes(int kind, int n, int k, int n_moduli);
int launch_split(int kind, int n, int k, double alpha, const double* A, long lda,
                 const double* gen, long ldgen, double beta, double* Q, long ldq, int n_moduli,
                 void* work, size_t lwork, cudaStream_t stream);
// As launch_split, also for KIND_DFT (A = B and Q = C as interleaved complex, lda/ldq in
// complex elements); with status_dev_out it does not synchronise (the device timeout flag
// is copied there at the end of the stream's work).
int launch_split_any(int kind, int n, int k, double alpha, const double* A, long lda,
                     const double* gen, long ldgen, double beta, double* Q, long ldq, int n_moduli,
                     void* work, size_t lwork, cudaStream_t stream, unsigned* status_dev_out);

// Library-owned device workspace (psmma_capi.cu): grow-only, one pool per (device, stream).
void* pool_get(size_t bytes, cudaStream_t stream, int* status);

// Per-phase tracing (psmma_capi.cu): when enabled, launchers record a CUDA event on the
// launch stream after each phase; psmma_profile_read turns them into milliseconds.
constexpr int PROF_MAX_PHASES = 16;
bool prof_enabled();
void prof_begin(cudaStream_t stream);
void prof_mark(cudaStream_t stream, const char* name);

}  // namespace psmma
