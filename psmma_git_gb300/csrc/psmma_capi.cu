// C ABI of libpsmma_gb300: argument checks with the reference's INFO numbering, dispatch
// to the FP64 and split kernels, host-pointer wrappers, Fortran-ABI shims and the
// library-owned workspace pools.
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <utility>

#include "psmma_internal.h"
#include "tcgen05_util.cuh"  // DEV_ERR_TIMEOUT

namespace psmma {

// ------------------------------------------------------------------------------------
// Workspace pools: grow-only device buffers, one per (device, stream).  A pool is only
// reallocated after its stream has drained, so work in flight never loses its buffer.
// ------------------------------------------------------------------------------------
namespace {
struct Pool {
  void* ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_pool_mu;
std::map<std::tuple<int, cudaStream_t, int>, Pool> g_pools;
}  // namespace

void* pool_get(size_t bytes, cudaStream_t stream, int* status, int slot) {
  *status = PSMMA_OK;
  if (bytes == 0) return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { *status = PSMMA_EDEVICE; return nullptr; }
  std::lock_guard<std::mutex> lk(g_pool_mu);
  Pool& pl = g_pools[std::make_tuple(dev, stream, slot)];
  if (pl.bytes >= bytes) return pl.ptr;
  if (pl.ptr) {
    if (cudaStreamSynchronize(stream) != cudaSuccess) { *status = PSMMA_EDEVICE; return nullptr; }
    cudaFree(pl.ptr);
    pl.ptr = nullptr;
    pl.bytes = 0;
  }
  size_t want = (bytes + (1u << 20) - 1) & ~((size_t)(1u << 20) - 1);
  if (cudaMalloc(&pl.ptr, want) != cudaSuccess) {
    cudaGetLastError();
    pl.ptr = nullptr;
    *status = PSMMA_ENOMEM;
    return nullptr;
  }
  pl.bytes = want;
  return pl.ptr;
}

// ------------------------------------------------------------------------------------
// Per-(device, stream) status words: the split path's asynchronous calls OR their device
// status (DEV_ERR_TIMEOUT when a bounded wait gave up) into the word of their stream;
// psmma_stream_status waits for the stream, reads and clears it.
// ------------------------------------------------------------------------------------
std::mutex g_stw_mu;
std::map<std::pair<int, cudaStream_t>, unsigned*> g_stw;

unsigned* stream_status_word(cudaStream_t stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_stw_mu);
  auto it = g_stw.find({dev, stream});
  if (it != g_stw.end()) return it->second;
  unsigned* w = nullptr;
  if (cudaMalloc(&w, 256) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemsetAsync(w, 0, sizeof(unsigned), stream) != cudaSuccess) {
    cudaFree(w);
    return nullptr;
  }
  g_stw[{dev, stream}] = w;
  return w;
}

// ------------------------------------------------------------------------------------
// Per-phase tracing with CUDA events on the launch stream (single recording slot).
// ------------------------------------------------------------------------------------
namespace {
std::mutex g_prof_mu;
bool g_prof_on = false;
int g_prof_n = 0;
cudaEvent_t g_prof_ev[PROF_MAX_PHASES + 1];
const char* g_prof_name[PROF_MAX_PHASES + 1];
bool g_prof_created = false;
}  // namespace

bool prof_enabled() { return g_prof_on; }

// Phases inside a stream capture are not traced (their events would belong to the graph).
static bool capturing(cudaStream_t stream) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

void prof_begin(cudaStream_t stream) {
  if (!g_prof_on || capturing(stream)) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_created) {
    for (int i = 0; i <= PROF_MAX_PHASES; ++i) cudaEventCreate(&g_prof_ev[i]);
    g_prof_created = true;
  }
  g_prof_n = 0;
  cudaEventRecord(g_prof_ev[0], stream);
  g_prof_name[0] = "begin";
  g_prof_n = 1;
}

void prof_mark(cudaStream_t stream, const char* name) {
  if (!g_prof_on || capturing(stream)) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (g_prof_n > PROF_MAX_PHASES) return;
  cudaEventRecord(g_prof_ev[g_prof_n], stream);
  g_prof_name[g_prof_n] = name;
  g_prof_n++;
}

namespace {

const psmma_opts kDefaultOpts = {PSMMA_PREC_FP64, 0, nullptr, 0, 0, {0, 0, 0, 0, 0, 0, 0}};

int check_opts(const psmma_opts* o, int kind) {
  if (o->precision != PSMMA_PREC_FP64 && o->precision != PSMMA_PREC_SPLIT) return PSMMA_EUNSUPPORTED;
  if (o->n_moduli != 0 && (o->n_moduli < 8 || o->n_moduli > 16)) return PSMMA_EUNSUPPORTED;
  if (o->block_levels < -1 || o->block_levels > 3) return PSMMA_EUNSUPPORTED;
  for (int i = 0; i < 7; i++)
    if (o->reserved[i] != 0) return PSMMA_EUNSUPPORTED;
  return PSMMA_OK;
}

// Argument checks of PSCAUCHY_COMPUTE / PSTOEPLITZ_COMPUTE / PSHANKEL_COMPUTE
// (pscauchy_compute.f90:234-255, 298-311 on a 1x1 grid where MP = N).
int check_real(int kind, int n, int k, double alpha, const double* A, int lda, const double* gen,
               int ldgen, double beta, const double* Q, int ldq) {
  if (n < 0) return -2;
  if (k < 0) return -3;
  if (lda < std::max(1, n)) return -9;
  if (ldq < std::max(1, n)) return -14;
  if (n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return 1;  // quick return
  if (k == 0) return 1;
  if (!Q) return PSMMA_ENULL;
  if (alpha != 0.0) {
    if (!A) return PSMMA_ENULL;
    if (!gen) return PSMMA_EGEN;
    long need = (kind == KIND_CAUCHY) ? (long)k : 2L * k - 1;
    if (ldgen < need) return PSMMA_EGEN;
  }
  return PSMMA_OK;
}

// Argument checks of PZMDFTL (pzmdftL.f90:182-205, 279-284 on a 1x1 grid).
int check_dft(int n, int k, double alpha, const void* B, int ldb, double beta, const void* C, int ldc) {
  if (n < 0) return -1;
  if (k < 0) return -2;
  if (ldb < std::max(1, n)) return -7;
  if (ldc < std::max(1, n)) return -10;
  if (n == 0 || k == 0 || (alpha == 0.0 && beta == 1.0)) return 1;  // quick return
  if (!C) return PSMMA_ENULL;
  if (alpha != 0.0 && !B) return PSMMA_ENULL;
  return PSMMA_OK;
}

// SMs of the current device (0 on error).
int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  return sms;
}

// Split-K partials of the FP64 path for a product with too few output tiles to fill the SMs:
// the caller's opts->work when it is large enough, else (no caller workspace) the stream's
// pool, slot 2.  NULL (no split) when the product fills the SMs or the caller's buffer is short.
void* f64_work(int M, int N, int K, const psmma_opts* o, cudaStream_t s, size_t* bytes, int* st) {
  *st = PSMMA_OK;
  *bytes = 0;
  const int sms = device_sms();
  const size_t need = sms ? f64_splitk_bytes(M, N, K, sms) : 0;
  if (!need) return nullptr;
  if (o->work) {
    if (o->lwork < need) return nullptr;
    *bytes = need;
    return o->work;
  }
  void* w = pool_get(need, s, st, 2);
  if (*st) return nullptr;
  *bytes = need;
  return w;
}

int run_real(int kind, int n, int k, double alpha, const double* A, int lda, const double* gen,
             int ldgen, double beta, double* Q, int ldq, const psmma_opts* opts, void* stream) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  int st = check_opts(o, kind);
  if (st) return st;
  st = check_real(kind, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (o->precision == PSMMA_PREC_SPLIT && alpha != 0.0) {
    size_t need = split_workspace_bytes(kind, n, k, o->n_moduli, o->block_levels);
    void* work = o->work;
    if (work) {
      if (o->lwork < need) return PSMMA_EWORKSPACE;
    } else {
      work = pool_get(need, s, &st);
      if (st) return st;
    }
    return launch_split(kind, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, o->n_moduli, work,
                        need, s, false, o->block_levels);
  }
  size_t wb = 0;
  void* w = f64_work(n, k, k, o, s, &wb, &st);
  if (st) return st;
  return launch_struct_f64_ws(n, k, k, alpha, A, lda, reference_gens(kind, gen, ldgen, k), beta, Q, ldq, w, wb, s);
}

int run_dft(int n, int k, double alpha, const psmma_complex* B, int ldb, double beta,
            psmma_complex* C, int ldc, const psmma_opts* opts, void* stream) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  int st = check_opts(o, KIND_DFT);
  if (st) return st;
  st = check_dft(n, k, alpha, B, ldb, beta, C, ldc);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (o->precision == PSMMA_PREC_SPLIT && alpha != 0.0) {
    size_t need = split_workspace_bytes(KIND_DFT, n, k, o->n_moduli);
    void* work = o->work;
    if (work) {
      if (o->lwork < need) return PSMMA_EWORKSPACE;
    } else {
      work = pool_get(need, s, &st);
      if (st) return st;
    }
    return launch_split_any(KIND_DFT, n, k, alpha, (const double*)B, ldb, nullptr, 0, beta, (double*)C, ldc,
                            o->n_moduli, work, need, s, nullptr);
  }
  if (alpha == 0.0) {  // C := beta C (B not read)
    GenSpec gs;
    gs.kind = KIND_DFT;
    return launch_struct_f64(2 * n, k, 2 * n, 0.0, nullptr, 2L * ldb, gs, beta, (double*)C, 2L * ldc, s);
  }
  const size_t need = dft_f64_workspace(n, k);
  void* work = o->work;
  if (work) {
    if (o->lwork < need) return PSMMA_EWORKSPACE;
  } else {
    work = pool_get(need, s, &st);
    if (st) return st;
  }
  return launch_dft_f64(n, k, alpha, (const double*)B, ldb, beta, (double*)C, ldc, work, need, s);
}

// ---- host-pointer wrappers -------------------------------------------------------------
struct HostArena {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy = nullptr;  // host<->device copies of the overlapped split path
  cudaEvent_t ev[28] = {};
  bool have_ev = false;
};
constexpr int kHostEvents = 28;
std::mutex g_host_mu;
std::map<int, HostArena> g_host;

// Returns a device buffer of >= bytes and the library stream of the current device.
void* host_arena(size_t bytes, cudaStream_t* stream, int* status) {
  *status = PSMMA_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { *status = PSMMA_EDEVICE; return nullptr; }
  HostArena& a = g_host[dev];
  if (!a.stream && cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking) != cudaSuccess) {
    *status = PSMMA_EDEVICE;
    return nullptr;
  }
  *stream = a.stream;
  if (a.bytes < bytes) {
    if (a.ptr) cudaFree(a.ptr);
    a.ptr = nullptr;
    a.bytes = 0;
    size_t want = (bytes + (1u << 20) - 1) & ~((size_t)(1u << 20) - 1);
    if (cudaMalloc(&a.ptr, want) != cudaSuccess) {
      cudaGetLastError();
      *status = PSMMA_ENOMEM;
      return nullptr;
    }
    a.bytes = want;
  }
  return a.ptr;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The copy stream and events of the current device's arena (created on first use).
int host_copy_stream(cudaStream_t* cs, cudaEvent_t** ev) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PSMMA_EDEVICE;
  HostArena& a = g_host[dev];
  if (!a.copy && cudaStreamCreateWithFlags(&a.copy, cudaStreamNonBlocking) != cudaSuccess) return PSMMA_EDEVICE;
  if (!a.have_ev) {
    for (int i = 0; i < kHostEvents; ++i)
      if (cudaEventCreateWithFlags(&a.ev[i], cudaEventDisableTiming) != cudaSuccess) return PSMMA_EDEVICE;
    a.have_ev = true;
  }
  *cs = a.copy;
  *ev = a.ev;
  return PSMMA_OK;
}

// Split-path workspace for a host-pointer call: the caller's opts->work or the pool of s.
void* host_split_work(size_t need, const psmma_opts* o, cudaStream_t s, int* st) {
  *st = PSMMA_OK;
  if (o->work) {
    if (o->lwork < need) { *st = PSMMA_EWORKSPACE; return nullptr; }
    return o->work;
  }
  return pool_get(need, s, st);
}

int host_real(int kind, int n, int k, double alpha, const double* A, int lda, const double* gen,
              int ldgen, double beta, double* Q, int ldq, const psmma_opts* opts) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  int st = check_opts(o, kind);
  if (st) return st;
  st = check_real(kind, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_host_mu);
  long glen = (alpha == 0.0) ? 0 : ((kind == KIND_CAUCHY) ? 4L * k : 2L * k - 1);
  size_t bA = align256((size_t)n * k * 8), bG = align256((size_t)glen * 8), bQ = align256((size_t)n * k * 8);
  cudaStream_t s;
  char* base = (char*)host_arena(bA + bG + bQ, &s, &st);
  if (st) return st;
  double* dA = (double*)base;
  double* dG = (double*)(base + bA);
  double* dQ = (double*)(base + bA + bG);
  bool ok = true;
  const bool overlapped = o->precision == PSMMA_PREC_SPLIT && alpha != 0.0;
  if (alpha != 0.0) {
    if (!overlapped)
      ok &= cudaMemcpy2DAsync(dA, (size_t)n * 8, A, (size_t)lda * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice, s) ==
            cudaSuccess;
    if (kind == KIND_CAUCHY)
      ok &= cudaMemcpy2DAsync(dG, (size_t)k * 8, gen, (size_t)ldgen * 8, (size_t)k * 8, 4, cudaMemcpyHostToDevice, s) == cudaSuccess;
    else
      ok &= cudaMemcpyAsync(dG, gen, (size_t)glen * 8, cudaMemcpyHostToDevice, s) == cudaSuccess;
  }
  if (o->precision == PSMMA_PREC_SPLIT && alpha != 0.0) {
    // generators are up (A and Q travel inside the overlapped pipeline)
    if (!ok) return PSMMA_EDEVICE;
    cudaStream_t cs;
    cudaEvent_t* ev;
    st = host_copy_stream(&cs, &ev);
    if (st) return st;
    const size_t need = split_workspace_bytes(kind, n, k, o->n_moduli, o->block_levels);
    void* work = host_split_work(need, o, s, &st);
    if (st) return st;
    st = launch_split_host(kind, n, k, alpha, A, lda, dA, dG, (kind == KIND_CAUCHY) ? k : (int)glen, beta, Q, ldq,
                           dQ, o->n_moduli, work, o->work ? o->lwork : need, s, cs, ev, kHostEvents, o->block_levels);
    if (st) {
      cudaStreamSynchronize(s);
      cudaStreamSynchronize(cs);
    }
    return st;
  }
  if (beta != 0.0)
    ok &= cudaMemcpy2DAsync(dQ, (size_t)n * 8, Q, (size_t)ldq * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (!ok) return PSMMA_EDEVICE;
  psmma_opts o2 = *o;
  st = run_real(kind, n, k, alpha, dA, n, dG, (kind == KIND_CAUCHY) ? k : (int)glen, beta, dQ, n, &o2, s);
  if (st) { cudaStreamSynchronize(s); return st; }
  ok &= cudaMemcpy2DAsync(Q, (size_t)ldq * 8, dQ, (size_t)n * 8, (size_t)n * 8, k, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  ok &= cudaStreamSynchronize(s) == cudaSuccess;
  return ok ? PSMMA_OK : PSMMA_EDEVICE;
}

// ---- accurate-denominator Cauchy (PSMMA_CAUCHYEIG) -----------------------------------------
GenSpec eig_gens(const double* F, const double* U, const double* V, const double* difl, const double* difr, int k) {
  GenSpec g;
  g.kind = KIND_CAUCHY_EIG;
  g.Dr = F;      // F(i), rows
  g.Ur = U;
  g.Fc = F;      // F(j), columns
  g.Fc1 = F + 1; // F(j+1)
  g.Vc = V;
  g.dl = difl;
  g.dr = difr;
  g.fc1_len = k - 1;
  g.diag_off = 0;
  return g;
}

// Argument checks of PSCAUCHYEIG_COMPUTE (pscauchyeig_compute.f90:231-250: N -> 1, K -> 2,
// LDA -> 7, LDC -> 17), with the leading dimensions checked against N as a 1x1 grid needs.
int check_eig(int n, int k, double alpha, const double* A, int lda, const double* F, const double* U,
              const double* V, const double* difl, const double* difr, double beta, const double* Q, int ldq) {
  if (n < 0) return -1;
  if (k < 0) return -2;
  if (lda < std::max(1, n)) return -7;
  if (ldq < std::max(1, n)) return -17;
  if (n == 0 || k == 0 || (alpha == 0.0 && beta == 1.0)) return 1;  // quick return
  if (!Q) return PSMMA_ENULL;
  if (alpha != 0.0) {
    if (!A) return PSMMA_ENULL;
    if (!F || !U || !V || !difl || (k > 1 && !difr)) return PSMMA_EGEN;
  }
  return PSMMA_OK;
}

int run_eig(int n, int k, double alpha, const double* A, int lda, const double* F, const double* U,
            const double* V, const double* difl, const double* difr, double beta, double* Q, int ldq,
            const psmma_opts* opts, void* stream) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  int st = check_opts(o, KIND_CAUCHY);
  if (st) return st;
  st = check_eig(n, k, alpha, A, lda, F, U, V, difl, difr, beta, Q, ldq);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const GenSpec gs = eig_gens(F, U, V, difl, difr, k);
  if (o->precision == PSMMA_PREC_SPLIT && alpha != 0.0) {
    size_t need = split_workspace_general(n, k, k, o->n_moduli, o->block_levels);
    void* work = o->work;
    if (work) {
      if (o->lwork < need) return PSMMA_EWORKSPACE;
    } else {
      work = pool_get(need, s, &st);
      if (st) return st;
    }
    unsigned* dstat = nullptr;
    return launch_split_general(n, k, k, alpha, A, lda, gs, beta, Q, ldq, o->n_moduli, work, need, s, dstat,
                                o->block_levels);
  }
  size_t wb = 0;
  void* w = f64_work(n, k, k, o, s, &wb, &st);
  if (st) return st;
  return launch_struct_f64_ws(n, k, k, alpha, A, lda, gs, beta, Q, ldq, w, wb, s);
}

int host_eig(int n, int k, double alpha, const double* A, int lda, const double* F, const double* U,
             const double* V, const double* difl, const double* difr, double beta, double* Q, int ldq,
             const psmma_opts* opts) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  int st = check_opts(o, KIND_CAUCHY);
  if (st) return st;
  st = check_eig(n, k, alpha, A, lda, F, U, V, difl, difr, beta, Q, ldq);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_host_mu);
  const size_t bA = align256((size_t)n * k * 8), bG = align256((size_t)5 * k * 8), bQ = align256((size_t)n * k * 8);
  cudaStream_t s;
  char* base = (char*)host_arena(bA + bG + bQ, &s, &st);
  if (st) return st;
  double* dA = (double*)base;
  double* dG = (double*)(base + bA);  // F, U, V, DIFL, DIFR, k each
  double* dQ = (double*)(base + bA + bG);
  bool ok = true;
  const bool overlapped = o->precision == PSMMA_PREC_SPLIT && alpha != 0.0;
  if (alpha != 0.0) {
    if (!overlapped)
      ok &= cudaMemcpy2DAsync(dA, (size_t)n * 8, A, (size_t)lda * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice, s) ==
            cudaSuccess;
    const double* src[5] = {F, U, V, difl, difr};
    for (int t = 0; t < 5; ++t)
      if (src[t]) ok &= cudaMemcpyAsync(dG + (size_t)t * k, src[t], (size_t)k * 8, cudaMemcpyHostToDevice, s) == cudaSuccess;
  }
  if (overlapped) {
    if (!ok) return PSMMA_EDEVICE;
    cudaStream_t cs;
    cudaEvent_t* ev;
    st = host_copy_stream(&cs, &ev);
    if (st) return st;
    const size_t need = split_workspace_general(n, k, k, o->n_moduli);
    void* work = host_split_work(need, o, s, &st);
    if (st) return st;
    const GenSpec gs = eig_gens(dG, dG + k, dG + 2 * (size_t)k, dG + 3 * (size_t)k, dG + 4 * (size_t)k, k);
    st = launch_split_host_general(n, k, k, alpha, A, lda, dA, gs, beta, Q, ldq, dQ, o->n_moduli, work,
                                   o->work ? o->lwork : need, s, cs, ev, kHostEvents);
    if (st) {
      cudaStreamSynchronize(s);
      cudaStreamSynchronize(cs);
    }
    return st;
  }
  if (beta != 0.0)
    ok &= cudaMemcpy2DAsync(dQ, (size_t)n * 8, Q, (size_t)ldq * 8, (size_t)n * 8, k, cudaMemcpyHostToDevice, s) ==
          cudaSuccess;
  if (!ok) return PSMMA_EDEVICE;
  st = run_eig(n, k, alpha, dA, n, dG, dG + k, dG + 2 * (size_t)k, dG + 3 * (size_t)k, dG + 4 * (size_t)k, beta, dQ,
               n, o, s);
  if (st) {
    cudaStreamSynchronize(s);
    return st;
  }
  ok &= cudaMemcpy2DAsync(Q, (size_t)ldq * 8, dQ, (size_t)n * 8, (size_t)n * 8, k, cudaMemcpyDeviceToHost, s) ==
        cudaSuccess;
  ok &= cudaStreamSynchronize(s) == cudaSuccess;
  return ok ? PSMMA_OK : PSMMA_EDEVICE;
}

int host_dft(int n, int k, double alpha, const psmma_complex* B, int ldb, double beta,
             psmma_complex* C, int ldc, const psmma_opts* opts) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  int st = check_opts(o, KIND_DFT);
  if (st) return st;
  st = check_dft(n, k, alpha, B, ldb, beta, C, ldc);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_host_mu);
  size_t bB = align256((size_t)n * k * 16), bC = bB;
  cudaStream_t s;
  char* base = (char*)host_arena(bB + bC, &s, &st);
  if (st) return st;
  psmma_complex* dB = (psmma_complex*)base;
  psmma_complex* dC = (psmma_complex*)(base + bB);
  bool ok = true;
  if (alpha != 0.0)
    ok &= cudaMemcpy2DAsync(dB, (size_t)n * 16, B, (size_t)ldb * 16, (size_t)n * 16, k, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (beta != 0.0)
    ok &= cudaMemcpy2DAsync(dC, (size_t)n * 16, C, (size_t)ldc * 16, (size_t)n * 16, k, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (!ok) return PSMMA_EDEVICE;
  st = run_dft(n, k, alpha, dB, n, beta, dC, n, o, s);
  if (st) { cudaStreamSynchronize(s); return st; }
  ok &= cudaMemcpy2DAsync(C, (size_t)ldc * 16, dC, (size_t)n * 16, (size_t)n * 16, k, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  ok &= cudaStreamSynchronize(s) == cudaSuccess;
  return ok ? PSMMA_OK : PSMMA_EDEVICE;
}

thread_local int g_last_status = PSMMA_OK;

}  // namespace

int check_real_args(int kind, int n, int k, double alpha, const double* A, int lda, const double* gen,
                    int ldgen, double beta, const double* Q, int ldq) {
  return check_real(kind, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq);
}

}  // namespace psmma

using namespace psmma;

extern "C" {

int psmma_cauchy(int n, int k, double alpha, const double* A, int lda, const double* gen, int ldgen,
                 double beta, double* Q, int ldq, const psmma_opts* opts, void* stream) {
  return run_real(KIND_CAUCHY, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts, stream);
}
int psmma_toeplitz(int n, int k, double alpha, const double* A, int lda, const double* gen,
                   int ldgen, double beta, double* Q, int ldq, const psmma_opts* opts, void* stream) {
  return run_real(KIND_TOEPLITZ, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts, stream);
}
int psmma_hankel(int n, int k, double alpha, const double* A, int lda, const double* gen, int ldgen,
                 double beta, double* Q, int ldq, const psmma_opts* opts, void* stream) {
  return run_real(KIND_HANKEL, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts, stream);
}
int pzmdftl(int n, int k, double alpha, const psmma_complex* B, int ldb, double beta,
            psmma_complex* C, int ldc, const psmma_opts* opts, void* stream) {
  return run_dft(n, k, alpha, B, ldb, beta, C, ldc, opts, stream);
}
int pzmdftl1(int n, int k, double alpha, const psmma_complex* B, int ldb, double beta,
             psmma_complex* C, int ldc, const psmma_opts* opts, void* stream) {
  return run_dft(n, k, alpha, B, ldb, beta, C, ldc, opts, stream);
}

int psmma_cauchy_host(int n, int k, double alpha, const double* A, int lda, const double* gen,
                      int ldgen, double beta, double* Q, int ldq, const psmma_opts* opts) {
  return host_real(KIND_CAUCHY, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts);
}
int psmma_toeplitz_host(int n, int k, double alpha, const double* A, int lda, const double* gen,
                        int ldgen, double beta, double* Q, int ldq, const psmma_opts* opts) {
  return host_real(KIND_TOEPLITZ, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts);
}
int psmma_hankel_host(int n, int k, double alpha, const double* A, int lda, const double* gen,
                      int ldgen, double beta, double* Q, int ldq, const psmma_opts* opts) {
  return host_real(KIND_HANKEL, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, opts);
}
int pzmdftl_host(int n, int k, double alpha, const psmma_complex* B, int ldb, double beta,
                 psmma_complex* C, int ldc, const psmma_opts* opts) {
  return host_dft(n, k, alpha, B, ldb, beta, C, ldc, opts);
}

// Fortran ABI: by-reference arguments, 1x1 grid descriptors (LLD = DESC(9)).
void psmma_cauchy_(const int* n, const int* k, const double* alpha, const double* A, const int*,
                   const int*, const int* desca, const double* B, const int* ldb, const double* beta,
                   double* Q, const int*, const int*, const int* descq, double*, const int*) {
  g_last_status = host_real(KIND_CAUCHY, *n, *k, *alpha, A, desca[8], B, *ldb, *beta, Q, descq[8], nullptr);
}
void psmma_toeplitz_(const int* n, const int* k, const double* alpha, const double* A, const int*,
                     const int*, const int* desca, const double* B, const int* ldb, const double* beta,
                     double* Q, const int*, const int*, const int* descq, double*, const int*) {
  g_last_status = host_real(KIND_TOEPLITZ, *n, *k, *alpha, A, desca[8], B, *ldb, *beta, Q, descq[8], nullptr);
}
void psmma_hankel_(const int* n, const int* k, const double* alpha, const double* A, const int*,
                   const int*, const int* desca, const double* B, const int* ldb, const double* beta,
                   double* Q, const int*, const int*, const int* descq, double*, const int*) {
  g_last_status = host_real(KIND_HANKEL, *n, *k, *alpha, A, desca[8], B, *ldb, *beta, Q, descq[8], nullptr);
}
int psmma_cauchyeig(int n, int k, double alpha, const double* A, int lda, const double* F, const double* D,
                    const double* U, const double* V, const double* difl, const double* difr, double beta,
                    double* Q, int ldq, const psmma_opts* opts, void* stream) {
  (void)D;  // the updated eigenvalues enter through DIFL/DIFR (CauchylikeEig does not read D)
  return run_eig(n, k, alpha, A, lda, F, U, V, difl, difr, beta, Q, ldq, opts, stream);
}
int psmma_cauchyeig_host(int n, int k, double alpha, const double* A, int lda, const double* F, const double* D,
                         const double* U, const double* V, const double* difl, const double* difr, double beta,
                         double* Q, int ldq, const psmma_opts* opts) {
  (void)D;
  return host_eig(n, k, alpha, A, lda, F, U, V, difl, difr, beta, Q, ldq, opts);
}
void psmma_cauchyeig_(const int* n, const int* k, const int*, const double* alpha, const double* A, const int*,
                      const int*, const int* desca, const double* F, const double* D, const double* U,
                      const double* V, const double* difl, const double* difr, const double* beta, double* Q,
                      const int*, const int*, const int* descq, double*, const int*) {
  (void)D;
  g_last_status = host_eig(*n, *k, *alpha, A, desca[8], F, U, V, difl, difr, *beta, Q, descq[8], nullptr);
}
void pzmdftl_(const int* n, const int* k, const int*, const int*, const double* alpha,
              const psmma_complex* B, const int* ldb, const double* beta, psmma_complex* C,
              const int* ldc, const int*, const int*, psmma_complex*, double*) {
  g_last_status = host_dft(*n, *k, *alpha, B, *ldb, *beta, C, *ldc, nullptr);
}
void pzmdftl1_(const int* n, const int* k, const int*, const int*, const double* alpha,
               const psmma_complex* B, const int* ldb, const double* beta, psmma_complex* C,
               const int* ldc, const int*, const int*, psmma_complex*, double*) {
  g_last_status = host_dft(*n, *k, *alpha, B, *ldb, *beta, C, *ldc, nullptr);
}
int psmma_last_status(void) { return g_last_status; }

size_t psmma_workspace_size(int kind, int n, int k, const psmma_opts* opts) {
  const psmma_opts* o = opts ? opts : &kDefaultOpts;
  if (n <= 0 || k <= 0) return 0;
  if (kind < KIND_CAUCHY || kind > KIND_CAUCHY_EIG || kind == KIND_DENSE) return 0;
  if (kind == KIND_CAUCHY_EIG)
    return o->precision == PSMMA_PREC_SPLIT ? split_workspace_general(n, k, k, o->n_moduli, o->block_levels)
                                            : f64_splitk_bytes(n, k, k, std::max(1, device_sms()));
  if (o->precision == PSMMA_PREC_SPLIT) return split_workspace_bytes(kind, n, k, o->n_moduli, o->block_levels);
  if (kind == KIND_DFT) return dft_f64_workspace(n, k);
  return f64_splitk_bytes(n, k, k, std::max(1, device_sms()));
}

int psmma_stream_status(void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PSMMA_EDEVICE;
  unsigned* w = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_stw_mu);
    auto it = g_stw.find({dev, s});
    if (it != g_stw.end()) w = it->second;
  }
  if (!w) return cudaStreamSynchronize(s) == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
  unsigned h = 0;
  if (cudaMemcpyAsync(&h, w, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PSMMA_EDEVICE;
  if (h == 0) return PSMMA_OK;
  if (cudaMemsetAsync(w, 0, sizeof(unsigned), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return PSMMA_EDEVICE;
  return (h & DEV_ERR_TIMEOUT) ? PSMMA_ETIMEDOUT : PSMMA_EDEVICE;
}

int psmma_stream_release(void* stream) {
  const int st = psmma_stream_status(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PSMMA_EDEVICE;
  unsigned* w = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_stw_mu);
    auto it = g_stw.find({dev, (cudaStream_t)stream});
    if (it != g_stw.end()) {
      w = it->second;
      g_stw.erase(it);
    }
  }
  if (w) cudaFree(w);  // the stream has drained (psmma_stream_status waited for it)
  return st;
}

void psmma_release_workspace(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (auto it = g_pools.begin(); it != g_pools.end();) {
      if (std::get<0>(it->first) == dev) {
        cudaStreamSynchronize(std::get<1>(it->first));
        cudaFree(it->second.ptr);
        it = g_pools.erase(it);
      } else {
        ++it;
      }
    }
  }
  std::lock_guard<std::mutex> lk(g_host_mu);
  auto it = g_host.find(dev);
  if (it != g_host.end() && it->second.ptr) {
    cudaStreamSynchronize(it->second.stream);
    cudaFree(it->second.ptr);
    it->second.ptr = nullptr;
    it->second.bytes = 0;
  }
}

const char* psmma_status_string(int status) {
  switch (status) {
    case PSMMA_OK: return "ok";
    case -1: return "argument N < 0 (PZMDFTL INFO=1)";
    case -2: return "argument N < 0 (PSCAUCHY_COMPUTE INFO=2) or K < 0 (PZMDFTL INFO=2)";
    case -3: return "argument K < 0 (PSCAUCHY_COMPUTE INFO=3)";
    case -7: return "LDB too small (PZMDFTL INFO=7)";
    case -9: return "LDA too small (PSCAUCHY_COMPUTE INFO=9)";
    case -10: return "LDC too small (PZMDFTL INFO=10)";
    case -14: return "LDQ too small (PSCAUCHY_COMPUTE INFO=14)";
    case PSMMA_EGEN: return "generator pointer NULL or generator length too small";
    case PSMMA_ENULL: return "matrix pointer NULL for a non-empty operand";
    case PSMMA_ENOMEM: return "device allocation failed";
    case PSMMA_EDEVICE: return "CUDA runtime error";
    case PSMMA_ETIMEDOUT: return "bounded device-side wait expired";
    case PSMMA_ESINGULAR: return "Cauchy denominator D(i)-F(j) is zero";
    case PSMMA_EUNSUPPORTED: return "unsupported option combination";
    case PSMMA_EWORKSPACE: return "workspace too small";
    case PSMMA_ERANGE: return "non-finite input or exponent out of range for the split path";
    case PSMMA_ESCRATCH: return "request exceeds the 96 MiB fixed scratch of psmma_cauchy_split_noalloc";
    default: return "unknown status";
  }
}

void psmma_set_profiling(int on) { g_prof_on = on != 0; }

int psmma_profile_read(float* ms, const char** names, int max_phases) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  int np = g_prof_n - 1;
  if (np <= 0) return 0;
  if (cudaEventSynchronize(g_prof_ev[g_prof_n - 1]) != cudaSuccess) return PSMMA_EDEVICE;
  int m = std::min(np, max_phases);
  for (int i = 0; i < m; ++i) {
    float t = 0.0f;
    cudaEventElapsedTime(&t, g_prof_ev[i], g_prof_ev[i + 1]);
    if (ms) ms[i] = t;
    if (names) names[i] = g_prof_name[i + 1];
  }
  return m;
}

int psmma_profile_read_timeline(float* ms, const char** names, int max_phases) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  int np = g_prof_n - 1;
  if (np <= 0) return 0;
  for (int i = 1; i < g_prof_n; ++i)  // marks may sit on several streams: wait for each
    if (cudaEventSynchronize(g_prof_ev[i]) != cudaSuccess) return PSMMA_EDEVICE;
  int m = std::min(np, max_phases);
  for (int i = 0; i < m; ++i) {
    float t = 0.0f;
    cudaEventElapsedTime(&t, g_prof_ev[0], g_prof_ev[i + 1]);
    if (ms) ms[i] = t;
    if (names) names[i] = g_prof_name[i + 1];
  }
  return m;
}

const char* psmma_version(void) { return "psmma-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
