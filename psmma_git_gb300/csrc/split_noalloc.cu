// psmma_cauchy_split_noalloc: the split-path Cauchy multiply with its workspace in a fixed
// device array of this library instead of memory allocated per call.
//
// Who needs it: callers that own all device memory through their own pool allocator and do
// not let a library call cudaMalloc/cudaFree (those calls synchronise the whole device and
// fragment the caller's pool), and callers on a latency-critical loop that cannot take that
// implicit synchronisation or an allocation failure in the middle of a run.  They pass A, the
// generators and Q as usual; every temporary of the split path lives in kNoAllocScratchBytes
// of statically allocated device memory, which every GPU that loads this library holds
// until the process exits.
//
// Limits and rules:
//  * requests whose split workspace exceeds kNoAllocScratchBytes are rejected with
//    PSMMA_ESCRATCH (96 MiB: n = k = 1024 with the default 14 moduli fits);
//  * all calls share the one array: calls whose work overlaps on the GPU (other streams,
//    other host threads) race on it and must be serialised by the caller; the buffers that
//    must start at zero are cleared by every call, the rest are overwritten;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress,
//    with that device current) and caches it until the process exits (a cudaDeviceReset,
//    which reloads the module, is not supported afterwards); make that first call before
//    any stream capture on that device;
//  * the call blocks: it waits for its work on the stream to finish and reads the device
//    status back (it may not allocate the per-stream status word of the asynchronous entry
//    points), so it returns with Q written;
//  * alpha = 0 scales Q by beta and reads neither A nor the generators, as psmma_cauchy and
//    the reference's DGEMM do.
#include <mutex>

#include "psmma_internal.h"

namespace psmma {
namespace {

constexpr size_t kNoAllocScratchBytes = 96ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once per device).
void* noalloc_scratch(int* status) {
  *status = PSMMA_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    *status = PSMMA_EDEVICE;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      *status = PSMMA_EDEVICE;
      return nullptr;
    }
    g_noalloc_ptr[dev] = p;
  }
  return g_noalloc_ptr[dev];
}

}  // namespace
}  // namespace psmma

using namespace psmma;

extern "C" int psmma_cauchy_split_noalloc(int n, int k, double alpha, const double* A, int lda,
                                          const double* gen, int ldgen, double beta, double* Q, int ldq,
                                          int n_moduli, void* stream) {
  // Argument checks and quick return of psmma_cauchy, with the numbering of PSCAUCHY_COMPUTE
  // (pscauchy_compute.f90:234-255).
  if (n_moduli != 0 && (n_moduli < 8 || n_moduli > 16)) return PSMMA_EUNSUPPORTED;
  int st = check_real_args(KIND_CAUCHY, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq);
  if (st == 1) return PSMMA_OK;
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (alpha == 0.0) {
    // Q := beta*Q: the DGEMM of pscauchy_compute.f90:406 with alpha = 0 reads neither operand.
    GenSpec none;
    st = launch_struct_f64_ws(n, k, k, 0.0, nullptr, lda, none, beta, Q, ldq, nullptr, 0, s);
    if (st) return st;
    return cudaStreamSynchronize(s) == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
  }
  const size_t need = split_workspace_bytes(KIND_CAUCHY, n, k, n_moduli);
  if (need > kNoAllocScratchBytes) return PSMMA_ESCRATCH;
  void* work = noalloc_scratch(&st);
  if (st) return st;
  return launch_split(KIND_CAUCHY, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, n_moduli, work,
                      kNoAllocScratchBytes, s, true);
}
