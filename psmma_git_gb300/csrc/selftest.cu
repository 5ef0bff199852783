// Self-test of the bounded device-side waits: a kernel waits on an mbarrier that nothing
// ever arrives on, with a short limit, and must come back with the timeout recorded in its
// status word instead of hanging.  No fault, trap or endless loop is involved; the CUDA
// context stays usable afterwards.
#include "psmma_internal.h"
#include "tcgen05_util.cuh"

namespace psmma {

__global__ void k_selftest_wait(unsigned* status, unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // expects one arrival that never comes
    abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_for(&bar, 0, status, &abort_flag, limit_ns);
}

}  // namespace psmma

using namespace psmma;

extern "C" int psmma_selftest_wait_timeout(unsigned long long limit_ns) {
  if (limit_ns == 0 || limit_ns > 10000000000ull) return PSMMA_EUNSUPPORTED;
  unsigned* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned)) != cudaSuccess) return PSMMA_ENOMEM;
  int st = PSMMA_OK;
  unsigned h = 0;
  if (cudaMemset(d, 0, sizeof(unsigned)) != cudaSuccess) st = PSMMA_EDEVICE;
  if (!st) {
    k_selftest_wait<<<1, 32>>>(d, limit_ns);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&h, d, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess)
      st = PSMMA_EDEVICE;
  }
  cudaFree(d);
  if (st) return st;
  return (h & DEV_ERR_TIMEOUT) ? PSMMA_ETIMEDOUT : PSMMA_OK;
}
