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

// ------------------------------------------------------------------------------------------
// Self-check of div_nr (FP64-exact quotients) and cauchy_entry (the split path's Cauchy entries
// u*v/x, double-float with div_split for operands outside its range) against the IEEE division on
// count seeded pairs: Cauchy-like operands u*v / (d - w) with |d - w| log-uniform in
// [1e-13, 1], plus arbitrary finite bit patterns (which exercise the fallback).
// ------------------------------------------------------------------------------------------
namespace psmma {

__device__ __forceinline__ unsigned long long splitmix(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double unit(unsigned long long r) { return (double)(r >> 11) * 0x1.0p-53; }

template <bool SPLIT>
__global__ void k_selftest_div(long long count, unsigned long long seed, unsigned long long* mism, int* max_ulp) {
  unsigned long long local = 0;
  int worst = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    unsigned long long s = seed ^ (0xD1B54A32D192ED03ull * (unsigned long long)(t + 1));
    double a, x, u = 1.0, v = 1.0;
    if ((t & 7) != 7) {
      u = 8.0 * unit(splitmix(s)) - 4.0;
      v = 8.0 * unit(splitmix(s)) - 4.0;
      const double d = unit(splitmix(s));
      const double gap = exp2(-43.2 * unit(splitmix(s)));  // 1e-13 .. 1
      const double w = (splitmix(s) & 1) ? d - gap : d + gap;
      a = u * v;
      x = d - w;
    } else {
      unsigned long long ba = splitmix(s), bx = splitmix(s);
      ba &= ~(0x7ffull << 52) | ((ba % 2046ull) << 52);  // finite exponents only
      bx &= ~(0x7ffull << 52) | (((bx >> 3) % 2046ull + 1) << 52);
      a = __longlong_as_double((long long)ba);
      x = __longlong_as_double((long long)bx);
      u = a;
    }
    if (x == 0.0) continue;
    const double q0 = a / x, q1 = SPLIT ? cauchy_entry(u, v, v_split(v), x) : div_nr(a, x);
    if (__double_as_longlong(q0) != __double_as_longlong(q1)) {
      ++local;
      const long long d = __double_as_longlong(q0) - __double_as_longlong(q1);
      const long long ad = d < 0 ? -d : d;
      worst = max(worst, (int)min(ad, 1ll << 30));
    }
  }
  if (local) atomicAdd(mism, local);
  if (worst) atomicMax(max_ulp, worst);
}

}  // namespace psmma

static int selftest_division(bool split, long long count, unsigned long long seed, unsigned long long* mismatches,
                             int* max_ulp) {
  if (count <= 0 || !mismatches || !max_ulp) return PSMMA_EUNSUPPORTED;
  unsigned long long* dm = nullptr;
  if (cudaMalloc(&dm, 16) != cudaSuccess) return PSMMA_ENOMEM;
  int st = PSMMA_OK;
  if (cudaMemset(dm, 0, 16) != cudaSuccess) st = PSMMA_EDEVICE;
  if (!st) {
    if (split)
      k_selftest_div<true><<<1216, 256>>>(count, seed, dm, (int*)(dm + 1));
    else
      k_selftest_div<false><<<1216, 256>>>(count, seed, dm, (int*)(dm + 1));
    unsigned long long h[2] = {0, 0};
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(h, dm, 16, cudaMemcpyDeviceToHost) != cudaSuccess)
      st = PSMMA_EDEVICE;
    *mismatches = h[0];
    *max_ulp = (int)(unsigned)h[1];
  }
  cudaFree(dm);
  return st;
}

extern "C" int psmma_selftest_division(long long count, unsigned long long seed, unsigned long long* mismatches,
                                       int* max_ulp) {
  return selftest_division(false, count, seed, mismatches, max_ulp);
}

extern "C" int psmma_selftest_division_split(long long count, unsigned long long seed,
                                             unsigned long long* mismatches, int* max_ulp) {
  return selftest_division(true, count, seed, mismatches, max_ulp);
}
