// Inline-PTX helpers for sm_103a: mbarriers with bounded waits, TMA tile loads, tcgen05
// (TMEM allocation, MMA, commit, TMEM loads) and the shared-memory / instruction
// descriptors of tcgen05.mma.  Every wait is bounded: on expiry it records an error in a
// global status word and returns false, so a kernel can drain and exit instead of hanging.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace psmma {

// Status bits written by device code into the per-call status word.
constexpr unsigned DEV_ERR_TIMEOUT = 1u;

// Time limit of one mbarrier wait.  Legitimate waits in these kernels last microseconds;
// 2 s means the pipeline is broken.  After the first expiry every CTA of the launch (and
// every later CTA, which checks the status word on entry) stops waiting and drains.
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool status_aborted(const unsigned* status) {
  return (*(const volatile unsigned*)status & DEV_ERR_TIMEOUT) != 0;
}

// Bounded wait for the phase with the given parity.  Returns false when the time limit
// expires (recording DEV_ERR_TIMEOUT) or when this CTA or the launch has already aborted.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, unsigned* status,
                                              volatile int* abort_flag, unsigned long long limit_ns) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*abort_flag || status_aborted(status)) {
        *abort_flag = 1;
        return false;
      }
      unsigned long long now = globaltimer_ns();
      if (t0 == 0) {
        t0 = now;
      } else if (now - t0 > limit_ns) {
        atomicOr(status, DEV_ERR_TIMEOUT);
        *abort_flag = 1;
        return false;
      }
    }
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned* status,
                                          volatile int* abort_flag) {
  return mbar_wait_for(bar, parity, status, abort_flag, WAIT_NS);
}

// Bounded wait that ignores the abort flags: used at exit to make sure this thread's own
// asynchronous copies and MMAs have completed before shared or tensor memory is released.
__device__ __forceinline__ bool mbar_wait_drain(uint64_t* bar, uint32_t parity, unsigned* status) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u) {
      unsigned long long now = globaltimer_ns();
      if (t0 == 0) {
        t0 = now;
      } else if (now - t0 > WAIT_NS) {
        atomicOr(status, DEV_ERR_TIMEOUT);
        return false;
      }
    }
  }
}

// ---- division ------------------------------------------------------------------------------
// a / x by Newton-Raphson refinement of the hardware reciprocal approximation and one
// residual correction (Markstein's method, IBM J. Res. Dev. 34(1), 1990): one step
// y <- y + y (1 - x y) squares the approximation's relative error; then q = a y and
// q' = q + y (a - x q), whose error is about that squared error times |q| -- the correctly
// rounded quotient except in rare ties (at most 1 ulp off; checked against the IEEE division
// by psmma_selftest_division).  Operands whose exponents are extreme
// (subnormal, huge, quotient near overflow or underflow, zero, Inf, NaN) take the IEEE
// division.  Cheaper than the IEEE division on GB300, whose FP64 pipe is narrow.
__device__ __forceinline__ double div_nr(double a, double x) {
  const int ea = (__double2hiint(a) >> 20) & 0x7ff, ex = (__double2hiint(x) >> 20) & 0x7ff;
  if (ea < 64 || ea > 1983 || ex < 64 || ex > 1983 || ea - ex > 900 || ex - ea > 900) return a / x;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  const double q = a * y;
  const double r = fma(-x, q, a);
  return fma(r, y, q);
}

// a / x for the split path's H: the FP32 reciprocal (1 ulp) of x rounded to a float, widened to
// a double with integer operations, one FP64 Newton step y <- y + y (1 - x y) (relative error
// about (2^-23)^2), then q = a y -- three FP64 operations instead of div_nr's five plus the
// FP64 reciprocal approximation.  The error (bounded by psmma_selftest_division_split) is about
// 2^-45: H is then rounded to at most 53 bits of each column's maximum, and a relative
// perturbation of 2^-45 of its entries changes the product's error by 0.2 %.  Operands outside
// [2^-100, 2^100] or with extreme quotients take div_nr.
__device__ __forceinline__ double div_split(double a, double x) {
  const int hx = __double2hiint(x);
  const int ea = (__double2hiint(a) >> 20) & 0x7ff, ex = (hx >> 20) & 0x7ff;
  if (ea < 64 || ea > 1983 || ex < 1023 - 100 || ex > 1023 + 100 || ea - ex > 900 || ex - ea > 900)
    return div_nr(a, x);
  // x as a float: sign, rebased exponent, 23 mantissa bits rounded to nearest (a carry into
  // the exponent is the correct rounding)
  const unsigned lo = (unsigned)__double2loint(x);
  const unsigned fx = (((unsigned)hx & 0x80000000u) | ((unsigned)(ex - 1023 + 127) << 23) |
                       (((unsigned)hx & 0xFFFFFu) << 3) | (lo >> 29)) +
                      ((lo >> 28) & 1u);
  float yf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(__uint_as_float(fx)));
  // the float reciprocal as a double (normal: |x| within 2^+-100)
  const unsigned uy = __float_as_uint(yf);
  const unsigned hy = (uy & 0x80000000u) | ((((uy >> 23) & 0xFFu) - 127u + 1023u) << 20) | ((uy & 0x7FFFFFu) >> 3);
  double y = __hiloint2double((int)hy, (int)((uy & 0x7u) << 29));
  const double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  return a * y;
}

// ---- double-float Cauchy entries -------------------------------------------------------------
// The significand of a normal double x (x * 2^-E, in [1, 2) with x's sign) as hi + lo floats,
// from its bits: hi = rounded to 24 significant bits (a rounding carry lands in the exponent
// field, which is what an add of the bits gives), lo = the remainder, a signed multiple of 2^-52
// of at most 2^28 units converted to a float: |lo| <= 2^-24 |hi|, |hi + lo - x 2^-E| <= 2^-49.
__device__ __forceinline__ float2 df_split_unit(double x) {
  const unsigned hx = (unsigned)__double2hiint(x), lx = (unsigned)__double2loint(x);
  const unsigned sgn = hx & 0x80000000u, up = (lx >> 28) & 1u;
  const float hi = __uint_as_float((sgn | (127u << 23) | ((hx & 0xFFFFFu) << 3) | (lx >> 29)) + up);
  const int rem = (int)(lx & 0x1FFFFFFFu) - (int)(up << 29);
  const float lo = __int2float_rn(rem) * 0x1.0p-52f;
  return make_float2(hi, sgn ? -lo : lo);
}

// The double nearest hi + lo (|lo| < 2^-20 |hi|, both normal or lo zero): both widened exactly
// from their bits, one FP64 add.
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  const unsigned bh = __float_as_uint(hi), bl = __float_as_uint(lo);
  const double dh = __hiloint2double((int)((bh & 0x80000000u) | ((((bh >> 23) & 0xFFu) + 896u) << 20) |
                                           ((bh & 0x7FFFFFu) >> 3)),
                                     (int)(bh << 29));
  if ((bl & 0x7F800000u) == 0u) return dh;
  const double dl = __hiloint2double((int)((bl & 0x80000000u) | ((((bl >> 23) & 0xFFu) + 896u) << 20) |
                                           ((bl & 0x7FFFFFu) >> 3)),
                                     (int)(bl << 29));
  return dh + dl;
}

// A column generator v of the split path's Cauchy entries: its significand split once per
// column and its exponent; ok for a normal v (else every entry of the column takes div_split).
struct VSplit {
  float2 s;
  int e;
  bool ok;
};
__device__ __forceinline__ VSplit v_split(double v) {
  VSplit r;
  const int f = (__double2hiint(v) >> 20) & 0x7FF;
  r.ok = f >= 1 && f <= 2046;
  r.e = f - 1023;
  r.s = df_split_unit(v);
  return r;
}

// u * v / x (x = D(i) - F(j), formed in FP64 by the caller) for the split path's H, in
// double-float arithmetic on the FP32 pipe: GB300 issues FP64 at about two lanes per SM per
// cycle, and this costs one FP64 add instead of div_split's product, two FMAs and product.
// The significands are split (df_split_unit) and the exponents added back at the end, so the
// result is exactly equivariant under power-of-two scalings of u, v and x.  With x = xh + xl:
// y0 = the FP32 reciprocal of xh, one Newton step against the whole x gives y1 with
// |1 - x y1| <~ 2^-24 (FP32 rounding of y1), e = 1 - x y1 from two FMAs (the first exact but
// for a rounding at 2^-48, the second at 2^-48), and 1/x = y1 + y1 e to about 2^-48 (e^2 and
// the rounding of y1 e); a = u v = ah + al by the usual FMA error terms, renormalised so that
// |al| <= 2^-24 |ah|, and q = a (y1 + y1 e) = qh + ql.  The low parts reach a few 2^-24 of the
// result, so their FP32 roundings set the relative error: about 2^-45.3 at most and 2^-49
// typically (div_split: 2^-44 and 2^-45); checked by psmma_selftest_division_split.  Zero,
// subnormal or non-finite operands, and quotients outside the normal range, take div_split.
// The operands cauchy_entry leaves to the FP64 division; out of line, so that the rare branch
// stays a branch (its FP64 instructions are not issued, predicated off, for every entry).
static __device__ __noinline__ double cauchy_entry_slow(double u, double v, double x) { return div_split(u * v, x); }

__device__ __forceinline__ double cauchy_entry(double u, double v, const VSplit& vs, double x) {
  const int fu = (__double2hiint(u) >> 20) & 0x7FF, fx = (__double2hiint(x) >> 20) & 0x7FF;
  if (!vs.ok || fu == 0 || fu == 0x7FF || fx == 0 || fx == 0x7FF) return cauchy_entry_slow(u, v, x);
  const float2 xs = df_split_unit(x), us = df_split_unit(u);
  float y0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(xs.x));
  const float y1 = fmaf(y0, fmaf(-xs.y, y0, fmaf(-xs.x, y0, 1.0f)), y0);
  const float e = fmaf(-xs.y, y1, fmaf(-xs.x, y1, 1.0f));
  const float p = us.x * vs.s.x;
  const float pl = fmaf(us.y, vs.s.y, fmaf(us.x, vs.s.y, fmaf(us.y, vs.s.x, fmaf(us.x, vs.s.x, -p))));
  const float ah = p + pl, al = pl - (ah - p);  // renormalised: |al| <= 2^-24 |ah|
  // a (y1 + y1 e) - ah y1 = (ah y1 - qh) + y1 (al + ah e + al e)
  const float qh = ah * y1;
  const float ql = fmaf(y1, fmaf(al, e, fmaf(ah, e, al)), fmaf(ah, y1, -qh));
  const double q = df_to_double(qh, ql);  // in (1/2, 4)
  const int eq = fu + vs.e - fx;           // exponent of u v / x over that of the significands'
  const int hq = __double2hiint(q);
  const int fq = ((hq >> 20) & 0x7FF) + eq;
  if (fq < 1 || fq > 2046) return cauchy_entry_slow(u, v, x);
  return __hiloint2double((int)((unsigned)hq + ((unsigned)eq << 20)), __double2loint(q));
}

// ---- TMA -------------------------------------------------------------------------------
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, "
      "%5}], [%2];\n" ::"r"(smem_u32(smem_dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(map) : "memory");
}

// ---- tcgen05 ------------------------------------------------------------------------------
// TMEM allocation: executed by one full warp; the allocated base address is written to smem.
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(smem_dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// D[tmem] (+)= A[smem desc] * B[smem desc], kind::f16 (BF16 inputs, FP32 accumulate).
__device__ __forceinline__ void tc_mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on an mbarrier when all prior tcgen05 async operations of this thread complete.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: thread t receives row (lane base + t).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// Shared-memory matrix descriptor of tcgen05.mma for a K-major operand stored with the
// 128-byte swizzle (rows of 128 B, 8-row atoms of 1024 B, atom stride 1024 B):
//   [0,14) start address >> 4, [16,30) leading byte offset >> 4 (unused for this layout),
//   [32,46) stride byte offset >> 4, [46,48) version = 1, [61,64) layout = 2 (128B swizzle).
__device__ __forceinline__ uint64_t sdesc_sw128_kmajor(uint32_t smem_addr) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)2u << 61;
  return d;
}

// Instruction descriptor of tcgen05.mma .kind::f16: D = F32, A = B = BF16, both K-major,
// dense, shape M x N:  [4,6) D format (1 = F32), [7,10) A format (1 = BF16),
// [10,13) B format (1 = BF16), [15] A major (0 = K), [16] B major (0 = K),
// [17,23) N >> 3, [24,29) M >> 4.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

}  // namespace psmma
