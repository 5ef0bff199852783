// Split path: the structured multiply Q = alpha*A*H + beta*Q computed exactly in modular
// integer arithmetic on the BF16 tensor cores (tcgen05), with FP64 scaling and
// recombination.
//
// Scheme (Chinese-remainder slicing of an integer-scaled product):
//   1. Each row i of A is scaled by a power of two 2^s_i and rounded to an integer with at
//      most P bits, A' = rint(A * 2^s); each column j of H likewise, H' = rint(H * 2^f).
//   2. For pairwise coprime moduli m_1..m_N <= 256 the residues A' mod m_l and H' mod m_l
//      lie in [-128, 128] and are exact in BF16.
//   3. One BF16 GEMM per modulus gives Z_l = A'H' mod m_l.  FP32 accumulation is exact
//      because the tensor memory accumulator is drained every 1024 k (|sum| <= 2^24) into
//      register-held int32 sums, reduced modulo m_l every 16 chunks.
//   4. Z = A'H' is recovered exactly by CRT (128-bit integer arithmetic, |Z| < 0.497 M with
//      M = prod m_l), scaled back by 2^-(s_i+f_j) and combined with alpha and beta in FP64.
// P is chosen on the device from the product bound |Z_ij| <= 2^(2P) * max_j(sum_k|H_kj| /
// max_k|H_kj|), so no host synchronisation is needed between the passes.
//
// H is generated on the device from the generators (formulas of Cauchylowrank.f90:509-521,
// Auxil_2p5D.f90:224-231, 309-316) in one pass; the caller never supplies a dense H.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstddef>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "psmma_internal.h"
#include "tcgen05_util.cuh"

namespace psmma {

constexpr int SPL_MAX_MODULI = 16;
constexpr int SPL_DEFAULT_MODULI = 14;
// Pairwise coprime: 2^8, 3*5*17, 11*23, 13*19 and primes.
static const int kModuli[SPL_MAX_MODULI] = {256, 255, 253, 251, 247, 241, 239, 233,
                                            229, 227, 223, 211, 199, 197, 193, 191};

struct CrtConsts {
  int nmod;
  int m[SPL_MAX_MODULI];
  float inv_m[SPL_MAX_MODULI];
  float mf[SPL_MAX_MODULI];   // m as a float
  float g23[SPL_MAX_MODULI];  // 2^23 mod m, symmetric (|g| <= m/2)
  float g38[SPL_MAX_MODULI];  // 2^38 mod m, symmetric
  float g14[SPL_MAX_MODULI], g28[SPL_MAX_MODULI], g42[SPL_MAX_MODULI];  // 2^14, 2^28, 2^42 mod m, symmetric
  unsigned long long C_lo[SPL_MAX_MODULI], C_hi[SPL_MAX_MODULI];  // CRT basis C_l < M
  float f[SPL_MAX_MODULI];                                        // C_l / M
  unsigned long long M_lo, M_hi;
  double log2M;
  unsigned climb[SPL_MAX_MODULI][4];   // C_l as four 32-bit limbs
  unsigned bias[4];                    // 128 * sum_l C_l mod 2^128 (residues enter offset by 128)
  int ffix[SPL_MAX_MODULI];            // round(2^19 * C_l / M): fixed-point quotient estimate
  unsigned long long biasl[4];         // sum_l 128 * climb[l][t], per limb, unreduced
  unsigned Mlimb[4];                   // M as four 32-bit limbs
  int top32;                           // sum_l 255 * climb[l][3] < 2^32: top limb summed in 32 bits
};

// Device-side parameters of one call (in the workspace).
constexpr int PARAMS_BLOCKS = 32;  // blocks of the single-product parameter pass

struct SplitDevParams {
  unsigned status;
  int PA, PH;                   // bits of the integer-scaled A (per row) and H (per column)
  unsigned long long rho_bits;  // max_j sum_k |H_kj| / max_k |H_kj| (bits of a positive double)
  unsigned done;                // parameter-pass blocks finished
  unsigned hbad;                // block-recursive products: some column of H is not finite
  double part[PARAMS_BLOCKS][6];  // their partial ratio maxima and sums, combined in block order
};

// ------------------------------------------------------------------------------------------
// Host: constants of the CRT for the first nmod moduli.
// ------------------------------------------------------------------------------------------
static long long inv_mod(long long a, long long m) {
  long long t = 0, nt = 1, r = m, nr = ((a % m) + m) % m;
  while (nr) {
    long long q = r / nr, tmp;
    tmp = t - q * nt; t = nt; nt = tmp;
    tmp = r - q * nr; r = nr; nr = tmp;
  }
  return (t % m + m) % m;
}

static CrtConsts make_consts(int nmod) {
  CrtConsts c;
  memset(&c, 0, sizeof(c));
  c.nmod = nmod;
  typedef unsigned __int128 u128;
  u128 M = 1;
  double l2 = 0.0;
  for (int l = 0; l < nmod; l++) {
    M *= (u128)kModuli[l];
    l2 += std::log2((double)kModuli[l]);
  }
  for (int l = 0; l < nmod; l++) {
    int m = kModuli[l];
    c.m[l] = m;
    c.inv_m[l] = 1.0f / (float)m;
    c.mf[l] = (float)m;
    const int g23 = (int)((1LL << 23) % m), g38 = (int)((1LL << 38) % m);
    c.g23[l] = (float)(g23 > m / 2 ? g23 - m : g23);
    c.g38[l] = (float)(g38 > m / 2 ? g38 - m : g38);
    const int g14 = (int)((1LL << 14) % m), g28 = (int)((1LL << 28) % m), g42 = (int)((1LL << 42) % m);
    c.g14[l] = (float)(g14 > m / 2 ? g14 - m : g14);
    c.g28[l] = (float)(g28 > m / 2 ? g28 - m : g28);
    c.g42[l] = (float)(g42 > m / 2 ? g42 - m : g42);
    u128 Ml = M / (u128)m;
    long long Ml_mod = (long long)(Ml % (u128)m);
    long long y = inv_mod(Ml_mod, m);
    u128 C = (Ml * (u128)y) % M;
    c.C_lo[l] = (unsigned long long)C;
    c.C_hi[l] = (unsigned long long)(C >> 64);
    // C / M as float: C < M < 2^126, take the top bits of both
    long double cf = (long double)C / (long double)M;
    c.f[l] = (float)cf;
  }
  c.M_lo = (unsigned long long)M;
  c.M_hi = (unsigned long long)(M >> 64);
  c.log2M = l2 - 1e-9;
  u128 bias = 0;
  for (int l = 0; l < nmod; l++) {
    u128 C = ((u128)c.C_hi[l] << 64) | c.C_lo[l];
    for (int t = 0; t < 4; t++) c.climb[l][t] = (unsigned)(C >> (32 * t));
    bias += (u128)128 * C;  // wraps modulo 2^128
  }
  for (int t = 0; t < 4; t++) c.bias[t] = (unsigned)(bias >> (32 * t));
  for (int t = 0; t < 4; t++) c.Mlimb[t] = (unsigned)(M >> (32 * t));
  for (int t = 0; t < 4; t++) {
    c.biasl[t] = 0;
    for (int l = 0; l < nmod; l++) c.biasl[t] += 128ull * c.climb[l][t];
  }
  c.top32 = 2 * c.biasl[3] < (1ull << 32);  // 255 <= 2 * 128
  for (int l = 0; l < nmod; l++) {
    u128 C = ((u128)c.C_hi[l] << 64) | c.C_lo[l];
    long double cf = (long double)C / (long double)M;
    c.ffix[l] = (int)std::llround((double)(cf * 524288.0L));  // |sum_l r_l ffix_l| < 16*128*2^19 = 2^30
  }
  return c;
}

// ------------------------------------------------------------------------------------------
// Workspace layout
// ------------------------------------------------------------------------------------------
static size_t al1k(size_t x) { return (x + 1023) & ~(size_t)1023; }

struct SplitLayout {
  int kp, kr;
  size_t off_params, off_amax, off_hmax, off_hsum, off_asq, off_hsq, off_wtab, off_ht, off_ra, off_rh, off_r,
      total;
  size_t off_rs = 0, off_gmax = 0, off_hall = 0;  // block products: A block sums, group / all-row column maxima
};

// M rows of A (and Q), K inner length, N columns of H (and Q).
static SplitLayout split_layout(int M, int K, int N, int nmod) {
  SplitLayout L;
  L.kp = (K + 63) / 64 * 64;
  L.kr = (N + 255) / 256 * 256;
  size_t o = 0;
  L.off_params = o; o += al1k(2 * sizeof(SplitDevParams));  // the call's parameters, then guessed PA/PH
  L.off_amax = o;   o += al1k((size_t)M * 8);
  L.off_hmax = o;   o += al1k((size_t)N * 8);
  L.off_hsum = o;   o += al1k((size_t)N * 8);
  L.off_asq = o;    o += al1k((size_t)M * 8);
  L.off_hsq = o;    o += al1k((size_t)N * 8);
  L.off_wtab = o;   o += al1k((size_t)(K / 2 + 1) * 16);
  L.off_ht = o;     o += al1k((size_t)N * L.kp * 8);
  L.off_ra = o;     o += al1k((size_t)nmod * M * L.kp * 2);
  L.off_rh = o;     o += al1k((size_t)nmod * N * L.kp * 2);
  L.off_r = o;      o += al1k((size_t)nmod * M * L.kr);
  L.total = o;
  return L;
}

// Rows of one split product: the residue and CRT passes tile rows in blocks of 64 and 32
// along the grid's y dimension (at most 65535 blocks), so M <= 32 * 65535; larger products
// are refused with PSMMA_EUNSUPPORTED rather than launched with a grid the device rejects.
constexpr int kSplitMaxRows = 32 * 65535;

static int resolve_nmod(int n_moduli) { return n_moduli == 0 ? SPL_DEFAULT_MODULI : n_moduli; }

// The DFT's split workspace: C^T = B^T F (k x n complex) as three real products of the 3M
// form, T1 = Br^T Fr, T2 = Bi^T Fi, T3 = (Br + Bi)^T (Fr + Fi): row maxima and sums of B's
// columns (M = k), column statistics of F (n), Ht = [Fr rows | Fi rows] (2n x kp doubles), three
// sets of A and H residue planes (product p at p * nmod planes), and output planes with Re in
// columns [0, n) and Im in [kr1, kr1 + n), kr1 = n rounded to 256 (the GEMMs' tile padding of
// the Re half stays out of the Im half).
static SplitLayout dft3_layout(int M, int n, int nmod) {
  SplitLayout L;
  L.kp = (n + 63) / 64 * 64;
  const int kr1 = (n + 255) / 256 * 256;
  L.kr = 2 * kr1;
  size_t o = 0;
  L.off_params = o; o += al1k(2 * sizeof(SplitDevParams));
  L.off_amax = o;   o += al1k((size_t)M * 8);
  L.off_hmax = o;   o += al1k((size_t)n * 8);
  L.off_hsum = o;   o += al1k((size_t)n * 8);
  L.off_asq = o;    o += al1k((size_t)M * 8);
  L.off_hsq = o;    o += al1k((size_t)n * 8);
  L.off_wtab = o;   o += al1k((size_t)(n + 1) * 16);
  L.off_ht = o;     o += al1k((size_t)2 * n * L.kp * 8);
  L.off_ra = o;     o += al1k((size_t)3 * nmod * M * L.kp * 2);
  L.off_rh = o;     o += al1k((size_t)3 * nmod * n * L.kp * 2);
  L.off_r = o;      o += al1k((size_t)nmod * M * L.kr);
  L.total = o;
  return L;
}

// Radix of the split DFT's first step (C = F_n B via F_(n/R) on R k columns): the largest R in
// {8, 4, 2} dividing n with n / R >= kDftMinInner (the modular GEMMs keep that inner length),
// else 1.
constexpr int kDftMinInner = 1024;
static int dft_radix(int n) {
  for (int R = 8; R >= 2; R >>= 1)
    if (n % R == 0 && n / R >= kDftMinInner) return R;
  return 1;
}

// Radix-R workspace: the core's (M = R k, n / R) layout, then B' (n x k complex) and the
// n-entry table w_n^t.
struct DftRadixLayout {
  size_t core, off_bp, off_w, total;
};
static DftRadixLayout dft_radix_layout(int n, int k, int R, int nmod) {
  DftRadixLayout D;
  D.core = al1k(dft3_layout(R * k, n / R, nmod).total);
  D.off_bp = D.core;
  D.off_w = D.off_bp + al1k((size_t)n * k * 16);
  D.total = D.off_w + al1k((size_t)n * 16);
  return D;
}

struct BlockChoice {  // levels of the Toeplitz / Hankel block step and the (padded) order
  int L, Np;
};
static BlockChoice block_choice(int kind, int N, int K, int req);
static SplitLayout block_layout(int M, int N, int L, int nmod);
static bool s2_use(int kind, int M, int K, int N, int req);
static SplitLayout s2_layout(int M, int K, int N, int rows, int nmod);

size_t split_workspace_bytes(int kind, int n, int k, int n_moduli, int block_req) {
  if (n <= 0 || k <= 0) return 0;
  if (kind == KIND_TOEPLITZ || kind == KIND_HANKEL) {
    const BlockChoice bc = block_choice(kind, k, k, block_req);
    const size_t plain = split_layout(n, k, k, resolve_nmod(n_moduli)).total;
    return bc.L > 0 ? std::max(plain, block_layout(n, bc.Np, bc.L, resolve_nmod(n_moduli)).total) : plain;
  }
  if (s2_use(kind, n, k, k, block_req))
    return std::max(split_layout(n, k, k, resolve_nmod(n_moduli)).total, s2_layout(n, k, k, n, resolve_nmod(n_moduli)).total);
  if (kind == KIND_DFT) {
    const int R = dft_radix(n);
    return R == 1 ? dft3_layout(k, n, resolve_nmod(n_moduli)).total
                  : dft_radix_layout(n, k, R, resolve_nmod(n_moduli)).total;
  }
  return split_layout(n, k, k, resolve_nmod(n_moduli)).total;
}

extern "C" int psmma_split_dft_radix(int n) { return n > 0 ? dft_radix(n) : 0; }

int dft_radix_for(int n) { return n > 0 ? dft_radix(n) : 1; }

size_t split_workspace_general(int M, int N, int K, int n_moduli, int block_req) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  const size_t plain = split_layout(M, K, N, resolve_nmod(n_moduli)).total;
  return s2_use(KIND_CAUCHY_EIG, M, K, N, block_req)
             ? std::max(plain, s2_layout(M, K, N, M, resolve_nmod(n_moduli)).total)
             : plain;
}

// ------------------------------------------------------------------------------------------
// Pass kernels
// ------------------------------------------------------------------------------------------
constexpr unsigned long long ABS_MASK = 0x7FFFFFFFFFFFFFFFull;
constexpr unsigned long long INF_BITS = 0x7FF0000000000000ull;
constexpr int NO_SCALE = -100000;

// The bound sums (row sums of squares of A, column sums of |H| and of H^2) are accumulated in
// FP32 on a per-thread power-of-two scale, because GB300 issues FP64 at about one operation
// per SM per cycle.  abs_scaled_up gives |x| * 2^-e as a float that is never below the true
// value (top 23 mantissa bits, rounded up; magnitudes under 2^-126 become 2^-126), from the
// bits of x on the integer pipe, and sets *big when |x| * 2^-e >= 2^56 (then the caller sums
// that thread's values in FP64 instead).  With round-up FP32 adds the sums stay upper bounds.
__device__ __forceinline__ float abs_scaled_up(unsigned long long ab, int e, bool* big) {
  const int fe = (int)(ab >> 52) - 1023 - e + 127;
  *big |= fe >= 127 + 56;
  const int fc = max(1, min(fe, 254));
  unsigned fb = ((unsigned)fc << 23) | ((unsigned)(ab >> 29) & 0x7FFFFFu);
  fb += (fe < 1 || (ab & 0x1FFFFFFFull) != 0ull) ? 1u : 0u;
  return ab ? __uint_as_float(fb) : 0.0f;
}

// Row max of |A| as the bits of a non-negative double (NaN/Inf compare above all finite) and
// row sums of squares (for the Cauchy-Schwarz bound of the integer product).
// Columns kk >= ka of A come from A2 (ld lda2) at kk - ka (ka = k: A alone).
__device__ __forceinline__ const double* acol(const double* A, long lda, const double* A2, long lda2, int ka,
                                              int kk) {
  return kk < ka ? A + (long)kk * lda : A2 + (long)(kk - ka) * lda2;
}

__device__ __forceinline__ void row_absmax_blk(const double* __restrict__ A, long lda, const double* A2, long lda2,
                                               int ka, int n, int k, int kchunk,
                                               unsigned long long* __restrict__ amax_bits,
                                               double* __restrict__ asq, int bx, int by) {
  int i = bx * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int k0 = by * kchunk, k1 = min(k, k0 + kchunk);
  unsigned long long mb = 0;
  float sq32 = 0.0f;
  int e = NO_SCALE;  // set by the first group with a nonzero entry
  bool big = false;
  int kk = k0;
  // eight independent loads in flight per thread (a warp reads 32 consecutive rows)
  for (; kk + 8 <= k1; kk += 8) {
    unsigned long long b[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      b[u] = (unsigned long long)__double_as_longlong(__ldg(acol(A, lda, A2, lda2, ka, kk + u) + i)) & ABS_MASK;
    unsigned long long gm = 0;
#pragma unroll
    for (int u = 0; u < 8; ++u) gm = b[u] > gm ? b[u] : gm;
    mb = gm > mb ? gm : mb;
    if (e == NO_SCALE && gm) e = (int)(gm >> 52) - 1023;
    if (e != NO_SCALE) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float f = abs_scaled_up(b[u], e, &big);
        sq32 = __fmaf_ru(f, f, sq32);
      }
    }
  }
  for (; kk < k1; ++kk) {
    const unsigned long long b =
        (unsigned long long)__double_as_longlong(__ldg(acol(A, lda, A2, lda2, ka, kk) + i)) & ABS_MASK;
    mb = b > mb ? b : mb;
    if (e == NO_SCALE && b) e = (int)(b >> 52) - 1023;
    if (e != NO_SCALE) {
      const float f = abs_scaled_up(b, e, &big);
      sq32 = __fmaf_ru(f, f, sq32);
    }
  }
  double sq = 0.0;
  if (big) {  // entries 2^56 times the thread's first ones (or Inf/NaN): FP64 sum
    for (kk = k0; kk < k1; ++kk) {
      const double a = __ldg(acol(A, lda, A2, lda2, ka, kk) + i);
      sq = fma(a, a, sq);
    }
  } else if (e != NO_SCALE) {
    sq = ldexp((double)sq32, 2 * e);
  }
  if (mb) atomicMax(amax_bits + i, mb);
  if (sq != 0.0) atomicAdd(asq + i, sq);
}

__global__ void k_row_absmax(const double* __restrict__ A, long lda, int n, int k, int kchunk,
                             unsigned long long* __restrict__ amax_bits, double* __restrict__ asq) {
  row_absmax_blk(A, lda, nullptr, 0, k, n, k, kchunk, amax_bits, asq, blockIdx.x, blockIdx.y);
}

// H pass 1: Ht[j][kk] = H(kk, j) in FP64, column max |H| and column sum |H|, and the global
// ratio rho = max_j sum/max over finite columns.  One block per column j.
template <int KIND>
// hmax_all != nullptr receives the column maximum over every generated row (with gs.srows the
// statistics cover the first srows rows only).
__device__ __forceinline__ void h_pass1_blk(const GenSpec& gs, int K, int kp, double* __restrict__ Ht,
                                            unsigned long long* __restrict__ hmax_bits, double* __restrict__ hsum,
                                            double* __restrict__ hsq, SplitDevParams* prm, int j,
                                            unsigned long long* __restrict__ hmax_all = nullptr) {
  double w = 0.0, v = 0.0, w1 = 0.0, dlj = 0.0, drj = 0.0;
  VSplit vs;
  vs.ok = false;
  if (KIND == KIND_CAUCHY || KIND == KIND_CAUCHY_EIG) {
    w = __ldg(gs.Fc + j);   // F(j)
    v = __ldg(gs.Vc + j);   // V(j)
    vs = v_split(v);
  }
  if (KIND == KIND_CAUCHY_EIG) {
    dlj = __ldg(gs.dl + j);  // DIFL(j)
    if (j < gs.fc1_len) {
      w1 = __ldg(gs.Fc1 + j);  // F(j+1)
      drj = __ldg(gs.dr + j);  // DIFR(j)
    }
  }
  unsigned long long mb = 0, mb_all = 0;
  float s32 = 0.0f, s2_32 = 0.0f;
  int e = NO_SCALE;  // set by the thread's first nonzero entry
  bool big = false;
  const long srows = gs.srows > 0 ? gs.srows : (long)kp;
  double* row = Ht + (long)j * kp;
  for (int kk = threadIdx.x; kk < kp; kk += blockDim.x) {
    double h = 0.0;
    if (kk < K) {
      if (KIND == KIND_CAUCHY) {
        if (gs.k1 > 0 && kk >= gs.k1) {
          const int t = kk - gs.k1;  // tail rows: dense, or Cauchy with the second row generators
          h = gs.B ? __ldg(gs.B + t + (long)j * gs.ldb) : cauchy_entry(__ldg(gs.Ur2 + t), v, vs, __ldg(gs.Dr2 + t) - w);
        } else {
          double d = __ldg(gs.Dr + kk), u = __ldg(gs.Ur + kk);
          h = cauchy_entry(u, v, vs, d - w);  // U(i)*V(j) / (D(i)-F(j))
        }
      } else if (KIND == KIND_CAUCHY_EIG) {
        if (gs.k1 > 0 && kk >= gs.k1) {
          // tail rows of merged products: dense, or CauchyEig rows in permuted order
          const int t = kk - gs.k1;
          h = gs.B ? __ldg(gs.B + t + (long)j * gs.ldb)
                   : cauchy_entry(__ldg(gs.Ur2 + t), v, vs,
                                  eig_den(__ldg(gs.Dr2 + t), w, w1, dlj, drj, __ldg(gs.rglob2 + t) - 1 <= gs.cg0 + j));
        } else {
          const double fi = __ldg(gs.Dr + kk), u = __ldg(gs.Ur + kk);
          const bool upper = gs.rglob ? (__ldg(gs.rglob + kk) - 1 <= gs.cg0 + j) : (kk - j <= gs.diag_off);
          h = cauchy_entry(u, v, vs, eig_den(fi, w, w1, dlj, drj, upper));
        }
      } else if (KIND == KIND_TOEPLITZ || KIND == KIND_HANKEL) {
        if (gs.k1 > 0 && kk >= gs.k1) {  // dense tail rows (the R P^T factor of a merged product)
          h = __ldg(gs.B + (kk - gs.k1) + (long)j * gs.ldb);
        } else {
          const long idx = KIND == KIND_TOEPLITZ ? (gs.order - 1) + j - kk : (long)kk + j;
          h = (gs.glen <= 0 || (idx >= 0 && idx < gs.glen)) ? __ldg(gs.g + idx) : 0.0;
        }
      } else {  // KIND_DENSE (the split DFT generates F in k_h_pass1_dft3)
        h = __ldg(gs.B + kk + (long)j * gs.ldb);
      }
    }
    row[kk] = h;
    unsigned long long b = (unsigned long long)__double_as_longlong(h) & ABS_MASK;
    mb_all = b > mb_all ? b : mb_all;
    if (kk >= srows) continue;
    mb = b > mb ? b : mb;
    if (e == NO_SCALE && b) e = (int)(b >> 52) - 1023;
    if (e != NO_SCALE) {
      const float f = abs_scaled_up(b, e, &big);
      s32 = __fadd_ru(s32, f);
      s2_32 = __fmaf_ru(f, f, s2_32);
    }
  }
  double s = 0.0, s2 = 0.0;
  if (big) {  // entries 2^56 times the thread's first one (or Inf/NaN): FP64 sums
    for (int kk = threadIdx.x; kk < srows; kk += blockDim.x) {
      const double h = row[kk];
      s += fabs(h);
      s2 = fma(h, h, s2);
    }
  } else if (e != NO_SCALE) {
    s = ldexp((double)s32, e);
    s2 = ldexp((double)s2_32, 2 * e);
  }
  __shared__ unsigned long long smax[32], smax_all[32];
  __shared__ double ssum[32], ssq[32];
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
    mb = ob > mb ? ob : mb;
    ob = __shfl_xor_sync(0xffffffffu, mb_all, o);
    mb_all = ob > mb_all ? ob : mb_all;
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) { smax[wid] = mb; smax_all[wid] = mb_all; ssum[wid] = s; ssq[wid] = s2; }
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    mb = ln < nw ? smax[ln] : 0ull;
    mb_all = ln < nw ? smax_all[ln] : 0ull;
    s = ln < nw ? ssum[ln] : 0.0;
    s2 = ln < nw ? ssq[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
      ob = __shfl_xor_sync(0xffffffffu, mb_all, o);
      mb_all = ob > mb_all ? ob : mb_all;
      s += __shfl_xor_sync(0xffffffffu, s, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (ln == 0) {
      if (hmax_all) hmax_all[j] = mb_all;
      hmax_bits[j] = mb;
      hsum[j] = s;
      hsq[j] = s2;
      if (mb > 0 && mb < INF_BITS && isfinite(s)) {
        double rho = s / __longlong_as_double((long long)mb);
        atomicMax(&prm->rho_bits, (unsigned long long)__double_as_longlong(rho));
      }
    }
  }
}

template <int KIND>
__global__ void k_h_pass1(GenSpec gs, int K, int kp, double* __restrict__ Ht,
                          unsigned long long* __restrict__ hmax_bits, double* __restrict__ hsum,
                          double* __restrict__ hsq, SplitDevParams* prm) {
  h_pass1_blk<KIND>(gs, K, kp, Ht, hmax_bits, hsum, hsq, prm, blockIdx.x);
}

// The same, also writing the column maxima over every generated row (the block step's
// exponents; hmax_bits then covers the first gs.srows rows).
template <int KIND>
__global__ void k_h_pass1_all(GenSpec gs, int K, int kp, double* __restrict__ Ht,
                              unsigned long long* __restrict__ hmax_bits, double* __restrict__ hsum,
                              double* __restrict__ hsq, SplitDevParams* prm,
                              unsigned long long* __restrict__ hmax_all) {
  h_pass1_blk<KIND>(gs, K, kp, Ht, hmax_bits, hsum, hsq, prm, blockIdx.x, hmax_all);
}

// Bits PA (rows of A) and PH (columns of H).  The integer product must satisfy
// |Z_ij| < 0.497 M for the CRT, with M = prod m_l: the symmetric reconstruction needs |Z| < M/2
// and the quotient estimate (ffix at 2^-19) errs by at most 16 * 128 * 0.5 * 2^-19 < 0.002 of M,
// a margin of 1.01 bits.  Two rigorous bounds of |Z_ij| =
// |sum_k A'_ik H'_kj| for |A'| <= 2^PA, |H'| <= 2^PH (rounding adds at most 1/2 per entry):
//   L1: 2^(PA+PH) * (rho + k 2^-9),      rho = max_j sum_k|H_kj| / max_k|H_kj|
//   CS: 2^(PA+PH) * (ra + sqrt(k)/512) * (rh + sqrt(k)/512),
//       ra = max_i ||A_i:||_2 / max_k|A_ik|, rh = max_j ||H_:j||_2 / max_k|H_kj|  (PA, PH >= 8).
// The budget PA + PH comes from the smaller bound.  It is split to balance the two rounding
// errors, ~2^-PA * c_A and ~2^-PH * c_H with c_A ~ rms_i(max|A_i:|)/rms(A),
// c_H ~ rms_j(max|H_:j|)/rms(H) (same constant factor): PH - PA = round(log2(c_H/c_A)).
// Partial maxima of the row / column ratios ||.||_2 / max|.| and sums of max^2 and ||.||_2^2
// over rows [i0, i1) of A and columns [j0, j1) of H; the block's totals land in thread 0's v.
__device__ __forceinline__ void params_partial(int i0, int i1, int j0, int j1, double rk,
                                               const unsigned long long* __restrict__ amax_bits,
                                               const double* __restrict__ asq,
                                               const unsigned long long* __restrict__ hmax_bits,
                                               const double* __restrict__ hsq, double v[6]) {
  double ra = 0.0, amx2 = 0.0, afro = 0.0, rh = 0.0, hmx2 = 0.0, hfro = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const unsigned long long b = amax_bits[i];
    if (b == 0 || b >= INF_BITS) continue;
    const double m = __longlong_as_double((long long)b), q = asq[i];
    const bool safe = m > 1e-140 && m < 1e140 && isfinite(q) && q > 0.0;
    ra = fmax(ra, safe ? sqrt(q) / m : rk);
    if (safe) { amx2 += m * m; afro += q; }
  }
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const unsigned long long b = hmax_bits[j];
    if (b == 0 || b >= INF_BITS) continue;
    const double m = __longlong_as_double((long long)b), q = hsq[j];
    const bool safe = m > 1e-140 && m < 1e140 && isfinite(q) && q > 0.0;
    rh = fmax(rh, safe ? sqrt(q) / m : rk);
    if (safe) { hmx2 += m * m; hfro += q; }
  }
  v[0] = ra; v[1] = amx2; v[2] = afro; v[3] = rh; v[4] = hmx2; v[5] = hfro;
  // block reduction: max for ra/rh, sums otherwise
  for (int o = 16; o > 0; o >>= 1)
    for (int t = 0; t < 6; ++t) {
      double w = __shfl_xor_sync(0xffffffffu, v[t], o);
      v[t] = (t == 0 || t == 3) ? fmax(v[t], w) : v[t] + w;
    }
  __shared__ double sv[6][32];
  const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0)
    for (int t = 0; t < 6; ++t) sv[t][wid] = v[t];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int t = 0; t < 6; ++t) {
      double acc = sv[t][0];
      for (int w = 1; w < nw; ++w) acc = (t == 0 || t == 3) ? fmax(acc, sv[t][w]) : acc + sv[t][w];
      v[t] = acc;
    }
  }
}

// PA and PH from the totals (thread 0).
__device__ __forceinline__ void params_finish(SplitDevParams* prm, double log2M, int k, const double v[6]) {
  const double rk = sqrt((double)k);
  double rho = __longlong_as_double((long long)prm->rho_bits);
  if (!(rho >= 1.0)) rho = rk * rk;
  const double l1 = log2(rho * 1.01 + (double)k / 512.0);
  const double cs = log2((v[0] * 1.01 + rk / 512.0) * (v[3] * 1.01 + rk / 512.0));
  const double bound = fmin(l1, (v[0] > 0.0 && v[3] > 0.0) ? cs : l1);
  int budget = (int)floor(log2M - 1.01 - bound);
  int d = 0;
  if (v[1] > 0.0 && v[2] > 0.0 && v[4] > 0.0 && v[5] > 0.0) {
    const double cA = sqrt(v[1] / v[2]), cH = sqrt(v[4] / v[5]);
    d = (int)lrint(log2(cH / cA));
    d = max(-12, min(12, d));
  }
  int PA = (budget - d) >> 1, PH = budget - PA;
  if (PH > 53) { PA += PH - 53; PH = 53; }
  if (PA > 53) { PH += PA - 53; PA = 53; }
  prm->PA = max(8, min(53, PA));
  prm->PH = max(8, min(53, PH));
}

// One block over all rows and columns (the grouped launches: one block per product).
__device__ __forceinline__ void split_params_blk(SplitDevParams* prm, double log2M, int n, int ncols, int k,
                                                 const unsigned long long* __restrict__ amax_bits,
                                                 const double* __restrict__ asq,
                                                 const unsigned long long* __restrict__ hmax_bits,
                                                 const double* __restrict__ hsq) {
  double v[6];
  params_partial(0, n, 0, ncols, sqrt((double)k), amax_bits, asq, hmax_bits, hsq, v);
  if (threadIdx.x == 0) params_finish(prm, log2M, k, v);
}

// PARAMS_BLOCKS blocks, each over a slice of the rows and columns (the square roots and
// divisions are FP64); the last block to finish combines the partials in block order, so the
// result does not depend on the finishing order.
__global__ void k_split_params(SplitDevParams* prm, double log2M, int n, int ncols, int k,
                               const unsigned long long* __restrict__ amax_bits, const double* __restrict__ asq,
                               const unsigned long long* __restrict__ hmax_bits, const double* __restrict__ hsq) {
  const int G = gridDim.x, b = blockIdx.x;
  const int i0 = (int)((long)n * b / G), i1 = (int)((long)n * (b + 1) / G);
  const int j0 = (int)((long)ncols * b / G), j1 = (int)((long)ncols * (b + 1) / G);
  double v[6];
  params_partial(i0, i1, j0, j1, sqrt((double)k), amax_bits, asq, hmax_bits, hsq, v);
  if (threadIdx.x == 0) {
    for (int t = 0; t < 6; ++t) prm->part[b][t] = v[t];
    __threadfence();
    if (atomicAdd(&prm->done, 1u) == (unsigned)G - 1) {
      __threadfence();
      double tot[6];
      for (int t = 0; t < 6; ++t) tot[t] = __ldcg(&prm->part[0][t]);
      for (int q = 1; q < G; ++q)
        for (int t = 0; t < 6; ++t) {
          const double x = __ldcg(&prm->part[q][t]);
          tot[t] = (t == 0 || t == 3) ? fmax(tot[t], x) : tot[t] + x;
        }
      params_finish(prm, log2M, k, tot);
    }
  }
}

// floor(log2 x) from the bits of a positive finite double, on the integer pipe (GB300's FP64
// pipe is narrow, and the library ilogb goes through it).
__device__ __forceinline__ int ilogb_bits(unsigned long long b) {
  const int ex = (int)(b >> 52);
  return ex ? ex - 1023 : 63 - __clzll((long long)b) - 1074;  // subnormal: b is the mantissa
}

// Exponent s such that |x * 2^s| < 2^P for all |x| <= amax (amax finite, > 0).
__device__ __forceinline__ int scale_exp(unsigned long long amax_bits, int P) {
  return P - 1 - ilogb_bits(amax_bits);
}

// rint(x * 2^e) (round half to even) for finite x with |x * 2^e| < 2^53, computed from the
// bits of x with integer operations only; *neg receives the sign.
__device__ __forceinline__ unsigned long long scaled_int(double x, int e, bool* neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  *neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  int E = -1074;
  if (ex != 0) {
    m |= 1ull << 52;
    E = ex - 1075;
  }
  const int sh = E + e;
  if (sh >= 0) return m << sh;  // the caller's bound keeps the result below 2^53
  const int k = -sh;
  if (k > 63) return 0;  // below one half
  // round half to even: m / 2^k + 1/2 - 2^-k, plus 2^-k when the last kept bit is odd
  return (m + ((1ull << (k - 1)) - 1) + ((m >> k) & 1)) >> k;
}

// Residues of neighbouring integers for every modulus, on the FP32 pipe.  A scaled integer
// x < 2^53 with sign s is cut into x0 = x mod 2^23, x1 = (x >> 23) mod 2^15 and x2 = x >> 38
// (< 2^15); the signed chunks s*x_i are exact floats.  With g1 = 2^23 mod m and g2 = 2^38 mod m
// taken symmetric (|g| <= m/2 <= 128), t = s*x0 + g1*s*x1 + g2*s*x2 is congruent to s*x modulo
// m and |t| < 2^23 + 2*128*2^15 = 2^24, so both FMAs are exact.  q = rint(t * fl(1/m)) comes from
// one FMA on the magic number 1.5*2^23 (|t*fl(1/m) - t/m| <= |t|/m * 2^-24 < 1/m), and
// r = t - q*m is one exact FMA with |r| < m/2 + 1, i.e. |r| <= 128 for every modulus <= 256
// (1/m is exact for m = 256).  An integer of at most 8 significant bits is its own BF16: the
// float's upper half.  The modulus loop is unrolled over the maximum count, so the per-modulus
// constants are kernel-parameter operands.
struct ResidueChunks {
  float c0, c1, c2;
};

__device__ __forceinline__ ResidueChunks residue_chunks(unsigned long long u, bool neg) {
  const float s = neg ? -1.0f : 1.0f, o = neg ? 8388608.0f : -8388608.0f;
  const unsigned lo = (unsigned)u, hi = (unsigned)(u >> 32);
  const unsigned x0 = lo & 0x7FFFFFu;
  const unsigned x1 = __funnelshift_r(lo, hi, 23) & 0x7FFFu;
  const unsigned x2 = hi >> 6;
  ResidueChunks c;
  c.c0 = fmaf(__uint_as_float(0x4B000000u | x0), s, o);  // s * (2^23 + x0) - s * 2^23
  c.c1 = fmaf(__uint_as_float(0x4B000000u | x1), s, o);
  c.c2 = fmaf(__uint_as_float(0x4B000000u | x2), s, o);
  return c;
}

__device__ __forceinline__ float residue_f(const ResidueChunks& c, float g23, float g38, float inv, float mf) {
  const float t = fmaf(c.c2, g38, fmaf(c.c1, g23, c.c0));
  const float q = fmaf(t, inv, 12582912.0f) - 12582912.0f;
  return fmaf(-q, mf, t);
}

__device__ __forceinline__ unsigned residue_bits(const ResidueChunks& c, float g23, float g38, float inv, float mf) {
  return __float_as_uint(residue_f(c, g23, g38, inv, mf));
}

// Residues of a signed integer V with |V| < 2^56 (a signed sum of up to eight scaled integers
// below 2^53): its magnitude cut into four 14-bit chunks c_i (exact floats by the same
// 2^23-offset trick, signed), t = c0 + g14 c1 + g28 c2 + g42 c3 with g = 2^(14 i) mod m taken
// symmetric is congruent to V and |t| < 2^14 * (1 + 3 * 128) < 2^23, so the FMAs are exact;
// quotient and remainder as in residue_f.
struct ResidueChunks4 {
  float c[4];
};

__device__ __forceinline__ ResidueChunks4 residue_chunks4(long long V) {
  const bool neg = V < 0;
  const unsigned long long u = neg ? (unsigned long long)(-V) : (unsigned long long)V;
  const float s = neg ? -1.0f : 1.0f, o = neg ? 8388608.0f : -8388608.0f;
  ResidueChunks4 r;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    r.c[i] = fmaf(__uint_as_float(0x4B000000u | (unsigned)((u >> (14 * i)) & 0x3FFFull)), s, o);
  return r;
}

__device__ __forceinline__ float residue4_f(const ResidueChunks4& c, float g14, float g28, float g42, float inv,
                                            float mf) {
  const float t = fmaf(c.c[3], g42, fmaf(c.c[2], g28, fmaf(c.c[1], g14, c.c[0])));
  const float q = fmaf(t, inv, 12582912.0f) - 12582912.0f;
  return fmaf(-q, mf, t);
}

// (a + b) mod m in [-128, 128] for residues |a|, |b| <= 128 (exact floats): the quotient
// rint((a + b) / m) is in {-1, 0, 1} and its float estimate is off by at most 2^-23.
__device__ __forceinline__ float residue_sum(float a, float b, float inv, float mf) {
  const float t = a + b;
  const float q = fmaf(t, inv, 12582912.0f) - 12582912.0f;
  return fmaf(-q, mf, t);
}

// The same for four neighbouring integers: one 8-byte store per plane.
__device__ __forceinline__ void write_residue_quad(const unsigned long long (&u)[4], const bool (&ng)[4],
                                                   const CrtConsts& cc, uint2* dst, size_t plane_u2) {
  ResidueChunks c[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) c[q] = residue_chunks(u[q], ng[q]);
#pragma unroll
  for (int l = 0; l < SPL_MAX_MODULI; ++l) {
    if (l < cc.nmod) {
      const float g23 = cc.g23[l], g38 = cc.g38[l], inv = cc.inv_m[l], mf = cc.mf[l];
      unsigned f[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) f[q] = residue_bits(c[q], g23, g38, inv, mf);
      *dst = make_uint2(__byte_perm(f[0], f[1], 0x7632), __byte_perm(f[2], f[3], 0x7632));
      dst += plane_u2;
    }
  }
}

// residues_H: consecutive kk per thread, and the grid width of a column
constexpr int RH_PER_THREAD = 4;
__host__ __device__ __forceinline__ int rh_blocks_x(int kp) { return (kp / RH_PER_THREAD + 127) / 128; }

// RA[l][i][kk] = residues of A' (bf16), rows i, K-major.  Block: TR (32 or 64) rows x 64 k,
// transposed through shared memory with element (k, r) at column (r + k/4) mod TR of row k, so
// that both the column-wise writes (the rows of one k) and the reads (16 threads, 4
// consecutive k each, of one row) touch 16 distinct 8-byte bank pairs per half-warp.
template <int TR = 32>
__device__ __forceinline__ void residues_A_blk(const double* __restrict__ A, long lda, const double* A2, long lda2,
                                               int ka, int n, int k, int kp,
                                               const unsigned long long* __restrict__ amax_bits,
                                               const SplitDevParams* prm, const CrtConsts& cc,
                                               __nv_bfloat16* __restrict__ RA, int bx, int by) {
  __shared__ double tile[64][TR];
  const int i0 = by * TR, k0 = bx * 64;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads: 8 x 32
  for (int kk = ty; kk < 64; kk += 8) {
    const int gk = k0 + kk;
#pragma unroll
    for (int rr = tx; rr < TR; rr += 32) {
      const int gi = i0 + rr;
      tile[kk][(rr + (kk >> 2)) & (TR - 1)] = (gi < n && gk < k) ? __ldg(acol(A, lda, A2, lda2, ka, gk) + gi) : 0.0;
    }
  }
  __syncthreads();
  const int P = prm->PA;
  const size_t plane = (size_t)n * kp;
  const int tq = threadIdx.x & 15, tr = threadIdx.x >> 4;  // 16 quads of k x 16 rows
  for (int r = tr; r < TR; r += 16) {
    int gi = i0 + r;
    if (gi >= n) continue;
    unsigned long long ab = amax_bits[gi];
    bool ok = ab > 0 && ab < INF_BITS;
    int e = ok ? scale_exp(ab, P) : 0;
    const int kk = 4 * tq;
    unsigned long long u[4];
    bool ng[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      ng[q] = false;
      u[q] = ok ? scaled_int(tile[kk + q][(r + tq) & (TR - 1)], e, &ng[q]) : 0ull;
    }
    write_residue_quad(u, ng, cc, (uint2*)(RA + (size_t)gi * kp + k0 + kk), plane / 4);
  }
}

__global__ void k_residues_A(const double* __restrict__ A, long lda, int n, int k, int kp,
                             const unsigned long long* __restrict__ amax_bits, const SplitDevParams* prm,
                             CrtConsts cc, __nv_bfloat16* __restrict__ RA) {
  residues_A_blk<64>(A, lda, nullptr, 0, k, n, k, kp, amax_bits, prm, cc, RA, blockIdx.x, blockIdx.y);
}

// Rows [64 by0, 64 (by0 + gridDim.y)) of A only (a row panel of the host pipeline).
__global__ void k_residues_A_rows(const double* __restrict__ A, long lda, int n, int k, int kp,
                                  const unsigned long long* __restrict__ amax_bits, const SplitDevParams* prm,
                                  CrtConsts cc, __nv_bfloat16* __restrict__ RA, int by0) {
  residues_A_blk<64>(A, lda, nullptr, 0, k, n, k, kp, amax_bits, prm, cc, RA, blockIdx.x, by0 + blockIdx.y);
}

// The guessed bit counts that a speculative host pipeline scales with.
__global__ void k_guess_params(SplitDevParams* g, int PA, int PH) {
  g->PA = PA;
  g->PH = PH;
}

// RH[l][j][kk] = residues of H' (bf16) from Ht[j][kk]; one thread per 4 consecutive kk.
__device__ __forceinline__ void residues_H_blk(const double* __restrict__ Ht, int ncols, int kp,
                                               const unsigned long long* __restrict__ hmax_bits,
                                               const SplitDevParams* prm, const CrtConsts& cc,
                                               __nv_bfloat16* __restrict__ RH, int bx, int by, int ph = -1,
                                               int krows = 1 << 30) {
  const int j = by;
  const int kk = RH_PER_THREAD * (bx * blockDim.x + threadIdx.x);
  if (kk >= kp) return;  // kp is a multiple of 64: a thread's four entries are all inside
  const int P = ph >= 0 ? ph : prm->PH;
  unsigned long long hb = hmax_bits[j];
  bool ok = hb > 0 && hb < INF_BITS;
  int e = ok ? scale_exp(hb, P) : 0;
  const double2 h01 = *(const double2*)(Ht + (size_t)j * kp + kk);
  const double2 h23 = *(const double2*)(Ht + (size_t)j * kp + kk + 2);
  const double hv[4] = {h01.x, h01.y, h23.x, h23.y};
  unsigned long long u[4];
  bool ng[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    ng[q] = false;
    u[q] = (ok && kk + q < krows) ? scaled_int(hv[q], e, &ng[q]) : 0ull;
  }
  const size_t plane = (size_t)ncols * kp;
  write_residue_quad(u, ng, cc, (uint2*)(RH + (size_t)j * kp + kk), plane / 4);
}

__global__ void k_residues_H(const double* __restrict__ Ht, int ncols, int kp,
                             const unsigned long long* __restrict__ hmax_bits, const SplitDevParams* prm,
                             CrtConsts cc, __nv_bfloat16* __restrict__ RH) {
  residues_H_blk(Ht, ncols, kp, hmax_bits, prm, cc, RH, blockIdx.y, blockIdx.x);  // x: column (any count)
}

// Speculative H residues: with guess >= 0 and !redo, the planes for PH = guess (before the
// parameter pass has run); with redo, nothing when the parameter pass chose PH == guess, else
// the planes for the chosen PH.
__global__ void k_residues_H_spec(const double* __restrict__ Ht, int ncols, int kp,
                                  const unsigned long long* __restrict__ hmax_bits, const SplitDevParams* prm,
                                  CrtConsts cc, __nv_bfloat16* __restrict__ RH, int guess, int redo) {
  if (redo && prm->PH == guess) return;
  residues_H_blk(Ht, ncols, kp, hmax_bits, prm, cc, RH, blockIdx.y, blockIdx.x, redo ? -1 : guess);
}

// ---- Block-recursive Toeplitz / Hankel products (split_core_block) --------------------------
// H (N x N) is cut into 2^L x 2^L blocks of width w = N / 2^L.  Columns j, j + w, ..., j + (2^L - 1) w
// form a group that shares one scaling exponent, from the group maximum gmax[j] of the column
// maxima, so that the integer-scaled H' keeps the block identities of the structure (Toeplitz:
// block (r, c) depends on c - r only; Hankel: on r + c) exactly.  The per-column maxima stay
// in hmax (the parameter pass's bounds hold for either exponent, which is never larger).
// prm->hbad turns the block step off for the call -- the gated kernels then take the single
// product with per-column exponents (k_residues_H_gated, the plain GEMM) -- when a column is
// not finite (zeroing it would break the identities; the single product returns NaN in exactly
// the non-finite columns) or when a nonzero column's maximum is more than 2^kBlockMaxSpread
// below its group's (its entries would lose that many bits to the shared exponent).
constexpr int kBlockMaxSpread = 4;
// hmax_bits here: the maxima over every row of the (possibly padded) H.
__global__ void k_group_colmax(const unsigned long long* __restrict__ hmax_bits,
                               unsigned long long* __restrict__ gmax_bits, int w, int nq, SplitDevParams* prm,
                               SplitDevParams* prm2) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= w) return;
  unsigned long long m = 0, mn = ~0ull;
  bool bad = false;
  for (int c = 0; c < nq; ++c) {
    const unsigned long long b = hmax_bits[g + (size_t)c * w];
    bad |= b >= INF_BITS;
    if (b < INF_BITS && b > m) m = b;
    if (b > 0 && b < mn) mn = b;
  }
  if (!bad && m > 0 && ilogb_bits(m) - ilogb_bits(mn) > kBlockMaxSpread) bad = true;
  if (bad) {
    prm->hbad = 1u;
    if (prm2) prm2->hbad = 1u;  // the guessed parameters of a speculative pipeline gate too
  }
  gmax_bits[g] = m;
}

// Signed sums of A's blocks that the leaf products take as their A operand.  Block q starts at
// row qrow[q] (relative to the pass's first row) and column qcol[q]; operand p adds the blocks
// of mask[p] and subtracts those of neg[p] (a subset of mask[p]).
constexpr int BLK_MAX_LEVELS = 3;
constexpr int BLK_MAX_LEAVES = 27;  // 3^BLK_MAX_LEVELS
struct BlockSums {
  int nsum;
  int wmask;  // blocks whose own residues are written to RA (the others are only summed)
  int mask[BLK_MAX_LEAVES], neg[BLK_MAX_LEAVES];
  int qrow[1 << BLK_MAX_LEVELS], qcol[1 << BLK_MAX_LEVELS];
};

// A residues of a block product: RA[l][r0 + qrow[q] + i][qcol[q] + kk] for every block q (as
// k_residues_A writes them) and RS[p][l][rs_r0 + i][kk] (planes of rs_rows rows) = the signed
// block sum p mod m_l, for i < rows, kk < w; columns from kvalid on read as zero (A padded
// with zero columns).  Each block row keeps its own exponent (rows of different blocks are different rows of
// A).  One CTA: 32 rows x 64 columns of each of the NQ blocks, transposed through shared memory
// (NQ tiles of 64 x 32 doubles, the swizzle of residues_A_blk); each thread keeps the signed
// scaled integers of its 4 columns of every block, so the sums need no second pass over A.
template <int NQ>
__global__ void __launch_bounds__(256) k_residues_A_blocks(const double* __restrict__ A, long lda, int M, int r0,
                                                           int rows, int w, int kp, int kvalid, int rs_rows, int rs_r0,
                                                           const unsigned long long* __restrict__ amax_bits,
                                                           const SplitDevParams* prm, CrtConsts cc,
                                                           __nv_bfloat16* __restrict__ RA,
                                                           __nv_bfloat16* __restrict__ RS,
                                                           const __grid_constant__ BlockSums bs) {
  constexpr int TR = 32;
  extern __shared__ double blk_tiles[];  // [NQ][64][TR]
  const int i0 = blockIdx.y * TR, k0 = blockIdx.x * 64;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q)
    for (int kk = ty; kk < 64; kk += 8) {
      const long gi = (long)r0 + bs.qrow[q] + i0 + tx;
      const long gk = (long)bs.qcol[q] + k0 + kk;
      blk_tiles[(q * 64 + kk) * TR + ((tx + (kk >> 2)) & (TR - 1))] =
          (i0 + tx < rows && gk < kvalid) ? __ldg(A + gk * lda + gi) : 0.0;
    }
  __syncthreads();
  const int P = prm->PA;
  const int nsum = prm->hbad ? 0 : bs.nsum;  // the single product needs no block sums
  const size_t plane = (size_t)M * kp, splane = (size_t)rs_rows * w;
  const int tq = threadIdx.x & 15, tr = threadIdx.x >> 4;
  for (int r = tr; r < TR; r += 16) {
    if (i0 + r >= rows) continue;
    const int kk = 4 * tq;
    long long sv[NQ][4];  // the signed scaled integers of the thread's 4 columns of every block
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const long gi = (long)r0 + bs.qrow[q] + i0 + r;
      const unsigned long long ab = amax_bits[gi];
      const bool ok = ab > 0 && ab < INF_BITS;
      const int e = ok ? scale_exp(ab, P) : 0;
      unsigned long long u[4];
      bool ng[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        ng[v] = false;
        u[v] = ok ? scaled_int(blk_tiles[(q * 64 + kk + v) * TR + ((r + tq) & (TR - 1))], e, &ng[v]) : 0ull;
        sv[q][v] = ng[v] ? -(long long)u[v] : (long long)u[v];
      }
      if ((bs.wmask >> q) & 1)
        write_residue_quad(u, ng, cc, (uint2*)(RA + (size_t)gi * kp + bs.qcol[q] + k0 + kk), plane / 4);
    }
    for (int p = 0; p < nsum; ++p) {
      const int mk = bs.mask[p], ngm = bs.neg[p];
      ResidueChunks4 c4[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        long long V = 0;
#pragma unroll
        for (int q = 0; q < NQ; ++q) V += ((mk >> q) & 1) ? (((ngm >> q) & 1) ? -sv[q][v] : sv[q][v]) : 0ll;
        c4[v] = residue_chunks4(V);
      }
      uint2* dst = (uint2*)(RS + (size_t)p * cc.nmod * splane + (size_t)(rs_r0 + i0 + r) * w + k0 + kk);
#pragma unroll
      for (int l = 0; l < SPL_MAX_MODULI; ++l) {
        if (l < cc.nmod) {
          const float g14 = cc.g14[l], g28 = cc.g28[l], g42 = cc.g42[l], inv = cc.inv_m[l], mf = cc.mf[l];
          unsigned f[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) f[v] = __float_as_uint(residue4_f(c4[v], g14, g28, g42, inv, mf));
          *dst = make_uint2(__byte_perm(f[0], f[1], 0x7632), __byte_perm(f[2], f[3], 0x7632));
          dst += splane / 4;
        }
      }
    }
  }
}

// H operands of the leaf products: leaf y is sum_t sign[y][t] * H'(kk' + koff[y][t], j' + joff[y][t])
// for kk' < wk, j' < wn, a signed sum of up to 2^L blocks of the integer-scaled H, each entry
// scaled with the group exponent of column j' (group != 0: the structured block step) or with
// its own column's (Strassen's step, which needs no structure).  Entries of a non-finite column
// count as zero (the recombination returns NaN there).
struct LeafTerms {
  int nterm[BLK_MAX_LEAVES];
  signed char sign[BLK_MAX_LEAVES][1 << BLK_MAX_LEVELS];
  int koff[BLK_MAX_LEAVES][1 << BLK_MAX_LEVELS], joff[BLK_MAX_LEAVES][1 << BLK_MAX_LEVELS];
};

// RHL[y][l][j'][kk'] (pitch wk) from Ht: grid (wn columns j', kk' blocks of 512, leaves y); one
// thread per 4 consecutive kk'.  hmax_bits: maxima over every row of the columns read (a term of
// an all-zero column is skipped).
template <int NT>
__global__ void __launch_bounds__(128) k_residues_H_leaf(const double* __restrict__ Ht, int kp, int wk, int wn,
                                                         const unsigned long long* __restrict__ hmax_bits,
                                                         const unsigned long long* __restrict__ gmax_bits,
                                                         int group, const SplitDevParams* prm, CrtConsts cc,
                                                         const __grid_constant__ LeafTerms lt,
                                                         __nv_bfloat16* __restrict__ RHL) {
  const int j = blockIdx.x, y = blockIdx.z;
  const int kk = RH_PER_THREAD * (blockIdx.y * blockDim.x + threadIdx.x);
  if (kk >= wk || prm->hbad) return;  // wk is a multiple of 64: a thread's four entries are all inside
  const int PH = prm->PH;
  const unsigned long long gb = group ? gmax_bits[j] : 0ull;
  const bool gok = !group || (gb > 0 && gb < INF_BITS);
  const int nt = lt.nterm[y];
  long long V[4] = {0, 0, 0, 0};  // exact: up to 8 terms below 2^53
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    if (t >= nt) break;
    const int col = j + lt.joff[y][t];
    const unsigned long long hb = hmax_bits[col];
    if (!gok || hb == 0 || hb >= INF_BITS) continue;
    const int e = scale_exp(group ? gb : hb, PH);
    const double* src = Ht + (size_t)col * kp + lt.koff[y][t] + kk;
    const double2 h01 = *(const double2*)src, h23 = *(const double2*)(src + 2);
    const double hv[4] = {h01.x, h01.y, h23.x, h23.y};
    const int sg = lt.sign[y][t];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      bool ng = false;
      const long long u = (long long)scaled_int(hv[v], e, &ng);
      V[v] += (ng != (sg < 0)) ? -u : u;
    }
  }
  ResidueChunks4 c4[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) c4[v] = residue_chunks4(V[v]);
  const size_t plane = (size_t)wn * wk;
  uint2* dst = (uint2*)(RHL + (size_t)y * cc.nmod * plane + (size_t)j * wk + kk);
#pragma unroll
  for (int l = 0; l < SPL_MAX_MODULI; ++l) {
    if (l < cc.nmod) {
      const float g14 = cc.g14[l], g28 = cc.g28[l], g42 = cc.g42[l], inv = cc.inv_m[l], mf = cc.mf[l];
      unsigned f[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) f[v] = __float_as_uint(residue4_f(c4[v], g14, g28, g42, inv, mf));
      *dst = make_uint2(__byte_perm(f[0], f[1], 0x7632), __byte_perm(f[2], f[3], 0x7632));
      dst += plane / 4;
    }
  }
}

// The seven H operands of Strassen's step (B00 + B11, B00, B01 - B11, B10 - B00, B11, B00 + B01,
// B10 + B11 in the order of the products) from the four blocks of Ht read once: RHS[y][l][j'][kk']
// (pitch wk) for j' < wn, kk' < wk; every entry scaled with its own column's exponent.  Grid (wn
// columns, kk' blocks of 512); one thread per 4 consecutive kk'.
__global__ void __launch_bounds__(128) k_residues_H_s2(const double* __restrict__ Ht, int kp, int wk, int wn,
                                                       const unsigned long long* __restrict__ hmax_bits,
                                                       const SplitDevParams* prm, CrtConsts cc,
                                                       __nv_bfloat16* __restrict__ RHS) {
  const int j = blockIdx.x;
  const int kk = RH_PER_THREAD * (blockIdx.y * blockDim.x + threadIdx.x);
  if (kk >= wk) return;
  const int PH = prm->PH;
  long long b[2][2][4];  // b[r][c][v]: block (r, c), the thread's 4 entries
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int col = j + c * wn;
    const unsigned long long hb = hmax_bits[col];
    const bool ok = hb > 0 && hb < INF_BITS;
    const int e = ok ? scale_exp(hb, PH) : 0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      double hv[4] = {0.0, 0.0, 0.0, 0.0};
      if (ok) {
        const double* src = Ht + (size_t)col * kp + r * wk + kk;
        const double2 h01 = *(const double2*)src, h23 = *(const double2*)(src + 2);
        hv[0] = h01.x; hv[1] = h01.y; hv[2] = h23.x; hv[3] = h23.y;
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        bool ng = false;
        const long long u = ok ? (long long)scaled_int(hv[v], e, &ng) : 0ll;
        b[r][c][v] = ng ? -u : u;
      }
    }
  }
  const size_t plane = (size_t)wn * wk;
#pragma unroll
  for (int y = 0; y < 7; ++y) {
    ResidueChunks4 c4[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const long long V = y == 0 ? b[0][0][v] + b[1][1][v] : y == 1 ? b[0][0][v] : y == 2 ? b[0][1][v] - b[1][1][v]
                        : y == 3 ? b[1][0][v] - b[0][0][v] : y == 4 ? b[1][1][v] : y == 5 ? b[0][0][v] + b[0][1][v]
                                                                                        : b[1][0][v] + b[1][1][v];
      c4[v] = residue_chunks4(V);
    }
    uint2* dst = (uint2*)(RHS + (size_t)y * cc.nmod * plane + (size_t)j * wk + kk);
#pragma unroll
    for (int l = 0; l < SPL_MAX_MODULI; ++l) {
      if (l < cc.nmod) {
        const float g14 = cc.g14[l], g28 = cc.g28[l], g42 = cc.g42[l], inv = cc.inv_m[l], mf = cc.mf[l];
        unsigned f[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) f[v] = __float_as_uint(residue4_f(c4[v], g14, g28, g42, inv, mf));
        *dst = make_uint2(__byte_perm(f[0], f[1], 0x7632), __byte_perm(f[2], f[3], 0x7632));
        dst += plane / 4;
      }
    }
  }
}

// The residues of the whole H (as k_residues_H) when prm->hbad is set; columns j = blockIdx.x +
// gridDim.x t.
// Rows from krows on (the padding of a padded H) get zero residues.
__global__ void k_residues_H_gated(const double* __restrict__ Ht, int ncols, int kp, int krows,
                                   const unsigned long long* __restrict__ hmax_bits, const SplitDevParams* prm,
                                   CrtConsts cc, __nv_bfloat16* __restrict__ RH) {
  if (!prm->hbad) return;
  for (int j = blockIdx.x; j < ncols; j += gridDim.x)
    residues_H_blk(Ht, ncols, kp, hmax_bits, prm, cc, RH, blockIdx.y, j, -1, krows);
}

// DFT A side: row i of the product (B^T) is column i of B, read contiguously (Bre = B as
// interleaved doubles, ldb2 = 2*ldb); its maximum and sum of squares run over both the real
// and the imaginary parts.  One block per row.
__global__ void k_row_absmax_dft(const double* __restrict__ Bre, long ldb2, int nn,
                                 unsigned long long* __restrict__ amax_bits, double* __restrict__ asq) {
  const int i = blockIdx.x;
  const double* col = Bre + (long)i * ldb2;
  unsigned long long mb = 0;
  // sum of squares in round-up FP32 on the thread's power-of-two scale (an upper bound), FP64
  // for a thread whose entries reach 2^56 times its first one
  float sq32 = 0.0f;
  int e = NO_SCALE;
  bool big = false;
  for (int t = threadIdx.x; t < 2 * nn; t += blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(__ldg(col + t)) & ABS_MASK;
    mb = b > mb ? b : mb;
    if (e == NO_SCALE && b) e = (int)(b >> 52) - 1023;
    if (e != NO_SCALE) {
      const float f = abs_scaled_up(b, e, &big);
      sq32 = __fmaf_ru(f, f, sq32);
    }
  }
  double sq = 0.0;
  if (big) {
    for (int t = threadIdx.x; t < 2 * nn; t += blockDim.x) {
      const double a = __ldg(col + t);
      sq = fma(a, a, sq);
    }
  } else if (e != NO_SCALE) {
    sq = ldexp((double)sq32, 2 * e);
  }
  __shared__ unsigned long long smax[32];
  __shared__ double ssq[32];
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
    mb = ob > mb ? ob : mb;
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
  }
  const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) { smax[wid] = mb; ssq[wid] = sq; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      mb = smax[w] > mb ? smax[w] : mb;
      sq += ssq[w];
    }
    amax_bits[i] = mb;
    asq[i] = sq;
  }
}

// The radix step's B' (as k_dft_deinterleave: B'(m, r k + c) = B(R m + r, c), ld n/R) and, in
// the same pass over B, the statistics k_row_absmax_dft takes of the product's rows (the
// columns of B').  Block c takes column c of B; with 256 a multiple of R, thread t meets only
// entries l = t mod R, i.e. row r k + c for r = t mod R, and the threads of one r are reduced
// together (lanes xor 16 .. R, then the eight warps).
template <int R>
__global__ void __launch_bounds__(256) k_dft_deinterleave_stats(const double2* __restrict__ B, long ldb, int n,
                                                                int k, double2* __restrict__ Bp,
                                                                unsigned long long* __restrict__ amax_bits,
                                                                double* __restrict__ asq) {
  static_assert(256 % R == 0 && R <= 32, "a thread meets one residue class of l mod R");
  const int nq = n / R;
  const int r = threadIdx.x % R;
  const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  __shared__ unsigned long long smax[8][R];
  __shared__ double ssq[8][R];
  for (int c = blockIdx.x; c < k; c += gridDim.x) {
    const double2* col = B + (long)c * ldb;
    double2* dst = Bp + ((size_t)r * k + c) * nq;
    unsigned long long mb = 0;
    // as k_row_absmax_dft: round-up FP32 squares on the thread's power-of-two scale, FP64 for a
    // thread whose entries reach 2^56 times its first one
    float sq32 = 0.0f;
    int e = NO_SCALE;
    bool big = false;
    for (int l = threadIdx.x; l < n; l += 256) {
      const double2 v = __ldg(col + l);
      dst[l / R] = v;
      const unsigned long long b0 = (unsigned long long)__double_as_longlong(v.x) & ABS_MASK;
      const unsigned long long b1 = (unsigned long long)__double_as_longlong(v.y) & ABS_MASK;
      mb = b0 > mb ? b0 : mb;
      mb = b1 > mb ? b1 : mb;
      if (e == NO_SCALE && (b0 | b1)) e = (int)((b0 ? b0 : b1) >> 52) - 1023;
      if (e != NO_SCALE) {
        const float f0 = abs_scaled_up(b0, e, &big), f1 = abs_scaled_up(b1, e, &big);
        sq32 = __fmaf_ru(f0, f0, sq32);
        sq32 = __fmaf_ru(f1, f1, sq32);
      }
    }
    double sq = 0.0;
    if (big) {
      for (int l = threadIdx.x; l < n; l += 256) {
        const double2 v = __ldg(col + l);
        sq = fma(v.x, v.x, sq);
        sq = fma(v.y, v.y, sq);
      }
    } else if (e != NO_SCALE) {
      sq = ldexp((double)sq32, 2 * e);
    }
    for (int o = 16; o >= R; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
      sq += __shfl_xor_sync(0xffffffffu, sq, o);
    }
    if (ln < R) {
      smax[wid][ln] = mb;
      ssq[wid][ln] = sq;
    }
    __syncthreads();
    if (threadIdx.x < R) {
      unsigned long long m2 = smax[0][threadIdx.x];
      double s2 = ssq[0][threadIdx.x];
      for (int w = 1; w < 8; ++w) {
        m2 = smax[w][threadIdx.x] > m2 ? smax[w][threadIdx.x] : m2;
        s2 += ssq[w][threadIdx.x];
      }
      amax_bits[(size_t)threadIdx.x * k + c] = m2;
      asq[(size_t)threadIdx.x * k + c] = s2;
    }
    __syncthreads();  // the shared partials are reused for the next column
  }
}

// The radix step around the 3M core: B (n x k complex, ldb) deinterleaved into Bp; the result
// C (n x k complex, ldc) = alpha F_n B + beta C from the core's residues with the table wn.
struct DftRadixSrc {
  const double2* B;
  long ldb;
  int n, k, R;
  double2* Bp;
  const double2* wn;
  double beta;
  double2* C;
  long ldc;
};

// ---- the DFT as three real products (3M form) ----------------------------------------------
// C^T = B^T F with F(j, l) = w^(j l), w = exp(-2 pi i / n), F symmetric: Re = T1 - T2 and
// Im = T3 - T1 - T2 for T1 = Br^T Fr, T2 = Bi^T Fi, T3 = (Br + Bi)^T (Fr + Fi).  Rows of A (columns
// of B) and columns of F are scaled as in the real embedding [Re B^T | Im B^T] x
// [[Fr, Fi], [-Fi, Fr]] (one exponent per complex row / column), so the integer products, and
// the result, are those of the embedding, with three BF16 GEMMs per modulus instead of four.

// Ht = [Fr rows | Fi rows] (row j: column j of F = row j), the column maxima over |Fr| and |Fi|,
// sum_l |Fr| + |Fi| and sum_l Fr^2 + Fi^2 (the statistics of the embedding's column j and
// n + j).  One block per column.
__global__ void __launch_bounds__(256) k_h_pass1_dft3(const double2* __restrict__ wtab, int nn, int kp,
                                                      double* __restrict__ Ht, unsigned long long* __restrict__ hmax_bits,
                                                      double* __restrict__ hsum, double* __restrict__ hsq,
                                                      SplitDevParams* prm) {
  const int j = blockIdx.x;
  double* rr = Ht + (size_t)j * kp;
  double* ri = Ht + ((size_t)nn + j) * kp;
  unsigned long long mb = 0;
  float s32 = 0.0f, s2_32 = 0.0f;
  int e = NO_SCALE;
  bool big = false;
  // table index t = (l j) mod n, advanced by (blockDim j) mod n per step (no division per entry)
  int t = (int)(((long long)threadIdx.x * j) % nn);
  const int step = (int)(((long long)blockDim.x * j) % nn);
  for (int l = threadIdx.x; l < kp; l += blockDim.x) {
    double2 wv = make_double2(0.0, 0.0);
    if (l < nn) {
      wv = __ldg(wtab + t);
      t += step;
      t -= t >= nn ? nn : 0;
    }
    rr[l] = wv.x;
    ri[l] = wv.y;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(part ? wv.y : wv.x) & ABS_MASK;
      mb = b > mb ? b : mb;
      if (e == NO_SCALE && b) e = (int)(b >> 52) - 1023;
      if (e != NO_SCALE) {
        const float f = abs_scaled_up(b, e, &big);
        s32 = __fadd_ru(s32, f);
        s2_32 = __fmaf_ru(f, f, s2_32);
      }
    }
  }
  double s = 0.0, s2 = 0.0;
  if (big) {
    for (int l = threadIdx.x; l < kp; l += blockDim.x) {
      s += fabs(rr[l]) + fabs(ri[l]);
      s2 = fma(rr[l], rr[l], fma(ri[l], ri[l], s2));
    }
  } else if (e != NO_SCALE) {
    s = ldexp((double)s32, e);
    s2 = ldexp((double)s2_32, 2 * e);
  }
  __shared__ unsigned long long smax[32];
  __shared__ double ssum[32], ssq[32];
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
    mb = ob > mb ? ob : mb;
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) { smax[wid] = mb; ssum[wid] = s; ssq[wid] = s2; }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    mb = ln < nw ? smax[ln] : 0ull;
    s = ln < nw ? ssum[ln] : 0.0;
    s2 = ln < nw ? ssq[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
      s += __shfl_xor_sync(0xffffffffu, s, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (ln == 0) {
      hmax_bits[j] = mb;
      hsum[j] = s;
      hsq[j] = s2;
      if (mb > 0 && mb < INF_BITS && isfinite(s)) {
        const double rho = s / __longlong_as_double((long long)mb);
        atomicMax(&prm->rho_bits, (unsigned long long)__double_as_longlong(rho));
      }
    }
  }
}

// Residues of Ar = Re B^T, Ai = Im B^T and Ar + Ai (the last as the sum of the first two's
// residues): row i is column i of B (interleaved complex, ldb2 doubles apart); a thread writes
// two neighbouring k of all three planes of every modulus.  RA holds product p's planes at
// p * nmod * M * kp.
__global__ void k_residues_A_dft3(const double* __restrict__ Bre, long ldb2, int nn, int kp,
                                  const unsigned long long* __restrict__ amax_bits, const SplitDevParams* prm,
                                  CrtConsts cc, __nv_bfloat16* __restrict__ RA, int M) {
  const int i = blockIdx.x;  // rows in x: M = R k can pass the 65535 limit of y
  const int kk = 2 * (blockIdx.y * blockDim.x + threadIdx.x);
  if (kk >= kp) return;
  const unsigned long long ab = amax_bits[i];
  const bool ok = ab > 0 && ab < INF_BITS;
  const int e = ok ? scale_exp(ab, prm->PA) : 0;
  const double* col = Bre + (long)i * ldb2;
  double2 z0 = make_double2(0.0, 0.0), z1 = make_double2(0.0, 0.0);
  if (kk < nn) z0 = __ldg((const double2*)(col + 2 * kk));
  if (kk + 1 < nn) z1 = __ldg((const double2*)(col + 2 * kk + 2));
  bool n0 = false, n1 = false, n2 = false, n3 = false;
  const ResidueChunks r0 = residue_chunks(ok ? scaled_int(z0.x, e, &n0) : 0ull, n0);
  const ResidueChunks r1 = residue_chunks(ok ? scaled_int(z1.x, e, &n1) : 0ull, n1);
  const ResidueChunks i0 = residue_chunks(ok ? scaled_int(z0.y, e, &n2) : 0ull, n2);
  const ResidueChunks i1 = residue_chunks(ok ? scaled_int(z1.y, e, &n3) : 0ull, n3);
  const size_t plane = (size_t)M * kp, prod = (size_t)cc.nmod * plane;
  uint32_t* dst = (uint32_t*)(RA + (size_t)i * kp + kk);
#pragma unroll
  for (int l = 0; l < SPL_MAX_MODULI; ++l) {
    if (l < cc.nmod) {
      const float g23 = cc.g23[l], g38 = cc.g38[l], inv = cc.inv_m[l], mf = cc.mf[l];
      const float a0 = residue_f(r0, g23, g38, inv, mf), a1 = residue_f(r1, g23, g38, inv, mf);
      const float b0 = residue_f(i0, g23, g38, inv, mf), b1 = residue_f(i1, g23, g38, inv, mf);
      const float c0 = residue_sum(a0, b0, inv, mf), c1 = residue_sum(a1, b1, inv, mf);
      uint32_t* d = dst + (size_t)l * plane / 2;
      d[0] = __byte_perm(__float_as_uint(a0), __float_as_uint(a1), 0x7632);
      d[prod / 2] = __byte_perm(__float_as_uint(b0), __float_as_uint(b1), 0x7632);
      d[prod] = __byte_perm(__float_as_uint(c0), __float_as_uint(c1), 0x7632);
    }
  }
}

// Residues of Fr, Fi and Fr + Fi from Ht with column j's common exponent: four consecutive l
// per thread; RH holds product p's planes at p * nmod * nn * kp.
__global__ void k_residues_H_dft3(const double* __restrict__ Ht, int nn, int kp,
                                  const unsigned long long* __restrict__ hmax_bits, const SplitDevParams* prm,
                                  CrtConsts cc, __nv_bfloat16* __restrict__ RH) {
  const int j = blockIdx.x;  // columns in x (any count)
  const int kk = RH_PER_THREAD * (blockIdx.y * blockDim.x + threadIdx.x);
  if (kk >= kp) return;  // kp is a multiple of 64
  const unsigned long long hb = hmax_bits[j];
  const bool ok = hb > 0 && hb < INF_BITS;
  const int e = ok ? scale_exp(hb, prm->PH) : 0;
  const double* pr = Ht + (size_t)j * kp + kk;
  const double* pi = Ht + ((size_t)nn + j) * kp + kk;
  const double2 r01 = *(const double2*)pr, r23 = *(const double2*)(pr + 2);
  const double2 i01 = *(const double2*)pi, i23 = *(const double2*)(pi + 2);
  const double vr[4] = {r01.x, r01.y, r23.x, r23.y}, vi[4] = {i01.x, i01.y, i23.x, i23.y};
  ResidueChunks cr[4], ci[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    bool a = false, b = false;
    cr[q] = residue_chunks(ok ? scaled_int(vr[q], e, &a) : 0ull, a);
    ci[q] = residue_chunks(ok ? scaled_int(vi[q], e, &b) : 0ull, b);
  }
  const size_t plane = (size_t)nn * kp, prod = (size_t)cc.nmod * plane;
  uint2* dst = (uint2*)(RH + (size_t)j * kp + kk);
#pragma unroll
  for (int l = 0; l < SPL_MAX_MODULI; ++l) {
    if (l < cc.nmod) {
      const float g23 = cc.g23[l], g38 = cc.g38[l], inv = cc.inv_m[l], mf = cc.mf[l];
      unsigned fr[4], fi[4], fs[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float a = residue_f(cr[q], g23, g38, inv, mf), b = residue_f(ci[q], g23, g38, inv, mf);
        fr[q] = __float_as_uint(a);
        fi[q] = __float_as_uint(b);
        fs[q] = __float_as_uint(residue_sum(a, b, inv, mf));
      }
      uint2* d = dst + (size_t)l * plane / 4;
      d[0] = make_uint2(__byte_perm(fr[0], fr[1], 0x7632), __byte_perm(fr[2], fr[3], 0x7632));
      d[prod / 4] = make_uint2(__byte_perm(fi[0], fi[1], 0x7632), __byte_perm(fi[2], fi[3], 0x7632));
      d[prod / 2] = make_uint2(__byte_perm(fs[0], fs[1], 0x7632), __byte_perm(fs[2], fs[3], 0x7632));
    }
  }
}

// ------------------------------------------------------------------------------------------
// The modular GEMM: for modulus l and a 128 x 256 output tile, R_l = (RA_l * RH_l^T) mod m_l.
// Warp roles (320 threads): warps 0-7 drain the accumulator (quadrant = warp % 4, column
// half = warp / 4), warp 8 issues TMA loads, warp 9 issues tcgen05.mma.  Two 256-column FP32
// accumulators in tensor memory alternate between 1024-deep k chunks.
// ------------------------------------------------------------------------------------------
constexpr int G_BM = 128, G_BN = 256, G_BK = 64;
constexpr int G_STAGES = 4;
// 16 x 64 = 1024 k per FP32 chunk: residues |r| <= 128 (|r| <= 127 for the odd moduli), so every
// partial sum is an integer with |sum| <= 1024 * 128 * 128 = 2^24, exact in FP32.
constexpr int G_CHUNK_KB = 16;
// Chunk sums are added as int32 and reduced modulo m every 16 chunks: |sum| <= 2^28 + 128.
constexpr int G_RED_CHUNKS = 16;
constexpr int G_EPI_WARPS = 8;
constexpr int G_THREADS = (G_EPI_WARPS + 2) * 32;
constexpr uint32_t G_A_BYTES = G_BM * G_BK * 2;

struct GemmArgs {
  int n, kr, nkb, tiles_m, tiles_n, group_m, nmod;  // (a grouped launch uses group_m, nmod)
  int tm0;  // one product: first row tile of this launch (row panels)
  // Epilogue of the 3M complex product (T1 = Ar Fr, T2 = Ai Fi, T3 = (Ar + Ai)(Fr + Fi)):
  // 0 stores the residues; 1 reads T1 where it stores and writes T1 - x there and -T1 - x at
  // +im_off bytes; 2 adds x to the residues already stored.
  int mode, im_off;
  // Block products (MULTI): each residue goes to ndst places, place d at row dst_row[d] and
  // column dst_col[d] of planes of r_rows rows, stored (dst_op 0), added (2) or subtracted (3);
  // only the product's first ncols columns are written (ncols = 0: every column of the tile).
  int ndst, ncols, r_rows;
  int dst_col[8], dst_row[8], dst_op[8];
  // gate != nullptr: the launch runs only when (*gate != 0) == gate_set (the block-recursive
  // products and their single-product fallback, chosen on the device)
  const unsigned* gate;
  int gate_set;
  int8_t* R;
  unsigned* status;
  int m[SPL_MAX_MODULI];
  float inv_m[SPL_MAX_MODULI];
};

// Tile t of the launch -> (modulus, row tile, column tile).  Moduli are outermost; inside a
// modulus group_m row tiles sweep all column tiles together (L2 reuse of both operands).
__device__ __forceinline__ void raster_tile(int tiles_m, int tiles_n, int group_m, int t, int& l, int& tm, int& tn) {
  const int per_mod = tiles_m * tiles_n;
  l = t / per_mod;
  const int b = t - l * per_mod;
  const int per_group = group_m * tiles_n;
  const int grp = b / per_group;
  const int first_m = grp * group_m;
  const int gm = min(group_m, tiles_m - first_m);
  const int rr = b - grp * per_group;
  tm = first_m + rr % gm;
  tn = rr / gm;
}

// One output tile of a launch: operands, destination and position.
struct TileInfo {
  const CUtensorMap* ta;
  const CUtensorMap* tb;
  int8_t* R;
  int n, kr, nkb, l, tm, tn;
};

// Tile source of a single product (tensor maps in parameter space).
struct OneGemm {
  CUtensorMap ta, tb;
  GemmArgs g;
  static constexpr bool kGlobalMaps = false;
  static constexpr int kSub = 1;
  static constexpr int kEpiWarps = G_EPI_WARPS;
  __device__ int total() const { return g.tiles_m * g.tiles_n * g.nmod; }
  __device__ TileInfo tile(int t) const {
    TileInfo ti;
    raster_tile(g.tiles_m, g.tiles_n, g.group_m, t, ti.l, ti.tm, ti.tn);
    ti.tm += g.tm0;
    ti.ta = &ta;
    ti.tb = &tb;
    ti.R = g.R;
    ti.n = g.n;
    ti.kr = g.kr;
    ti.nkb = g.nkb;
    return ti;
  }
};

// One product of a grouped launch; tiles [t0, t0 + tiles_m * tiles_n * nmod).
struct GemmDesc {
  CUtensorMap ta, tb;
  int8_t* R;
  int n, kr, nkb, tiles_m, tiles_n, t0;
};

// Tile source of a grouped launch: the products' descriptors (and tensor maps) in global memory.
struct GroupGemm {
  GemmArgs g;  // nmod, group_m, status, moduli
  const GemmDesc* d;
  int count, total_tiles;
  static constexpr bool kGlobalMaps = true;
  static constexpr int kSub = 1;
  static constexpr int kEpiWarps = G_EPI_WARPS;
  __device__ int total() const { return total_tiles; }
  __device__ TileInfo tile(int t) const {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (d[mid].t0 <= t) lo = mid; else hi = mid - 1;
    }
    const GemmDesc& e = d[lo];
    TileInfo ti;
    raster_tile(e.tiles_m, e.tiles_n, g.group_m, t - e.t0, ti.l, ti.tm, ti.tn);
    ti.ta = &e.ta;
    ti.tb = &e.tb;
    ti.R = e.R;
    ti.n = e.n;
    ti.kr = e.kr;
    ti.nkb = e.nkb;
    return ti;
  }
};

// The three real products of a 3M complex product in one launch (T1 = Ar Fr, T2 = Ai Fi,
// T3 = (Ar + Ai)(Fr + Fi); operand maps ta[p], tb[p]), each of one chunk (k <= 1024): a tile's
// three products run back to back on the alternating accumulators and its epilogue writes
// Re = T1 - T2 and Im = T3 - T1 - T2 (Im at +im_off bytes) once, reading no residues back.
struct Gemm3M {
  CUtensorMap ta[3], tb[3];
  GemmArgs g;
  static constexpr bool kGlobalMaps = false;
  static constexpr int kSub = 3;
  // sixteen epilogue warps (64 columns each): the drain's residue arithmetic is the limit
  // here, and four warps per scheduler hide its latencies better than two
  static constexpr int kEpiWarps = 16;
  __device__ int total() const { return g.tiles_m * g.tiles_n * g.nmod; }
  __device__ TileInfo tile(int t) const {
    TileInfo ti;
    raster_tile(g.tiles_m, g.tiles_n, g.group_m, t, ti.l, ti.tm, ti.tn);
    ti.ta = &ta[0];
    ti.tb = &tb[0];
    ti.R = g.R;
    ti.n = g.n;
    ti.kr = g.kr;
    ti.nkb = g.nkb;
    return ti;
  }
};

// s mod m in [-128, 127] for |s| <= 2^28 + 128 and m <= 256: the float quotient estimate is
// within 0.3 of s / m, so q is off by at most one and one correction on each side suffices.
__device__ __forceinline__ int mod_sym(int s, int m, float inv_m) {
  const int q = __float2int_rn(__int2float_rn(s) * inv_m);
  int x = s - q * m;
  x = (x > 127) ? x - m : x;
  x = (x < -128) ? x + m : x;
  return x;
}

// s mod m in [-128, 127] for |s| <= 256 and 191 <= m <= 256 (every modulus of the split path):
// one conditional subtraction or addition of m (s - m >= -65 above 127, s + m <= 127 below -128).
__device__ __forceinline__ int mod_sym_small(int s, int m) {
  s -= s > 127 ? m : 0;
  s += s < -128 ? m : 0;
  return s;
}

// v mod m in [-128, 127] for an integer v held exactly in FP32 (|v| <= 2^24) and m <= 256, on the
// FP32 pipe, as the bits of x + 1.5 * 2^23 (the residue x is their low byte, as an int8).  Adding
// 1.5 * 2^23 rounds to an integer and leaves it in the low mantissa bits; q = round(v * fl(1/m))
// is within 0.5 + 1/m of v / m, so |v - q m| <= m/2 + 1 and one correction on each side
// suffices; v - q m is exact in the FMA.  The intrinsics keep the steps apart (no contraction).
constexpr float kRound23 = 12582912.0f;  // 1.5 * 2^23
__device__ __forceinline__ uint32_t mod_sym_f_bits(float v, float mf, float inv_m) {
  const float q = __fsub_rn(__fadd_rn(__fmul_rn(v, inv_m), kRound23), kRound23);
  float x = __fmaf_rn(-q, mf, v);
  x = x > 127.0f ? x - mf : x;
  x = x < -128.0f ? x + mf : x;
  return __float_as_uint(__fadd_rn(x, kRound23));
}

// (v + a) mod m likewise, for integers v (|v| <= 2^24) and a (|a| <= 256) held in FP32: the
// quotient comes from the rounded sum (within 1 of v + a), the remainder (v - q m) + a exactly,
// |x| <= 0.52 m.
__device__ __forceinline__ uint32_t mod_sym_f_bits_add(float v, float a, float mf, float inv_m) {
  const float t = __fadd_rn(v, a);
  const float q = __fsub_rn(__fadd_rn(__fmul_rn(t, inv_m), kRound23), kRound23);
  float x = __fadd_rn(__fmaf_rn(-q, mf, v), a);
  x = x > 127.0f ? x - mf : x;
  x = x < -128.0f ? x + mf : x;
  return __float_as_uint(__fadd_rn(x, kRound23));
}

// The low bytes of four words, packed (byte j from word j).
__device__ __forceinline__ uint32_t pack_low_bytes(uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
  return __byte_perm(__byte_perm(b0, b1, 0x0040), __byte_perm(b2, b3, 0x0040), 0x5410);
}

// Byte j of w, a residue offset by 128 (u = x + 128), back to x as a float: 0x4B4000uu is the
// float 1.5 * 2^23 + u.
__device__ __forceinline__ float offset_byte_f(uint32_t w, int j) {
  return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B400000u, 0x7650 + j)), kRound23 + 128.0f);
}

// Epilogue of the 3M complex product's second and third GEMMs: combine this tile's residues x
// (in [-128, 127]) with those already in the output plane, 16 bytes at a time.
// mode 1: old = T1 -> store (T1 - x) mod m, and (-T1 - x) mod m at dst + im_off;
// mode 2: old = -T1 - T2 -> store (old + x) mod m.
// Only the first `valid` columns (a multiple of 16) are touched.
template <int HALF>
__device__ __forceinline__ void store_combined(int8_t* dst, const int (&res)[HALF], int mode, int im_off, int m,
                                               int valid = HALF) {
  // every 16-byte load issued before the first store (the stores at dst + im_off may alias the
  // later loads for all the compiler knows, which would serialise the round trips)
  uint4 ov[HALF / 16];
#pragma unroll
  for (int v = 0; v < HALF / 16; ++v) ov[v] = v * 16 < valid ? *(const uint4*)(dst + v * 16) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
  for (int v = 0; v < HALF / 16; ++v) {
    if (v * 16 >= valid) break;
    const uint32_t ow[4] = {ov[v].x, ov[v].y, ov[v].z, ov[v].w};
    uint32_t w1[4], w2[4];
#pragma unroll
    for (int t4 = 0; t4 < 4; ++t4) {
      w1[t4] = 0u;
      w2[t4] = 0u;
#pragma unroll
      for (int bb = 0; bb < 4; ++bb) {
        const int old = (int)(int8_t)(ow[t4] >> (8 * bb));
        const int x = res[v * 16 + t4 * 4 + bb];
        const int a = mod_sym_small(mode == 1 ? old - x : old + x, m);
        w1[t4] |= (uint32_t)(uint8_t)(int8_t)a << (8 * bb);
        if (mode == 1) w2[t4] |= (uint32_t)(uint8_t)(int8_t)mod_sym_small(-old - x, m) << (8 * bb);
      }
    }
    *(uint4*)(dst + v * 16) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
    if (mode == 1) *(uint4*)(dst + im_off + v * 16) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
  }
}

template <int BN>
struct GemmShape {
  static constexpr uint32_t B_BYTES = BN * G_BK * 2;
  static constexpr size_t SMEM = 1024 + (size_t)G_STAGES * (G_A_BYTES + B_BYTES) + 256;
  static constexpr uint32_t TMEM_COLS = 2 * BN;  // two accumulators (a power of two >= 32)
};

__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(m) : "memory");
}

// Persistent: one CTA per SM walks tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...  The
// stage ring and the two TMEM accumulators continue across tiles (and, in a grouped launch,
// across products), so the loads and MMAs of the next tile overlap the drain and residue
// store of the previous one.  BN: output tile width (256, or 64 for narrow products).
// MULTI: the block-recursive products' epilogue (GemmArgs::ndst, dst_col, ncols); without it
// every residue goes to one place and the epilogue keeps fewer registers live.
template <int BN, class TS, bool MULTI = false>
__global__ void __launch_bounds__((TS::kEpiWarps + 2) * 32, 1) k_crt_gemm(const __grid_constant__ TS ts) {
  constexpr int EPI = TS::kEpiWarps;  // warps 0 .. EPI-1 drain, EPI issues TMA, EPI + 1 the MMAs
  using S = GemmShape<BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base;
  uint8_t* sB = base + G_STAGES * G_A_BYTES;
  uint64_t* bars = (uint64_t*)(sB + G_STAGES * S::B_BYTES);
  uint64_t* full = bars;
  uint64_t* empty = bars + G_STAGES;
  uint64_t* acc_full = bars + 2 * G_STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  const GemmArgs& g = ts.g;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < G_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], EPI * 32);
    }
    mbar_init(mma_done, 1);
    // a launch whose pipeline already timed out does no further work, nor one gated off
    const bool gated_off = g.gate != nullptr && ((*(const volatile unsigned*)g.gate != 0u) != (g.gate_set != 0));
    *abort_flag = (status_aborted(g.status) || gated_off) ? 1 : 0;
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, S::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const int total = *abort_flag ? 0 : ts.total();

  if (warp == EPI) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0, issued = 0;
      bool ok = true;
      const CUtensorMap* last = nullptr;
      for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
        const TileInfo ti = ts.tile(t);
        if (ti.ta != last) {
          if (TS::kGlobalMaps) {
            tensormap_acquire(ti.ta);
            tensormap_acquire(ti.tb);
          }
#pragma unroll
          for (int sub = 0; sub < TS::kSub; ++sub) {
            prefetch_tmap(ti.ta + sub);
            prefetch_tmap(ti.tb + sub);
          }
          last = ti.ta;
        }
        for (int sub = 0; sub < TS::kSub && ok; ++sub) {
          for (int kb = 0; kb < ti.nkb; ++kb, ++it) {
            const int s = it % G_STAGES;
            if (!mbar_wait(&empty[s], ((it / G_STAGES) & 1) ^ 1, g.status, abort_flag)) { ok = false; break; }
            mbar_arrive_expect_tx(&full[s], G_A_BYTES + S::B_BYTES);
            tma_load_3d(sA + s * G_A_BYTES, ti.ta + sub, &full[s], kb * G_BK, ti.tm * G_BM, ti.l);
            tma_load_3d(sB + s * S::B_BYTES, ti.tb + sub, &full[s], kb * G_BK, ti.tn * BN, ti.l);
            issued = it + 1;
          }
        }
      }
      // every issued copy must have landed before the CTA may exit
      for (int q = max(0, issued - G_STAGES); q < issued; ++q)
        mbar_wait_drain(&full[q % G_STAGES], (q / G_STAGES) & 1, g.status);
    }
    __syncwarp();
  } else if (warp == EPI + 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(G_BM, BN);
      int it = 0, c = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
        const int nkb = ts.tile(t).nkb;
        const int cpt = (nkb + G_CHUNK_KB - 1) / G_CHUNK_KB;  // chunks of each product of this tile
        for (int cc = 0; cc < TS::kSub * cpt && ok; ++cc, ++c) {
          const int buf = c & 1;
          const uint32_t use = (uint32_t)(c >> 1);
          if (!mbar_wait(&acc_empty[buf], (use & 1) ^ 1, g.status, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t dt = tmem_base + (uint32_t)(buf * BN);
          const int kb0 = (cc % cpt) * G_CHUNK_KB;
          const int kend = min(nkb, kb0 + G_CHUNK_KB);
          uint32_t acc = 0;
          for (int kb = kb0; kb < kend; ++kb, ++it) {
            const int s = it % G_STAGES;
            if (!mbar_wait(&full[s], (it / G_STAGES) & 1, g.status, abort_flag)) { ok = false; break; }
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + s * G_A_BYTES), b0 = smem_u32(sB + s * S::B_BYTES);
#pragma unroll
            for (int kk = 0; kk < G_BK / 16; ++kk) {
              tc_mma_bf16(dt, sdesc_sw128_kmajor(a0 + kk * 32), sdesc_sw128_kmajor(b0 + kk * 32), idesc, acc);
              acc = 1;
            }
            tc_commit(&empty[s]);
          }
          if (ok) tc_commit(&acc_full[buf]);
        }
      }
      // all tcgen05 work of this thread must complete before TMEM is released
      tc_commit(mma_done);
      mbar_wait_drain(mma_done, 0, g.status);
    }
    __syncwarp();
  } else {
    // ---------------- accumulator drain (epilogue) ----------------
    // warp w drains TMEM lanes 32 (w mod 4) .. +31 (its quadrant's rows) and the columns
    // [h HALF, (h + 1) HALF) of the tile, h = w / 4
    constexpr int HALF = BN / (EPI / 4);  // columns per epilogue warp
    const int q = warp & 3, h = warp >> 2;
    int c = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
      const TileInfo ti = ts.tile(t);
      const int cpt = (ti.nkb + G_CHUNK_KB - 1) / G_CHUNK_KB;
      const int mi = g.m[ti.l];
      const float inv_m = g.inv_m[ti.l];
      if constexpr (TS::kSub == 3) {
        // T1 -> x1 (kept); T2 -> Re = x1 - T2 (stored) and s = -x1 - T2 (kept); T3 -> Im = s + T3
        // (stored).  Residues on the FP32 pipe from the exact sums; kept residues are bytes
        // offset by 128, four to a word.  The epilogue work is spread over the three drains,
        // each within the next product's MMA time.
        const int i = ti.tm * G_BM + q * 32 + lane;
        const int col0 = ti.tn * BN + h * HALF;
        const float mf = (float)mi;
        int8_t* dst = ti.R + ((size_t)ti.l * ti.n + (size_t)min(i, ti.n - 1)) * ti.kr + (size_t)col0;
        uint32_t p1[HALF / 4], ps[HALF / 4];
#pragma unroll
        for (int sub = 0; sub < 3; ++sub) {
          const int buf = c & 1;
          const uint32_t use = (uint32_t)(c >> 1);
          if (!mbar_wait(&acc_full[buf], use & 1, g.status, abort_flag)) { ok = false; break; }
          ++c;
          tc_fence_after();
          const bool store = sub > 0 && !*abort_flag && i < ti.n;
#pragma unroll
          for (int cb = 0; cb < HALF / 32; ++cb) {
            uint32_t r[32];
            tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN + h * HALF + cb * 32), r);
            tmem_ld_wait();
            uint32_t wa[8], wb[8];
#pragma unroll
            for (int e4 = 0; e4 < 8; ++e4) {
              uint32_t ba[4], bb4[4];
#pragma unroll
              for (int bb = 0; bb < 4; ++bb) {
                const float v = __uint_as_float(r[4 * e4 + bb]);
                if (sub == 0) {
                  ba[bb] = mod_sym_f_bits(v, mf, inv_m);
                } else if (sub == 1) {
                  const float x1 = offset_byte_f(p1[cb * 8 + e4], bb);
                  ba[bb] = mod_sym_f_bits_add(-v, x1, mf, inv_m);   // x1 - T2
                  bb4[bb] = mod_sym_f_bits_add(-v, -x1, mf, inv_m);  // -x1 - T2
                } else {
                  ba[bb] = mod_sym_f_bits_add(v, offset_byte_f(ps[cb * 8 + e4], bb), mf, inv_m);  // s + T3
                }
              }
              wa[e4] = pack_low_bytes(ba[0], ba[1], ba[2], ba[3]);
              if (sub == 0) p1[cb * 8 + e4] = wa[e4] ^ 0x80808080u;
              if (sub == 1) {
                wb[e4] = pack_low_bytes(bb4[0], bb4[1], bb4[2], bb4[3]);
                ps[cb * 8 + e4] = wb[e4] ^ 0x80808080u;
              }
            }
            if (store) {
              int8_t* o = dst + (sub == 2 ? g.im_off : 0) + cb * 32;
              *(uint4*)o = make_uint4(wa[0], wa[1], wa[2], wa[3]);
              *(uint4*)(o + 16) = make_uint4(wa[4], wa[5], wa[6], wa[7]);
            }
          }
          tc_fence_before();
          mbar_arrive(&acc_empty[buf]);
        }
      } else {
        // int32 running sums of the chunks' exact FP32 sums (|chunk| <= 2^24), reduced to
        // [-128, 127] every G_RED_CHUNKS chunks and at the end of the tile
        int res[HALF];
#pragma unroll
        for (int e = 0; e < HALF; ++e) res[e] = 0;
        for (int cc = 0; cc < cpt; ++cc, ++c) {
          const int buf = c & 1;
          const uint32_t use = (uint32_t)(c >> 1);
          if (!mbar_wait(&acc_full[buf], use & 1, g.status, abort_flag)) { ok = false; break; }
          tc_fence_after();
#pragma unroll
          for (int cb = 0; cb < HALF / 32; ++cb) {
            uint32_t r[32];
            tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN + h * HALF + cb * 32), r);
            tmem_ld_wait();
#pragma unroll
            for (int e = 0; e < 32; ++e) res[cb * 32 + e] += __float2int_rn(__uint_as_float(r[e]));
          }
          tc_fence_before();
          mbar_arrive(&acc_empty[buf]);
          if ((cc % G_RED_CHUNKS) == G_RED_CHUNKS - 1 || cc == cpt - 1) {
#pragma unroll
            for (int e = 0; e < HALF; ++e) res[e] = mod_sym(res[e], mi, inv_m);
          }
        }
        const int i = ti.tm * G_BM + q * 32 + lane;
        if (MULTI) {
          // per place every 16-byte load issued before the first add: one round trip per place
          const int col0 = ti.tn * BN + h * HALF;
          const int valid = g.ncols > 0 ? g.ncols - col0 : HALF;  // columns of this half in the product
          if (ok && !*abort_flag && i < ti.n && valid > 0) {
            // the residues packed to bytes (32 registers instead of 128); the volatile move keeps
            // the compiler from re-deriving them from the int32 sums inside the place loop,
            // which would keep all 128 sums live there and spill
            uint32_t pk[HALF / 4];
#pragma unroll
            for (int e4 = 0; e4 < HALF / 4; ++e4) {
              const uint32_t pv = (uint32_t)(uint8_t)(int8_t)res[4 * e4] |
                                  ((uint32_t)(uint8_t)(int8_t)res[4 * e4 + 1] << 8) |
                                  ((uint32_t)(uint8_t)(int8_t)res[4 * e4 + 2] << 16) |
                                  ((uint32_t)(uint8_t)(int8_t)res[4 * e4 + 3] << 24);
              asm volatile("mov.b32 %0, %1;" : "=r"(pk[e4]) : "r"(pv));
            }
            const int nd = g.ndst > 0 ? g.ndst : 1;
            const size_t plane_rows = g.r_rows > 0 ? (size_t)g.r_rows : (size_t)ti.n;
            for (int d = 0; d < nd; ++d) {
              int8_t* dst = ti.R + ((size_t)ti.l * plane_rows + i + (g.ndst > 0 ? g.dst_row[d] : 0)) * ti.kr +
                            (size_t)col0 + (g.ndst > 0 ? g.dst_col[d] : 0);
              const int op = g.ndst > 0 ? g.dst_op[d] : g.mode;
              if (op >= 2) {
                uint4 o[HALF / 16];
#pragma unroll
                for (int v = 0; v < HALF / 16; ++v)
                  o[v] = v * 16 < valid ? *(const uint4*)(dst + v * 16) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (int v = 0; v < HALF / 16; ++v) {
                  if (v * 16 >= valid) break;
                  const uint32_t ow[4] = {o[v].x, o[v].y, o[v].z, o[v].w};
                  uint32_t nw[4];
#pragma unroll
                  for (int t4 = 0; t4 < 4; ++t4) {
                    nw[t4] = 0u;
#pragma unroll
                    for (int bb = 0; bb < 4; ++bb) {
                      const int x = (int)(int8_t)(pk[4 * v + t4] >> (8 * bb));
                      const int a = (int)(int8_t)(ow[t4] >> (8 * bb)) + (op == 3 ? -x : x);
                      nw[t4] |= (uint32_t)(uint8_t)(int8_t)mod_sym_small(a, mi) << (8 * bb);
                    }
                  }
                  *(uint4*)(dst + v * 16) = make_uint4(nw[0], nw[1], nw[2], nw[3]);
                }
              } else {
#pragma unroll
                for (int v = 0; v < HALF / 16; ++v)
                  if (v * 16 < valid)
                    *(uint4*)(dst + v * 16) = make_uint4(pk[4 * v], pk[4 * v + 1], pk[4 * v + 2], pk[4 * v + 3]);
              }
            }
          }
          continue;
        }
        const int col0 = ti.tn * BN + h * HALF;
        const int valid = HALF;
        const int nd = 1;
        for (int d = 0; d < nd && ok && !*abort_flag && i < ti.n && valid > 0; ++d) {
          int8_t* dst = ti.R + ((size_t)ti.l * ti.n + i) * ti.kr + (size_t)col0;
          if (g.mode != 0) {
            store_combined<HALF>(dst, res, g.mode, g.im_off, mi, valid);
            continue;
          }
#pragma unroll
          for (int v = 0; v < HALF / 16; ++v) {
            if (v * 16 >= valid) break;
            uint32_t w[4];
#pragma unroll
            for (int t4 = 0; t4 < 4; ++t4) {
              uint32_t b0 = (uint32_t)(uint8_t)(int8_t)res[v * 16 + t4 * 4 + 0];
              uint32_t b1 = (uint32_t)(uint8_t)(int8_t)res[v * 16 + t4 * 4 + 1];
              uint32_t b2 = (uint32_t)(uint8_t)(int8_t)res[v * 16 + t4 * 4 + 2];
              uint32_t b3 = (uint32_t)(uint8_t)(int8_t)res[v * 16 + t4 * 4 + 3];
              w[t4] = b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
            }
            *(uint4*)(dst + v * 16) = make_uint4(w[0], w[1], w[2], w[3]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem_base, S::TMEM_COLS);
}

// ------------------------------------------------------------------------------------------
// CRT recombination + FP64 epilogue: Q(i,j) = alpha * Z_ij * 2^-(s_i+f_j) + beta * Q(i,j).
// 32 x 32 output tile per block (32 x 8 threads), transposed through shared memory so that
// both the residue reads (row-major) and the Q writes (column-major) are coalesced.
// ------------------------------------------------------------------------------------------
typedef unsigned __int128 u128;

// m * 2^x with the sign, for results outside the normal range; out of line, so that its FP64
// instructions are not issued (predicated off) for every element.
static __device__ __noinline__ double scaled_outside_normal(unsigned long long m, int x, bool neg) {
  const double v = ldexp((double)m, x);
  return neg ? -v : v;
}

// (hi:lo) * 2^-e as a double, (hi:lo) a non-negative 128-bit integer in two words, rounded
// to nearest even from the bits; results outside the normal range go through ldexp.
__device__ __forceinline__ double u128w_scaled(unsigned long long hi, unsigned long long lo, bool neg, int e) {
  if ((hi | lo) == 0) return 0.0;
  // normalise so that the leading bit is bit 63 of `top`; `rest` keeps the bits below
  int p;
  unsigned long long top, rest;
  if (hi) {
    const int s = __clzll((long long)hi);
    p = 127 - s;
    top = s ? (hi << s) | (lo >> (64 - s)) : hi;
    rest = s ? (lo << s) : lo;
  } else {
    const int s = __clzll((long long)lo);
    p = 63 - s;
    top = lo << s;
    rest = 0;
  }
  unsigned long long m = top >> 11;  // 53 bits
  const unsigned long long low11 = top & 0x7FFull;
  const bool sticky = (low11 & 0x3FFull) != 0 || rest != 0;
  if ((low11 & 0x400ull) && (sticky || (m & 1))) {
    ++m;
    if (m == (1ull << 53)) {
      m >>= 1;
      ++p;
    }
  }
  const int field = p - e + 1023;
  if (field >= 1 && field <= 2046) {
    unsigned long long bits = ((unsigned long long)field << 52) | (m & 0xFFFFFFFFFFFFFull);
    if (neg) bits |= 1ull << 63;
    return __longlong_as_double((long long)bits);
  }
  return scaled_outside_normal(m, p - 52 - e, neg);
}

// One block: 32 rows x 128 columns (32 x 8 threads); a thread recombines 4 neighbouring
// columns of one row per pass from 32-bit loads (4 residues) of each plane, so each warp
// request moves 128 bytes.  Per modulus and element: four 32x32->64-bit multiply-adds for
// the limbs of sum_l (r_l + 128) C_l and one for the fixed-point quotient estimate.
constexpr int CRT_TI = 32, CRT_TJ = 128;

// The column of C^T that residue column rc of the 3M DFT layout holds (Re: rc < nn, Im: from
// kr/2), or -1 for the padding between and after.
__device__ __forceinline__ int dft_col(int rc, int nn, int kr) {
  if (rc < nn) return rc;
  const int im = rc - (kr >> 1);
  return (im >= 0 && im < nn) ? im : -1;
}

// The CRT of four neighbouring columns of one row: the residue words of the moduli at rp (a
// 4-byte aligned address in the first plane; planes plane_w words apart), ab the row's maximum
// (its exponent with PA), hb / fexp the columns' maxima and exponents; val = Z 2^-(s + f), NaN
// for a non-finite row or column, 0 for a zero one.
template <bool TOP32>
__device__ __forceinline__ void crt_row4(const int8_t* __restrict__ rp, size_t plane_w, const CrtConsts& cc,
                                         unsigned long long ab, int PA, const unsigned long long (&hb)[4],
                                         const int (&fexp)[4], double (&val)[4]) {
  const int sexp = (ab != 0 && ab < INF_BITS) ? scale_exp(ab, PA) : 0;
  unsigned long long acc[4][4];
  unsigned acc3[4];
  int qi[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    qi[c] = 0;
    acc3[c] = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) acc[c][t] = 0;
  }
  const uint32_t* src = (const uint32_t*)rp;
  // all residue words first (the loads are then in flight together), then the sums
  uint32_t wl[SPL_MAX_MODULI];
#pragma unroll
  for (int l = 0; l < SPL_MAX_MODULI; ++l) wl[l] = (l < cc.nmod) ? __ldg(src + (size_t)l * plane_w) : 0u;
#pragma unroll
  for (int l = 0; l < SPL_MAX_MODULI; ++l) {
    if (l >= cc.nmod) break;
    const uint32_t w4 = wl[l];
    const int ff = cc.ffix[l];
    const unsigned c0 = cc.climb[l][0], c1 = cc.climb[l][1], c2 = cc.climb[l][2], c3 = cc.climb[l][3];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int r = (int)(int8_t)(w4 >> (8 * c));
      qi[c] += r * ff;
      const unsigned ur = (unsigned)(r + 128);
      acc[c][0] += (unsigned long long)ur * c0;
      acc[c][1] += (unsigned long long)ur * c1;
      acc[c][2] += (unsigned long long)ur * c2;
      if (TOP32)
        acc3[c] += ur * c3;
      else
        acc[c][3] += (unsigned long long)ur * c3;
    }
  }
  if (TOP32) {
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c][3] = acc3[c];
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    if (ab >= INF_BITS || hb[c] >= INF_BITS) {
      val[c] = __longlong_as_double(0x7FF8000000000000ll);  // NaN: non-finite input row/column
    } else if (ab != 0 && hb[c] != 0) {
      // Z = sum_l r_l C_l - q*M in signed 64-bit limbs (|limb terms| < 2^46), then carries
      const long long q = (long long)((qi[c] + (1 << 18)) >> 19);
      long long z0 = (long long)acc[c][0] - (long long)cc.biasl[0] - q * (long long)cc.Mlimb[0];
      long long z1 = (long long)acc[c][1] - (long long)cc.biasl[1] - q * (long long)cc.Mlimb[1];
      long long z2 = (long long)acc[c][2] - (long long)cc.biasl[2] - q * (long long)cc.Mlimb[2];
      long long z3 = (long long)acc[c][3] - (long long)cc.biasl[3] - q * (long long)cc.Mlimb[3];
      z1 += z0 >> 32;
      z2 += z1 >> 32;
      z3 += z2 >> 32;  // exact: z3 holds the sign and top bits of Z (|Z| < 2^126)
      const unsigned long long L0 = (unsigned long long)z0 & 0xFFFFFFFFull;
      const unsigned long long L1 = (unsigned long long)z1 & 0xFFFFFFFFull;
      const unsigned long long L2 = (unsigned long long)z2 & 0xFFFFFFFFull;
      unsigned long long hi = ((unsigned long long)z3 << 32) | L2, lo = (L1 << 32) | L0;
      const bool neg = z3 < 0;
      if (neg) {  // two's-complement negate of the 128-bit value
        lo = ~lo + 1;
        hi = ~hi + (lo == 0 ? 1 : 0);
      }
      val[c] = u128w_scaled(hi, lo, neg, sexp + fexp[c]);
    }
  }
}

// DFT_OUT: the product is C^T (rows = columns of C, k = n its column count) with Re in R
// columns [0, n) and Im in [kr/2, kr/2 + n) (the 3M layout); Re / Im of element (i, j) go to
// the interleaved complex C at 2j / 2j + 1 + i*ldq (ldq in doubles); column j's exponent is
// that of hmax_bits[j].
// TOP32 (cc.top32): the sum over the moduli of (r_l + 128) times the top 32-bit limb of C_l
// stays below 2^32 (true for M < 2^112: every top limb is below 2^16), so it is kept in 32 bits.
template <bool DFT_OUT, bool TOP32 = false>
__device__ __forceinline__ void crt_combine_blk(const int8_t* __restrict__ R, int n, int k, int kr,
                                                const CrtConsts& cc, const unsigned long long* __restrict__ amax_bits,
                                                const unsigned long long* __restrict__ hmax_bits,
                                                const SplitDevParams* prm, double alpha, double beta,
                                                double* __restrict__ Q, long ldq, int bx, int by,
                                                const unsigned long long* __restrict__ gmax_bits = nullptr,
                                                int gw = 1) {
  // element (jl, il) of the tile at column (il + jl/4) mod 32 of row jl: the row-wise writes
  // (4 columns per thread) and the column-wise reads both hit distinct bank pairs
  __shared__ double tile[CRT_TJ][CRT_TI];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = by * CRT_TI, j0 = bx * CRT_TJ;
  const int PA = prm->PA, PH = prm->PH;
  const int jb = j0 + 4 * tx;
  const int kcols = DFT_OUT ? kr : k;  // residue columns covered
  unsigned long long hb[4];
  int fexp[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int hc = DFT_OUT ? dft_col(jb + c, k, kr) : (jb + c < k ? jb + c : -1);
    hb[c] = hc >= 0 ? hmax_bits[hc] : 0ull;
    // block-recursive products: finite columns scaled with their group's exponent
    if (gmax_bits != nullptr && hc >= 0 && hb[c] < INF_BITS && !prm->hbad) hb[c] = gmax_bits[hc % gw];
    fexp[c] = (hb[c] != 0 && hb[c] < INF_BITS) ? scale_exp(hb[c], PH) : 0;
  }
  const size_t plane_w = (size_t)n * kr / 4;
  for (int a = 0; a < CRT_TI / 8; ++a) {
    const int il = ty + 8 * a, i = i0 + il;
    double val[4] = {0.0, 0.0, 0.0, 0.0};
    if (i < n && jb < kcols) crt_row4<TOP32>(R + (size_t)i * kr + jb, plane_w, cc, amax_bits[i], PA, hb, fexp, val);
#pragma unroll
    for (int c = 0; c < 4; ++c) tile[4 * tx + c][(il + tx) & 31] = val[c];
  }
  __syncthreads();
  const bool scale = alpha != 1.0, accumulate = beta != 0.0;  // uniform: decided once
  if (!DFT_OUT && !scale && !accumulate) {
    // Q = Z 2^-(s+f): a loop of its own, without the FP64 epilogue (instructions predicated off
    // would still be issued to GB300's narrow FP64 pipe)
    const int i = i0 + tx;
    for (int b = 0; b < CRT_TJ / 8; ++b) {
      const int jl = ty + 8 * b, jj = j0 + jl;
      if (i < n && jj < k) Q[i + (long)jj * ldq] = tile[jl][(tx + (jl >> 2)) & 31];
    }
  } else if (!DFT_OUT) {
    const int i = i0 + tx;
    for (int b = 0; b < CRT_TJ / 8; ++b) {
      const int jl = ty + 8 * b, jj = j0 + jl;
      if (i < n && jj < k) {
        double* qp = Q + i + (long)jj * ldq;
        double v = tile[jl][(tx + (jl >> 2)) & 31];
        if (scale) v *= alpha;
        if (accumulate) v = fma(beta, *qp, v);
        *qp = v;
      }
    }
  } else {
    for (int a = 0; a < CRT_TI / 8; ++a) {
      const int il = ty + 8 * a, i = i0 + il;
      if (i >= n) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int jj = jb + c, hc = dft_col(jj, k, kr);
        if (hc < 0) continue;
        double* qp = Q + (long)i * ldq + 2 * hc + (jj >= (kr >> 1) ? 1 : 0);
        double v = tile[4 * tx + c][(il + tx) & 31];
        if (scale) v *= alpha;
        if (accumulate) v = fma(beta, *qp, v);
        *qp = v;
      }
    }
  }
}

template <bool DFT_OUT, bool TOP32>
__global__ void __launch_bounds__(256, 3) k_crt_combine(const int8_t* __restrict__ R, int n, int k, int kr,
                                                     CrtConsts cc, const unsigned long long* __restrict__ amax_bits,
                                                     const unsigned long long* __restrict__ hmax_bits,
                                                     const SplitDevParams* prm, double alpha, double beta,
                                                     double* __restrict__ Q, long ldq, int by0) {
  crt_combine_blk<DFT_OUT, TOP32>(R, n, k, kr, cc, amax_bits, hmax_bits, prm, alpha, beta, Q, ldq, blockIdx.x,
                                  by0 + blockIdx.y);
}

// The recombination of the block-recursive products (group exponents unless prm->hbad).
template <bool TOP32>
__global__ void __launch_bounds__(256, 3) k_crt_combine_blocks(const int8_t* __restrict__ R, int n, int k, int kr,
                                                            CrtConsts cc,
                                                            const unsigned long long* __restrict__ amax_bits,
                                                            const unsigned long long* __restrict__ hmax_bits,
                                                            const unsigned long long* __restrict__ gmax_bits, int gw,
                                                            const SplitDevParams* prm, double alpha, double beta,
                                                            double* __restrict__ Q, long ldq, int by0) {
  crt_combine_blk<false, TOP32>(R, n, k, kr, cc, amax_bits, hmax_bits, prm, alpha, beta, Q, ldq, blockIdx.x,
                                by0 + blockIdx.y, gmax_bits, gw);
}

// ------------------------------------------------------------------------------------------
// Host orchestration
// ------------------------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

static bool make_tmap(CUtensorMap* map, void* ptr, int kp, int rows, int nmod, int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)nmod};
  cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)rows * kp * 2};
  cuuint32_t box[3] = {(cuuint32_t)G_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, ptr, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

static CrtConsts get_consts(int nmod) {
  static std::mutex cmu;
  static CrtConsts consts[SPL_MAX_MODULI + 1];
  static bool have[SPL_MAX_MODULI + 1] = {false};
  std::lock_guard<std::mutex> lk(cmu);
  if (!have[nmod]) {
    consts[nmod] = make_consts(nmod);
    have[nmod] = true;
  }
  return consts[nmod];
}

struct SplitBuffers {
  SplitDevParams* prm;
  SplitDevParams* prm_guess;  // PA/PH of a speculative host pipeline (only those two fields are read)
  unsigned long long *amax, *hmax;
  double *hsum, *asq, *hsq, *Ht;
  double2* wtab;
  __nv_bfloat16 *RA, *RH;
  int8_t* R;
};

static SplitBuffers split_buffers(char* w, const SplitLayout& L) {
  SplitBuffers b;
  b.prm = (SplitDevParams*)(w + L.off_params);
  b.prm_guess = b.prm + 1;
  b.amax = (unsigned long long*)(w + L.off_amax);
  b.hmax = (unsigned long long*)(w + L.off_hmax);
  b.hsum = (double*)(w + L.off_hsum);
  b.asq = (double*)(w + L.off_asq);
  b.hsq = (double*)(w + L.off_hsq);
  b.wtab = (double2*)(w + L.off_wtab);
  b.Ht = (double*)(w + L.off_ht);
  b.RA = (__nv_bfloat16*)(w + L.off_ra);
  b.RH = (__nv_bfloat16*)(w + L.off_rh);
  b.R = (int8_t*)(w + L.off_r);
  return b;
}

int launch_split_any(int kind, int n, int k, double alpha, const double* A, long lda, const double* gen,
                     long ldgen, double beta, double* Q, long ldq, int n_moduli, void* work, size_t lwork,
                     cudaStream_t stream, unsigned* status_dev_out, int block_levels);

int launch_split(int kind, int n, int k, double alpha, const double* A, long lda, const double* gen, long ldgen,
                 double beta, double* Q, long ldq, int n_moduli, void* work, size_t lwork, cudaStream_t stream,
                 bool wait_status, int block_levels) {
  return launch_split_any(kind, n, k, alpha, A, lda, gen, ldgen, beta, Q, ldq, n_moduli, work, lwork, stream,
                          wait_status ? kStatusWait : nullptr, block_levels);
}

// The device status of a call ORed into the stream's status word.
__global__ void k_status_or(unsigned* acc, const unsigned* st) {
  const unsigned v = *st;
  if (v) atomicOr(acc, v);
}

// The device status of a split call: status_dev_out == nullptr ORs it into the stream's status
// word (no synchronisation), kStatusWait waits and returns it, any other pointer receives a copy
// of it (no synchronisation).
// ---- the DFT with a radix-R first step -------------------------------------------------------
// With l = R m + r and j = j' + (n/R) s (r, s < R; m, j' < n/R),
//   C(j' + (n/R) s, c) = sum_r w_R^(s r) w_n^(j' r) P_r(j', c),   P_r = F_(n/R) B(r::R, :),
// so the dense product becomes F_(n/R) times the R k columns B' = [B(0::R, :) | ... | B(R-1::R, :)]:
// n^2 k / R complex multiply-adds instead of n^2 k.  The twiddles w_n^(j' r) come from the exact
// table (j' r < n, no reduction), then R-point butterflies (w_2 = -1, w_4 = -i: additions only).

// B' (n/R x R k complex, ld n/R): B'(m, r k + c) = B(R m + r, c).  One thread per element of B
// (coalesced reads along a column; each warp writes R runs of 32 / R consecutive elements).
__global__ void k_dft_deinterleave(const double2* __restrict__ B, long ldb, int n, int k, int R,
                                   double2* __restrict__ Bp) {
  const int nq = n / R;
  for (int c = blockIdx.y; c < k; c += gridDim.y) {
    const double2* col = B + (long)c * ldb;
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += gridDim.x * blockDim.x) {
      const int r = l % R, m = l / R;
      Bp[((size_t)r * k + c) * nq + m] = __ldg(col + l);
    }
  }
}

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// The 4-point DFT with w_4 = -i: y0 = t0 + t2, y2 = t0 - t2, y1 = t1 - i t3, y3 = t1 + i t3 for
// t0 = x0 + x2, t1 = x0 - x2, t2 = x1 + x3, t3 = x1 - x3.
__device__ __forceinline__ void dft4(double2 x0, double2 x1, double2 x2, double2 x3, double2& y0, double2& y1,
                                     double2& y2, double2& y3) {
  const double2 t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = csub(x1, x3);
  y0 = cadd(t0, t2);
  y2 = csub(t0, t2);
  y1 = make_double2(t1.x + t3.y, t1.y - t3.x);
  y3 = make_double2(t1.x - t3.y, t1.y + t3.x);
}

// Y = DFT_R X (R = 2, 4, 8): the R-point butterflies.
template <int R>
__device__ __forceinline__ void radix_butterfly(const double2 (&X)[R], double2 (&Y)[R]) {
  if (R == 2) {
    Y[0] = cadd(X[0], X[1]);
    Y[1] = csub(X[0], X[1]);
  } else if (R == 4) {
    dft4(X[0], X[1 % R], X[2 % R], X[3 % R], Y[0], Y[1 % R], Y[2 % R], Y[3 % R]);
  } else {
    // w_8 = (1 - i)/sqrt(2): a_r = X_r + X_(r+4) and b_r = w_8^r (X_r - X_(r+4)) give the
    // even outputs Y_2t = DFT4(a)_t and the odd ones Y_(2t+1) = DFT4(b)_t
    double2 a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      a[r] = cadd(X[r % R], X[(r + 4) % R]);
      b[r] = csub(X[r % R], X[(r + 4) % R]);
    }
    const double h = 0.70710678118654752440;  // 1/sqrt(2)
    b[1] = make_double2(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));   // * (1 - i)/sqrt(2)
    b[2] = make_double2(b[2].y, -b[2].x);                                // * -i
    b[3] = make_double2(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));  // * (-1 - i)/sqrt(2)
    dft4(a[0], a[1], a[2], a[3], Y[0], Y[2 % R], Y[4 % R], Y[6 % R]);
    dft4(b[0], b[1], b[2], b[3], Y[1 % R], Y[3 % R], Y[5 % R], Y[7 % R]);
  }
}

// p w, complex.
__device__ __forceinline__ double2 twiddle(double2 p, double2 w) {
  return make_double2(fma(p.x, w.x, -p.y * w.y), fma(p.x, w.y, p.y * w.x));
}

// C(j' + nq s, c) = sum_r w_R^(s r) X_r + beta C, X_r = w_n^(j' r) P(j', r k + c) (P already
// carries alpha).  One thread per (j', c), j' fastest: coalesced reads of P and writes of C.
template <int R>
__global__ void k_dft_radix_combine(const double2* __restrict__ P, int nq, int k, const double2* __restrict__ wn,
                                    double beta, double2* __restrict__ C, long ldc) {
  for (int c = blockIdx.y; c < k; c += gridDim.y) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nq; j += gridDim.x * blockDim.x) {
      double2 X[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const double2 p = __ldg(P + ((size_t)r * k + c) * nq + j);
        if (r == 0) {
          X[r] = p;
        } else {
          X[r] = twiddle(p, __ldg(wn + j * r));
        }
      }
      double2 Y[R];
      radix_butterfly<R>(X, Y);
      double2* out = C + (long)c * ldc + j;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        double2 y = Y[q];
        if (beta != 0.0) {
          const double2 o = out[(size_t)q * nq];
          y = make_double2(fma(beta, o.x, y.x), fma(beta, o.y, y.y));
        }
        out[(size_t)q * nq] = y;
      }
    }
  }
}

// The radix step's CRT, twiddles and butterflies in one pass (P = alpha F_nq B' never reaches
// HBM).  Block (bx, by) recombines the product rows r k + c (r < R, c among the block's 32 / R
// columns of B) over the 64 columns j' = 64 bx + ..., Re and Im (residue columns j' and
// kr/2 + j'), into shared memory, then each thread takes (c, j') pairs in turn and writes
// C(j' + nq s, c) = sum_r w_R^(s r) w_n^(j' r) alpha P(j', r k + c) + beta C(j' + nq s, c).  The
// CRT is integer work and the butterflies FP64 work: four blocks per SM (64 registers, a few
// spilled) overlap the two better than three at 74 registers (n = 8192: 2.23 -> 1.98 ms).
constexpr int RDX_TJ = 64;
template <int R, bool TOP32>
__global__ void __launch_bounds__(256, 4) k_crt_dft_radix(const int8_t* __restrict__ Rres, int M, int nq, int kr,
                                                       CrtConsts cc, const unsigned long long* __restrict__ amax_bits,
                                                       const unsigned long long* __restrict__ hmax_bits,
                                                       const SplitDevParams* prm, double alpha,
                                                       const double2* __restrict__ wn, double beta,
                                                       double2* __restrict__ C, long ldc, int k) {
  constexpr int CPB = 32 / R;  // columns of B per block
  __shared__ double2 tile[32][RDX_TJ];
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * 32 + tx;
  const int j0 = blockIdx.x * RDX_TJ;
  const int PA = prm->PA, PH = prm->PH;
  // this thread's four residue columns: j' = j0 + jl0 + e, Re (tx < 16) or Im
  const bool im = tx >= 16;
  const int jl0 = 4 * (tx & 15);
  const int rc = (im ? kr / 2 : 0) + j0 + jl0;
  unsigned long long hb[4];
  int fexp[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int j = j0 + jl0 + e;
    hb[e] = j < nq ? hmax_bits[j] : 0ull;
    fexp[e] = (hb[e] != 0 && hb[e] < INF_BITS) ? scale_exp(hb[e], PH) : 0;
  }
  const size_t plane_w = (size_t)M * kr / 4;
  const bool scale = alpha != 1.0, accumulate = beta != 0.0;
  for (int cb = blockIdx.y * CPB; cb < k; cb += gridDim.y * CPB) {
    for (int a = 0; a < 4; ++a) {
      const int il = ty + 8 * a;
      const int c = cb + il % CPB, i = (il / CPB) * k + c;
      double val[4] = {0.0, 0.0, 0.0, 0.0};
      if (c < k && j0 + jl0 < nq) crt_row4<TOP32>(Rres + (size_t)i * kr + rc, plane_w, cc, amax_bits[i], PA, hb, fexp, val);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        // rotated (selects, not a dynamic index): a warp's eight-byte stores spread over the banks
        const int er = (e + tx) & 3;
        double v = er == 0 ? val[0] : er == 1 ? val[1] : er == 2 ? val[2] : val[3];
        if (scale) v *= alpha;
        double* slot = (double*)&tile[il][jl0 + er];
        slot[im ? 1 : 0] = v;
      }
    }
    __syncthreads();
    for (int p = t; p < CPB * RDX_TJ; p += 256) {
      const int cl = p / RDX_TJ, jl = p % RDX_TJ;
      const int c = cb + cl, j = j0 + jl;
      if (c < k && j < nq) {
        double2 X[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const double2 v = tile[r * CPB + cl][jl];
          X[r] = r == 0 ? v : twiddle(v, __ldg(wn + j * r));
        }
        double2 Y[R];
        radix_butterfly<R>(X, Y);
        double2* out = C + (long)c * ldc + j;
#pragma unroll
        for (int q = 0; q < R; ++q) {
          double2 y = Y[q];
          if (accumulate) {
            const double2 o = out[(size_t)q * nq];
            y = make_double2(fma(beta, o.x, y.x), fma(beta, o.y, y.y));
          }
          out[(size_t)q * nq] = y;
        }
      }
    }
    __syncthreads();  // the tile is refilled for the next columns
  }
}

int launch_dft_deinterleave(const double2* B, long ldb, int n, int k, int R, double2* Bp, cudaStream_t stream) {
  const dim3 gd((n + 255) / 256 < 64 ? (n + 255) / 256 : 64, k < 65535 ? k : 65535);
  k_dft_deinterleave<<<gd, 256, 0, stream>>>(B, ldb, n, k, R, Bp);
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

int launch_dft_radix_combine(const double2* P, int nq, int k, const double2* wn, double beta, double2* C, long ldc,
                             int R, cudaStream_t stream) {
  const dim3 gc((nq + 255) / 256 < 64 ? (nq + 255) / 256 : 64, k < 65535 ? k : 65535);
  if (R == 8)
    k_dft_radix_combine<8><<<gc, 256, 0, stream>>>(P, nq, k, wn, beta, C, ldc);
  else if (R == 4)
    k_dft_radix_combine<4><<<gc, 256, 0, stream>>>(P, nq, k, wn, beta, C, ldc);
  else if (R == 2)
    k_dft_radix_combine<2><<<gc, 256, 0, stream>>>(P, nq, k, wn, beta, C, ldc);
  else
    return PSMMA_EUNSUPPORTED;
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

static int split_status(SplitDevParams* prm, cudaStream_t stream, unsigned* status_dev_out) {
  if (status_dev_out && status_dev_out != kStatusWait) {
    if (cudaMemcpyAsync(status_dev_out, &prm->status, sizeof(unsigned), cudaMemcpyDeviceToDevice, stream) !=
        cudaSuccess)
      return PSMMA_EDEVICE;
    return PSMMA_OK;
  }
  if (!status_dev_out) {
    // asynchronous: the status joins the stream's word, reported by psmma_stream_status
    unsigned* acc = stream_status_word(stream);
    if (acc) {
      k_status_or<<<1, 1, 0, stream>>>(acc, &prm->status);
      return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
    }
  }
  unsigned st = 0;  // kStatusWait (or no status word): wait for the call and read its status
  if (cudaMemcpyAsync(&st, &prm->status, sizeof(st), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return PSMMA_EDEVICE;
  if (st & DEV_ERR_TIMEOUT) return PSMMA_ETIMEDOUT;
  return PSMMA_OK;
}

// Core of the split path: Q (M x N) = alpha * A (M x K, column-major, lda) * H (K x N) + beta * Q
// (column-major, ldq), H generated from gs (any kind but the DFT: split_core_dft3).
static int split_core(int M, int N, int K, double alpha, const double* A, long lda, const GenSpec& gs, double beta,
                      double* Q, long ldq, int nmod, void* work, size_t lwork, cudaStream_t stream,
                      unsigned* status_dev_out) {
  if (gs.kind == KIND_DFT) return PSMMA_EUNSUPPORTED;  // split_core_dft3
  if (nmod < 8 || nmod > SPL_MAX_MODULI) return PSMMA_EUNSUPPORTED;
  if (K >= (1 << 24) || M > kSplitMaxRows || N >= (1 << 30)) return PSMMA_EUNSUPPORTED;
  SplitLayout L = split_layout(M, K, N, nmod);
  if (lwork < L.total || !work) return PSMMA_EWORKSPACE;
  char* w = (char*)work;
  const SplitBuffers b = split_buffers(w, L);
  const CrtConsts cc = get_consts(nmod);

  prof_begin(stream);
  if (cudaMemsetAsync(w, 0, L.off_wtab, stream) != cudaSuccess) return PSMMA_EDEVICE;  // params, maxima, sums

  // ---- A side: row maxima and norms
  {
    const int kchunk = 1024;
    dim3 g1((M + 127) / 128, (K + kchunk - 1) / kchunk);
    k_row_absmax<<<g1, 128, 0, stream>>>(A, lda, M, K, kchunk, b.amax, b.asq);
  }
  prof_mark(stream, "row_scale");
  // ---- H side: generate, column maxima / sums / norms
  switch (gs.kind) {
    case KIND_CAUCHY: k_h_pass1<KIND_CAUCHY><<<N, 256, 0, stream>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_TOEPLITZ: k_h_pass1<KIND_TOEPLITZ><<<N, 256, 0, stream>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_HANKEL: k_h_pass1<KIND_HANKEL><<<N, 256, 0, stream>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_DENSE: k_h_pass1<KIND_DENSE><<<N, 256, 0, stream>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_CAUCHY_EIG: k_h_pass1<KIND_CAUCHY_EIG><<<N, 256, 0, stream>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    default: return PSMMA_EUNSUPPORTED;
  }
  prof_mark(stream, "h_generate");
  k_split_params<<<PARAMS_BLOCKS, 512, 0, stream>>>(b.prm, cc.log2M, M, N, K, b.amax, b.asq, b.hmax, b.hsq);
  prof_mark(stream, "params");
  k_residues_A<<<dim3(L.kp / 64, (M + 63) / 64), 256, 0, stream>>>(A, lda, M, K, L.kp, b.amax, b.prm, cc, b.RA);
  prof_mark(stream, "residues_A");
  k_residues_H<<<dim3(N, rh_blocks_x(L.kp)), 128, 0, stream>>>(b.Ht, N, L.kp, b.hmax, b.prm, cc, b.RH);
  prof_mark(stream, "residues_H");

  OneGemm og;
  memset(&og, 0, sizeof(og));
  if (!make_tmap(&og.ta, b.RA, L.kp, M, nmod, G_BM) || !make_tmap(&og.tb, b.RH, L.kp, N, nmod, G_BN))
    return PSMMA_EDEVICE;
  GemmArgs& ga = og.g;
  ga.n = M;
  ga.kr = L.kr;
  ga.nkb = L.kp / G_BK;
  ga.tiles_m = (M + G_BM - 1) / G_BM;
  ga.tiles_n = (N + G_BN - 1) / G_BN;
  ga.group_m = 16;
  ga.R = b.R;
  ga.status = &b.prm->status;
  for (int l = 0; l < nmod; ++l) { ga.m[l] = cc.m[l]; ga.inv_m[l] = cc.inv_m[l]; }
  using Shape = GemmShape<G_BN>;
  if (set_smem_attr(k_crt_gemm<G_BN, OneGemm>, (int)Shape::SMEM) != cudaSuccess)
    return PSMMA_EDEVICE;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PSMMA_EDEVICE;
  ga.nmod = nmod;
  const int total_tiles = ga.tiles_m * ga.tiles_n * nmod;
  k_crt_gemm<G_BN, OneGemm><<<std::min(sms, total_tiles), G_THREADS, Shape::SMEM, stream>>>(og);
  prof_mark(stream, "modular_gemm");

  dim3 gc((N + CRT_TJ - 1) / CRT_TJ, (M + CRT_TI - 1) / CRT_TI);
  (cc.top32 ? k_crt_combine<false, true> : k_crt_combine<false, false>)<<<gc, dim3(32, 8), 0, stream>>>(
      b.R, M, N, L.kr, cc, b.amax, b.hmax, b.prm, alpha, beta, Q, ldq, 0);
  prof_mark(stream, "crt_combine");
  if (cudaGetLastError() != cudaSuccess) return PSMMA_EDEVICE;

  return split_status(b.prm, stream, status_dev_out);
}

// ---- Block-recursive Toeplitz / Hankel products --------------------------------------------
// With A = [X1 X2] (column halves) and H = [Y00 Y01; Y10 Y11] (Y_rc: rows block r, columns block
// c), Q = [Q1 Q2] takes three half-size products instead of four:
//   Toeplitz (Y11 = Y00):  P = (X1 + X2) Y00,  Q1 = P + X2 (Y10 - Y00),  Q2 = P + X1 (Y01 - Y00);
//   Hankel   (Y10 = Y01):  P = (X1 + X2) Y01,  Q1 = P + X1 (Y00 - Y01),  Q2 = P + X2 (Y11 - Y01).
// Sums and differences of Toeplitz (Hankel) blocks are Toeplitz (Hankel) again, so the step
// repeats on each of the three products: L levels give 3^L leaf products of width w = N / 2^L,
// (3/4)^L of the modular GEMM work.  All of it is exact integer arithmetic modulo m_l on the
// residues of the scaled A' and H' (the shared group exponents keep H' structured), so the
// recombined Z = A'H' is the same integer matrix the single product gives.  Each leaf's A
// operand is a sum of A's column blocks, its H operand a signed sum of up to 2^L blocks of H',
// and its result goes to (is added to) 1 to 2^L column blocks of the output residues; the
// first leaf (the sums at every level) covers every block and stores, the others add.
struct BlkNode {
  int amask;  // column blocks of A (at the node's level) summed into its A operand
  int nterm;
  int sign[1 << BLK_MAX_LEVELS], r[1 << BLK_MAX_LEVELS], c[1 << BLK_MAX_LEVELS];  // H blocks (r, c)
  int ndst;
  int dst[1 << BLK_MAX_LEVELS];  // output column blocks
};

static void block_expand(int kind, int level, int L, const BlkNode& nd, std::vector<BlkNode>& leaves) {
  if (level == L) {
    leaves.push_back(nd);
    return;
  }
  // per choice: A halves (0 both, 1 first, 2 second), H terms (sign, row block, column block of
  // the node's 2 x 2 split), output halves (0 both, 1 first, 2 second)
  struct Choice {
    int ahalf, nt, s[2], a[2], b[2], dsel;
  };
  static const Choice kToeplitz[3] = {{0, 1, {1, 0}, {0, 0}, {0, 0}, 0},
                                      {2, 2, {1, -1}, {1, 0}, {0, 0}, 1},
                                      {1, 2, {1, -1}, {0, 0}, {1, 0}, 2}};
  static const Choice kHankel[3] = {{0, 1, {1, 0}, {0, 0}, {1, 0}, 0},
                                    {1, 2, {1, -1}, {0, 0}, {0, 1}, 1},
                                    {2, 2, {1, -1}, {1, 0}, {1, 1}, 2}};
  const Choice* ch = kind == KIND_TOEPLITZ ? kToeplitz : kHankel;
  for (int x = 0; x < 3; ++x) {
    const Choice& cb = ch[x];
    BlkNode c;
    memset(&c, 0, sizeof(c));
    for (int p = 0; p < 32; ++p)
      if ((nd.amask >> p) & 1) {
        if (cb.ahalf != 2) c.amask |= 1 << (2 * p);
        if (cb.ahalf != 1) c.amask |= 1 << (2 * p + 1);
      }
    for (int t = 0; t < nd.nterm; ++t)
      for (int u = 0; u < cb.nt; ++u) {
        c.sign[c.nterm] = nd.sign[t] * cb.s[u];
        c.r[c.nterm] = 2 * nd.r[t] + cb.a[u];
        c.c[c.nterm] = 2 * nd.c[t] + cb.b[u];
        ++c.nterm;
      }
    for (int d = 0; d < nd.ndst; ++d) {
      if (cb.dsel != 2) c.dst[c.ndst++] = 2 * nd.dst[d];
      if (cb.dsel != 1) c.dst[c.ndst++] = 2 * nd.dst[d] + 1;
    }
    block_expand(kind, level + 1, L, c, leaves);
  }
}

static std::vector<BlkNode> block_leaves(int kind, int L) {
  BlkNode root;
  memset(&root, 0, sizeof(root));
  root.amask = 1;
  root.nterm = 1;
  root.sign[0] = 1;
  root.ndst = 1;
  std::vector<BlkNode> leaves;
  block_expand(kind, 0, L, root, leaves);
  return leaves;
}

// Leaves need w = Np / 2^L to be a multiple of 64 (whole k blocks and 128-byte operand offsets),
// so an order N that 64 * 2^L does not divide is padded to Np: H extended by the zero-extended
// generator (still Toeplitz / Hankel), A by zero columns, and only N columns recombined.
// req (psmma_opts::block_levels): 0 = automatic -- the L <= kBlockAutoLevels with w >=
// kBlockMinLeaf that minimises the GEMM work (Np / N)^2 (3/4)^L, if that is at most
// kBlockMaxWork (below w = 4096 the modular GEMMs' per-tile epilogue, 2 drains at k = 2048,
// weighs about as much as their MMAs and the step stops paying); -1 = none; 1..3 = that many
// levels.
constexpr int kBlockMinLeaf = 4096;
constexpr int kBlockAutoLevels = 2;
constexpr double kBlockMaxWork = 0.85;
static int round_up(int x, int m) { return (x + m - 1) / m * m; }
static BlockChoice block_choice(int kind, int N, int K, int req) {
  if ((kind != KIND_TOEPLITZ && kind != KIND_HANKEL) || N != K || req < 0 || N <= 0) return {0, N};
  if (req > 0) {
    const int L = std::min(req, BLK_MAX_LEVELS);
    return {L, round_up(N, 64 << L)};
  }
  BlockChoice best = {0, N};
  double best_work = kBlockMaxWork;
  for (int L = 1; L <= kBlockAutoLevels; ++L) {
    const int Np = round_up(N, 64 << L);
    const double work = (double)Np * Np / ((double)N * N) * std::pow(0.75, L);
    if ((Np >> L) >= kBlockMinLeaf && work <= best_work) {
      best = {L, Np};
      best_work = work;
    }
  }
  return best;
}
static int block_levels(int kind, int N, int K, int req) { return block_choice(kind, N, K, req).L; }

static bool s2_use(int kind, int M, int K, int N, int req);

extern "C" int psmma_split_block_levels(int kind, int n, int k) {
  if (n <= 0 || k <= 0) return 0;
  return (kind == KIND_TOEPLITZ || kind == KIND_HANKEL) ? block_levels(kind, k, k, 0) : (s2_use(kind, n, k, k, 0) ? 1 : 0);
}

static int ipow3(int L) { return L == 0 ? 1 : 3 * ipow3(L - 1); }

// The split layout with the H residues replaced by the 3^L leaf operands (w x w each) followed
// by the A block sums (3^L - 2^L planes of M x w); the region also holds the whole H's residues
// of the single-product fallback.  The group maxima come last.
static SplitLayout block_layout(int M, int N, int L, int nmod) {
  const int w = N >> L, nleaf = ipow3(L), nsum = nleaf - (1 << L);
  SplitLayout B;
  B.kp = (N + 63) / 64 * 64;
  B.kr = (N + 255) / 256 * 256;
  size_t o = 0;
  B.off_params = o; o += al1k(2 * sizeof(SplitDevParams));
  B.off_amax = o;   o += al1k((size_t)M * 8);
  B.off_hmax = o;   o += al1k((size_t)N * 8);
  B.off_hsum = o;   o += al1k((size_t)N * 8);
  B.off_asq = o;    o += al1k((size_t)M * 8);
  B.off_hsq = o;    o += al1k((size_t)N * 8);
  B.off_wtab = o;   o += al1k(16);
  B.off_ht = o;     o += al1k((size_t)N * B.kp * 8);
  B.off_ra = o;     o += al1k((size_t)nmod * M * B.kp * 2);
  B.off_rh = o;
  B.off_rs = o + al1k((size_t)nleaf * nmod * w * w * 2);
  o += std::max(al1k((size_t)nleaf * nmod * w * w * 2) + al1k((size_t)nsum * nmod * M * w * 2),
                al1k((size_t)nmod * N * B.kp * 2));
  B.off_r = o;      o += al1k((size_t)nmod * M * B.kr);
  B.off_gmax = o;   o += al1k((size_t)w * 8);
  B.off_hall = o;   o += al1k((size_t)N * 8);
  B.total = o;
  return B;
}

// Tensor map of residue planes [nmod][rows][pitch] (bf16), the first `inner` entries of each row.
static bool make_tmap_view(CUtensorMap* map, void* ptr, int inner, long pitch, int rows, int nmod, long plane,
                           int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)inner, (cuuint64_t)rows, (cuuint64_t)nmod};
  cuuint64_t strides[2] = {(cuuint64_t)pitch * 2, (cuuint64_t)plane * 2};
  cuuint32_t box[3] = {(cuuint32_t)G_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, ptr, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The launches of the block step for one call, shared by the device-pointer call (all rows at
// once) and the host-pointer pipeline (row panels).  pk: the parameters the kernels scale with
// and gate on (hbad) -- the call's, or the guessed ones of a speculative pipeline.
struct BlockRun {
  int M, N, Np, L, w, NQ, nmod, nleaf, sms;
  GenSpec gs;
  SplitLayout Lo;
  SplitBuffers b;
  __nv_bfloat16* RS;
  unsigned long long *gmax, *hall;
  CrtConsts cc;
  std::vector<BlkNode> leaves;
  std::vector<int> a_sum;
  BlockSums bs;
  LeafTerms lt;

  int init(int M_, int N_, int Np_, int L_, const GenSpec& gs_in, int nmod_, void* work, size_t lwork) {
    M = M_; N = N_; Np = Np_; L = L_; nmod = nmod_;
    if (nmod < 8 || nmod > SPL_MAX_MODULI) return PSMMA_EUNSUPPORTED;
    if (Np >= (1 << 24) || M > kSplitMaxRows || L < 1 || L > BLK_MAX_LEVELS || Np < N || Np % (64 << L) != 0)
      return PSMMA_EUNSUPPORTED;
    gs = gs_in;
    if (Np > N) {
      gs.glen = 2L * N - 1;  // the padding reads the generator zero-extended
      gs.srows = N;          // and only the real rows count in the column statistics
    }
    w = Np >> L;
    NQ = 1 << L;
    Lo = block_layout(M, Np, L, nmod);
    if (lwork < Lo.total || !work) return PSMMA_EWORKSPACE;
    char* wk = (char*)work;
    b = split_buffers(wk, Lo);
    RS = (__nv_bfloat16*)(wk + Lo.off_rs);
    gmax = (unsigned long long*)(wk + Lo.off_gmax);
    hall = (unsigned long long*)(wk + Lo.off_hall);
    cc = get_consts(nmod);
    leaves = block_leaves(gs.kind, L);
    nleaf = (int)leaves.size();
    // A operands: one block (a view of RA) or a sum plane (RS), numbered in leaf order
    memset(&bs, 0, sizeof(bs));
    for (int q = 0; q < NQ; ++q) bs.qcol[q] = q * w;  // column blocks of every row
    bs.wmask = (1 << NQ) - 1;
    a_sum.assign(nleaf, -1);
    for (int y = 0; y < nleaf; ++y) {
      const int mk = leaves[y].amask;
      if ((mk & (mk - 1)) == 0) continue;
      int p = 0;
      while (p < bs.nsum && bs.mask[p] != mk) ++p;
      if (p == bs.nsum) bs.mask[bs.nsum++] = mk;
      a_sum[y] = p;
    }
    memset(&lt, 0, sizeof(lt));
    for (int y = 0; y < nleaf; ++y) {
      lt.nterm[y] = leaves[y].nterm;
      for (int t = 0; t < leaves[y].nterm; ++t) {
        lt.sign[y][t] = (signed char)leaves[y].sign[t];
        lt.koff[y][t] = leaves[y].r[t] * w;
        lt.joff[y][t] = leaves[y].c[t] * w;
      }
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return PSMMA_EDEVICE;
    using Shape = GemmShape<G_BN>;
    if (set_smem_attr(k_crt_gemm<G_BN, OneGemm, true>, (int)Shape::SMEM) != cudaSuccess ||
        set_smem_attr(k_crt_gemm<G_BN, OneGemm>, (int)Shape::SMEM) != cudaSuccess)
      return PSMMA_EDEVICE;
    const int smem = NQ * 64 * 32 * 8;
    const cudaError_t e = NQ == 2 ? set_smem_attr(k_residues_A_blocks<2>, smem)
                          : NQ == 4 ? set_smem_attr(k_residues_A_blocks<4>, smem)
                                    : set_smem_attr(k_residues_A_blocks<8>, smem);
    return e == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
  }

  // Ht, the column statistics (real rows) and all-row maxima, the group maxima and the gate.
  void h_side(SplitDevParams* prm2, cudaStream_t s) {
    if (gs.kind == KIND_TOEPLITZ)
      k_h_pass1_all<KIND_TOEPLITZ><<<Np, 256, 0, s>>>(gs, Np, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm, hall);
    else
      k_h_pass1_all<KIND_HANKEL><<<Np, 256, 0, s>>>(gs, Np, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm, hall);
    k_group_colmax<<<(w + 255) / 256, 256, 0, s>>>(hall, gmax, w, NQ, b.prm, prm2);
  }

  // The leaves' H operands, or (gated) the whole H's residues for the single product.
  void h_operands(const SplitDevParams* pk, cudaStream_t s) {
    const dim3 gh(w, rh_blocks_x(w), nleaf);
    if (NQ == 2)
      k_residues_H_leaf<2><<<gh, 128, 0, s>>>(b.Ht, Lo.kp, w, w, hall, gmax, 1, pk, cc, lt, b.RH);
    else if (NQ == 4)
      k_residues_H_leaf<4><<<gh, 128, 0, s>>>(b.Ht, Lo.kp, w, w, hall, gmax, 1, pk, cc, lt, b.RH);
    else
      k_residues_H_leaf<8><<<gh, 128, 0, s>>>(b.Ht, Lo.kp, w, w, hall, gmax, 1, pk, cc, lt, b.RH);
    k_residues_H_gated<<<dim3(std::min(Np, 608), rh_blocks_x(Lo.kp)), 128, 0, s>>>(b.Ht, Np, Lo.kp, N, b.hmax, pk,
                                                                                   cc, b.RH);
  }

  // Block residues and sums of rows [r0, r0 + rows) of A (leading dimension lda).
  void a_residues(const double* A, long lda, int r0, int rows, const SplitDevParams* pk, cudaStream_t s) {
    const dim3 ga(w / 64, (rows + 31) / 32);
    const int smem = NQ * 64 * 32 * 8;
    if (NQ == 2)
      k_residues_A_blocks<2><<<ga, 256, smem, s>>>(A, lda, M, r0, rows, w, Lo.kp, N, M, r0, b.amax, pk, cc, b.RA, RS,
                                                    bs);
    else if (NQ == 4)
      k_residues_A_blocks<4><<<ga, 256, smem, s>>>(A, lda, M, r0, rows, w, Lo.kp, N, M, r0, b.amax, pk, cc, b.RA, RS,
                                                    bs);
    else
      k_residues_A_blocks<8><<<ga, 256, smem, s>>>(A, lda, M, r0, rows, w, Lo.kp, N, M, r0, b.amax, pk, cc, b.RA, RS,
                                                    bs);
  }

  // The leaf products of rows [r0, r0 + rows) (r0 a multiple of the 128-row tile) into R, and
  // (gated) the single product of those rows.
  int products(int r0, int rows, const SplitDevParams* pk, cudaStream_t s) {
    using Shape = GemmShape<G_BN>;
    for (int y = 0; y < nleaf; ++y) {
      const BlkNode& lf = leaves[y];
      OneGemm og;
      memset(&og, 0, sizeof(og));
      bool ok;
      if (a_sum[y] < 0) {
        int q = 0;
        while (!((lf.amask >> q) & 1)) ++q;
        ok = make_tmap_view(&og.ta, b.RA + (size_t)r0 * Lo.kp + (size_t)q * w, w, Lo.kp, rows, nmod, (long)M * Lo.kp,
                            G_BM);
      } else {
        ok = make_tmap_view(&og.ta, RS + (size_t)a_sum[y] * nmod * M * w + (size_t)r0 * w, w, w, rows, nmod,
                            (long)M * w, G_BM);
      }
      ok = ok && make_tmap_view(&og.tb, b.RH + (size_t)y * nmod * w * w, w, w, w, nmod, (long)w * w, G_BN);
      if (!ok) return PSMMA_EDEVICE;
      GemmArgs& ga = og.g;
      ga.n = rows;
      ga.kr = Lo.kr;
      ga.nkb = w / G_BK;
      ga.tiles_m = (rows + G_BM - 1) / G_BM;
      ga.tiles_n = (w + G_BN - 1) / G_BN;
      ga.group_m = 16;
      ga.nmod = nmod;
      ga.R = b.R;
      ga.status = &b.prm->status;
      for (int l = 0; l < nmod; ++l) { ga.m[l] = cc.m[l]; ga.inv_m[l] = cc.inv_m[l]; }
      ga.r_rows = M;
      ga.ndst = lf.ndst;
      for (int d = 0; d < lf.ndst; ++d) {
        ga.dst_row[d] = r0;
        ga.dst_col[d] = lf.dst[d] * w;
        ga.dst_op[d] = y == 0 ? 0 : 2;  // the first leaf covers every block (block_expand takes the sums first)
      }
      ga.ncols = w;
      ga.gate = &pk->hbad;
      ga.gate_set = 0;
      const int total_tiles = ga.tiles_m * ga.tiles_n * nmod;
      k_crt_gemm<G_BN, OneGemm, true><<<std::min(sms, total_tiles), G_THREADS, Shape::SMEM, s>>>(og);
    }
    // the single product, when some column of H is not finite or spreads too far
    OneGemm og;
    memset(&og, 0, sizeof(og));
    if (!make_tmap(&og.ta, b.RA, Lo.kp, M, nmod, G_BM) || !make_tmap(&og.tb, b.RH, Lo.kp, Np, nmod, G_BN))
      return PSMMA_EDEVICE;
    GemmArgs& ga = og.g;
    ga.n = M;
    ga.kr = Lo.kr;
    ga.nkb = Lo.kp / G_BK;
    ga.tm0 = r0 / G_BM;
    ga.tiles_m = (rows + G_BM - 1) / G_BM;
    ga.tiles_n = (Np + G_BN - 1) / G_BN;
    ga.group_m = 16;
    ga.nmod = nmod;
    ga.R = b.R;
    ga.status = &b.prm->status;
    for (int l = 0; l < nmod; ++l) { ga.m[l] = cc.m[l]; ga.inv_m[l] = cc.inv_m[l]; }
    ga.gate = &pk->hbad;
    ga.gate_set = 1;
    k_crt_gemm<G_BN, OneGemm><<<std::min(sms, ga.tiles_m * ga.tiles_n * nmod), G_THREADS, Shape::SMEM, s>>>(og);
    return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
  }

  // The recombination of rows [r0, r0 + rows) (r0 a multiple of CRT_TI) into Q (rows from r0).
  void crt(int r0, int rows, double alpha, double beta, double* Q, long ldq, const SplitDevParams* pk,
           cudaStream_t s) {
    const dim3 gc((N + CRT_TJ - 1) / CRT_TJ, (rows + CRT_TI - 1) / CRT_TI);
    (cc.top32 ? k_crt_combine_blocks<true> : k_crt_combine_blocks<false>)<<<gc, dim3(32, 8), 0, s>>>(
        b.R, M, N, Lo.kr, cc, b.amax, b.hmax, gmax, w, pk, alpha, beta, Q, ldq, r0 / CRT_TI);
  }
};

// Q (M x N) = alpha * A (M x N) * H + beta * Q for Toeplitz / Hankel H (N x N) with L >= 1 levels
// of the block step on the order Np >= N (block_choice; padded when Np > N).
static int split_core_block(int M, int N, int Np, int L, double alpha, const double* A, long lda,
                            const GenSpec& gs_in, double beta, double* Q, long ldq, int nmod, void* work,
                            size_t lwork, cudaStream_t stream, unsigned* status_dev_out) {
  BlockRun br;
  int st = br.init(M, N, Np, L, gs_in, nmod, work, lwork);
  if (st != PSMMA_OK) return st;
  const SplitBuffers& b = br.b;
  prof_begin(stream);
  if (cudaMemsetAsync(work, 0, br.Lo.off_wtab, stream) != cudaSuccess) return PSMMA_EDEVICE;
  {
    const int kchunk = 1024;
    dim3 g1((M + 127) / 128, (N + kchunk - 1) / kchunk);
    k_row_absmax<<<g1, 128, 0, stream>>>(A, lda, M, N, kchunk, b.amax, b.asq);
  }
  prof_mark(stream, "row_scale");
  br.h_side(nullptr, stream);
  prof_mark(stream, "h_generate");
  k_split_params<<<PARAMS_BLOCKS, 512, 0, stream>>>(b.prm, br.cc.log2M, M, Np, Np, b.amax, b.asq, b.hmax, b.hsq);
  prof_mark(stream, "params");
  br.a_residues(A, lda, 0, M, b.prm, stream);
  prof_mark(stream, "residues_A");
  br.h_operands(b.prm, stream);
  prof_mark(stream, "residues_H");
  st = br.products(0, M, b.prm, stream);
  if (st != PSMMA_OK) return st;
  prof_mark(stream, "modular_gemm");
  br.crt(0, M, alpha, beta, Q, ldq, b.prm, stream);
  prof_mark(stream, "crt_combine");
  if (cudaGetLastError() != cudaSuccess) return PSMMA_EDEVICE;
  return split_status(b.prm, stream, status_dev_out);
}

// ---- Strassen's step on the residue planes -----------------------------------------------
// Over any ring, the 2 x 2 block product C = A B takes seven block products instead of eight:
//   M1 = (A00 + A11)(B00 + B11)   M2 = (A10 + A11) B00   M3 = A00 (B01 - B11)   M4 = A11 (B10 - B00)
//   M5 = (A00 + A01) B11          M6 = (A10 - A00)(B00 + B01)                   M7 = (A01 - A11)(B10 + B11)
//   C00 = M1 + M4 - M5 + M7   C01 = M3 + M5   C10 = M2 + M4   C11 = M1 - M2 + M3 + M6.
// Applied to the residue planes of the integer-scaled A' (rows of a panel, columns K) and H'
// modulo each m_l, it is exact and needs no structure: the recombined Z = A'H' is the same
// integer matrix, so the result is the single product's bit for bit, with 7/8 of its modular
// GEMM work.  A blocks are numbered q = 2 row-block + column-block; H blocks (r, c) are the row
// (k) and column blocks.  Products run in this order; each output block's first contribution
// stores and has a positive sign, the later ones add or subtract.
struct S2Prod {
  int amask, aneg;           // A blocks summed / subtracted
  int nh, hs[2], hr[2], hc[2];  // H terms
  int nd, drb[2], dcb[2], dop[2];  // output blocks (row block, column block), operation
};
static const S2Prod kStrassen[7] = {
    {0x9, 0x0, 2, {1, 1}, {0, 1}, {0, 1}, 2, {0, 1}, {0, 1}, {0, 0}},   // M1 -> C00, C11 (stores)
    {0xC, 0x0, 1, {1, 0}, {0, 0}, {0, 0}, 2, {1, 1}, {0, 1}, {0, 3}},   // M2 -> C10 (store), C11 -
    {0x1, 0x0, 2, {1, -1}, {0, 1}, {1, 1}, 2, {0, 1}, {1, 1}, {0, 2}},  // M3 -> C01 (store), C11 +
    {0x8, 0x0, 2, {1, -1}, {1, 0}, {0, 0}, 2, {0, 1}, {0, 0}, {2, 2}},  // M4 -> C00 +, C10 +
    {0x3, 0x0, 1, {1, 0}, {1, 0}, {1, 0}, 2, {0, 0}, {0, 1}, {3, 2}},   // M5 -> C00 -, C01 +
    {0x5, 0x1, 2, {1, 1}, {0, 0}, {0, 1}, 1, {1, 0}, {1, 0}, {2, 0}},   // M6 -> C11 +
    {0xA, 0x8, 2, {1, 1}, {1, 1}, {0, 1}, 1, {0, 0}, {0, 0}, {2, 0}},   // M7 -> C00 +
};

// Strassen's step for a product of M rows, K inner, N columns: M even, K and N multiples of
// 128 (block widths of whole 64-column k blocks, 16-byte output offsets).  Only on request
// (psmma_opts::block_levels = 1): its operands take 7/4 of the residue planes' HBM traffic, and
// at n = 16384 those passes cost about what the eighth of the modular GEMM work saves.
static bool s2_fits(int M, int K, int N) { return M % 2 == 0 && K % 128 == 0 && N % 128 == 0 && M >= 2; }
// Strassen's step is for the unstructured kinds (Toeplitz and Hankel take their own block step).
static bool s2_use(int kind, int M, int K, int N, int req) {
  if (kind != KIND_CAUCHY && kind != KIND_CAUCHY_EIG && kind != KIND_DENSE) return false;
  return req > 0 && s2_fits(M, K, N);
}

// Workspace: the split layout with the H residues replaced by the seven H operands (N/2 x K/2
// each) and the five A block sums (rows / 2 x K/2 each) of a pass over `rows` rows.
static SplitLayout s2_layout(int M, int K, int N, int rows, int nmod) {
  SplitLayout B = split_layout(M, K, N, nmod);
  const size_t rh = al1k((size_t)7 * nmod * (N / 2) * (K / 2) * 2);
  const size_t rs = al1k((size_t)5 * nmod * (rows / 2) * (K / 2) * 2);
  // split_layout's H residue region [off_rh, off_r) becomes the H operands, then the sums
  const size_t tail = B.total - B.off_r;
  B.off_rs = B.off_rh + rh;
  const size_t off_r = B.off_rs + rs;
  B.total = off_r + tail;
  B.off_r = off_r;
  return B;
}

// Prepared state of Strassen's step for one call: operand numbering and the constant parts of
// the seven GEMM launches.
struct S2State {
  int M, K, N, nmod, kp, kr, sms;
  __nv_bfloat16 *RA, *RS, *RHL;
  int8_t* R;
  unsigned* status;
  int a_sum[7];  // A operand: sum plane index, or -1 for a block of RA
  BlockSums bs;  // qrow filled per pass
  CrtConsts cc;
};

static void s2_prepare(S2State& st) {
  memset(&st.bs, 0, sizeof(st.bs));
  for (int y = 0; y < 7; ++y) {
    const int mk = kStrassen[y].amask;
    st.a_sum[y] = -1;
    if ((mk & (mk - 1)) == 0 && kStrassen[y].aneg == 0) continue;
    st.a_sum[y] = st.bs.nsum;
    st.bs.mask[st.bs.nsum] = mk;
    st.bs.neg[st.bs.nsum] = kStrassen[y].aneg;
    ++st.bs.nsum;
  }
  for (int q = 0; q < 4; ++q) st.bs.qcol[q] = (q & 1) * (st.K / 2);
  for (int y = 0; y < 7; ++y)
    if (st.a_sum[y] < 0) st.bs.wmask |= kStrassen[y].amask;  // A00 and A11: read in place
}

// The seven H operands from Ht, in the order of kStrassen (k_residues_H_s2 writes that order).
static void s2_h_operands(const S2State& st, const double* Ht, const unsigned long long* hmax, const SplitDevParams* prm,
                          cudaStream_t stream) {
  const dim3 gh(st.N / 2, rh_blocks_x(st.K / 2));
  k_residues_H_s2<<<gh, 128, 0, stream>>>(Ht, st.kp, st.K / 2, st.N / 2, hmax, prm, st.cc, st.RHL);
}

// Rows [r0, r0 + P) (P even) of A: block residues and sums, then the seven products into the
// residue planes of R.  pk: the bit counts to scale A with.
static int s2_pass(S2State& st, const double* A, long lda, const unsigned long long* amax, const SplitDevParams* pk,
                   int r0, int P, cudaStream_t stream) {
  const int h = P / 2, wk = st.K / 2, wn = st.N / 2;
  BlockSums bs = st.bs;
  for (int q = 0; q < 4; ++q) bs.qrow[q] = (q >> 1) * h;
  const int smem = 4 * 64 * 32 * 8;
  if (set_smem_attr(k_residues_A_blocks<4>, smem) != cudaSuccess) return PSMMA_EDEVICE;
  k_residues_A_blocks<4><<<dim3(wk / 64, (h + 31) / 32), 256, smem, stream>>>(A, lda, st.M, r0, h, wk, st.kp, st.K,
                                                                               h, 0, amax, pk, st.cc, st.RA, st.RS,
                                                                               bs);
  prof_mark(stream, "residues_A");
  using Shape = GemmShape<G_BN>;
  if (set_smem_attr(k_crt_gemm<G_BN, OneGemm, true>, (int)Shape::SMEM) != cudaSuccess) return PSMMA_EDEVICE;
  for (int y = 0; y < 7; ++y) {
    const S2Prod& pr = kStrassen[y];
    OneGemm og;
    memset(&og, 0, sizeof(og));
    bool ok;
    if (st.a_sum[y] < 0) {
      const int q = __builtin_ctz(pr.amask);
      ok = make_tmap_view(&og.ta, st.RA + (size_t)(r0 + (q >> 1) * h) * st.kp + (q & 1) * wk, wk, st.kp, h, st.nmod,
                          (long)st.M * st.kp, G_BM);
    } else {
      ok = make_tmap_view(&og.ta, st.RS + (size_t)st.a_sum[y] * st.nmod * h * wk, wk, wk, h, st.nmod, (long)h * wk,
                          G_BM);
    }
    ok = ok && make_tmap_view(&og.tb, st.RHL + (size_t)y * st.nmod * wn * wk, wk, wk, wn, st.nmod, (long)wn * wk, G_BN);
    if (!ok) return PSMMA_EDEVICE;
    GemmArgs& ga = og.g;
    ga.n = h;
    ga.kr = st.kr;
    ga.nkb = wk / G_BK;
    ga.tiles_m = (h + G_BM - 1) / G_BM;
    ga.tiles_n = (wn + G_BN - 1) / G_BN;
    ga.group_m = 16;
    ga.nmod = st.nmod;
    ga.R = st.R;
    ga.status = st.status;
    for (int l = 0; l < st.nmod; ++l) { ga.m[l] = st.cc.m[l]; ga.inv_m[l] = st.cc.inv_m[l]; }
    ga.ncols = wn;
    ga.r_rows = st.M;
    ga.ndst = pr.nd;
    for (int d = 0; d < pr.nd; ++d) {
      ga.dst_row[d] = r0 + pr.drb[d] * h;
      ga.dst_col[d] = pr.dcb[d] * wn;
      ga.dst_op[d] = pr.dop[d];
    }
    const int total_tiles = ga.tiles_m * ga.tiles_n * st.nmod;
    k_crt_gemm<G_BN, OneGemm, true><<<std::min(st.sms, total_tiles), G_THREADS, Shape::SMEM, stream>>>(og);
    prof_mark(stream, "modular_gemm");
  }
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

// Device-pointer split multiply with Strassen's step over all M rows.
static int split_core_s2(int M, int N, int K, double alpha, const double* A, long lda, const GenSpec& gs, double beta,
                         double* Q, long ldq, int nmod, void* work, size_t lwork, cudaStream_t stream,
                         unsigned* status_dev_out) {
  if (nmod < 8 || nmod > SPL_MAX_MODULI) return PSMMA_EUNSUPPORTED;
  if (K >= (1 << 24) || M > kSplitMaxRows || N >= (1 << 30) || !s2_fits(M, K, N)) return PSMMA_EUNSUPPORTED;
  const SplitLayout Lo = s2_layout(M, K, N, M, nmod);
  if (lwork < Lo.total || !work) return PSMMA_EWORKSPACE;
  char* wk = (char*)work;
  const SplitBuffers b = split_buffers(wk, Lo);
  S2State st;
  st.M = M; st.K = K; st.N = N; st.nmod = nmod; st.kp = Lo.kp; st.kr = Lo.kr;
  st.RA = b.RA; st.RS = (__nv_bfloat16*)(wk + Lo.off_rs); st.RHL = b.RH; st.R = b.R;
  st.status = &b.prm->status;
  st.cc = get_consts(nmod);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&st.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PSMMA_EDEVICE;
  s2_prepare(st);

  prof_begin(stream);
  if (cudaMemsetAsync(wk, 0, Lo.off_wtab, stream) != cudaSuccess) return PSMMA_EDEVICE;
  {
    const int kchunk = 1024;
    dim3 g1((M + 127) / 128, (K + kchunk - 1) / kchunk);
    k_row_absmax<<<g1, 128, 0, stream>>>(A, lda, M, K, kchunk, b.amax, b.asq);
  }
  prof_mark(stream, "row_scale");
  switch (gs.kind) {
    case KIND_CAUCHY: k_h_pass1<KIND_CAUCHY><<<N, 256, 0, stream>>>(gs, K, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_TOEPLITZ: k_h_pass1<KIND_TOEPLITZ><<<N, 256, 0, stream>>>(gs, K, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_HANKEL: k_h_pass1<KIND_HANKEL><<<N, 256, 0, stream>>>(gs, K, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_DENSE: k_h_pass1<KIND_DENSE><<<N, 256, 0, stream>>>(gs, K, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_CAUCHY_EIG: k_h_pass1<KIND_CAUCHY_EIG><<<N, 256, 0, stream>>>(gs, K, Lo.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    default: return PSMMA_EUNSUPPORTED;
  }
  prof_mark(stream, "h_generate");
  k_split_params<<<PARAMS_BLOCKS, 512, 0, stream>>>(b.prm, st.cc.log2M, M, N, K, b.amax, b.asq, b.hmax, b.hsq);
  prof_mark(stream, "params");
  s2_h_operands(st, b.Ht, b.hmax, b.prm, stream);
  prof_mark(stream, "residues_H");
  const int rc = s2_pass(st, A, lda, b.amax, b.prm, 0, M, stream);
  if (rc != PSMMA_OK) return rc;
  dim3 gc((N + CRT_TJ - 1) / CRT_TJ, (M + CRT_TI - 1) / CRT_TI);
  (st.cc.top32 ? k_crt_combine<false, true> : k_crt_combine<false, false>)<<<gc, dim3(32, 8), 0, stream>>>(
      b.R, M, N, Lo.kr, st.cc, b.amax, b.hmax, b.prm, alpha, beta, Q, ldq, 0);
  prof_mark(stream, "crt_combine");
  if (cudaGetLastError() != cudaSuccess) return PSMMA_EDEVICE;
  return split_status(b.prm, stream, status_dev_out);
}

// Host-pointer multiply with the copies overlapped (pinned host memory makes them
// asynchronous).  dA (M x K) and dQ (M x N) are device buffers with leading dimension M; Q is
// read from the host first when beta != 0.  Synchronises both streams.  The modular GEMM and
// the CRT run in row panels of whole 128-row tiles, and each finished panel of Q goes back to
// the host on the copy stream `cs` while the next panel multiplies.  Two ways to get A up:
//  - without guesses (or beta != 0): A goes up in column chunks while H is generated on `s`;
//    each chunk's row maxima / norms start as soon as it has landed, and the residue passes
//    wait for the parameter pass.  The H residues need PH, which the parameter pass sets from
//    A's statistics as well; with ph_guess (the PH a previous call of the same shape chose)
//    they are computed while A is still being uploaded and recomputed after the parameter
//    pass only if the guess was wrong.
//  - with pa_guess and ph_guess (beta == 0): A goes up in the GEMM's row panels of whole rows,
//    and each panel's row maxima, residues (scaled with the guessed PA), GEMM and CRT start as
//    soon as its rows have landed, so the upload hides behind the H passes and the products.
//    The parameter pass runs last; if its PA or PH differs from the guesses, the residues,
//    products and downloads are redone with the computed ones (A is resident by then), so
//    the result is always the one the computed parameters give.
// *pa_out / *ph_out receive the PA / PH of the call.
static int split_core_host(int M, int N, int K, double alpha, const double* A_h, long lda_h, double* dA,
                           const GenSpec& gs, double beta, double* Q_h, long ldq_h, double* dQ, int nmod, void* work,
                           size_t lwork, cudaStream_t s, cudaStream_t cs, cudaEvent_t* ev, int nev, int pa_guess,
                           int ph_guess, int* pa_out, int* ph_out) {
  if (gs.kind == KIND_DFT) return PSMMA_EUNSUPPORTED;
  if (nmod < 8 || nmod > SPL_MAX_MODULI) return PSMMA_EUNSUPPORTED;
  if (K >= (1 << 24) || M > kSplitMaxRows || N >= (1 << 30)) return PSMMA_EUNSUPPORTED;
  // A column chunks; GEMM / CRT / download row panels: eighths of the row tiles, the first
  // one cut to two row tiles (its pitched upload runs beside the H passes' HBM traffic and
  // gates the first product) and the last one halved three times (8 + 4 + 2 + 2 of 16 tiles:
  // the download left after the last product is short)
  constexpr int NCH = 4, NP = 12;
  if (nev < 2 * NP + 3) return PSMMA_EUNSUPPORTED;
  static_assert(NCH <= NP, "column chunks and row panels share the upload events");
  SplitLayout L = split_layout(M, K, N, nmod);
  if (lwork < L.total || !work) return PSMMA_EWORKSPACE;
  char* w = (char*)work;
  const SplitBuffers b = split_buffers(w, L);
  const CrtConsts cc = get_consts(nmod);
  const bool spec = pa_guess >= 8 && ph_guess >= 8 && beta == 0.0;
  cudaEvent_t* ev_up = ev;               // NP: column chunks or row panels of A landed
  cudaEvent_t* ev_panel = ev + NP;       // NP: panels of Q ready
  cudaEvent_t ev_start = ev[2 * NP], ev_q = ev[2 * NP + 1], ev_done = ev[2 * NP + 2];
  bool ok = true;
  // the copy stream starts after everything already queued on s
  ok &= cudaEventRecord(ev_start, s) == cudaSuccess;
  ok &= cudaStreamWaitEvent(cs, ev_start, 0) == cudaSuccess;
  prof_begin(s);
  ok &= cudaMemsetAsync(w, 0, L.off_wtab, s) == cudaSuccess;
  if (spec) k_guess_params<<<1, 1, 0, s>>>(b.prm_guess, pa_guess, ph_guess);
  // ---- H side (needs no A)
  switch (gs.kind) {
    case KIND_CAUCHY: k_h_pass1<KIND_CAUCHY><<<N, 256, 0, s>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_TOEPLITZ: k_h_pass1<KIND_TOEPLITZ><<<N, 256, 0, s>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_HANKEL: k_h_pass1<KIND_HANKEL><<<N, 256, 0, s>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    case KIND_CAUCHY_EIG: k_h_pass1<KIND_CAUCHY_EIG><<<N, 256, 0, s>>>(gs, K, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm); break;
    default: return PSMMA_EUNSUPPORTED;
  }
  const dim3 grh(N, rh_blocks_x(L.kp));
  if (ph_guess >= 8)
    k_residues_H_spec<<<grh, 128, 0, s>>>(b.Ht, N, L.kp, b.hmax, b.prm, cc, b.RH, ph_guess, 0);
  prof_mark(s, "h_side");

  OneGemm og;
  memset(&og, 0, sizeof(og));
  if (!make_tmap(&og.ta, b.RA, L.kp, M, nmod, G_BM) || !make_tmap(&og.tb, b.RH, L.kp, N, nmod, G_BN))
    return PSMMA_EDEVICE;
  GemmArgs& ga = og.g;
  ga.n = M;
  ga.kr = L.kr;
  ga.nkb = L.kp / G_BK;
  ga.tiles_n = (N + G_BN - 1) / G_BN;
  ga.group_m = 16;
  ga.R = b.R;
  ga.status = &b.prm->status;
  ga.nmod = nmod;
  for (int l = 0; l < nmod; ++l) { ga.m[l] = cc.m[l]; ga.inv_m[l] = cc.inv_m[l]; }
  using Shape = GemmShape<G_BN>;
  if (set_smem_attr(k_crt_gemm<G_BN, OneGemm>, (int)Shape::SMEM) != cudaSuccess)
    return PSMMA_EDEVICE;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PSMMA_EDEVICE;
  const int tiles_m = (M + G_BM - 1) / G_BM;
  int pb[NP + 1], npanels = 0;  // panel p: row tiles [pb[p], pb[p + 1])
  {
    const int tp = (tiles_m + 7) / 8;
    pb[0] = 0;
    if (tp >= 4 && tiles_m > tp) {
      pb[1] = 2;
      pb[2] = tp;
      npanels = 2;
    }
    while (tiles_m - pb[npanels] > tp) { pb[npanels + 1] = pb[npanels] + tp; ++npanels; }
    for (int rest = tiles_m - pb[npanels], cut = 0; rest > 0; ++cut) {
      const int t = cut < 3 ? (rest + 1) / 2 : rest;
      pb[npanels + 1] = pb[npanels] + t;
      ++npanels;
      rest -= t;
    }
  }
  static_assert(G_BM % CRT_TI == 0 && G_BM % 64 == 0, "row panels must cover whole CRT and residue blocks");
  const int kchunk = 1024;
  // GEMM + CRT of panel p (rows [r0, r1)) with the bit counts in *pk, then its download
  auto panel = [&](int p, const SplitDevParams* pk) {
    const int t0 = pb[p], t1 = pb[p + 1];
    ga.tm0 = t0;
    ga.tiles_m = t1 - t0;
    const int total_tiles = ga.tiles_m * ga.tiles_n * nmod;
    k_crt_gemm<G_BN, OneGemm><<<std::min(sms, total_tiles), G_THREADS, Shape::SMEM, s>>>(og);
    const int r0 = t0 * G_BM, r1 = std::min(M, t1 * G_BM);
    dim3 gc((N + CRT_TJ - 1) / CRT_TJ, (r1 - r0 + CRT_TI - 1) / CRT_TI);
    (cc.top32 ? k_crt_combine<false, true> : k_crt_combine<false, false>)<<<gc, dim3(32, 8), 0, s>>>(
        b.R, M, N, L.kr, cc, b.amax, b.hmax, pk, alpha, beta, dQ, M, r0 / CRT_TI);
    prof_mark(s, "panel_gemm_crt");
    ok &= cudaEventRecord(ev_panel[p], s) == cudaSuccess;
    ok &= cudaStreamWaitEvent(cs, ev_panel[p], 0) == cudaSuccess;
    ok &= cudaMemcpy2DAsync(Q_h + r0, (size_t)ldq_h * 8, dQ + r0, (size_t)M * 8, (size_t)(r1 - r0) * 8, (size_t)N,
                            cudaMemcpyDeviceToHost, cs) == cudaSuccess;
    prof_mark(cs, "q_panel_down");
  };
  // the parameters, then the caller's view of them once both streams are done
  // status, PA, PH: read back into pinned memory (a pageable destination would take the
  // driver's staged path behind the stream's other copies); host calls are serialised
  static SplitDevParams* head_pinned = nullptr;
  if (!head_pinned && cudaHostAlloc((void**)&head_pinned, sizeof(SplitDevParams), cudaHostAllocPortable) != cudaSuccess) {
    head_pinned = nullptr;
    return PSMMA_ENOMEM;
  }
  SplitDevParams& head = *head_pinned;
  auto finish = [&]() {
    if (cudaGetLastError() != cudaSuccess) ok = false;
    ok &= cudaMemcpyAsync(head_pinned, b.prm, offsetof(SplitDevParams, rho_bits), cudaMemcpyDeviceToHost, s) ==
          cudaSuccess;
    prof_mark(s, "params_head");
    prof_mark(cs, "q_download_tail");  // on the copy stream: the end of the last download
    ok &= cudaEventRecord(ev_done, cs) == cudaSuccess;
    ok &= cudaStreamSynchronize(s) == cudaSuccess;
    ok &= cudaEventSynchronize(ev_done) == cudaSuccess;
  };

  if (spec) {
    // ---- A in row panels: each panel is multiplied as soon as its rows have landed (all
    // uploads are queued on the copy stream ahead of the downloads)
    for (int p = 0; p < npanels; ++p) {
      const int r0 = pb[p] * G_BM, r1 = std::min(M, pb[p + 1] * G_BM);
      ok &= cudaMemcpy2DAsync(dA + r0, (size_t)M * 8, A_h + r0, (size_t)lda_h * 8, (size_t)(r1 - r0) * 8,
                              (size_t)K, cudaMemcpyHostToDevice, cs) == cudaSuccess;
      ok &= cudaEventRecord(ev_up[p], cs) == cudaSuccess;
      prof_mark(cs, "a_panel_up");
    }
    for (int p = 0; p < npanels; ++p) {
      const int r0 = pb[p] * G_BM, r1 = std::min(M, pb[p + 1] * G_BM);
      ok &= cudaStreamWaitEvent(s, ev_up[p], 0) == cudaSuccess;
      // a panel has few rows: shorter K chunks keep enough blocks in flight
      const int kc = 256;
      dim3 g1((r1 - r0 + 127) / 128, (K + kc - 1) / kc);
      k_row_absmax<<<g1, 128, 0, s>>>(dA + r0, M, r1 - r0, K, kc, b.amax + r0, b.asq + r0);
      k_residues_A_rows<<<dim3(L.kp / 64, (r1 - r0 + 63) / 64), 256, 0, s>>>(dA, M, M, K, L.kp, b.amax,
                                                                             b.prm_guess, cc, b.RA, r0 / 64);
      prof_mark(s, "panel_rows");
      panel(p, b.prm_guess);
    }
    k_split_params<<<PARAMS_BLOCKS, 512, 0, s>>>(b.prm, cc.log2M, M, N, K, b.amax, b.asq, b.hmax, b.hsq);
    finish();
    if (!ok) return PSMMA_EDEVICE;
    if (head.status & DEV_ERR_TIMEOUT) return PSMMA_ETIMEDOUT;
    if (pa_out) *pa_out = head.PA;
    if (ph_out) *ph_out = head.PH;
    if (head.PA == pa_guess && head.PH == ph_guess) return PSMMA_OK;
    // a wrong guess: everything after the parameter pass again, with the computed bit counts
    prof_mark(s, "redo_wrong_guess");
    k_residues_A<<<dim3(L.kp / 64, (M + 63) / 64), 256, 0, s>>>(dA, M, M, K, L.kp, b.amax, b.prm, cc, b.RA);
    k_residues_H<<<grh, 128, 0, s>>>(b.Ht, N, L.kp, b.hmax, b.prm, cc, b.RH);
    ok &= cudaEventRecord(ev_start, s) == cudaSuccess;
    ok &= cudaStreamWaitEvent(cs, ev_start, 0) == cudaSuccess;
    for (int p = 0; p < npanels; ++p) panel(p, b.prm);
    finish();
    if (!ok) return PSMMA_EDEVICE;
    return (head.status & DEV_ERR_TIMEOUT) ? PSMMA_ETIMEDOUT : PSMMA_OK;
  }

  // ---- A in column chunks (multiples of the 1024-column row-norm chunk)
  const int cols_per = std::max(kchunk, (K + NCH * kchunk - 1) / (NCH * kchunk) * kchunk);
  for (int ch = 0; ch < NCH; ++ch) {
    const int c0 = ch * cols_per, c1 = std::min(K, c0 + cols_per);
    if (c0 >= c1) break;
    ok &= cudaMemcpy2DAsync(dA + (size_t)c0 * M, (size_t)M * 8, A_h + (size_t)c0 * lda_h, (size_t)lda_h * 8,
                            (size_t)M * 8, (size_t)(c1 - c0), cudaMemcpyHostToDevice, cs) == cudaSuccess;
    ok &= cudaEventRecord(ev_up[ch], cs) == cudaSuccess;
    prof_mark(cs, "a_chunk_up");
    ok &= cudaStreamWaitEvent(s, ev_up[ch], 0) == cudaSuccess;
    dim3 g1((M + 127) / 128, (c1 - c0 + kchunk - 1) / kchunk);
    k_row_absmax<<<g1, 128, 0, s>>>(dA + (size_t)c0 * M, M, M, c1 - c0, kchunk, b.amax, b.asq);
  }
  if (beta != 0.0) {
    ok &= cudaMemcpy2DAsync(dQ, (size_t)M * 8, Q_h, (size_t)ldq_h * 8, (size_t)M * 8, (size_t)N,
                            cudaMemcpyHostToDevice, cs) == cudaSuccess;
    ok &= cudaEventRecord(ev_q, cs) == cudaSuccess;
  }
  if (!ok) return PSMMA_EDEVICE;
  prof_mark(s, "a_upload_rows");
  k_split_params<<<PARAMS_BLOCKS, 512, 0, s>>>(b.prm, cc.log2M, M, N, K, b.amax, b.asq, b.hmax, b.hsq);
  k_residues_A<<<dim3(L.kp / 64, (M + 63) / 64), 256, 0, s>>>(dA, M, M, K, L.kp, b.amax, b.prm, cc, b.RA);
  if (ph_guess >= 8)
    k_residues_H_spec<<<grh, 128, 0, s>>>(b.Ht, N, L.kp, b.hmax, b.prm, cc, b.RH, ph_guess, 1);
  else
    k_residues_H<<<grh, 128, 0, s>>>(b.Ht, N, L.kp, b.hmax, b.prm, cc, b.RH);
  prof_mark(s, "params_residues");
  if (beta != 0.0 && cudaStreamWaitEvent(s, ev_q, 0) != cudaSuccess) return PSMMA_EDEVICE;
  for (int p = 0; p < npanels; ++p) panel(p, b.prm);
  finish();
  if (!ok) return PSMMA_EDEVICE;
  if (pa_out) *pa_out = head.PA;
  if (ph_out) *ph_out = head.PH;
  if (head.status & DEV_ERR_TIMEOUT) return PSMMA_ETIMEDOUT;
  return PSMMA_OK;
}

// The host-pointer pipeline of split_core_host with the Toeplitz / Hankel block step: the same
// uploads, row panels, speculative bit counts and downloads; per panel the A block residues,
// the leaf products and the recombination.  The H side (generation, group maxima, the leaves'
// H operands) runs once, before the panels.
static int split_core_host_block(int M, int N, int Np, int L, double alpha, const double* A_h, long lda_h,
                                 double* dA, const GenSpec& gs, double beta, double* Q_h, long ldq_h, double* dQ,
                                 int nmod, void* work, size_t lwork, cudaStream_t s, cudaStream_t cs,
                                 cudaEvent_t* ev, int nev, int pa_guess, int ph_guess, int* pa_out, int* ph_out) {
  constexpr int NCH = 4, NP = 12;
  if (nev < 2 * NP + 3) return PSMMA_EUNSUPPORTED;
  BlockRun br;
  const int st0 = br.init(M, N, Np, L, gs, nmod, work, lwork);
  if (st0 != PSMMA_OK) return st0;
  const SplitBuffers& b = br.b;
  const bool spec = pa_guess >= 8 && ph_guess >= 8 && beta == 0.0;
  cudaEvent_t* ev_up = ev;
  cudaEvent_t* ev_panel = ev + NP;
  cudaEvent_t ev_start = ev[2 * NP], ev_q = ev[2 * NP + 1], ev_done = ev[2 * NP + 2];
  bool ok = true;
  ok &= cudaEventRecord(ev_start, s) == cudaSuccess;
  ok &= cudaStreamWaitEvent(cs, ev_start, 0) == cudaSuccess;
  prof_begin(s);
  ok &= cudaMemsetAsync(work, 0, br.Lo.off_wtab, s) == cudaSuccess;
  if (spec) k_guess_params<<<1, 1, 0, s>>>(b.prm_guess, pa_guess, ph_guess);
  br.h_side(spec ? b.prm_guess : nullptr, s);
  if (spec) br.h_operands(b.prm_guess, s);
  prof_mark(s, "h_side");
  // row panels of whole 128-row tiles, as split_core_host cuts them
  const int tiles_m = (M + G_BM - 1) / G_BM;
  int pb[NP + 1], npanels = 0;
  {
    const int tp = (tiles_m + 7) / 8;
    pb[0] = 0;
    if (tp >= 4 && tiles_m > tp) {
      pb[1] = 2;
      pb[2] = tp;
      npanels = 2;
    }
    while (tiles_m - pb[npanels] > tp) { pb[npanels + 1] = pb[npanels] + tp; ++npanels; }
    for (int rest = tiles_m - pb[npanels], cut = 0; rest > 0; ++cut) {
      const int t = cut < 3 ? (rest + 1) / 2 : rest;
      pb[npanels + 1] = pb[npanels] + t;
      ++npanels;
      rest -= t;
    }
  }
  auto panel = [&](int p, const SplitDevParams* pk) {
    const int r0 = pb[p] * G_BM, r1 = std::min(M, pb[p + 1] * G_BM);
    ok &= br.products(r0, r1 - r0, pk, s) == PSMMA_OK;
    br.crt(r0, r1 - r0, alpha, beta, dQ, M, pk, s);
    prof_mark(s, "panel_gemm_crt");
    ok &= cudaEventRecord(ev_panel[p], s) == cudaSuccess;
    ok &= cudaStreamWaitEvent(cs, ev_panel[p], 0) == cudaSuccess;
    ok &= cudaMemcpy2DAsync(Q_h + r0, (size_t)ldq_h * 8, dQ + r0, (size_t)M * 8, (size_t)(r1 - r0) * 8, (size_t)N,
                            cudaMemcpyDeviceToHost, cs) == cudaSuccess;
    prof_mark(cs, "q_panel_down");
  };
  static SplitDevParams* head_pinned = nullptr;  // host calls are serialised
  if (!head_pinned && cudaHostAlloc((void**)&head_pinned, sizeof(SplitDevParams), cudaHostAllocPortable) != cudaSuccess) {
    head_pinned = nullptr;
    return PSMMA_ENOMEM;
  }
  SplitDevParams& head = *head_pinned;
  auto finish = [&]() {
    if (cudaGetLastError() != cudaSuccess) ok = false;
    ok &= cudaMemcpyAsync(head_pinned, b.prm, offsetof(SplitDevParams, rho_bits), cudaMemcpyDeviceToHost, s) ==
          cudaSuccess;
    prof_mark(s, "params_head");
    prof_mark(cs, "q_download_tail");
    ok &= cudaEventRecord(ev_done, cs) == cudaSuccess;
    ok &= cudaStreamSynchronize(s) == cudaSuccess;
    ok &= cudaEventSynchronize(ev_done) == cudaSuccess;
  };
  if (spec) {
    for (int p = 0; p < npanels; ++p) {
      const int r0 = pb[p] * G_BM, r1 = std::min(M, pb[p + 1] * G_BM);
      ok &= cudaMemcpy2DAsync(dA + r0, (size_t)M * 8, A_h + r0, (size_t)lda_h * 8, (size_t)(r1 - r0) * 8,
                              (size_t)N, cudaMemcpyHostToDevice, cs) == cudaSuccess;
      ok &= cudaEventRecord(ev_up[p], cs) == cudaSuccess;
      prof_mark(cs, "a_panel_up");
    }
    for (int p = 0; p < npanels; ++p) {
      const int r0 = pb[p] * G_BM, r1 = std::min(M, pb[p + 1] * G_BM);
      ok &= cudaStreamWaitEvent(s, ev_up[p], 0) == cudaSuccess;
      const int kc = 256;
      dim3 g1((r1 - r0 + 127) / 128, (N + kc - 1) / kc);
      k_row_absmax<<<g1, 128, 0, s>>>(dA + r0, M, r1 - r0, N, kc, b.amax + r0, b.asq + r0);
      br.a_residues(dA, M, r0, r1 - r0, b.prm_guess, s);
      prof_mark(s, "panel_rows");
      panel(p, b.prm_guess);
    }
    k_split_params<<<PARAMS_BLOCKS, 512, 0, s>>>(b.prm, br.cc.log2M, M, Np, Np, b.amax, b.asq, b.hmax, b.hsq);
    finish();
    if (!ok) return PSMMA_EDEVICE;
    if (head.status & DEV_ERR_TIMEOUT) return PSMMA_ETIMEDOUT;
    if (pa_out) *pa_out = head.PA;
    if (ph_out) *ph_out = head.PH;
    if (head.PA == pa_guess && head.PH == ph_guess) return PSMMA_OK;
    // a wrong guess: the operands and products again with the computed bit counts
    prof_mark(s, "redo_wrong_guess");
    br.a_residues(dA, M, 0, M, b.prm, s);
    br.h_operands(b.prm, s);
    ok &= cudaEventRecord(ev_start, s) == cudaSuccess;
    ok &= cudaStreamWaitEvent(cs, ev_start, 0) == cudaSuccess;
    for (int p = 0; p < npanels; ++p) panel(p, b.prm);
    finish();
    if (!ok) return PSMMA_EDEVICE;
    return (head.status & DEV_ERR_TIMEOUT) ? PSMMA_ETIMEDOUT : PSMMA_OK;
  }
  // A in column chunks, its row statistics as each lands
  const int kchunk = 1024;
  const int cols_per = std::max(kchunk, (N + NCH * kchunk - 1) / (NCH * kchunk) * kchunk);
  for (int ch = 0; ch < NCH; ++ch) {
    const int c0 = ch * cols_per, c1 = std::min(N, c0 + cols_per);
    if (c0 >= c1) break;
    ok &= cudaMemcpy2DAsync(dA + (size_t)c0 * M, (size_t)M * 8, A_h + (size_t)c0 * lda_h, (size_t)lda_h * 8,
                            (size_t)M * 8, (size_t)(c1 - c0), cudaMemcpyHostToDevice, cs) == cudaSuccess;
    ok &= cudaEventRecord(ev_up[ch], cs) == cudaSuccess;
    prof_mark(cs, "a_chunk_up");
    ok &= cudaStreamWaitEvent(s, ev_up[ch], 0) == cudaSuccess;
    dim3 g1((M + 127) / 128, (c1 - c0 + kchunk - 1) / kchunk);
    k_row_absmax<<<g1, 128, 0, s>>>(dA + (size_t)c0 * M, M, M, c1 - c0, kchunk, b.amax, b.asq);
  }
  if (beta != 0.0) {
    ok &= cudaMemcpy2DAsync(dQ, (size_t)M * 8, Q_h, (size_t)ldq_h * 8, (size_t)M * 8, (size_t)N,
                            cudaMemcpyHostToDevice, cs) == cudaSuccess;
    ok &= cudaEventRecord(ev_q, cs) == cudaSuccess;
  }
  if (!ok) return PSMMA_EDEVICE;
  prof_mark(s, "a_upload_rows");
  k_split_params<<<PARAMS_BLOCKS, 512, 0, s>>>(b.prm, br.cc.log2M, M, Np, Np, b.amax, b.asq, b.hmax, b.hsq);
  br.a_residues(dA, M, 0, M, b.prm, s);
  br.h_operands(b.prm, s);
  prof_mark(s, "params_residues");
  if (beta != 0.0 && cudaStreamWaitEvent(s, ev_q, 0) != cudaSuccess) return PSMMA_EDEVICE;
  for (int p = 0; p < npanels; ++p) panel(p, b.prm);
  finish();
  if (!ok) return PSMMA_EDEVICE;
  if (pa_out) *pa_out = head.PA;
  if (ph_out) *ph_out = head.PH;
  if (head.status & DEV_ERR_TIMEOUT) return PSMMA_ETIMEDOUT;
  return PSMMA_OK;
}

struct PhKey {
  int M, N, K, kind, nmod;
  bool operator<(const PhKey& o) const {
    return std::tie(M, N, K, kind, nmod) < std::tie(o.M, o.N, o.K, o.kind, o.nmod);
  }
};
static std::mutex g_ph_mu;
static std::map<PhKey, std::pair<int, int>> g_ph;  // (PA, PH) of the last call of the shape

static int split_core_host_cached(int M, int N, int K, double alpha, const double* A_h, long lda_h, double* dA,
                                  const GenSpec& gs, double beta, double* Q_h, long ldq_h, double* dQ, int nmod,
                                  void* work, size_t lwork, cudaStream_t s, cudaStream_t cs, cudaEvent_t* ev,
                                  int nev, int block_req = -1) {
  const BlockChoice bc = gs.k1 == 0 ? block_choice(gs.kind, N, K, block_req) : BlockChoice{0, N};
  const PhKey key{M, bc.L > 0 ? bc.Np : N, K, gs.kind * 4 + bc.L, nmod};
  int pa_guess = -1, ph_guess = -1;
  {
    std::lock_guard<std::mutex> lk(g_ph_mu);
    auto it = g_ph.find(key);
    if (it != g_ph.end()) std::tie(pa_guess, ph_guess) = it->second;
  }
  int pa = -1, ph = -1;
  const int st = bc.L > 0 ? split_core_host_block(M, N, bc.Np, bc.L, alpha, A_h, lda_h, dA, gs, beta, Q_h, ldq_h,
                                                  dQ, nmod, work, lwork, s, cs, ev, nev, pa_guess, ph_guess, &pa,
                                                  &ph)
                          : split_core_host(M, N, K, alpha, A_h, lda_h, dA, gs, beta, Q_h, ldq_h, dQ, nmod, work,
                                            lwork, s, cs, ev, nev, pa_guess, ph_guess, &pa, &ph);
  if (!st && pa >= 8 && ph >= 8) {
    std::lock_guard<std::mutex> lk(g_ph_mu);
    if (g_ph.size() > 256) g_ph.clear();
    g_ph[key] = {pa, ph};
  }
  return st;
}

int launch_split_host(int kind, int n, int k, double alpha, const double* A_h, long lda_h, double* dA,
                      const double* dgen, long ldgen, double beta, double* Q_h, long ldq_h, double* dQ,
                      int n_moduli, void* work, size_t lwork, cudaStream_t s, cudaStream_t cs, cudaEvent_t* ev,
                      int nev, int block_levels) {
  const GenSpec gs = reference_gens(kind, dgen, ldgen, k);
  return split_core_host_cached(n, k, k, alpha, A_h, lda_h, dA, gs, beta, Q_h, ldq_h, dQ, resolve_nmod(n_moduli),
                                work, lwork, s, cs, ev, nev, block_levels);
}

int launch_split_host_general(int M, int N, int K, double alpha, const double* A_h, long lda_h, double* dA,
                              const GenSpec& gs, double beta, double* Q_h, long ldq_h, double* dQ, int n_moduli,
                              void* work, size_t lwork, cudaStream_t s, cudaStream_t cs, cudaEvent_t* ev, int nev) {
  return split_core_host_cached(M, N, K, alpha, A_h, lda_h, dA, gs, beta, Q_h, ldq_h, dQ, resolve_nmod(n_moduli),
                                work, lwork, s, cs, ev, nev);
}

// kind != DFT: Q (n x k) = alpha * A (n x k) * H (k x k) + beta * Q.
// C (n x k complex, ldc) = alpha * F * B + beta * C on the split path, F(j, l) = w^(j l): the
// rows of the product are the k columns of B (M = k), three real products per modulus (3M).
// src != nullptr: B is src->Bp, deinterleaved from src->B here (with the row statistics).
static int dft3_enqueue(int M, int nn, double alpha, const double* B, long ldb, double beta, double* C, long ldc,
                        int nmod, void* work, size_t lwork, cudaStream_t stream, SplitDevParams** prm_out,
                        const DftRadixSrc* src = nullptr) {
  if (nmod < 8 || nmod > SPL_MAX_MODULI) return PSMMA_EUNSUPPORTED;
  if (2 * nn >= (1 << 24) || M > kSplitMaxRows) return PSMMA_EUNSUPPORTED;
  const SplitLayout L = dft3_layout(M, nn, nmod);
  if (lwork < L.total || !work) return PSMMA_EWORKSPACE;
  char* w = (char*)work;
  const SplitBuffers b = split_buffers(w, L);
  const CrtConsts cc = get_consts(nmod);

  prof_begin(stream);
  if (cudaMemsetAsync(w, 0, L.off_wtab, stream) != cudaSuccess) return PSMMA_EDEVICE;  // params, maxima, sums
  if (src) {
    const int gx = src->k < 8192 ? src->k : 8192;
    if (src->R == 8)
      k_dft_deinterleave_stats<8><<<gx, 256, 0, stream>>>(src->B, src->ldb, src->n, src->k, src->Bp, b.amax, b.asq);
    else if (src->R == 4)
      k_dft_deinterleave_stats<4><<<gx, 256, 0, stream>>>(src->B, src->ldb, src->n, src->k, src->Bp, b.amax, b.asq);
    else if (src->R == 2)
      k_dft_deinterleave_stats<2><<<gx, 256, 0, stream>>>(src->B, src->ldb, src->n, src->k, src->Bp, b.amax, b.asq);
    else
      return PSMMA_EUNSUPPORTED;
    prof_mark(stream, "deinterleave_row_scale");
  } else {
    k_row_absmax_dft<<<M, 256, 0, stream>>>(B, 2 * ldb, nn, b.amax, b.asq);
    prof_mark(stream, "row_scale");
  }
  int st = launch_dft_table(b.wtab, nn, stream);
  if (st) return st;
  k_h_pass1_dft3<<<nn, 256, 0, stream>>>(b.wtab, nn, L.kp, b.Ht, b.hmax, b.hsum, b.hsq, b.prm);
  prof_mark(stream, "h_generate");
  // the bounds are those of the real embedding: n columns, inner dimension 2n
  k_split_params<<<PARAMS_BLOCKS, 512, 0, stream>>>(b.prm, cc.log2M, M, nn, 2 * nn, b.amax, b.asq, b.hmax, b.hsq);
  prof_mark(stream, "params");
  k_residues_A_dft3<<<dim3(M, (L.kp / 2 + 127) / 128), 128, 0, stream>>>(B, 2 * ldb, nn, L.kp, b.amax, b.prm, cc,
                                                                         b.RA, M);
  prof_mark(stream, "residues_A");
  k_residues_H_dft3<<<dim3(nn, rh_blocks_x(L.kp)), 128, 0, stream>>>(b.Ht, nn, L.kp, b.hmax, b.prm, cc, b.RH);
  prof_mark(stream, "residues_H");

  using Shape = GemmShape<G_BN>;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PSMMA_EDEVICE;
  const int kr1 = L.kr / 2;
  if (L.kp / G_BK <= G_CHUNK_KB) {
    // one chunk per product: the three products in one launch, Re and Im written once
    if (set_smem_attr(k_crt_gemm<G_BN, Gemm3M>, (int)Shape::SMEM) != cudaSuccess) return PSMMA_EDEVICE;
    Gemm3M g3;
    memset(&g3, 0, sizeof(g3));
    for (int p = 0; p < 3; ++p)
      if (!make_tmap(&g3.ta[p], b.RA + (size_t)p * nmod * M * L.kp, L.kp, M, nmod, G_BM) ||
          !make_tmap(&g3.tb[p], b.RH + (size_t)p * nmod * nn * L.kp, L.kp, nn, nmod, G_BN))
        return PSMMA_EDEVICE;
    GemmArgs& ga = g3.g;
    ga.n = M;
    ga.kr = L.kr;
    ga.nkb = L.kp / G_BK;
    ga.tiles_m = (M + G_BM - 1) / G_BM;
    ga.tiles_n = (nn + G_BN - 1) / G_BN;
    ga.group_m = 16;
    ga.R = b.R;
    ga.status = &b.prm->status;
    ga.nmod = nmod;
    ga.im_off = kr1;
    for (int l = 0; l < nmod; ++l) { ga.m[l] = cc.m[l]; ga.inv_m[l] = cc.inv_m[l]; }
    const int total_tiles = ga.tiles_m * ga.tiles_n * nmod;
    k_crt_gemm<G_BN, Gemm3M><<<std::min(sms, total_tiles), (Gemm3M::kEpiWarps + 2) * 32, Shape::SMEM, stream>>>(g3);
    prof_mark(stream, "gemm_3m");
  }
  if (L.kp / G_BK > G_CHUNK_KB && set_smem_attr(k_crt_gemm<G_BN, OneGemm>, (int)Shape::SMEM) != cudaSuccess)
    return PSMMA_EDEVICE;
  // T1 into the Re half; T2: Re = T1 - T2, Im = -T1 - T2; T3: Im += T3
  for (int p = 0; p < 3 && L.kp / G_BK > G_CHUNK_KB; ++p) {
    OneGemm og;
    memset(&og, 0, sizeof(og));
    __nv_bfloat16* ra = b.RA + (size_t)p * nmod * M * L.kp;
    __nv_bfloat16* rh = b.RH + (size_t)p * nmod * nn * L.kp;
    if (!make_tmap(&og.ta, ra, L.kp, M, nmod, G_BM) || !make_tmap(&og.tb, rh, L.kp, nn, nmod, G_BN))
      return PSMMA_EDEVICE;
    GemmArgs& ga = og.g;
    ga.n = M;
    ga.kr = L.kr;
    ga.nkb = L.kp / G_BK;
    ga.tiles_m = (M + G_BM - 1) / G_BM;
    ga.tiles_n = (nn + G_BN - 1) / G_BN;
    ga.group_m = 16;
    ga.R = b.R + (p == 2 ? kr1 : 0);
    ga.status = &b.prm->status;
    ga.nmod = nmod;
    ga.mode = p;
    ga.im_off = kr1;
    for (int l = 0; l < nmod; ++l) { ga.m[l] = cc.m[l]; ga.inv_m[l] = cc.inv_m[l]; }
    const int total_tiles = ga.tiles_m * ga.tiles_n * nmod;
    k_crt_gemm<G_BN, OneGemm><<<std::min(sms, total_tiles), G_THREADS, Shape::SMEM, stream>>>(og);
    prof_mark(stream, p == 0 ? "gemm_T1" : p == 1 ? "gemm_T2_combine" : "gemm_T3_combine");
  }
  if (src) {
    const int cpb = 32 / src->R;
    const int by = (src->k + cpb - 1) / cpb;
    const dim3 gr((nn + RDX_TJ - 1) / RDX_TJ, by < 65535 ? by : 65535);
#define PSMMA_CRT_RADIX(RR, T32)                                                                             \
  k_crt_dft_radix<RR, T32><<<gr, dim3(32, 8), 0, stream>>>(b.R, M, nn, L.kr, cc, b.amax, b.hmax, b.prm, alpha, \
                                                          src->wn, src->beta, src->C, src->ldc, src->k)
    if (src->R == 8) {
      if (cc.top32) PSMMA_CRT_RADIX(8, true); else PSMMA_CRT_RADIX(8, false);
    } else if (src->R == 4) {
      if (cc.top32) PSMMA_CRT_RADIX(4, true); else PSMMA_CRT_RADIX(4, false);
    } else {
      if (cc.top32) PSMMA_CRT_RADIX(2, true); else PSMMA_CRT_RADIX(2, false);
    }
#undef PSMMA_CRT_RADIX
    prof_mark(stream, "crt_radix_combine");
  } else {
    dim3 gc(L.kr / CRT_TJ, (M + CRT_TI - 1) / CRT_TI);
    (cc.top32 ? k_crt_combine<true, true> : k_crt_combine<true, false>)<<<gc, dim3(32, 8), 0, stream>>>(
        b.R, M, nn, L.kr, cc, b.amax, b.hmax, b.prm, alpha, beta, C, 2 * ldc, 0);
    prof_mark(stream, "crt_combine");
  }
  if (cudaGetLastError() != cudaSuccess) return PSMMA_EDEVICE;
  *prm_out = b.prm;
  return PSMMA_OK;
}

// C (n x k complex, ldc) = alpha * F_n * B + beta * C: with R = dft_radix(n) > 1 the modular
// products run on F_(n/R) and the R k columns of B' (k_dft_deinterleave), their result P =
// alpha F_(n/R) B' goes to the workspace, and k_dft_radix_combine applies the twiddles, the
// R-point butterflies and beta; R = 1 is the plain 3M product.
static int split_core_dft3(int k, int n, double alpha, const double* B, long ldb, double beta, double* C,
                           long ldc, int nmod, void* work, size_t lwork, cudaStream_t stream,
                           unsigned* status_dev_out) {
  const int R = dft_radix(n);
  SplitDevParams* prm = nullptr;
  int st;
  if (R == 1) {
    st = dft3_enqueue(k, n, alpha, B, ldb, beta, C, ldc, nmod, work, lwork, stream, &prm);
  } else {
    if ((long)k * R > kSplitMaxRows) return PSMMA_EUNSUPPORTED;
    const DftRadixLayout D = dft_radix_layout(n, k, R, nmod);
    if (!work || lwork < D.total) return PSMMA_EWORKSPACE;
    char* w = (char*)work;
    double2* Bp = (double2*)(w + D.off_bp);
    double2* wn = (double2*)(w + D.off_w);
    const int nq = n / R;
    st = launch_dft_table(wn, n, stream);
    if (st) return st;
    const DftRadixSrc src{(const double2*)B, ldb, n, k, R, Bp, wn, beta, (double2*)C, ldc};
    st = dft3_enqueue(R * k, nq, alpha, (const double*)Bp, nq, 0.0, nullptr, 0, nmod, work, D.core, stream, &prm,
                      &src);
    if (st) return st;
  }
  if (st) return st;
  return split_status(prm, stream, status_dev_out);
}

// kind == DFT: C (n x k complex, ldq) = alpha * F (n x n) * B (n x k complex, lda) + beta * C,
//   computed as C^T = B^T F in the 3M form (split_core_dft3).
int launch_split_any(int kind, int n, int k, double alpha, const double* A, long lda, const double* gen,
                     long ldgen, double beta, double* Q, long ldq, int n_moduli, void* work, size_t lwork,
                     cudaStream_t stream, unsigned* status_dev_out, int block_req) {
  const int nmod = resolve_nmod(n_moduli);
  if (kind == KIND_DFT) return split_core_dft3(k, n, alpha, A, lda, beta, Q, ldq, nmod, work, lwork, stream, status_dev_out);
  const GenSpec gs = reference_gens(kind, gen, ldgen, k);
  const BlockChoice bc = block_choice(kind, k, k, block_req);
  if (bc.L > 0 && gs.k1 == 0)
    return split_core_block(n, k, bc.Np, bc.L, alpha, A, lda, gs, beta, Q, ldq, nmod, work, lwork, stream,
                            status_dev_out);
  if (s2_use(kind, n, k, k, block_req) && gs.k1 == 0)
    return split_core_s2(n, k, k, alpha, A, lda, gs, beta, Q, ldq, nmod, work, lwork, stream, status_dev_out);
  return split_core(n, k, k, alpha, A, lda, gs, beta, Q, ldq, nmod, work, lwork, stream, status_dev_out);
}

int launch_split_general(int M, int N, int K, double alpha, const double* A, long lda, const GenSpec& gs,
                         double beta, double* Q, long ldq, int n_moduli, void* work, size_t lwork,
                         cudaStream_t stream, unsigned* status_dev_out, int block_req) {
  if (gs.kind == KIND_DFT) return PSMMA_EUNSUPPORTED;
  if (s2_use(KIND_CAUCHY_EIG, M, K, N, block_req) && gs.k1 == 0)
    return split_core_s2(M, N, K, alpha, A, lda, gs, beta, Q, ldq, resolve_nmod(n_moduli), work, lwork, stream,
                         status_dev_out);
  return split_core(M, N, K, alpha, A, lda, gs, beta, Q, ldq, resolve_nmod(n_moduli), work, lwork, stream,
                    status_dev_out);
}


// ------------------------------------------------------------------------------------------
// Grouped split path: many independent products (uneven sizes) in one launch per phase --
// one persistent modular GEMM over the tiles of all products per tile width -- for the
// batched merge level.  Device-side descriptors are copied once (prepare); the launches
// (enqueue) are then plain kernel launches that a stream capture can record.
// ------------------------------------------------------------------------------------------
struct GProb {
  int M, N, K, kp, kr, bn;
  double alpha, beta;
  const double* A;
  long lda;
  const double* A2;
  long lda2;
  int ka;
  GenSpec gs;
  double* Q;
  long ldq;
  SplitDevParams* prm;
  unsigned long long *amax, *hmax;
  double *hsum, *asq, *hsq, *Ht;
  __nv_bfloat16 *RA, *RH;
  int8_t* R;
  int b_row, b_h, b_ra, b_rh, b_crt;  // first block of this product in each grouped launch
};

// Product owning block `blk` of grouped launch W (largest first-block <= blk).
template <int W>
__device__ __forceinline__ int gfind(const GProb* d, int count, int blk) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const GProb& e = d[mid];
    const int key = W == 0 ? e.b_row : W == 1 ? e.b_h : W == 2 ? e.b_ra : W == 3 ? e.b_rh : e.b_crt;
    if (key <= blk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

constexpr int G_ROW_KCHUNK = 1024;

// Each CTA of a grouped pass kernel walks a run of consecutive logical blocks (one binary
// search per CTA, then a linear advance across product boundaries): a lookup per logical block
// (seven dependent loads of the descriptor table before any data moves) had made the small
// blocks of these passes latency-bound.  Runs per kernel: rows 2, H columns 2, residue and CRT
// tiles 8, H residue strips 16.
template <int W>
__device__ __forceinline__ int gkey(const GProb& e) {
  return W == 0 ? e.b_row : W == 1 ? e.b_h : W == 2 ? e.b_ra : W == 3 ? e.b_rh : e.b_crt;
}
template <int W>
struct GRun {
  int b, end, p;
  __device__ GRun(const GProb* d, int count, int total, int chunk) {
    b = blockIdx.x * chunk;
    end = min(b + chunk, total);
    p = b < end ? gfind<W>(d, count, b) : 0;
  }
  // the product owning logical block b (the last one whose first block is <= b)
  __device__ __forceinline__ const GProb& owner(const GProb* d, int count) {
    while (p + 1 < count && gkey<W>(d[p + 1]) <= b) ++p;
    return d[p];
  }
};
constexpr int G_RUN_ROW = 2, G_RUN_H = 2, G_RUN_RA = 8, G_RUN_RH = 16, G_RUN_CRT = 8;

__global__ void __launch_bounds__(128) k_g_row_absmax(const GProb* d, int count, int total) {
  for (GRun<0> r(d, count, total, G_RUN_ROW); r.b < r.end; ++r.b) {
    const GProb& e = r.owner(d, count);
    const int local = r.b - e.b_row, gx = (e.M + 127) / 128;
    row_absmax_blk(e.A, e.lda, e.A2, e.lda2, e.ka, e.M, e.K, G_ROW_KCHUNK, e.amax, e.asq, local % gx, local / gx);
  }
}

__global__ void __launch_bounds__(256) k_g_h_pass1(const GProb* d, int count, int total) {
  for (GRun<1> r(d, count, total, G_RUN_H); r.b < r.end; ++r.b) {
    const GProb& e = r.owner(d, count);
    const int j = r.b - e.b_h;
    switch (e.gs.kind) {
      case KIND_CAUCHY: h_pass1_blk<KIND_CAUCHY>(e.gs, e.K, e.kp, e.Ht, e.hmax, e.hsum, e.hsq, e.prm, j); break;
      case KIND_TOEPLITZ: h_pass1_blk<KIND_TOEPLITZ>(e.gs, e.K, e.kp, e.Ht, e.hmax, e.hsum, e.hsq, e.prm, j); break;
      case KIND_HANKEL: h_pass1_blk<KIND_HANKEL>(e.gs, e.K, e.kp, e.Ht, e.hmax, e.hsum, e.hsq, e.prm, j); break;
      case KIND_CAUCHY_EIG: h_pass1_blk<KIND_CAUCHY_EIG>(e.gs, e.K, e.kp, e.Ht, e.hmax, e.hsum, e.hsq, e.prm, j); break;
      default: h_pass1_blk<KIND_DENSE>(e.gs, e.K, e.kp, e.Ht, e.hmax, e.hsum, e.hsq, e.prm, j); break;
    }
    __syncthreads();  // the block's shared reduction buffers are reused by the next column
  }
}

__global__ void __launch_bounds__(1024) k_g_split_params(const GProb* d, double log2M) {
  const GProb& e = d[blockIdx.x];
  split_params_blk(e.prm, log2M, e.M, e.N, e.K, e.amax, e.asq, e.hmax, e.hsq);
}

__global__ void __launch_bounds__(256) k_g_residues_A(const GProb* d, int count, int total, CrtConsts cc) {
  for (GRun<2> r(d, count, total, G_RUN_RA); r.b < r.end; ++r.b) {
    const GProb& e = r.owner(d, count);
    const int local = r.b - e.b_ra, gx = e.kp / 64;
    residues_A_blk<64>(e.A, e.lda, e.A2, e.lda2, e.ka, e.M, e.K, e.kp, e.amax, e.prm, cc, e.RA, local % gx,
                       local / gx);
    __syncthreads();  // the shared tile is refilled for the next block
  }
}

__global__ void __launch_bounds__(128) k_g_residues_H(const GProb* d, int count, int total, CrtConsts cc) {
  for (GRun<3> r(d, count, total, G_RUN_RH); r.b < r.end; ++r.b) {
    const GProb& e = r.owner(d, count);
    const int local = r.b - e.b_rh, gx = rh_blocks_x(e.kp);
    residues_H_blk(e.Ht, e.N, e.kp, e.hmax, e.prm, cc, e.RH, local % gx, local / gx);
  }
}

template <bool TOP32>
__global__ void __launch_bounds__(256, 3) k_g_crt_combine(const GProb* d, int count, int total, CrtConsts cc) {
  for (GRun<4> r(d, count, total, G_RUN_CRT); r.b < r.end; ++r.b) {
    const GProb& e = r.owner(d, count);
    const int local = r.b - e.b_crt, gx = (e.N + CRT_TJ - 1) / CRT_TJ;
    crt_combine_blk<false, TOP32>(e.R, e.M, e.N, e.kr, cc, e.amax, e.hmax, e.prm, e.alpha, e.beta, e.Q, e.ldq,
                                  local % gx, local / gx);
    __syncthreads();  // the shared transpose tile is reused by the next block
  }
}

namespace {

// Bump allocation over a workspace (base 0: measure only).
struct WsBump {
  uintptr_t base, off = 0;
  explicit WsBump(void* b) : base((uintptr_t)b) {}
  template <class T>
  T* take(size_t count, size_t align) {
    off = (off + align - 1) & ~(uintptr_t)(align - 1);
    T* p = (T*)(base + off);
    off += count * sizeof(T);
    return p;
  }
};

// Lays out (and, with a real base, fills) the group's descriptors and buffers.
int plan_group(const SplitProblem* P, int count, int nmod, const SplitTune& tune, WsBump& w,
               std::vector<GProb>* probs, std::vector<GemmDesc>* gd, SplitGroup* g) {
  GProb* d_probs = w.take<GProb>(count, 256);
  GemmDesc* d_gc[3];
  for (int c = 0; c < 3; ++c) d_gc[c] = w.take<GemmDesc>(count, 128);
  // small region: status word, then per product params, maxima and sums (zeroed by one memset)
  const uintptr_t small0 = (w.off + 1023) & ~(uintptr_t)1023;
  unsigned* status = w.take<unsigned>(256, 1024);
  std::vector<GProb> pr(count);
  for (int i = 0; i < count; ++i) {
    GProb& e = pr[i];
    const SplitProblem& q = P[i];
    e.M = q.M; e.N = q.N; e.K = q.K;
    e.kp = (q.K + 63) / 64 * 64;
    e.bn = (q.N <= tune.narrow_max) ? 64 : (q.N <= tune.mid_max) ? 128 : 256;
    e.kr = (q.N + 255) / 256 * 256;  // row stride of the residue products (any tile width)
    e.alpha = q.alpha; e.beta = q.beta;
    e.A = q.A; e.lda = q.lda; e.gs = q.gs; e.Q = q.Q; e.ldq = q.ldq;
    e.A2 = q.A2; e.lda2 = q.lda2;
    e.ka = (q.ka > 0 && q.A2) ? q.ka : q.K;
    e.prm = w.take<SplitDevParams>(1, 256);
    e.amax = w.take<unsigned long long>(q.M, 256);
    e.asq = w.take<double>(q.M, 256);
    e.hmax = w.take<unsigned long long>(q.N, 256);
    e.hsum = w.take<double>(q.N, 256);
    e.hsq = w.take<double>(q.N, 256);
  }
  const uintptr_t small1 = (w.off + 1023) & ~(uintptr_t)1023;
  int b_row = 0, b_h = 0, b_ra = 0, b_rh = 0, b_crt = 0;
  for (int i = 0; i < count; ++i) {
    GProb& e = pr[i];
    e.Ht = w.take<double>((size_t)e.N * e.kp, 1024);
    e.RA = w.take<__nv_bfloat16>((size_t)nmod * e.M * e.kp, 1024);
    e.RH = w.take<__nv_bfloat16>((size_t)nmod * e.N * e.kp, 1024);
    e.R = w.take<int8_t>((size_t)nmod * e.M * e.kr, 1024);
    e.b_row = b_row; b_row += ((e.M + 127) / 128) * ((e.K + G_ROW_KCHUNK - 1) / G_ROW_KCHUNK);
    e.b_h = b_h;     b_h += e.N;
    e.b_ra = b_ra;   b_ra += (e.kp / 64) * ((e.M + 63) / 64);
    e.b_rh = b_rh;   b_rh += rh_blocks_x(e.kp) * e.N;
    e.b_crt = b_crt; b_crt += ((e.N + CRT_TJ - 1) / CRT_TJ) * ((e.M + CRT_TI - 1) / CRT_TI);
  }
  g->count = count;
  g->nmod = nmod;
  g->group_m = tune.group_m;
  g->d_probs = d_probs;
  for (int c = 0; c < 3; ++c) g->d_gemm[c] = d_gc[c];
  g->blocks_row = b_row; g->blocks_h = b_h; g->blocks_ra = b_ra; g->blocks_rh = b_rh; g->blocks_crt = b_crt;
  g->small = (void*)(w.base + small0);  // small0, small1 are offsets from the base
  g->small_bytes = small1 - small0;
  g->status = status;
  if (!probs) return PSMMA_OK;
  // GEMM descriptors per tile width, larger products first (their tiles start the sweep)
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (double)pr[a].M * pr[a].N * pr[a].K > (double)pr[b].M * pr[b].N * pr[b].K;
  });
  for (int c = 0; c < 3; ++c) gd[c].clear();
  int tiles[3] = {0, 0, 0};
  for (int i : order) {
    const GProb& e = pr[i];
    const int cls = e.bn == 64 ? 1 : e.bn == 128 ? 2 : 0;
    GemmDesc x;
    memset(&x, 0, sizeof(x));
    if (!make_tmap(&x.ta, e.RA, e.kp, e.M, nmod, G_BM) || !make_tmap(&x.tb, e.RH, e.kp, e.N, nmod, e.bn))
      return PSMMA_EDEVICE;
    x.R = e.R;
    x.n = e.M;
    x.kr = e.kr;
    x.nkb = e.kp / G_BK;
    x.tiles_m = (e.M + G_BM - 1) / G_BM;
    x.tiles_n = (e.N + e.bn - 1) / e.bn;
    x.t0 = tiles[cls];
    tiles[cls] += x.tiles_m * x.tiles_n * nmod;
    gd[cls].push_back(x);
  }
  for (int c = 0; c < 3; ++c) {
    g->n_gemm[c] = (int)gd[c].size();
    g->tiles[c] = tiles[c];
  }
  *probs = pr;
  return PSMMA_OK;
}

}  // namespace

size_t split_group_bytes(const SplitProblem* P, int count, int n_moduli) {
  if (count <= 0) return 0;
  SplitGroup g;
  WsBump w(nullptr);
  plan_group(P, count, resolve_nmod(n_moduli), SplitTune(), w, nullptr, nullptr, &g);
  return w.off + 4096;
}

int split_group_prepare(const SplitProblem* P, int count, int n_moduli, const SplitTune& tune, void* work,
                        size_t lwork, cudaStream_t stream, SplitGroup* g) {
  const int nmod = resolve_nmod(n_moduli);
  if (nmod < 8 || nmod > SPL_MAX_MODULI) return PSMMA_EUNSUPPORTED;
  if (count <= 0) {
    *g = SplitGroup();
    return PSMMA_OK;
  }
  for (int i = 0; i < count; ++i) {
    const SplitProblem& q = P[i];
    if (q.M <= 0 || q.N <= 0 || q.K <= 0 || q.gs.kind == KIND_DFT) return PSMMA_EUNSUPPORTED;
    if (q.K >= (1 << 24) || q.M >= (1 << 30) || q.N >= (1 << 30)) return PSMMA_EUNSUPPORTED;
  }
  if (!work || lwork < split_group_bytes(P, count, n_moduli)) return PSMMA_EWORKSPACE;
  WsBump w((void*)(((uintptr_t)work + 255) & ~(uintptr_t)255));
  std::vector<GProb> pr;
  std::vector<GemmDesc> gd[3];
  int st = plan_group(P, count, nmod, tune, w, &pr, gd, g);
  if (st) return st;
  if (cudaMemcpyAsync(g->d_probs, pr.data(), sizeof(GProb) * count, cudaMemcpyHostToDevice, stream) != cudaSuccess)
    return PSMMA_EDEVICE;
  for (int c = 0; c < 3; ++c)
    if (!gd[c].empty() && cudaMemcpyAsync(g->d_gemm[c], gd[c].data(), sizeof(GemmDesc) * gd[c].size(),
                                          cudaMemcpyHostToDevice, stream) != cudaSuccess)
      return PSMMA_EDEVICE;
  return PSMMA_OK;
}

template <int BN>
static int launch_group_gemm(const SplitGroup& g, int cls, const CrtConsts& cc, int sms, cudaStream_t stream) {
  if (g.n_gemm[cls] == 0) return PSMMA_OK;
  using Shape = GemmShape<BN>;
  GroupGemm ts;
  memset(&ts, 0, sizeof(ts));
  ts.g.nmod = g.nmod;
  ts.g.group_m = g.group_m;
  ts.g.status = g.status;
  for (int l = 0; l < g.nmod; ++l) {
    ts.g.m[l] = cc.m[l];
    ts.g.inv_m[l] = cc.inv_m[l];
  }
  ts.d = (const GemmDesc*)g.d_gemm[cls];
  ts.count = g.n_gemm[cls];
  ts.total_tiles = g.tiles[cls];
  if (set_smem_attr(k_crt_gemm<BN, GroupGemm>, (int)Shape::SMEM) != cudaSuccess)
    return PSMMA_EDEVICE;
  k_crt_gemm<BN, GroupGemm><<<std::min(sms, ts.total_tiles), G_THREADS, Shape::SMEM, stream>>>(ts);
  return PSMMA_OK;
}

int split_group_enqueue(const SplitGroup& g, cudaStream_t stream, unsigned* status_out) {
  if (g.count == 0) return PSMMA_OK;
  const CrtConsts cc = get_consts(g.nmod);
  const GProb* d = (const GProb*)g.d_probs;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PSMMA_EDEVICE;
  if (cudaMemsetAsync(g.small, 0, g.small_bytes, stream) != cudaSuccess) return PSMMA_EDEVICE;
  auto runs = [](int total, int chunk) { return (unsigned)((total + chunk - 1) / chunk); };
  if (g.blocks_row > 0) k_g_row_absmax<<<runs(g.blocks_row, G_RUN_ROW), 128, 0, stream>>>(d, g.count, g.blocks_row);
  prof_mark(stream, "g_row_scale");
  if (g.blocks_h > 0) k_g_h_pass1<<<runs(g.blocks_h, G_RUN_H), 256, 0, stream>>>(d, g.count, g.blocks_h);
  prof_mark(stream, "g_h_generate");
  k_g_split_params<<<g.count, 1024, 0, stream>>>(d, cc.log2M);
  prof_mark(stream, "g_params");
  if (g.blocks_ra > 0) k_g_residues_A<<<runs(g.blocks_ra, G_RUN_RA), 256, 0, stream>>>(d, g.count, g.blocks_ra, cc);
  prof_mark(stream, "g_residues_A");
  if (g.blocks_rh > 0) k_g_residues_H<<<runs(g.blocks_rh, G_RUN_RH), 128, 0, stream>>>(d, g.count, g.blocks_rh, cc);
  prof_mark(stream, "g_residues_H");
  int st = launch_group_gemm<256>(g, 0, cc, sms, stream);
  prof_mark(stream, "g_gemm_256");
  if (!st) st = launch_group_gemm<128>(g, 2, cc, sms, stream);
  prof_mark(stream, "g_gemm_128");
  if (!st) st = launch_group_gemm<64>(g, 1, cc, sms, stream);
  prof_mark(stream, "g_gemm_64");
  if (st) return st;
  if (g.blocks_crt > 0)
    (cc.top32 ? k_g_crt_combine<true> : k_g_crt_combine<false>)<<<runs(g.blocks_crt, G_RUN_CRT), dim3(32, 8), 0,
                                                                   stream>>>(d, g.count, g.blocks_crt, cc);
  prof_mark(stream, "g_crt_combine");
  if (cudaGetLastError() != cudaSuccess) return PSMMA_EDEVICE;
  if (status_out &&
      cudaMemcpyAsync(status_out, g.status, sizeof(unsigned), cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
    return PSMMA_EDEVICE;
  return PSMMA_OK;
}

}  // namespace psmma
