// FP64 plain path: structured multiply on FP64 tensor-core MMA (mma.sync .f64) with the
// structured operand generated tile by tile in shared memory, never read from HBM.
//
// Real kinds (Cauchy, Toeplitz, Hankel):  Q(n x k) = alpha * A(n x k) * H(k x k) + beta * Q
//   A streams from HBM (column-major, lda); H's tile is rebuilt from the generators.
//   Tile formulas follow the reference's tile builders:
//     Cauchy   H(i,j) = U(i)*V(j) / (D(i)-F(j))     Cauchylowrank.f90:509-521 (Cauchylike),
//              generator columns [D,F,U,V]          Auxil_2p5D.f90:138-141 (ConstCauchy)
//     Toeplitz H(i,j) = G(K+j-i)                    Auxil_2p5D.f90:224-231 (ConstToeplitz)
//     Hankel   H(i,j) = G(i+j-1)                    Auxil_2p5D.f90:309-316 (ConstHankel)
//   The reference's ring over process columns (pscauchy_compute.f90:355-423) visits every
//   k-block of A once; here the k-loop of one thread block does the same.
//
// DFT (pzmdftL.f90): C(n x k) = alpha * F(n x n) * B(n x k) + beta * C, F(j,l) = w^(j*l).
//   Viewing interleaved complex B and C as real (2n x k) column-major arrays with twice the
//   leading dimension, the product is the real GEMM C' = F' * B' where F' (2n x 2n) holds
//   the 2x2 blocks [[Re F, -Im F], [Im F, Re F]].  F' tiles are generated from a table
//   w^t, t = 0..n-1, indexed by the exact integer (j*l) mod n.
#include "psmma_internal.h"
#include "tcgen05_util.cuh"  // div_nr

#include <vector>

namespace psmma {

// ------------------------------------------------------------------------------------
// Tile geometry.  256 threads = 8 warps as 2 (M) x 4 (N); warp tile 64 x 32.
// ------------------------------------------------------------------------------------
constexpr int F64_BM = 128;
constexpr int F64_BN = 128;
constexpr int F64_BK = 16;
constexpr int F64_THREADS = 256;
constexpr int F64_WM = 64;                  // warp tile rows
constexpr int F64_WN = 32;                  // warp tile cols
constexpr int F64_MT = F64_WM / 16;         // m16 fragments per warp
constexpr int F64_NT = F64_WN / 8;          // n8 fragments per warp
constexpr int F64_APAD = F64_BM + 8;        // smem row stride (doubles) of the A tile [k][i]
constexpr int F64_BPAD = F64_BN + 8;        // smem row stride (doubles) of the B tile [k][j]
constexpr int F64_SMEM_A = F64_BK * F64_APAD;
constexpr int F64_SMEM_B = F64_BK * F64_BPAD;
constexpr size_t F64_SMEM_BYTES = 2 * (F64_SMEM_A + F64_SMEM_B) * sizeof(double);

struct F64Args {
  int M, N, K;               // GEMM sizes of the real view
  double alpha, beta;
  const double* X; long ldx;  // streamed operand (A for real kinds, B' for DFT)
  double* C; long ldc;        // output (Q or C')
  GenSpec gs;                       // generators of the structured operand
  // split K (single products that fill too few waves): block z of the launch covers
  // k in [z*kc, (z+1)*kc) and writes alpha * its partial sum to W + z * ldw * N (ld ldw)
  int kc = 0;
  double* W = nullptr;
  long ldw = 0;
};

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool pred) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = pred ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

// m16n8k16 FP64 MMA.  Fragment layout (g = lane/4, t = lane%4):
//   a[r]: A[g + 8*(r&1)][t + 4*(r>>1)], r = 0..7
//   b[r]: B[t + 4*r][g],                r = 0..3
//   c[0..1]: C[g][2t + {0,1}], c[2..3]: C[g+8][2t + {0,1}]
__device__ __forceinline__ void dmma16816(double (&c)[4], const double (&a)[8], const double (&b)[4]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
      "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
      : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
      : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
        "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
}

// One BK-deep step of the warp tile from smem tiles As[k][i] and Bs[k][j].
__device__ __forceinline__ void warp_mma_step(double (&acc)[F64_MT][F64_NT][4], const double* As,
                                              const double* Bs, int wm0, int wn0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  double b[F64_NT][4];
#pragma unroll
  for (int nt = 0; nt < F64_NT; nt++)
#pragma unroll
    for (int r = 0; r < 4; r++) b[nt][r] = Bs[(t + 4 * r) * F64_BPAD + wn0 + nt * 8 + g];
#pragma unroll
  for (int mt = 0; mt < F64_MT; mt++) {
    double a[8];
#pragma unroll
    for (int r = 0; r < 8; r++) a[r] = As[(t + 4 * (r >> 1)) * F64_APAD + wm0 + mt * 16 + g + 8 * (r & 1)];
#pragma unroll
    for (int nt = 0; nt < F64_NT; nt++) dmma16816(acc[mt][nt], a, b[nt]);
  }
}

// ---- streamed-operand loaders -----------------------------------------------------------
// A tile (real kinds): As[kk][ii] = A[(m0+ii) + (k0+kk)*lda], zero outside M x K.
__device__ __forceinline__ void load_A_tile(double* As, const F64Args& p, int m0, int k0, int tid) {
#pragma unroll
  for (int e = tid; e < F64_BM * F64_BK; e += F64_THREADS) {
    int ii = e % F64_BM, kk = e / F64_BM;
    int gi = m0 + ii, gk = k0 + kk;
    bool ok = gi < p.M && gk < p.K;
    const double* src = ok ? p.X + (long)gi + (long)gk * p.ldx : p.X;
    cp_async8(&As[kk * F64_APAD + ii], src, ok);
  }
}
// B tile (DFT): Bs[kk][jj] = B'[(k0+kk) + (n0+jj)*ldb'], zero outside K x N.
__device__ __forceinline__ void load_B_tile(double* Bs, const F64Args& p, int n0, int k0, int tid) {
#pragma unroll
  for (int e = tid; e < F64_BN * F64_BK; e += F64_THREADS) {
    int kk = e % F64_BK, jj = e / F64_BK;
    int gk = k0 + kk, gj = n0 + jj;
    bool ok = gk < p.K && gj < p.N;
    const double* src = ok ? p.X + (long)gk + (long)gj * p.ldx : p.X;
    cp_async8(&Bs[kk * F64_BPAD + jj], src, ok);
  }
}

// B tile (dense H): Bs[kk][jj] = H[(k0+kk) + (n0+jj)*ldb], zero outside K x N.
__device__ __forceinline__ void load_Hd_tile(double* Bs, const F64Args& p, int n0, int k0, int tid) {
#pragma unroll
  for (int e = tid; e < F64_BN * F64_BK; e += F64_THREADS) {
    int kk = e % F64_BK, jj = e / F64_BK;
    int gk = k0 + kk, gj = n0 + jj;
    bool ok = gk < p.K && gj < p.N;
    const double* src = ok ? p.gs.B + (long)gk + (long)gj * p.gs.ldb : p.gs.B;
    cp_async8(&Bs[kk * F64_BPAD + jj], src, ok);
  }
}

// ---- generated-operand builders -----------------------------------------------------------
// H tile (real kinds): Bs[kk][jj] = H(k0+kk, n0+jj) (0-based), zero outside K x N.
// Each thread owns one column jj and BK/2 consecutive rows.
struct ColGen {
  double F, V, F1, dl, dr;  // this thread's column generators
  VSplit vs;                // V(j) split for the double-float entries
};

template <int KIND>
__device__ __forceinline__ void gen_H_tile(double* Bs, const F64Args& p, int n0, int k0, int tid,
                                           const ColGen& cg) {
  const double colF = cg.F, colV = cg.V;
  const int jj = tid % F64_BN;
  const int kh = tid / F64_BN;  // 0 or 1
  const int gj = n0 + jj;
#pragma unroll
  for (int q = 0; q < F64_BK / 2; q++) {
    int kk = kh * (F64_BK / 2) + q;
    int gk = k0 + kk;
    double h = 0.0;
    if (gk < p.K && gj < p.N) {
      if (KIND == KIND_CAUCHY) {
        double d = __ldg(p.gs.Dr + gk);               // D(i)
        double u = __ldg(p.gs.Ur + gk);               // U(i)
        h = cauchy_entry(u, colV, cg.vs, d - colF);   // U(i)*V(j) / (D(i)-F(j))
      } else if (KIND == KIND_CAUCHY_EIG) {
        const double fi = __ldg(p.gs.Dr + gk), u = __ldg(p.gs.Ur + gk);
        const bool upper = p.gs.rglob ? (__ldg(p.gs.rglob + gk) - 1 <= p.gs.cg0 + gj) : (gk - gj <= p.gs.diag_off);
        h = cauchy_entry(u, colV, cg.vs, eig_den(fi, colF, cg.F1, cg.dl, cg.dr, upper));
      } else if (KIND == KIND_TOEPLITZ) {
        h = __ldg(p.gs.g + (p.gs.order - 1) + gj - gk);  // G(K + j - i), 1-based
      } else {
        h = __ldg(p.gs.g + gk + gj);                     // G(i + j - 1), 1-based
      }
    }
    Bs[kk * F64_BPAD + jj] = h;
  }
}

// F' tile (DFT): As[kk][ii] = F'(m0+ii, k0+kk), F'(2r+a, 2l+b) = [[Re,-Im],[Im,Re]][a][b] of
// w^(r*l mod n).  Each thread owns one row ii and BK/2 consecutive k columns (one complex l
// per pair of columns).
__device__ __forceinline__ void gen_F_tile(double* As, const F64Args& p, int m0, int k0, int tid) {
  const int ii = tid % F64_BM;
  const int kh = tid / F64_BM;  // 0 or 1
  const int gi = m0 + ii;
  const long n = p.gs.n_dft;
  const int r = gi >> 1, a = gi & 1;
#pragma unroll
  for (int q = 0; q < F64_BK / 4; q++) {
    int kk = kh * (F64_BK / 2) + 2 * q;   // even column: b = 0, next: b = 1
    int gk = k0 + kk;
    int l = gk >> 1;
    double v0 = 0.0, v1 = 0.0;
    if (gi < p.M && gk < p.K) {
      long t = ((long)r * (long)l) % n;
      double2 w = __ldg(p.gs.wtab + t);
      // row 2r  : [ Re, -Im ];  row 2r+1: [ Im, Re ]
      v0 = a ? w.y : w.x;
      v1 = a ? w.x : -w.y;
    }
    As[kk * F64_APAD + ii] = v0;
    As[(kk + 1) * F64_APAD + ii] = v1;
  }
}

// One 128 x 128 output tile (bx, by) of the product described by p.
template <int KIND>
__device__ __forceinline__ void struct_f64_tile(const F64Args& p, int bx, int by, int bz = 0) {
  extern __shared__ __align__(16) double smem[];
  double* As0 = smem;
  double* Bs0 = smem + F64_SMEM_A;
  double* As1 = smem + F64_SMEM_A + F64_SMEM_B;
  double* Bs1 = As1 + F64_SMEM_A;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = bx * F64_BM, n0 = by * F64_BN;
  const int wm0 = (warp & 1) * F64_WM, wn0 = (warp >> 1) * F64_WN;

  ColGen cg{0.0, 0.0, 0.0, 0.0, 0.0, VSplit{}};
  if (KIND == KIND_CAUCHY || KIND == KIND_CAUCHY_EIG) {
    int gj = n0 + (tid % F64_BN);
    if (gj < p.N) {
      cg.F = __ldg(p.gs.Fc + gj);   // F(j)
      cg.V = __ldg(p.gs.Vc + gj);   // V(j)
      if (KIND == KIND_CAUCHY_EIG) {
        cg.dl = __ldg(p.gs.dl + gj);  // DIFL(j)
        if (gj < p.gs.fc1_len) {
          cg.F1 = __ldg(p.gs.Fc1 + gj);  // F(j+1)
          cg.dr = __ldg(p.gs.dr + gj);   // DIFR(j)
        }
      }
    }
    cg.vs = v_split(cg.V);
  }

  double acc[F64_MT][F64_NT][4];
#pragma unroll
  for (int i = 0; i < F64_MT; i++)
#pragma unroll
    for (int j = 0; j < F64_NT; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[i][j][r] = 0.0;

  // k-steps of this block (all of K, or split z's share of kc)
  const int kt0 = p.W ? bz * (p.kc / F64_BK) : 0;
  const int nk = p.W ? min((p.K + F64_BK - 1) / F64_BK, (bz + 1) * (p.kc / F64_BK)) : (p.K + F64_BK - 1) / F64_BK;
  auto stage = [&](int kt, double* As, double* Bs) {
    int k0 = kt * F64_BK;
    if (KIND == KIND_DFT) {
      load_B_tile(Bs, p, n0, k0, tid);
      cp_async_commit();
      gen_F_tile(As, p, m0, k0, tid);
    } else if (KIND == KIND_DENSE) {
      load_A_tile(As, p, m0, k0, tid);
      load_Hd_tile(Bs, p, n0, k0, tid);
      cp_async_commit();
    } else {
      load_A_tile(As, p, m0, k0, tid);
      cp_async_commit();
      gen_H_tile<KIND>(Bs, p, n0, k0, tid, cg);
    }
  };

  if (kt0 < nk) {
    stage(kt0, As0, Bs0);
    cp_async_wait_all();
    __syncthreads();
  }
  for (int kt = kt0; kt < nk; kt++) {
    const int ph = (kt - kt0) & 1;
    double* As = ph ? As1 : As0;
    double* Bs = ph ? Bs1 : Bs0;
    if (kt + 1 < nk) stage(kt + 1, ph ? As0 : As1, ph ? Bs0 : Bs1);
    warp_mma_step(acc, As, Bs, wm0, wn0, lane);
    cp_async_wait_all();
    __syncthreads();
  }

  // Epilogue: C = alpha*acc + beta*C (beta == 0: C is not read).
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < F64_MT; mt++)
#pragma unroll
    for (int nt = 0; nt < F64_NT; nt++)
#pragma unroll
      for (int r = 0; r < 4; r++) {
        int gi = m0 + wm0 + mt * 16 + g + 8 * (r >> 1);
        int gj = n0 + wn0 + nt * 8 + 2 * t + (r & 1);
        if (gi < p.M && gj < p.N) {
          if (p.W) {  // split K: this split's partial, combined by k_splitk_reduce
            p.W[(long)bz * p.ldw * p.N + (long)gi + (long)gj * p.ldw] = p.alpha * acc[mt][nt][r];
          } else {
            double* cp = p.C + (long)gi + (long)gj * p.ldc;
            double v = p.alpha * acc[mt][nt][r];
            if (p.beta != 0.0) v = fma(p.beta, *cp, v);
            *cp = v;
          }
        }
      }
}

template <int KIND>
__global__ void __launch_bounds__(F64_THREADS, 1) k_struct_f64(F64Args p) {
  struct_f64_tile<KIND>(p, blockIdx.x, blockIdx.y, blockIdx.z);
}

// C := beta * C + sum_z W_z over the S split-K partials, in split order (deterministic).
__global__ void k_splitk_reduce(double* __restrict__ C, long ldc, const double* __restrict__ W, long ldw, int M,
                                int N, int S, double beta) {
  const long total = (long)M * N;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long i = e % M, j = e / M;
    double v = W[i + j * ldw];
    for (int z = 1; z < S; ++z) v += W[(long)z * ldw * N + i + j * ldw];
    double* cp = C + i + j * ldc;
    if (beta != 0.0) v = fma(beta, *cp, v);
    *cp = v;
  }
}

// Grouped: block b belongs to the product with the largest first block t0 <= b.
template <int KIND>
__global__ void __launch_bounds__(F64_THREADS, 1)
    k_struct_f64_group(const F64Args* __restrict__ ps, const int* __restrict__ t0, int count) {
  const int b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t0[mid] <= b) lo = mid; else hi = mid - 1;
  }
  const F64Args& p = ps[lo];
  const int local = b - t0[lo], gx = (p.M + F64_BM - 1) / F64_BM;
  struct_f64_tile<KIND>(p, local % gx, local / gx);
}

// C := beta * C for an M x N column-major block (alpha == 0 path).
__global__ void k_scale(double* C, long ldc, int M, int N, double beta) {
  long total = (long)M * N;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    long i = e % M, j = e / M;
    double* cp = C + i + j * ldc;
    *cp = (beta == 0.0) ? 0.0 : beta * *cp;
  }
}

// w^t = exp(-2*pi*i*t/n), t = 0..n-1, from sincospi of the exact fraction 2t/n.
__global__ void k_dft_table(double2* w, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)t / (double)n, &s, &c);
    w[t] = make_double2(c, -s);
  }
}

// Splits of K that fill the SMs in whole waves when the output has few tiles (fewer than 16
// waves; one CTA per SM): the count S (1..16, at least 128 k per split) maximising the useful
// fraction of the last wave, with a charge of 0.2 % per extra split for the partials' traffic
// (S M N doubles written and summed: about 10 us per split at n = 2048, 0.06 % of the product)
// and the jobs' pipeline fill.  n = 2048: 256 tiles x 16 splits = 26.9 waves (0.998 of the
// last wave used, against 0.963 at 4 splits); n = 4096: 1024 tiles x 4 = 26.9 waves.
int f64_splitk_count(int M, int N, int K, int sms) {
  const long tiles = (long)((M + F64_BM - 1) / F64_BM) * ((N + F64_BN - 1) / F64_BN);
  if (tiles >= 16L * sms || K < 256) return 1;
  int best = 1;
  double best_v = -1.0;
  for (int S = 1; S <= 16 && K / S >= 128; ++S) {
    const long jobs = tiles * S;
    const double eff = (double)jobs / (double)(((jobs + sms - 1) / sms) * sms);
    const double v = eff - 0.002 * (S - 1);
    if (v > best_v + 1e-9) { best_v = v; best = S; }
  }
  return best;
}

size_t f64_splitk_bytes(int M, int N, int K, int sms) {
  const int S = f64_splitk_count(M, N, K, sms);
  return S > 1 ? (size_t)S * (size_t)M * (size_t)N * sizeof(double) : 0;
}

int launch_struct_f64(int M, int N, int K, double alpha, const double* X, long ldx, const GenSpec& gs,
                      double beta, double* C, long ldc, cudaStream_t stream) {
  return launch_struct_f64_ws(M, N, K, alpha, X, ldx, gs, beta, C, ldc, nullptr, 0, stream);
}

int launch_struct_f64_ws(int M, int N, int K, double alpha, const double* X, long ldx, const GenSpec& gs,
                         double beta, double* C, long ldc, void* work, size_t lwork, cudaStream_t stream) {
  const int kind = gs.kind;
  if (M == 0 || N == 0) return PSMMA_OK;
  if (alpha == 0.0 || K == 0) {
    if (beta == 1.0) return PSMMA_OK;
    int blocks = (int)std::min<long>(((long)M * N + 255) / 256, 152L * 16);
    k_scale<<<blocks, 256, 0, stream>>>(C, ldc, M, N, beta);
    return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
  }
  F64Args p;
  p.M = M; p.N = N; p.K = K; p.alpha = alpha; p.beta = beta;
  p.X = X; p.ldx = ldx; p.C = C; p.ldc = ldc;
  p.gs = gs;
  dim3 grid((M + F64_BM - 1) / F64_BM, (N + F64_BN - 1) / F64_BN);
  if (grid.y > 65535) return PSMMA_EUNSUPPORTED;
  if (work) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return PSMMA_EDEVICE;
    const int S = f64_splitk_count(M, N, K, sms);
    if (S > 1 && lwork >= f64_splitk_bytes(M, N, K, sms)) {
      p.kc = ((K + S - 1) / S + F64_BK - 1) / F64_BK * F64_BK;
      p.W = (double*)work;
      p.ldw = M;
      grid.z = (K + p.kc - 1) / p.kc;
    }
  }
  prof_begin(stream);
  switch (kind) {
#define PSMMA_LAUNCH_F64(KD)                                                                  \
  case KD: {                                                                                  \
    static bool attr_set = false;                                                             \
    if (!attr_set) {                                                                          \
      if (set_smem_attr(k_struct_f64<KD>, (int)F64_SMEM_BYTES) != cudaSuccess)                           \
        return PSMMA_EDEVICE;                                                                 \
      attr_set = true;                                                                        \
    }                                                                                         \
    k_struct_f64<KD><<<grid, F64_THREADS, F64_SMEM_BYTES, stream>>>(p);                       \
    break;                                                                                    \
  }
    PSMMA_LAUNCH_F64(KIND_CAUCHY)
    PSMMA_LAUNCH_F64(KIND_TOEPLITZ)
    PSMMA_LAUNCH_F64(KIND_HANKEL)
    PSMMA_LAUNCH_F64(KIND_DFT)
    PSMMA_LAUNCH_F64(KIND_DENSE)
    PSMMA_LAUNCH_F64(KIND_CAUCHY_EIG)
#undef PSMMA_LAUNCH_F64
    default:
      return PSMMA_EUNSUPPORTED;
  }
  if (p.W) {
    const long total = (long)M * N;
    const int blocks = (int)std::min<long>((total + 255) / 256, 152L * 16);
    k_splitk_reduce<<<blocks, 256, 0, stream>>>(C, ldc, p.W, p.ldw, M, N, (int)grid.z, beta);
  }
  prof_mark(stream, "struct_gemm_f64");
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

int launch_dft_table(double2* w, int n, cudaStream_t stream) {
  int blocks = std::max(1, std::min((n + 255) / 256, 1024));
  k_dft_table<<<blocks, 256, 0, stream>>>(w, n);
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}


// ---- the DFT on the FP64 path ---------------------------------------------------------------
// C (n x k complex) = alpha F_n B + beta C as the real GEMM C' = F' B' of the embedding, F'
// generated tile by tile from the table w^t.  With R = dft_radix_for(n) > 1 (the split path's
// rule) the embedding is F_(n/R)'s, applied to the R k columns B(r::R, :), and the twiddles and
// R-point butterflies follow in one pass: n^2 k / R complex multiply-adds instead of n^2 k.
// Workspace: the n-entry table (plain); B' and P (n x k complex each) and the tables of n and
// n / R entries (radix).
size_t dft_f64_workspace(int n, int k) {
  if (n <= 0 || k <= 0) return 0;
  const size_t a = 256;
  auto al = [&](size_t x) { return (x + a - 1) / a * a; };
  const int R = dft_radix_for(n);
  if (R == 1) return al((size_t)n * 16);
  return 2 * al((size_t)n * k * 16) + al((size_t)n * 16) + al((size_t)(n / R) * 16);
}

int launch_dft_f64(int n, int k, double alpha, const double* B, long ldb, double beta, double* C, long ldc,
                   void* work, size_t lwork, cudaStream_t stream) {
  if (n <= 0 || k <= 0) return PSMMA_OK;
  if (lwork < dft_f64_workspace(n, k) || !work) return PSMMA_EWORKSPACE;
  const int R = dft_radix_for(n);
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  char* w = (char*)work;
  GenSpec gs;
  gs.kind = KIND_DFT;
  if (R == 1) {
    double2* wtab = (double2*)w;
    int st = launch_dft_table(wtab, n, stream);
    if (st) return st;
    gs.n_dft = n;
    gs.wtab = wtab;
    // real view: C'(2n x k) = F'(2n x 2n) * B'(2n x k), leading dimensions doubled
    return launch_struct_f64(2 * n, k, 2 * n, alpha, B, 2 * ldb, gs, beta, C, 2 * ldc, stream);
  }
  const int nq = n / R;
  if ((long)R * k > 65535L * F64_BN) return PSMMA_EUNSUPPORTED;  // the kernel's grid y covers R k columns
  double2* Bp = (double2*)w;
  double2* P = (double2*)(w + al((size_t)n * k * 16));
  double2* wn = (double2*)(w + 2 * al((size_t)n * k * 16));
  double2* wq = (double2*)((char*)wn + al((size_t)n * 16));
  int st = launch_dft_deinterleave((const double2*)B, ldb, n, k, R, Bp, stream);
  if (!st) st = launch_dft_table(wq, nq, stream);
  if (!st) st = launch_dft_table(wn, n, stream);
  if (st) return st;
  gs.n_dft = nq;
  gs.wtab = wq;
  st = launch_struct_f64(2 * nq, R * k, 2 * nq, alpha, (const double*)Bp, 2L * nq, gs, 0.0, (double*)P, 2L * nq,
                         stream);
  if (st) return st;
  return launch_dft_radix_combine(P, nq, k, wn, beta, (double2*)C, ldc, R, stream);
}

size_t f64_group_bytes(int count) {
  if (count <= 0) return 0;
  return ((sizeof(F64Args) * count + 255) & ~(size_t)255) + sizeof(int) * count + 512;
}

int f64_group_prepare(const F64Prob* P, int count, void* dev, cudaStream_t stream, F64Group* g) {
  *g = F64Group();
  if (count <= 0) return PSMMA_OK;
  std::vector<F64Args> args(count);
  std::vector<int> t0(count);
  int blocks = 0;
  for (int i = 0; i < count; ++i) {
    const F64Prob& q = P[i];
    if (q.M <= 0 || q.N <= 0 || q.K <= 0 || q.gs.kind != P[0].gs.kind) return PSMMA_EUNSUPPORTED;
    if (q.gs.kind != KIND_CAUCHY && q.gs.kind != KIND_DENSE && q.gs.kind != KIND_CAUCHY_EIG &&
        q.gs.kind != KIND_TOEPLITZ && q.gs.kind != KIND_HANKEL)
      return PSMMA_EUNSUPPORTED;
    if (q.gs.k1 > 0) return PSMMA_EUNSUPPORTED;  // tail rows: split path only
    F64Args& a = args[i];
    a.M = q.M; a.N = q.N; a.K = q.K; a.alpha = q.alpha; a.beta = q.beta;
    a.X = q.X; a.ldx = q.ldx; a.C = q.C; a.ldc = q.ldc; a.gs = q.gs;
    t0[i] = blocks;
    const long nb = (long)((q.M + F64_BM - 1) / F64_BM) * ((q.N + F64_BN - 1) / F64_BN);
    if (blocks + nb > 0x7fffffffL) return PSMMA_EUNSUPPORTED;
    blocks += (int)nb;
  }
  uintptr_t base = ((uintptr_t)dev + 255) & ~(uintptr_t)255;
  F64Args* d_args = (F64Args*)base;
  int* d_t0 = (int*)(base + ((sizeof(F64Args) * count + 255) & ~(size_t)255));
  if (cudaMemcpyAsync(d_args, args.data(), sizeof(F64Args) * count, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaMemcpyAsync(d_t0, t0.data(), sizeof(int) * count, cudaMemcpyHostToDevice, stream) != cudaSuccess)
    return PSMMA_EDEVICE;
  g->count = count;
  g->kind = P[0].gs.kind;
  g->blocks = blocks;
  g->d_args = d_args;
  g->d_t0 = d_t0;
  return PSMMA_OK;
}

template <int KIND>
static int f64_group_launch(const F64Group& g, const F64Args* a, cudaStream_t stream) {
  if (set_smem_attr(k_struct_f64_group<KIND>, (int)F64_SMEM_BYTES) != cudaSuccess)
    return PSMMA_EDEVICE;
  k_struct_f64_group<KIND><<<g.blocks, F64_THREADS, F64_SMEM_BYTES, stream>>>(a, g.d_t0, g.count);
  return PSMMA_OK;
}

int f64_group_enqueue(const F64Group& g, cudaStream_t stream) {
  if (g.count == 0) return PSMMA_OK;
  const F64Args* a = (const F64Args*)g.d_args;
  int st;
  const char* name;
  switch (g.kind) {
    case KIND_CAUCHY: st = f64_group_launch<KIND_CAUCHY>(g, a, stream); name = "f64_group_cauchy"; break;
    case KIND_CAUCHY_EIG: st = f64_group_launch<KIND_CAUCHY_EIG>(g, a, stream); name = "f64_group_cauchyeig"; break;
    case KIND_TOEPLITZ: st = f64_group_launch<KIND_TOEPLITZ>(g, a, stream); name = "f64_group_toeplitz"; break;
    case KIND_HANKEL: st = f64_group_launch<KIND_HANKEL>(g, a, stream); name = "f64_group_hankel"; break;
    default: st = f64_group_launch<KIND_DENSE>(g, a, stream); name = "f64_group_dense"; break;
  }
  if (st) return st;
  prof_mark(stream, name);
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

}  // namespace psmma
