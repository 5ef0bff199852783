// Block-cyclic redistribution between two ScaLAPACK layouts over the same processes.
//
// PSMMA_CAUCHY / TOEPLITZ / HANKEL / CAUCHYEIG with REDIST = .TRUE. move A from its
// block-cyclic layout to a blocked one and Q back with two PDGEMR2D calls
// (psmma_cauchy.f90:113-162, psmma_toeplitz.f90:137-157, psmma_cauchyeig.f90:166-200).  Here
// the same copy is a plan built once on the host, a pack kernel that gathers a rank's
// elements into one contiguous buffer per peer, one all-to-all exchange that the caller
// runs (MPI_Alltoallv, NCCL, torch.distributed), and an unpack kernel that scatters the
// received buffers into the destination's local array.  Both kernels are HBM-bound copies:
// 2 x element size bytes per element plus the cached row/column maps.
//
// The pair (source rank s, destination rank d) exchanges the sub-matrix elements whose row
// is owned by s's process row in A's layout and by d's process row in B's layout, and
// whose column likewise: a Cartesian product of a row set and a column set.  Both sides
// order it column-major by increasing global index, so the packing rank and the unpacking
// rank agree on every element's place without exchanging indices.
#include "psmma_internal.h"

#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace psmma {
namespace {

// ScaLAPACK TOOLS, restated from their documented definitions with 0-based process and
// index arguments: NUMROC (local count), INDXL2G (local to global), INDXG2P (owner).
int numroc0(int n, int nb, int iproc, int isrc, int nprocs) {
  const int mydist = (nprocs + iproc - isrc) % nprocs;
  const int nblocks = n / nb;
  int r = (nblocks / nprocs) * nb;
  const int extra = nblocks % nprocs;
  if (mydist < extra) r += nb;
  else if (mydist == extra) r += n % nb;
  return r;
}
long l2g0(long l, int nb, int p, int src, int nprocs) {
  const int dist = (p - src + nprocs) % nprocs;
  return ((l / nb) * nprocs + dist) * nb + l % nb;
}
int g2p0(long g, int nb, int src, int nprocs) { return (int)((src + g / nb) % nprocs); }

struct Layout {
  int M = 0, N = 0, MB = 1, NB = 1, RSRC = 0, CSRC = 0, LLD = 1;
  int nprow = 1, npcol = 1, order = 0;
  int myrow = 0, mycol = 0, lrows = 0, lcols = 0;
  int rank_of(int pr, int pc) const { return order == 0 ? pr * npcol + pc : pc * nprow + pr; }
};

// Checks one descriptor / sub-matrix / grid triple; the codes follow ScaLAPACK's CHK1MAT:
// -(100 * descriptor position + entry) for a bad descriptor entry, -(position) for a bad
// sub-matrix start or grid.
int make_layout(const int* desc, int i0, int j0, int m, int n, const psmma_grid& g, int rank, int dpos, int ipos,
                int jpos, int gpos, Layout* L) {
  if (g.nprow < 1 || g.npcol < 1 || (g.order != 0 && g.order != 1)) return -gpos;
  if (rank < 0 || rank >= g.nprow * g.npcol) return -gpos;
  if (!desc) return -(100 * dpos + 1);
  if (desc[0] != 1) return -(100 * dpos + 1);
  if (desc[2] < 0) return -(100 * dpos + 3);
  if (desc[3] < 0) return -(100 * dpos + 4);
  if (desc[4] < 1) return -(100 * dpos + 5);
  if (desc[5] < 1) return -(100 * dpos + 6);
  if (desc[6] < 0 || desc[6] >= g.nprow) return -(100 * dpos + 7);
  if (desc[7] < 0 || desc[7] >= g.npcol) return -(100 * dpos + 8);
  L->M = desc[2];
  L->N = desc[3];
  L->MB = desc[4];
  L->NB = desc[5];
  L->RSRC = desc[6];
  L->CSRC = desc[7];
  L->LLD = desc[8];
  L->nprow = g.nprow;
  L->npcol = g.npcol;
  L->order = g.order;
  L->myrow = g.order == 0 ? rank / g.npcol : rank % g.nprow;
  L->mycol = g.order == 0 ? rank % g.npcol : rank / g.nprow;
  L->lrows = numroc0(L->M, L->MB, L->myrow, L->RSRC, L->nprow);
  L->lcols = numroc0(L->N, L->NB, L->mycol, L->CSRC, L->npcol);
  if (L->LLD < std::max(1, L->lrows)) return -(100 * dpos + 9);
  if (i0 < 1 || (m > 0 && (long)i0 - 1 + m > L->M)) return -ipos;
  if (j0 < 1 || (n > 0 && (long)j0 - 1 + n > L->N)) return -jpos;
  return 0;
}

// For each local index of `from` (rows or columns): the process coordinate that owns the
// same sub-matrix element in `to` (or -1 outside the sub-matrix) and its position among
// the local indices of `from` that go to that coordinate; cnt[p] counts them.
void build_map(int nloc, int nb, int me, int src, int nprocs, long sub0, long count, int nb_to, int src_to,
               int nprocs_to, long sub0_to, std::vector<int2>& map, std::vector<int>& cnt) {
  map.assign(std::max(nloc, 0), make_int2(-1, 0));
  cnt.assign(nprocs_to, 0);
  for (int l = 0; l < nloc; ++l) {
    const long g = l2g0(l, nb, me, src, nprocs) - sub0;
    if (g < 0 || g >= count) continue;
    const int p = g2p0(g + sub0_to, nb_to, src_to, nprocs_to);
    map[l] = make_int2(p, cnt[p]++);
  }
}

constexpr int RD_THREADS = 256;
constexpr int RD_COLS = 8;  // columns per block: a thread reuses its row map entry

// out[displ[peer] + cpos * rcnt[rpart] + rpos] = in[i + j * ld] for every local (i, j)
// inside the sub-matrix, peer = the rank at (rpart, cpart) of the other layout's grid.
template <typename T>
__global__ void __launch_bounds__(RD_THREADS) k_pack(const T* __restrict__ in, long ld, int lrows, int lcols,
                                                     const int2* __restrict__ rmap, const int2* __restrict__ cmap,
                                                     const int* __restrict__ rcnt,
                                                     const long long* __restrict__ displ, int npr, int npc,
                                                     int order, T* __restrict__ out) {
  const int i = blockIdx.x * RD_THREADS + threadIdx.x;
  if (i >= lrows) return;
  const int2 r = rmap[i];
  if (r.x < 0) return;
  const long long rc = rcnt[r.x];
  const int j1 = min(lcols, (int)(blockIdx.y + 1) * RD_COLS);
  for (int j = blockIdx.y * RD_COLS; j < j1; ++j) {
    const int2 c = cmap[j];
    if (c.x < 0) continue;
    const int peer = order == 0 ? r.x * npc + c.x : c.x * npr + r.x;
    out[displ[peer] + c.y * rc + r.y] = in[i + j * ld];
  }
}

// The inverse: out[i + j * ld] = in[displ[peer] + cpos * rcnt[rpart] + rpos].
template <typename T>
__global__ void __launch_bounds__(RD_THREADS) k_unpack(const T* __restrict__ in, const int2* __restrict__ rmap,
                                                       const int2* __restrict__ cmap, const int* __restrict__ rcnt,
                                                       const long long* __restrict__ displ, int npr, int npc,
                                                       int order, int lrows, int lcols, T* __restrict__ out,
                                                       long ld) {
  const int i = blockIdx.x * RD_THREADS + threadIdx.x;
  if (i >= lrows) return;
  const int2 r = rmap[i];
  if (r.x < 0) return;
  const long long rc = rcnt[r.x];
  const int j1 = min(lcols, (int)(blockIdx.y + 1) * RD_COLS);
  for (int j = blockIdx.y * RD_COLS; j < j1; ++j) {
    const int2 c = cmap[j];
    if (c.x < 0) continue;
    const int peer = order == 0 ? r.x * npc + c.x : c.x * npr + r.x;
    out[i + j * ld] = in[displ[peer] + c.y * rc + r.y];
  }
}

// Generator rows in a new order: TB(i, :) = B(perm[i] - 1, :) (Redist2P5's gather,
// Auxil_2p5D.f90:352-357).
__global__ void k_permute_rows(const double* __restrict__ B, long ldb, int ncb, int k, const int* __restrict__ perm,
                               double* __restrict__ TB, long ldtb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  const long src = perm[i] - 1;
  for (int j = 0; j < ncb; ++j) TB[i + j * ldtb] = B[src + j * ldb];
}

}  // namespace
}  // namespace psmma

using namespace psmma;

struct psmma_redist_plan {
  int m = 0, n = 0, nprocs = 0, rank = 0;
  Layout A, B;
  // pack side (this rank's local array in A's layout): maps to B's process rows / cols
  std::vector<int2> arow, acol;
  std::vector<int> arow_cnt, acol_cnt;
  // unpack side (this rank's local array in B's layout): maps to A's process rows / cols
  std::vector<int2> brow, bcol;
  std::vector<int> brow_cnt, bcol_cnt;
  std::vector<long long> send_counts, send_displ, recv_counts, recv_displ;
  // device copies, made on the first pack / unpack
  int device = -1;
  void* dmem = nullptr;
  int2 *d_arow = nullptr, *d_acol = nullptr, *d_brow = nullptr, *d_bcol = nullptr;
  int *d_arow_cnt = nullptr, *d_brow_cnt = nullptr;
  long long *d_send_displ = nullptr, *d_recv_displ = nullptr;
};

namespace {

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

int upload(psmma_redist_plan* p, cudaStream_t stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PSMMA_EDEVICE;
  if (p->dmem && p->device == dev) return PSMMA_OK;
  if (p->dmem) return PSMMA_EUNSUPPORTED;  // a plan serves the device it was first used on
  struct Part { const void* src; size_t bytes; void** dst; };
  Part parts[] = {
      {p->arow.data(), p->arow.size() * sizeof(int2), (void**)&p->d_arow},
      {p->acol.data(), p->acol.size() * sizeof(int2), (void**)&p->d_acol},
      {p->brow.data(), p->brow.size() * sizeof(int2), (void**)&p->d_brow},
      {p->bcol.data(), p->bcol.size() * sizeof(int2), (void**)&p->d_bcol},
      {p->arow_cnt.data(), p->arow_cnt.size() * sizeof(int), (void**)&p->d_arow_cnt},
      {p->brow_cnt.data(), p->brow_cnt.size() * sizeof(int), (void**)&p->d_brow_cnt},
      {p->send_displ.data(), p->send_displ.size() * sizeof(long long), (void**)&p->d_send_displ},
      {p->recv_displ.data(), p->recv_displ.size() * sizeof(long long), (void**)&p->d_recv_displ},
  };
  size_t total = 0;
  for (const Part& q : parts) total += align16(std::max<size_t>(q.bytes, 16));
  void* mem = nullptr;
  if (cudaMalloc(&mem, total) != cudaSuccess) {
    cudaGetLastError();
    return PSMMA_ENOMEM;
  }
  size_t off = 0;
  for (const Part& q : parts) {
    *q.dst = (char*)mem + off;
    if (q.bytes && cudaMemcpyAsync(*q.dst, q.src, q.bytes, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
      cudaFree(mem);
      return PSMMA_EDEVICE;
    }
    off += align16(std::max<size_t>(q.bytes, 16));
  }
  p->dmem = mem;
  p->device = dev;
  return PSMMA_OK;
}

template <typename T>
int launch_pack(const psmma_redist_plan* p, const T* A, T* out, cudaStream_t st) {
  const int lr = p->A.lrows, lc = p->A.lcols;
  if (lr == 0 || lc == 0) return PSMMA_OK;
  const unsigned gy = (unsigned)((lc + RD_COLS - 1) / RD_COLS);
  if (gy > 65535u) return PSMMA_EUNSUPPORTED;
  dim3 grid((lr + RD_THREADS - 1) / RD_THREADS, gy);
  k_pack<T><<<grid, RD_THREADS, 0, st>>>(A, p->A.LLD, lr, lc, p->d_arow, p->d_acol, p->d_arow_cnt, p->d_send_displ,
                                         p->B.nprow, p->B.npcol, p->B.order, out);
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

template <typename T>
int launch_unpack(const psmma_redist_plan* p, const T* in, T* B, cudaStream_t st) {
  const int lr = p->B.lrows, lc = p->B.lcols;
  if (lr == 0 || lc == 0) return PSMMA_OK;
  const unsigned gy = (unsigned)((lc + RD_COLS - 1) / RD_COLS);
  if (gy > 65535u) return PSMMA_EUNSUPPORTED;
  dim3 grid((lr + RD_THREADS - 1) / RD_THREADS, gy);
  k_unpack<T><<<grid, RD_THREADS, 0, st>>>(in, p->d_brow, p->d_bcol, p->d_brow_cnt, p->d_recv_displ, p->A.nprow,
                                           p->A.npcol, p->A.order, lr, lc, B, p->B.LLD);
  return cudaGetLastError() == cudaSuccess ? PSMMA_OK : PSMMA_EDEVICE;
}

}  // namespace

extern "C" {

int psmma_numroc(int n, int nb, int iproc, int isrcproc, int nprocs) {
  if (n < 0 || nb < 1 || nprocs < 1) return 0;
  return numroc0(n, nb, ((iproc % nprocs) + nprocs) % nprocs, ((isrcproc % nprocs) + nprocs) % nprocs, nprocs);
}

int psmma_redist_plan_create(int m, int n, const int* desca, int ia, int ja, psmma_grid ga, const int* descb,
                             int ib, int jb, psmma_grid gb, int rank, psmma_redist_plan** out) {
  if (!out) return -12;
  *out = nullptr;
  if (m < 0) return -1;
  if (n < 0) return -2;
  Layout LA, LB;
  int info = make_layout(desca, ia, ja, m, n, ga, rank, 3, 4, 5, 6, &LA);
  if (info) return info;
  info = make_layout(descb, ib, jb, m, n, gb, rank, 7, 8, 9, 10, &LB);
  if (info) return info;
  if (ga.nprow * ga.npcol != gb.nprow * gb.npcol) return -10;
  psmma_redist_plan* p = new (std::nothrow) psmma_redist_plan();
  if (!p) return PSMMA_ENOMEM;
  p->m = m;
  p->n = n;
  p->nprocs = ga.nprow * ga.npcol;
  p->rank = rank;
  p->A = LA;
  p->B = LB;
  // rows of my A-local array -> B's process rows; columns -> B's process columns
  build_map(LA.lrows, LA.MB, LA.myrow, LA.RSRC, LA.nprow, ia - 1, m, LB.MB, LB.RSRC, LB.nprow, ib - 1, p->arow,
            p->arow_cnt);
  build_map(LA.lcols, LA.NB, LA.mycol, LA.CSRC, LA.npcol, ja - 1, n, LB.NB, LB.CSRC, LB.npcol, jb - 1, p->acol,
            p->acol_cnt);
  // rows of my B-local array -> A's process rows; columns -> A's process columns
  build_map(LB.lrows, LB.MB, LB.myrow, LB.RSRC, LB.nprow, ib - 1, m, LA.MB, LA.RSRC, LA.nprow, ia - 1, p->brow,
            p->brow_cnt);
  build_map(LB.lcols, LB.NB, LB.mycol, LB.CSRC, LB.npcol, jb - 1, n, LA.NB, LA.CSRC, LA.npcol, ja - 1, p->bcol,
            p->bcol_cnt);
  const int P = p->nprocs;
  p->send_counts.assign(P, 0);
  p->recv_counts.assign(P, 0);
  for (int pr = 0; pr < LB.nprow; ++pr)
    for (int pc = 0; pc < LB.npcol; ++pc)
      p->send_counts[LB.rank_of(pr, pc)] = (long long)p->arow_cnt[pr] * p->acol_cnt[pc];
  for (int pr = 0; pr < LA.nprow; ++pr)
    for (int pc = 0; pc < LA.npcol; ++pc)
      p->recv_counts[LA.rank_of(pr, pc)] = (long long)p->brow_cnt[pr] * p->bcol_cnt[pc];
  p->send_displ.assign(P, 0);
  p->recv_displ.assign(P, 0);
  for (int q = 1; q < P; ++q) {
    p->send_displ[q] = p->send_displ[q - 1] + p->send_counts[q - 1];
    p->recv_displ[q] = p->recv_displ[q - 1] + p->recv_counts[q - 1];
  }
  *out = p;
  return PSMMA_OK;
}

int psmma_redist_counts(const psmma_redist_plan* p, long long* send_counts, long long* recv_counts) {
  if (!p) return -1;
  if (send_counts) std::memcpy(send_counts, p->send_counts.data(), sizeof(long long) * p->nprocs);
  if (recv_counts) std::memcpy(recv_counts, p->recv_counts.data(), sizeof(long long) * p->nprocs);
  return PSMMA_OK;
}

int psmma_redist_local_shape(const psmma_redist_plan* p, int* a_rows, int* a_cols, int* b_rows, int* b_cols) {
  if (!p) return -1;
  if (a_rows) *a_rows = p->A.lrows;
  if (a_cols) *a_cols = p->A.lcols;
  if (b_rows) *b_rows = p->B.lrows;
  if (b_cols) *b_cols = p->B.lcols;
  return PSMMA_OK;
}

int psmma_redist_maps(const psmma_redist_plan* p, int which, int* part, int* pos) {
  if (!p) return -1;
  const std::vector<int2>* v = which == 0 ? &p->arow : which == 1 ? &p->acol : which == 2 ? &p->brow
                             : which == 3 ? &p->bcol : nullptr;
  if (!v) return -2;
  for (size_t i = 0; i < v->size(); ++i) {
    if (part) part[i] = (*v)[i].x;
    if (pos) pos[i] = (*v)[i].y;
  }
  return (int)v->size();
}

int psmma_redist_pack(psmma_redist_plan* p, const void* A, void* sendbuf, int elem_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!p) return -1;
  if (elem_bytes != 8 && elem_bytes != 16) return -4;
  long long total = 0;
  for (long long c : p->send_counts) total += c;
  if (total == 0) return PSMMA_OK;
  if (!A) return -2;
  if (!sendbuf) return -3;
  int st = upload(p, stream);
  if (st) return st;
  return elem_bytes == 8 ? launch_pack(p, (const double*)A, (double*)sendbuf, stream)
                         : launch_pack(p, (const double2*)A, (double2*)sendbuf, stream);
}

int psmma_redist_unpack(psmma_redist_plan* p, const void* recvbuf, void* B, int elem_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!p) return -1;
  if (elem_bytes != 8 && elem_bytes != 16) return -4;
  long long total = 0;
  for (long long c : p->recv_counts) total += c;
  if (total == 0) return PSMMA_OK;
  if (!recvbuf) return -2;
  if (!B) return -3;
  int st = upload(p, stream);
  if (st) return st;
  return elem_bytes == 8 ? launch_unpack(p, (const double*)recvbuf, (double*)B, stream)
                         : launch_unpack(p, (const double2*)recvbuf, (double2*)B, stream);
}

int psmma_redist_plan_destroy(psmma_redist_plan* p) {
  if (!p) return PSMMA_OK;
  if (p->dmem) {
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != p->device) cudaSetDevice(p->device);
    cudaFree(p->dmem);
    if (cur != p->device) cudaSetDevice(cur);
  }
  delete p;
  return PSMMA_OK;
}

// ---- 2.5D index helpers (Auxil_2p5D.f90:315-459) ---------------------------------------

// Redist2P5a (Auxil_2p5D.f90:362-390): the 1-based global indices 1..k ordered by process
// column, the columns taken as I + J * (npcol / npzc) for I < npcol / npzc (outer) and
// J < npzc (inner), each contributing its block-cyclic slice (ConstIndex) in order.
int psmma_redist2p5_index(int k, int nb, int npzc, int npcol, int* pindex) {
  if (k < 0) return -1;
  if (nb < 1) return -2;
  if (npzc < 1) return -3;
  if (npcol < 1) return -4;
  if (npcol % npzc != 0) return -3;  // the reference prints "NPZC must divide NPCOL" and returns
  if (k > 0 && !pindex) return -5;
  const int lnpcol = npcol / npzc;
  int t = 0;
  for (int i = 0; i < lnpcol; ++i)
    for (int j = 0; j < npzc; ++j) {
      const int col = i + j * lnpcol;
      const int loc = numroc0(k, nb, col, 0, npcol);
      for (int l = 0; l < loc; ++l) pindex[t++] = (int)l2g0(l, nb, col, 0, npcol) + 1;
    }
  return t == k ? PSMMA_OK : PSMMA_EDEVICE;
}

// ConstIndex1 (Auxil_2p5D.f90:392-419): process column mycol's full block segments of a
// permuted index list, cindex = pindex(mycol*nb + s*npcol*nb + (1..nb)) for the first
// ICEIL(n, nb) / npcol segments.  Where that count includes a partial last block the
// reference reads pindex past n; here the segment stops at n.  Returns the count written.
int psmma_const_index1(int n, int nb, int mycol, int npcol, const int* pindex, int* cindex) {
  if (n < 0 || nb < 1 || npcol < 1 || mycol < 0 || mycol >= npcol) return -1;
  const int knb = (n + nb - 1) / nb;
  const int nfseg = knb / npcol;
  long start = (long)mycol * nb;
  int t = 0;
  for (int s = 0; s < nfseg; ++s, start += (long)npcol * nb)
    for (int l = 0; l < nb && start + l < n; ++l) cindex[t++] = pindex[start + l];
  return t;
}

// Redist2P5 (Auxil_2p5D.f90:315-360) on the device: TB(i, :) = B(pindex(i), :) for the
// 2.5D order of the generator rows, i < k, ncb columns.
int psmma_redist2p5(int k, int nb, int npzc, int npcol, const double* B, int ldb, int ncb, double* TB, int ldtb,
                    void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (k < 0) return -1;
  if (ncb < 0) return -7;
  if (ldb < std::max(1, k)) return -6;
  if (ldtb < std::max(1, k)) return -9;
  std::vector<int> h(std::max(k, 1));
  int st = psmma_redist2p5_index(k, nb, npzc, npcol, h.data());
  if (st) return st;
  if (k == 0 || ncb == 0) return PSMMA_OK;
  if (!B || !TB) return PSMMA_ENULL;
  int* d = nullptr;
  if (cudaMallocAsync((void**)&d, sizeof(int) * k, stream) != cudaSuccess) {
    cudaGetLastError();
    return PSMMA_ENOMEM;
  }
  if (cudaMemcpyAsync(d, h.data(), sizeof(int) * k, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
    cudaFreeAsync(d, stream);
    return PSMMA_EDEVICE;
  }
  k_permute_rows<<<(k + 255) / 256, 256, 0, stream>>>(B, ldb, ncb, k, d, TB, ldtb);
  const bool ok = cudaGetLastError() == cudaSuccess;
  // the pageable copy above is staged before cudaMemcpyAsync returns; h may go
  cudaFreeAsync(d, stream);
  return ok ? PSMMA_OK : PSMMA_EDEVICE;
}

}  // extern "C"
