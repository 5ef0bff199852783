"""Descriptor interop: the reference's routines on a block-cyclic matrix spread over an
NPROW x NPCOL process grid, one GPU per process.

The reference takes A and Q as local pieces of ScaLAPACK block-cyclic matrices (DESCA, DESCQ)
and, with REDIST = .TRUE., copies A to a blocked layout and Q back with PDGEMR2D
(psmma_cauchy.f90:113-162).  Its multiply then shifts blocks of A around the process grid
(the SPMMA ring of PSCAUCHY_COMPUTE).  On GB300 the whole product of a row panel
Q[I, :] = alpha * A[I, :] * H + beta * Q[I, :] fits one GPU and needs only the replicated
O(k) generators, so the distributed call here is:

1. redistribute A (and Q when beta != 0) from the caller's layout to row panels over all
   ranks (an NPROCS x 1 grid) -- one all-to-all, packed and unpacked by the library's GPU
   kernels (:class:`RedistPlan`);
2. multiply each panel on its GPU (``psmma_<kind>``) with no further exchange;
3. redistribute the Q panels back to the caller's layout -- one all-to-all.

When the caller's grid already has one process column and Q's rows are distributed like A's,
step 1 and 3 are skipped: every rank multiplies its local rows in place.  The DFT multiply
(F on the left) uses column panels instead.

Semantics kept from the reference: A is read from its (1,1) element (IA, JA are ignored, as
both branches of psmma_cauchy.f90 do); with ``redist=True`` Q is written at (IQ, JQ) of the
DESCQ layout (psmma_cauchy.f90:157); with ``redist=False`` Q has A's distribution and DESCQ's
leading dimension, and IQ, JQ are ignored (psmma_cauchy.f90:99-101 passes only DESCA and LDQ).

The exchange is ``torch.distributed.all_to_all_single`` by default (NCCL on GPUs); any callable
with the same contract can replace it (``exchange=``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import PsmmaError, PsmmaGrid, load

__all__ = ["Grid", "numroc", "descinit", "local_shape", "RedistPlan", "redistribute", "all_to_all",
           "pstructured", "pzmdftl_distributed", "redist2p5_index", "redist2p5", "const_index1"]


@dataclass(frozen=True)
class Grid:
    """A BLACS process grid: ``order`` 'R' numbers ranks row-major (BLACS_GRIDINIT 'R', the
    reference tests' choice, Test/psmma_testcauchy.f90:77), 'C' column-major."""
    nprow: int
    npcol: int
    order: str = "R"

    @property
    def nprocs(self) -> int:
        return self.nprow * self.npcol

    @property
    def row_major(self) -> bool:
        return self.order.upper().startswith("R")

    def coords(self, rank: int) -> tuple[int, int]:
        if self.row_major:
            return rank // self.npcol, rank % self.npcol
        return rank % self.nprow, rank // self.nprow

    def rank_of(self, prow: int, pcol: int) -> int:
        return prow * self.npcol + pcol if self.row_major else pcol * self.nprow + prow

    def c(self) -> PsmmaGrid:
        return PsmmaGrid(self.nprow, self.npcol, 0 if self.row_major else 1)


def numroc(n: int, nb: int, iproc: int, isrcproc: int, nprocs: int) -> int:
    """ScaLAPACK NUMROC (0-based process numbers), from the library."""
    return int(load().psmma_numroc(n, nb, iproc, isrcproc, nprocs))


def descinit(m: int, n: int, mb: int, nb: int, rsrc: int, csrc: int, grid: Grid, rank: int,
             lld: int | None = None) -> tuple:
    """ScaLAPACK DESCINIT's descriptor (CTXT_ unused): LLD defaults to max(1, local rows)."""
    pr, _ = grid.coords(rank)
    if lld is None:
        lld = max(1, numroc(m, mb, pr, rsrc, grid.nprow))
    return (1, 0, m, n, mb, nb, rsrc, csrc, lld)


def local_shape(desc, grid: Grid, rank: int) -> tuple[int, int]:
    pr, pc = grid.coords(rank)
    return (numroc(desc[2], desc[4], pr, desc[6], grid.nprow), numroc(desc[3], desc[5], pc, desc[7], grid.npcol))


def _desc_arr(desc):
    if len(desc) != 9:
        raise ValueError("a descriptor has 9 entries")
    return (C.c_int * 9)(*[int(x) for x in desc])


class RedistPlan:
    """PDGEMR2D's copy of the sub-matrix A(ia:ia+m-1, ja:ja+n-1) of layout (desca, grid_a) to
    B(ib:..., jb:...) of layout (descb, grid_b), seen from one rank: per-peer counts, and the
    GPU pack / unpack around one all-to-all (psmma_redist_* in include/psmma.h)."""

    def __init__(self, m: int, n: int, desca, grid_a: Grid, descb, grid_b: Grid, rank: int,
                 ia: int = 1, ja: int = 1, ib: int = 1, jb: int = 1):
        lib = load()
        self._lib = lib
        self.m, self.n, self.rank = m, n, rank
        self.desca, self.descb = tuple(desca), tuple(descb)
        self.grid_a, self.grid_b = grid_a, grid_b
        h = C.c_void_p()
        st = lib.psmma_redist_plan_create(m, n, _desc_arr(desca), ia, ja, grid_a.c(), _desc_arr(descb), ib, jb,
                                          grid_b.c(), rank, C.byref(h))
        if st != 0:
            raise PsmmaError(st, "psmma_redist_plan_create")
        self._h = h
        P = grid_a.nprocs
        sc, rc = (C.c_longlong * P)(), (C.c_longlong * P)()
        lib.psmma_redist_counts(h, sc, rc)
        self.send_counts = [int(x) for x in sc]
        self.recv_counts = [int(x) for x in rc]
        a_r, a_c, b_r, b_c = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        lib.psmma_redist_local_shape(h, C.byref(a_r), C.byref(a_c), C.byref(b_r), C.byref(b_c))
        self.a_shape = (a_r.value, a_c.value)
        self.b_shape = (b_r.value, b_c.value)

    def maps(self, which: int) -> tuple[np.ndarray, np.ndarray]:
        """(part, pos) of map ``which`` (0/1: rows/cols of the a-local array, 2/3: of the
        b-local array)."""
        cnt = self._lib.psmma_redist_maps(self._h, which, None, None)
        part = np.zeros(max(cnt, 1), dtype=np.int32)
        pos = np.zeros(max(cnt, 1), dtype=np.int32)
        self._lib.psmma_redist_maps(self._h, which, part.ctypes.data_as(C.POINTER(C.c_int)),
                                    pos.ctypes.data_as(C.POINTER(C.c_int)))
        return part[:cnt], pos[:cnt]

    @staticmethod
    def _check_local(x, ld: int, shape, name: str):
        import torch
        if not x.is_cuda:
            raise ValueError(f"{name}: expected a CUDA tensor")
        if x.dtype not in (torch.float64, torch.complex128):
            raise TypeError(f"{name}: expected float64 or complex128, got {x.dtype}")
        if x.dim() != 2 or tuple(x.shape) != tuple(shape):
            raise ValueError(f"{name}: local array of shape {tuple(shape)} expected, got {tuple(x.shape)}")
        if shape[0] > 1 and x.stride(0) != 1:
            raise ValueError(f"{name}: expected a column-major local array (stride(0) == 1)")
        if shape[1] > 1 and x.stride(1) != ld:
            raise ValueError(f"{name}: leading dimension {x.stride(1)} differs from the descriptor's LLD {ld}")

    @staticmethod
    def _check_buf(buf, like, count: int, name: str):
        if not buf.is_cuda or buf.dtype != like.dtype or buf.device != like.device:
            raise ValueError(f"{name}: expected a CUDA {like.dtype} tensor on {like.device}")
        if not buf.is_contiguous() or buf.numel() < count:
            raise ValueError(f"{name}: expected a contiguous buffer of at least {count} elements")

    def pack(self, A_local, sendbuf, stream=None):
        """Gathers this rank's elements of A into ``sendbuf`` (segments in rank order)."""
        from . import _stream_ptr
        self._check_local(A_local, self.desca[8], self.a_shape, "A")
        self._check_buf(sendbuf, A_local, sum(self.send_counts), "sendbuf")
        eb = A_local.element_size()
        st = self._lib.psmma_redist_pack(self._h, C.c_void_p(A_local.data_ptr()), C.c_void_p(sendbuf.data_ptr()),
                                         eb, _stream_ptr(stream))
        if st != 0:
            raise PsmmaError(st, "psmma_redist_pack")

    def unpack(self, recvbuf, B_local, stream=None):
        """Scatters the received segments into this rank's local array of B."""
        from . import _stream_ptr
        self._check_local(B_local, self.descb[8], self.b_shape, "B")
        self._check_buf(recvbuf, B_local, sum(self.recv_counts), "recvbuf")
        eb = B_local.element_size()
        st = self._lib.psmma_redist_unpack(self._h, C.c_void_p(recvbuf.data_ptr()), C.c_void_p(B_local.data_ptr()),
                                           eb, _stream_ptr(stream))
        if st != 0:
            raise PsmmaError(st, "psmma_redist_unpack")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.psmma_redist_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuMover:
    """Pack / unpack on the GPU (the library's kernels)."""

    @staticmethod
    def pack(plan: RedistPlan, A_local, sendbuf):
        plan.pack(A_local, sendbuf)

    @staticmethod
    def unpack(plan: RedistPlan, recvbuf, B_local):
        plan.unpack(recvbuf, B_local)


def all_to_all(send, send_counts, recv, recv_counts, group=None):
    """One all-to-all with per-rank element counts (torch.distributed; NCCL on GPUs).
    Complex buffers travel as their float64 view."""
    import torch
    import torch.distributed as dist
    f = 1
    if send.is_complex():
        send, recv, f = torch.view_as_real(send).reshape(-1), torch.view_as_real(recv).reshape(-1), 2
    dist.all_to_all_single(recv, send, [c * f for c in recv_counts], [c * f for c in send_counts], group=group)


def redistribute(plan: RedistPlan, A_local, B_local, *, exchange=None, group=None, mover=None):
    """B_local := this rank's part of B after PDGEMR2D of A (pack, one all-to-all, unpack)."""
    import torch
    exchange = exchange or all_to_all
    mover = mover or GpuMover
    ref = A_local if A_local is not None else B_local
    send = torch.empty(max(sum(plan.send_counts), 1), dtype=ref.dtype, device=ref.device)
    recv = torch.empty(max(sum(plan.recv_counts), 1), dtype=ref.dtype, device=ref.device)
    if sum(plan.send_counts):
        mover.pack(plan, A_local, send)
    exchange(send[:sum(plan.send_counts)], plan.send_counts, recv[:sum(plan.recv_counts)], plan.recv_counts,
             group)
    if sum(plan.recv_counts):
        mover.unpack(plan, recv, B_local)
    return B_local


_PLANS: dict = {}


def _plan(m, n, desca, grid_a, descb, grid_b, rank, ia=1, ja=1, ib=1, jb=1) -> RedistPlan:
    key = (m, n, tuple(desca), grid_a, tuple(descb), grid_b, rank, ia, ja, ib, jb)
    p = _PLANS.get(key)
    if p is None:
        if len(_PLANS) >= 64:
            _PLANS.pop(next(iter(_PLANS))).close()
        p = _PLANS[key] = RedistPlan(m, n, desca, grid_a, descb, grid_b, rank, ia, ja, ib, jb)
    return p


def _local_empty(desc, grid: Grid, rank: int, like):
    import torch
    r, c = local_shape(desc, grid, rank)
    base = torch.zeros((max(c, 1), desc[8]), dtype=like.dtype, device=like.device)
    return base.t()[:r, :c]


def _panel_layout(n: int, k: int, nprocs: int, rank: int, by_rows: bool = True):
    """Row panels (NPROCS x 1 grid, blocks of ceil(n / NPROCS) rows) or column panels."""
    if by_rows:
        g = Grid(nprocs, 1, "R")
        mb = max(1, -(-n // nprocs))
        return g, descinit(n, k, mb, max(1, k), 0, 0, g, rank)
    g = Grid(1, nprocs, "R")
    nb = max(1, -(-k // nprocs))
    return g, (1, 0, n, k, max(1, n), nb, 0, 0, max(1, n))


def _library_compute(kind: str, precision, n_moduli):
    import psmma_git_gb300 as P
    if kind == "cauchyeig":
        def run(rows, k, alpha, A, gen, beta, Q):
            F, U, V, difl, difr = gen
            return P.psmma_cauchyeig(rows, k, alpha, A, F, U, V, difl, difr, beta, Q, precision=precision,
                                     n_moduli=n_moduli)
        return run
    fn = getattr(P, "psmma_" + kind)
    return lambda rows, k, alpha, A, gen, beta, Q: fn(rows, k, alpha, A, gen, beta, Q, precision=precision,
                                                      n_moduli=n_moduli)


def pstructured(kind: str, n: int, k: int, alpha: float, A_local, desca, gen, beta: float, Q_local, descq,
                grid: Grid, rank: int, *, iq: int = 1, jq: int = 1, redist: bool = True,
                precision="split", n_moduli: int = 0, group=None, exchange=None, mover=None, compute=None):
    """PSMMA_CAUCHY / TOEPLITZ / HANKEL / CAUCHYEIG (kind 'cauchy', 'toeplitz', 'hankel',
    'cauchyeig') on this rank's local pieces of A (n x k, layout desca) and Q (layout descq),
    grid ``grid``.  ``gen`` is the replicated generator operand of the single-GPU call
    (for 'cauchyeig' the tuple (F, U, V, DIFL, DIFR)).  Returns Q_local."""
    if kind not in ("cauchy", "toeplitz", "hankel", "cauchyeig"):
        raise ValueError(f"unknown kind {kind!r}")
    if n < 0:
        raise PsmmaError(-2, "pstructured")
    if k < 0:
        raise PsmmaError(-3, "pstructured")
    # descriptor extents (INFO as ScaLAPACK: -(100 * position + entry), DESCA is argument 7,
    # DESCQ argument 14 of PSMMA_CAUCHY)
    if desca[2] < n:
        raise PsmmaError(-703, "pstructured")
    if desca[3] < k:
        raise PsmmaError(-704, "pstructured")
    compute = compute or _library_compute(kind, precision, n_moduli)
    if not redist:
        # Q shares A's distribution, with DESCQ's leading dimension; IQ, JQ are ignored
        descq = tuple(desca[:8]) + (descq[8],)
        iq = jq = 1
    if descq[2] < iq - 1 + n:
        raise PsmmaError(-1403, "pstructured")
    if descq[3] < jq - 1 + k:
        raise PsmmaError(-1404, "pstructured")
    if n == 0 or k == 0:
        return Q_local
    pr, pc = grid.coords(rank)
    same_rows = (grid.npcol == 1 and desca[4] == descq[4] and desca[6] == descq[6] and iq == 1)
    if same_rows:
        # one process column: every rank holds whole rows of A and of Q; multiply in place
        rows = numroc(n, desca[4], pr, desca[6], grid.nprow)
        if rows:
            compute(rows, k, alpha, A_local[:rows, :k], gen, beta, Q_local[:rows, jq - 1:jq - 1 + k])
        return Q_local
    gT, dT = _panel_layout(n, k, grid.nprocs, rank)
    pA = _plan(n, k, desca, grid, dT, gT, rank)
    A_T = _local_empty(dT, gT, rank, A_local)
    redistribute(pA, A_local, A_T, exchange=exchange, group=group, mover=mover)
    Q_T = _local_empty(dT, gT, rank, A_local)
    if beta != 0.0:
        pQin = _plan(n, k, descq, grid, dT, gT, rank, ia=iq, ja=jq)
        redistribute(pQin, Q_local, Q_T, exchange=exchange, group=group, mover=mover)
    rows = Q_T.shape[0]
    if rows:
        compute(rows, k, alpha, A_T, gen, beta, Q_T)
    pQ = _plan(n, k, dT, gT, descq, grid, rank, ib=iq, jb=jq)
    redistribute(pQ, Q_T, Q_local, exchange=exchange, group=group, mover=mover)
    return Q_local


def pzmdftl_distributed(n: int, k: int, nb: int, kb: int, alpha: float, B_local, beta: float, C_local,
                        imrow: int, imcol: int, grid: Grid, rank: int, *, precision="split", n_moduli: int = 0,
                        group=None, exchange=None, mover=None, compute=None):
    """PZMDFTL (pzmdftL.f90:1-2) on a block-cyclic B and C (N x K, blocks NB x KB, first block on
    process (IMROW, IMCOL)): C := alpha * F * B + beta * C by column panels.  The local arrays'
    leading dimensions are their column strides.  Returns C_local."""
    if n < 0:
        raise PsmmaError(-1, "pzmdftl_distributed")
    if k < 0:
        raise PsmmaError(-2, "pzmdftl_distributed")
    if n == 0 or k == 0:
        return C_local
    if compute is None:
        import psmma_git_gb300 as lib

        def compute(cols, alpha_, B, beta_, Cm):
            return lib.pzmdftl(n, cols, alpha_, B, beta_, Cm, precision=precision, n_moduli=n_moduli)
    pr, _ = grid.coords(rank)
    lrows = numroc(n, nb, pr, imrow, grid.nprow)
    ldb = B_local.stride(1) if B_local.dim() == 2 and B_local.shape[1] > 1 else max(1, lrows)
    ldc = C_local.stride(1) if C_local.dim() == 2 and C_local.shape[1] > 1 else max(1, lrows)
    dB = (1, 0, n, k, nb, kb, imrow, imcol, ldb)
    dC = (1, 0, n, k, nb, kb, imrow, imcol, ldc)
    if grid.nprow == 1:
        # one process row: every rank holds whole columns; multiply in place
        cols = B_local.shape[1]
        if cols:
            compute(cols, alpha, B_local, beta, C_local)
        return C_local
    gT, dT = _panel_layout(n, k, grid.nprocs, rank, by_rows=False)
    B_T = _local_empty(dT, gT, rank, B_local)
    redistribute(_plan(n, k, dB, grid, dT, gT, rank), B_local, B_T, exchange=exchange, group=group, mover=mover)
    C_T = _local_empty(dT, gT, rank, B_local)
    if beta != 0.0:
        redistribute(_plan(n, k, dC, grid, dT, gT, rank), C_local, C_T, exchange=exchange, group=group,
                     mover=mover)
    cols = C_T.shape[1]
    if cols:
        compute(cols, alpha, B_T, beta, C_T)
    redistribute(_plan(n, k, dT, gT, dC, grid, rank), C_T, C_local, exchange=exchange, group=group, mover=mover)
    return C_local


# ---- 2.5D helpers (Auxil_2p5D.f90:315-419) ---------------------------------------------
def redist2p5_index(k: int, nb: int, npzc: int, npcol: int) -> np.ndarray:
    """Redist2P5a: the 1-based indices 1..k in the 2.5D process-column order."""
    out = np.zeros(max(k, 1), dtype=np.int32)
    st = load().psmma_redist2p5_index(k, nb, npzc, npcol, out.ctypes.data_as(C.POINTER(C.c_int)))
    if st != 0:
        raise PsmmaError(st, "psmma_redist2p5_index")
    return out[:k]


def const_index1(n: int, nb: int, mycol: int, npcol: int, pindex: np.ndarray) -> np.ndarray:
    """ConstIndex1: process column mycol's full block segments of a permuted index list."""
    p = np.ascontiguousarray(pindex, dtype=np.int32)
    out = np.zeros(max(n, 1), dtype=np.int32)
    cnt = load().psmma_const_index1(n, nb, mycol, npcol, p.ctypes.data_as(C.POINTER(C.c_int)),
                                    out.ctypes.data_as(C.POINTER(C.c_int)))
    if cnt < 0:
        raise PsmmaError(cnt, "psmma_const_index1")
    return out[:cnt]


def redist2p5(k: int, nb: int, npzc: int, npcol: int, B, TB=None, stream=None):
    """Redist2P5 on the device: TB(i, :) = B(pindex(i), :) for a column-major CUDA tensor B
    (k x ncb, e.g. the Cauchy generators [D|F|U|V]).  Returns TB."""
    import torch
    from . import _stream_ptr, fortran_empty
    if not B.is_cuda or B.dtype != torch.float64:
        raise TypeError("B: expected a CUDA float64 tensor")
    ncb = B.shape[1]
    ldb = B.stride(1) if ncb > 1 else max(1, B.shape[0])
    if TB is None:
        TB = fortran_empty(k, ncb, torch.float64, B.device)
    ldtb = TB.stride(1) if ncb > 1 else max(1, TB.shape[0])
    st = load().psmma_redist2p5(k, nb, npzc, npcol, C.c_void_p(B.data_ptr()), ldb, ncb, C.c_void_p(TB.data_ptr()),
                                ldtb, _stream_ptr(stream))
    if st != 0:
        raise PsmmaError(st, "psmma_redist2p5")
    return TB
