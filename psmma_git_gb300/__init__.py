"""psmma_git_gb300 -- PSMMA's structured multiply on one GB300 (sm_103a).

Python mirror of the reference's public routines, calling the C ABI of
``libpsmma_gb300.so`` (include/psmma.h) through ctypes:

* :func:`psmma_cauchy`   -- PSMMA_CAUCHY   (psmma_cauchy.f90:2-3):   Q := alpha*A*H + beta*Q,
  H(i,j) = U(i)*V(j)/(D(i)-F(j)), generators ``[D|F|U|V]`` as a (ldgen x 4) array.
* :func:`psmma_toeplitz` -- PSMMA_TOEPLITZ (psmma_toeplitz.f90:2-3): H(i,j) = G(K+j-i).
* :func:`psmma_hankel`   -- PSMMA_HANKEL   (psmma_hankel.f90:2-3):   H(i,j) = G(i+j-1).
* :func:`pzmdftl` / :func:`pzmdftl1` -- PZMDFTL / PZMDFTL1 (pzmdftL.f90:1-2):
  C := alpha*F*B + beta*C with F the N-by-N DFT matrix, w = exp(-2*pi*i/N).
* :func:`psmma_cauchyeig` -- PSMMA_CAUCHYEIG (psmma_cauchyeig.f90:2-3): the eigensolver's Cauchy
  multiply with accurate denominators (F(i) - F(j)) - DIFL(j) / (F(i) - F(j+1)) - DIFR(j).
* :func:`cauchy_batch_lowrank` -- the low-rank branch of PSCAUCHY_COMPUTE
  (pscauchy_compute.f90:371-391) for a batch of Cauchy multiplies: off-diagonal blocks
  compressed by RRQR (Compress_RRQR) or the structured RRLU (compress_cauchy).

Matrices are column-major.  Device operands are ``torch`` CUDA tensors with unit row
stride (``t.stride(0) == 1``, leading dimension ``t.stride(1)``), as made by
:func:`fortran_empty`; host operands are Fortran-ordered ``numpy`` arrays, which take the
copy-in/compute/copy-out path.  Errors raise :class:`PsmmaError` carrying the status code
(argument errors use the reference's PXERBLA INFO numbers, negated).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (COMPRESS_RRLU, COMPRESS_RRQR, KIND_CAUCHY, KIND_DFT, KIND_HANKEL, KIND_TOEPLITZ,
                   PREC_FP64, PREC_SPLIT, PsmmaBatchItem, PsmmaBatchStats, PsmmaError, PsmmaOpts,
                   PsmmaTuneResult, load, status_string)

__all__ = [
    "psmma_cauchy", "psmma_toeplitz", "psmma_hankel", "pzmdftl", "pzmdftl1", "fortran_empty",
    "workspace_size", "PsmmaError", "PREC_FP64", "PREC_SPLIT", "load", "status_string",
    "make_opts", "psmma_cauchyeig", "cauchy_batch_lowrank", "batch_workspace_size", "tune_batch",
    "toeplitz_batch_lowrank", "stream_status",
]

_PREC = {"fp64": PREC_FP64, "split": PREC_SPLIT, PREC_FP64: PREC_FP64, PREC_SPLIT: PREC_SPLIT}


def make_opts(precision="fp64", n_moduli: int = 0, work=None, lwork: int = 0, block_levels: int = 0) -> PsmmaOpts:
    o = PsmmaOpts()
    o.precision = _PREC[precision]
    o.n_moduli = n_moduli
    o.block_levels = block_levels
    if work is not None:
        o.work = C.c_void_p(work.data_ptr())
        o.lwork = lwork or work.numel() * work.element_size()
    return o


def fortran_empty(n: int, k: int, dtype=None, device="cuda", ld: int | None = None):
    """A column-major (n x k) torch tensor with leading dimension ``ld`` (default n)."""
    import torch
    ld = n if ld is None else ld
    dtype = dtype or torch.float64
    base = torch.empty((k, max(ld, 1)), dtype=dtype, device=device)
    return base.t()[:n, :]


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _dev(x, name: str, dtype):
    """(pointer, leading dimension) of a column-major CUDA tensor."""
    import torch
    if not x.is_cuda:
        raise ValueError(f"{name}: expected a CUDA tensor")
    if x.dtype != dtype:
        raise TypeError(f"{name}: expected {dtype}, got {x.dtype}")
    if x.dim() == 1:
        return x.data_ptr(), x.numel()
    if x.dim() != 2 or (x.stride(0) != 1 and x.shape[0] > 1):
        raise ValueError(f"{name}: expected a column-major 2-D tensor (stride(0) == 1)")
    ld = x.stride(1) if x.shape[1] > 1 else max(x.shape[0], 1)
    return x.data_ptr(), ld


def _host(x, name: str, dtype):
    if not isinstance(x, np.ndarray) or x.dtype != dtype:
        raise TypeError(f"{name}: expected a numpy {np.dtype(dtype)} array")
    if x.ndim == 1:
        return x.ctypes.data, x.size
    if not x.flags.f_contiguous and x.shape[0] > 1 and x.shape[1] > 1:
        # column-major with a leading dimension: a Fortran-ordered view of a larger array
        if x.strides[0] != x.itemsize:
            raise ValueError(f"{name}: expected a column-major (Fortran-ordered) array")
    ld = x.strides[1] // x.itemsize if x.shape[1] > 1 else max(x.shape[0], 1)
    return x.ctypes.data, ld


def _stream_ptr(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _real(kind: int, name: str, n, k, alpha, A, gen, beta, Q, precision, n_moduli, stream, work, block_levels=0):
    lib = load()
    opts = make_opts(precision, n_moduli, work, block_levels=block_levels)
    if _is_torch(Q):
        import torch
        pa, lda = _dev(A, "A", torch.float64) if A is not None else (0, max(1, n))
        pg, ldg = (0, 0) if gen is None else _dev(gen, "gen", torch.float64)
        if gen is not None and kind == KIND_CAUCHY and gen.dim() == 1:
            ldg = gen.numel() // 4
        pq, ldq = _dev(Q, "Q", torch.float64)
        fn = getattr(lib, name)
        st = fn(n, k, float(alpha), C.c_void_p(pa), lda, C.c_void_p(pg), ldg, float(beta),
                C.c_void_p(pq), ldq, C.byref(opts), _stream_ptr(stream))
    else:
        pa, lda = _host(A, "A", np.float64) if A is not None else (0, max(1, n))
        pg, ldg = (0, 0) if gen is None else _host(gen, "gen", np.float64)
        if gen is not None and kind == KIND_CAUCHY and gen.ndim == 1:
            ldg = gen.size // 4
        pq, ldq = _host(Q, "Q", np.float64)
        fn = getattr(lib, name + "_host")
        st = fn(n, k, float(alpha), C.c_void_p(pa), lda, C.c_void_p(pg), ldg, float(beta),
                C.c_void_p(pq), ldq, C.byref(opts))
    if st != 0:
        raise PsmmaError(st, name)
    return Q


def psmma_cauchy(n, k, alpha, A, gen, beta, Q, *, precision="fp64", n_moduli=0, stream=None, work=None,
                 block_levels=0):
    """Q := alpha*A*H + beta*Q with H(i,j) = U(i)*V(j)/(D(i)-F(j)), gen = [D|F|U|V].  block_levels:
    the split path's Strassen step on the residue planes (0 = automatic, -1 = none, 1 = one)."""
    return _real(KIND_CAUCHY, "psmma_cauchy", n, k, alpha, A, gen, beta, Q, precision, n_moduli, stream, work,
                 block_levels)


def psmma_toeplitz(n, k, alpha, A, gen, beta, Q, *, precision="fp64", n_moduli=0, stream=None, work=None,
                   block_levels=0):
    """Q := alpha*A*H + beta*Q with H(i,j) = G(K+j-i) (1-based), len(G) = 2K-1.  block_levels:
    the split path's block step (0 = automatic, -1 = none, 1..3 = that many levels)."""
    return _real(KIND_TOEPLITZ, "psmma_toeplitz", n, k, alpha, A, gen, beta, Q, precision, n_moduli, stream, work,
                 block_levels)


def psmma_hankel(n, k, alpha, A, gen, beta, Q, *, precision="fp64", n_moduli=0, stream=None, work=None,
                 block_levels=0):
    """Q := alpha*A*H + beta*Q with H(i,j) = G(i+j-1) (1-based), len(G) = 2K-1.  block_levels as
    for psmma_toeplitz."""
    return _real(KIND_HANKEL, "psmma_hankel", n, k, alpha, A, gen, beta, Q, precision, n_moduli, stream, work,
                 block_levels)


def _dft(name: str, n, k, alpha, B, beta, Cm, stream, work, precision="fp64", n_moduli=0):
    lib = load()
    opts = make_opts(precision, n_moduli, work)
    if _is_torch(Cm):
        import torch
        pb, ldb = _dev(B, "B", torch.complex128) if B is not None else (0, max(1, n))
        pc, ldc = _dev(Cm, "C", torch.complex128)
        st = getattr(lib, name)(n, k, float(alpha), C.c_void_p(pb), ldb, float(beta), C.c_void_p(pc),
                                ldc, C.byref(opts), _stream_ptr(stream))
    else:
        pb, ldb = _host(B, "B", np.complex128) if B is not None else (0, max(1, n))
        pc, ldc = _host(Cm, "C", np.complex128)
        st = lib.pzmdftl_host(n, k, float(alpha), C.c_void_p(pb), ldb, float(beta), C.c_void_p(pc),
                              ldc, C.byref(opts))
    if st != 0:
        raise PsmmaError(st, name)
    return Cm


def pzmdftl(n, k, alpha, B, beta, Cm, *, precision="fp64", n_moduli=0, stream=None, work=None):
    """C := alpha*F*B + beta*C, F(j,l) = exp(-2*pi*i*(j-1)*(l-1)/N), F on the left."""
    return _dft("pzmdftl", n, k, alpha, B, beta, Cm, stream, work, precision, n_moduli)


def pzmdftl1(n, k, alpha, B, beta, Cm, *, precision="fp64", n_moduli=0, stream=None, work=None):
    """PZMDFTL1 (RRQR variant in the reference); the same exact product here."""
    return _dft("pzmdftl1", n, k, alpha, B, beta, Cm, stream, work, precision, n_moduli)


def stream_status(stream=None) -> None:
    """Waits for the stream and raises PsmmaError if a split-path call on it recorded a
    device-side timeout since the last check (device-pointer calls return without waiting)."""
    st = load().psmma_stream_status(_stream_ptr(stream))
    if st != 0:
        raise PsmmaError(st, "psmma_stream_status")


def workspace_size(kind: int, n: int, k: int, precision="fp64", n_moduli: int = 0, block_levels: int = 0) -> int:
    opts = make_opts(precision, n_moduli, block_levels=block_levels)
    return int(load().psmma_workspace_size(kind, n, k, C.byref(opts)))


_COMPRESS = {"rrqr": COMPRESS_RRQR, "rrlu": COMPRESS_RRLU, COMPRESS_RRQR: COMPRESS_RRQR,
             COMPRESS_RRLU: COMPRESS_RRLU}


def _batch_items(problems):
    import torch
    items = (PsmmaBatchItem * max(1, len(problems)))()
    for i, (A, gen, Q) in enumerate(problems):
        n = Q.shape[0]
        pa, lda = _dev(A, "A", torch.float64)
        pg, ldg = _dev(gen, "gen", torch.float64)
        if gen.dim() == 1:
            ldg = gen.numel()  # a generator vector (Toeplitz G): its length
        pq, ldq = _dev(Q, "Q", torch.float64)
        items[i].n, items[i].A, items[i].lda = n, pa, max(lda, 1)
        items[i].gen, items[i].ldgen = pg, ldg
        items[i].Q, items[i].ldq = pq, max(ldq, 1)
    return items


def cauchy_batch_lowrank(problems, alpha, beta, *, compressor="rrqr", tol=1e-14, precision="fp64",
                         n_moduli=0, stream=None, work=None, eig=False):
    """Q_i := alpha*A_i*H_i + beta*Q_i for problems = [(A_i, gen_i, Q_i), ...] (n_i x n_i CUDA
    tensors, gen_i = [D|F|U|V]), H_i split 2 x 2 with its off-diagonal blocks compressed by
    ``compressor`` ("rrqr" or "rrlu") at ``tol``.  With eig=True the H_i are the eigensolver's
    matrices (psmma_cauchyeig) and gen_i = [F|U|V|DIFL|DIFR].  Returns (ranks,
    stats): two ranks per problem with n >= 2 (blocks H(1:h, h+1:n), H(h+1:n, 1:h)) and a dict
    of flop counts."""
    lib = load()
    items = _batch_items(problems)
    opts = make_opts(precision, n_moduli, work)
    nb = sum(2 for (_, _, Q) in problems if Q.shape[0] >= 2)
    ranks = (C.c_int * max(1, nb))()
    stats = PsmmaBatchStats()
    fn = lib.psmma_cauchyeig_batch_lowrank if eig else lib.psmma_cauchy_batch_lowrank
    st = fn(len(problems), items, float(alpha), float(beta), _COMPRESS[compressor], float(tol), C.byref(opts), ranks,
            C.byref(stats), _stream_ptr(stream))
    if st != 0:
        raise PsmmaError(st, "psmma_cauchy_batch_lowrank")
    info = {"effective_flops": stats.effective_flops, "executed_flops": stats.executed_flops,
            "compress_flops": stats.compress_flops, "n_blocks": stats.n_blocks, "max_rank": stats.max_rank,
            "full_rank_blocks": stats.full_rank_blocks, "graph_reused": bool(stats.graph_reused)}
    return list(ranks)[:nb], info


def toeplitz_batch_lowrank(problems, alpha, beta, *, tol=1e-14, precision="fp64", n_moduli=0, stream=None,
                           work=None):
    """The merge level of Toeplitz multiplies: problems = [(A_i, G_i, Q_i), ...] with G_i the
    2n_i - 1 generator of psmma_toeplitz; off-diagonal blocks compressed by RRQR at ``tol``.
    Returns (ranks, stats) as cauchy_batch_lowrank."""
    lib = load()
    items = _batch_items(problems)
    opts = make_opts(precision, n_moduli, work)
    nb = sum(2 for (_, _, Q) in problems if Q.shape[0] >= 2)
    ranks = (C.c_int * max(1, nb))()
    stats = PsmmaBatchStats()
    st = lib.psmma_toeplitz_batch_lowrank(len(problems), items, float(alpha), float(beta), float(tol),
                                          C.byref(opts), ranks, C.byref(stats), _stream_ptr(stream))
    if st != 0:
        raise PsmmaError(st, "psmma_toeplitz_batch_lowrank")
    info = {"effective_flops": stats.effective_flops, "executed_flops": stats.executed_flops,
            "compress_flops": stats.compress_flops, "n_blocks": stats.n_blocks, "max_rank": stats.max_rank,
            "full_rank_blocks": stats.full_rank_blocks, "graph_reused": bool(stats.graph_reused)}
    return list(ranks)[:nb], info


def batch_workspace_size(problems, *, compressor="rrqr", precision="fp64", n_moduli=0) -> int:
    opts = make_opts(precision, n_moduli)
    items = _batch_items(problems)
    return int(load().psmma_batch_workspace_size(len(problems), items, _COMPRESS[compressor], C.byref(opts)))


def tune_batch(problems, alpha=1.0, beta=0.0, *, compressor="rrqr", tol=1e-14, precision="split", n_moduli=0,
               stream=None) -> dict:
    """Autotunes the grouped split GEMM on this batch (overwrites the Q_i) and returns the chosen
    configuration; later cauchy_batch_lowrank calls on batches of the same signature use it."""
    lib = load()
    items = _batch_items(problems)
    opts = make_opts(precision, n_moduli)
    res = PsmmaTuneResult()
    st = lib.psmma_tune_batch(len(problems), items, float(alpha), float(beta), _COMPRESS[compressor], float(tol),
                              C.byref(opts), C.byref(res), _stream_ptr(stream))
    if st != 0:
        raise PsmmaError(st, "psmma_tune_batch")
    return {"narrow_max": res.narrow_max, "mid_max": res.mid_max, "group_m": res.group_m,
            "candidates": res.candidates, "ms_best": res.ms_best, "ms_default": res.ms_default}


def psmma_cauchyeig(n, k, alpha, A, F, U, V, difl, difr, beta, Q, *, D=None, precision="fp64", n_moduli=0,
                    stream=None, work=None, block_levels=0):
    """Q := alpha*A*H + beta*Q, H(i,j) = U(i)V(j) / (F(i) - D(j)) with the denominators formed from
    DIFL(j) = D(j) - F(j) and DIFR(j) = D(j) - F(j+1) (CauchylikeEig).  Vectors of length k."""
    lib = load()
    opts = make_opts(precision, n_moduli, work, block_levels=block_levels)
    vecs = [F, D, U, V, difl, difr]
    if _is_torch(Q):
        import torch
        pa, lda = _dev(A, "A", torch.float64) if A is not None else (0, max(1, n))
        ptr = [C.c_void_p(x.data_ptr()) if x is not None else None for x in vecs]
        pq, ldq = _dev(Q, "Q", torch.float64)
        st = lib.psmma_cauchyeig(n, k, float(alpha), C.c_void_p(pa), lda, *ptr, float(beta), C.c_void_p(pq), ldq,
                                 C.byref(opts), _stream_ptr(stream))
    else:
        pa, lda = _host(A, "A", np.float64) if A is not None else (0, max(1, n))
        keep = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None for x in vecs]
        ptr = [C.c_void_p(x.ctypes.data) if x is not None else None for x in keep]
        pq, ldq = _host(Q, "Q", np.float64)
        st = lib.psmma_cauchyeig_host(n, k, float(alpha), C.c_void_p(pa), lda, *ptr, float(beta), C.c_void_p(pq),
                                      ldq, C.byref(opts))
    if st != 0:
        raise PsmmaError(st, "psmma_cauchyeig")
    return Q
