"""CPU oracle for PSMMA's structured multiply -- TEST INFRASTRUCTURE ONLY.

This module restates, on the CPU, the algorithm of the reference (shengguolsg/PSMMA_Git,
Fortran 90 + MPI + ScaLAPACK) for the structured multiply Q = alpha*A*H + beta*Q and the
DFT multiply C = alpha*F*B + beta*C.  It is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.  Nothing in
``psmma_git_gb300`` uses it.

Parity status.  The reference cannot be compiled here or on the GPU host (no Fortran
compiler, MPI, BLACS or ScaLAPACK) and its tests are unseeded (``random_number`` without
a seed) with no stored answers, so there are no golden output vectors to copy.  Parity is
pinned instead by
  * closed-form known answers for the reference tests' own deterministic fixtures: the
    Toeplitz generator of Test/psmma_testtoeplitz.f90:38-46 (H = N^2 I + (i-j)) and the
    all-ones B of Test/pzfox_fft2.f90:99 (F*1 = N e_1);
  * exact rational arithmetic (``fractions.Fraction``) on the Cauchy recipe of
    Test/psmma_testcauchy.f90:37-53 at small N;
  * this restatement of the reference's ring algorithm (process grid emulated), checked
    against the exact products above.
The fixtures and answers are committed under tests/golden/ with the script that made them.

Third-party arithmetic.  DGEMM/ZGEMM and the LAPACK routines (DGEQP3, DORGQR, ZGEQP3,
ZUNMQR, ZGESVD) come from MKL or OpenBLAS in the reference builds (SLMakes/SLmake.inc*);
here they are numpy/scipy (scipy-openblas).  ``NUMROC``, ``INDXL2G`` and ``PDGEMR2D`` are
ScaLAPACK's; they are restated from their documented definitions (PDGEMR2D as "assemble the
global matrices, copy the sub-matrix, distribute again", sharing nothing with the library's
per-peer plan).
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

try:
    import scipy.linalg as sla
except Exception:  # pragma: no cover - scipy is present in both environments
    sla = None

# REAL(4) literals of the reference converted to double, as Fortran does.
TOL_RRLU = float(np.float32(1.0e-17))   # Auxil_2p5D.f90:946  tol = 1.0E-17
TOL_RRQR = float(np.float32(1.0e-13))   # Auxil_2p5D.f90:1140 TOL = 1.0E-13
TOL_DFT = float(np.float32(1.0e-13))    # pzmdftL.f90:324, pzmdftL1.f90:361


# ---------------------------------------------------------------------------------------
# Index bookkeeping
# ---------------------------------------------------------------------------------------
def numroc(n: int, nb: int, iproc: int, isrcproc: int, nprocs: int) -> int:
    """ScaLAPACK NUMROC: rows/cols of an n-vector in blocks of nb owned by process iproc."""
    mydist = (nprocs + iproc - isrcproc) % nprocs
    nblocks = n // nb
    r = (nblocks // nprocs) * nb
    extra = nblocks % nprocs
    if mydist < extra:
        r += nb
    elif mydist == extra:
        r += n % nb
    return r


def const_index(n: int, nb: int, mycol: int, npcol: int) -> np.ndarray:
    """ConstIndex (Auxil_2p5D.f90:2-66): 1-based global indices of process column mycol's
    block-cyclic slice of 1..n."""
    knb = n // nb
    nfseg = knb // npcol
    cstart = mycol * nb + 1
    gap = npcol * nb
    out = []
    for _ in range(nfseg):
        out.extend(range(cstart, cstart + nb))
        cstart += gap
    left = n - nfseg * gap - mycol * nb
    if left > 0:
        ln = min(nb, left)
        out.extend(range(cstart, cstart + ln))
    return np.asarray(out, dtype=np.int64)


def is_intersect(set_a: np.ndarray, set_b: np.ndarray) -> bool:
    """is_intersect (Auxil_2p5D.f90:752-792).  Despite its name it returns True when the
    two sets are DISJOINT (is_inters starts .TRUE. and is set .FALSE. on a common element);
    the caller stores the result in ``islowrank``."""
    return len(np.intersect1d(set_a, set_b)) == 0


# ---------------------------------------------------------------------------------------
# Block-cyclic layouts and their redistribution (PDGEMR2D, the 2.5D index helpers)
# ---------------------------------------------------------------------------------------
def indxl2g(l: int, nb: int, iproc: int, isrcproc: int, nprocs: int) -> int:
    """ScaLAPACK INDXL2G (1-based local l -> 1-based global index), from its definition."""
    return nprocs * nb * ((l - 1) // nb) + (l - 1) % nb + ((nprocs + iproc - isrcproc) % nprocs) * nb + 1


def grid_coords(rank: int, nprow: int, npcol: int, order: str = "R") -> tuple[int, int]:
    """BLACS grid coordinates of a rank ('R': row-major numbering, 'C': column-major)."""
    if order.upper().startswith("R"):
        return rank // npcol, rank % npcol
    return rank % nprow, rank // nprow


def bc_local(G: np.ndarray, desc, nprow: int, npcol: int, myrow: int, mycol: int) -> np.ndarray:
    """Process (myrow, mycol)'s local array of the global matrix G in layout desc
    (DTYPE, CTXT, M, N, MB, NB, RSRC, CSRC, LLD): the fill loop of the reference tests,
    A(i,j) = G(indxl2g(i), indxl2g(j)) (Test/psmma_testcauchy.f90:93-101)."""
    _, _, M, N, MB, NB, RS, CS, _ = desc
    lr = numroc(M, MB, myrow, RS, nprow)
    lc = numroc(N, NB, mycol, CS, npcol)
    rows = [indxl2g(i, MB, myrow, RS, nprow) - 1 for i in range(1, lr + 1)]
    cols = [indxl2g(j, NB, mycol, CS, npcol) - 1 for j in range(1, lc + 1)]
    return np.asarray(G)[np.ix_(rows, cols)].copy()


def bc_global(locals_: dict, desc, nprow: int, npcol: int, order: str = "R", fill=0.0) -> np.ndarray:
    """Assembles the global M x N matrix from every rank's local array (dict rank -> array)."""
    _, _, M, N, MB, NB, RS, CS, _ = desc
    first = next(iter(locals_.values()))
    G = np.full((M, N), fill, dtype=first.dtype)
    for rank, L in locals_.items():
        pr, pc = grid_coords(rank, nprow, npcol, order)
        lr = numroc(M, MB, pr, RS, nprow)
        lc = numroc(N, NB, pc, CS, npcol)
        rows = [indxl2g(i, MB, pr, RS, nprow) - 1 for i in range(1, lr + 1)]
        cols = [indxl2g(j, NB, pc, CS, npcol) - 1 for j in range(1, lc + 1)]
        G[np.ix_(rows, cols)] = L[:lr, :lc]
    return G


def pdgemr2d(m: int, n: int, A_locals: dict, ia: int, ja: int, desca, grid_a, B_locals: dict, ib: int, jb: int,
             descb, grid_b) -> dict:
    """PDGEMR2D's result: B(ib:ib+m-1, jb:jb+n-1) := A(ia:ia+m-1, ja:ja+n-1), every other
    element of B unchanged.  grid_* = (nprow, npcol, order).  Works on the assembled global
    matrices, so it shares nothing with the library's per-peer plan."""
    GA = bc_global(A_locals, desca, *grid_a)
    GB = bc_global(B_locals, descb, *grid_b)
    GB[ib - 1:ib - 1 + m, jb - 1:jb - 1 + n] = GA[ia - 1:ia - 1 + m, ja - 1:ja - 1 + n]
    out = {}
    for rank in B_locals:
        pr, pc = grid_coords(rank, *grid_b)
        out[rank] = bc_local(GB, descb, grid_b[0], grid_b[1], pr, pc)
    return out


def redist2p5a(k: int, nb: int, npzc: int, npcol: int) -> np.ndarray:
    """Redist2P5a (Auxil_2p5D.f90:362-390): 1..k ordered by process column, the columns taken
    as I + J*(npcol/npzc), I outer, J inner, each contributing its ConstIndex slice."""
    if npcol % npzc:
        raise ValueError("NPZC must divide NPCOL")
    lnpcol = npcol // npzc
    out = []
    for i in range(lnpcol):
        for j in range(npzc):
            out.extend(const_index(k, nb, i + j * lnpcol, npcol).tolist())
    return np.asarray(out, dtype=np.int64)


def const_index1(n: int, nb: int, mycol: int, npcol: int, pindex) -> list:
    """ConstIndex1 (Auxil_2p5D.f90:392-419): nfseg = ICEIL(n, nb) / npcol full segments of nb
    entries of pindex starting at mycol*nb + 1, stride npcol*nb.  Entries past n (which the
    reference would read out of bounds when the last block is partial) are returned as None."""
    knb = -(-n // nb)
    nfseg = knb // npcol
    cstart = mycol * nb
    out = []
    for _ in range(nfseg):
        for t in range(cstart, cstart + nb):
            out.append(int(pindex[t]) if t < n else None)
        cstart += npcol * nb
    return out


# ---------------------------------------------------------------------------------------
# Tile builders
# ---------------------------------------------------------------------------------------
def cauchy_like(D, F, U, V) -> np.ndarray:
    """Cauchylike (Cauchylowrank.f90:509-521): A(i,j) = U(i)*V(j) / (D(i)-F(j))."""
    D, F, U, V = (np.asarray(x, dtype=np.float64) for x in (D, F, U, V))
    return (U[:, None] * V[None, :]) / (D[:, None] - F[None, :])


def const_cauchy(gen: np.ndarray, rindex, cindex) -> np.ndarray:
    """ConstCauchy (Auxil_2p5D.f90:68-151): generator columns [D, F, U, V] (:138-141);
    rindex/cindex are 1-based."""
    r = np.asarray(rindex) - 1
    c = np.asarray(cindex) - 1
    return cauchy_like(gen[r, 0], gen[c, 1], gen[r, 2], gen[c, 3])


def const_toeplitz(g: np.ndarray, k: int, rindex, cindex) -> np.ndarray:
    """ConstToeplitz (Auxil_2p5D.f90:153-236): T(i,j) = G(K + C_j - R_i), 1-based."""
    r = np.asarray(rindex)[:, None]
    c = np.asarray(cindex)[None, :]
    return np.asarray(g, dtype=np.float64)[k + c - r - 1]


def const_hankel(g: np.ndarray, k: int, rindex, cindex) -> np.ndarray:
    """ConstHankel (Auxil_2p5D.f90:238-322): T(i,j) = G(R_i + C_j - 1), 1-based."""
    r = np.asarray(rindex)[:, None]
    c = np.asarray(cindex)[None, :]
    return np.asarray(g, dtype=np.float64)[r + c - 2]


def dense_h(kind: str, gen, k: int) -> np.ndarray:
    """The whole K-by-K structured matrix (what the reference tests form explicitly,
    e.g. psmma_testcauchy.f90:95-102)."""
    idx = np.arange(1, k + 1)
    if kind == "cauchy":
        return const_cauchy(np.asarray(gen).reshape(4, -1).T if np.ndim(gen) == 1 else gen, idx, idx)
    if kind == "toeplitz":
        return const_toeplitz(gen, k, idx, idx)
    if kind == "hankel":
        return const_hankel(gen, k, idx, idx)
    raise ValueError(kind)


def dft_matrix(n: int) -> np.ndarray:
    """F(j,k) = w^((j-1)(k-1)), w = exp(-2*pi*i/n), from the exact exponent (j*k mod n)."""
    j = np.arange(n, dtype=np.int64)
    t = np.outer(j, j) % n
    return np.exp(-2j * np.pi * t / n)


# ---------------------------------------------------------------------------------------
# Cauchy structured RRLU (Cauchylowrank.f90)
# ---------------------------------------------------------------------------------------
def _cauchy_max(D, F, u):
    """CauchyMax (Cauchylowrank.f90:166-188): largest |u(i)/(D(i)-F)| and its 1-based index."""
    lk = np.abs(u / (D - F))
    jj = int(np.argmax(lk))
    return float(lk[jj]), jj + 1


def _cauchy_pivt_g(D, F, u, v, PL, PU, k, A, M, N):
    """CauchyPivtG (Cauchylowrank.f90:191-243): alternating row/column partial pivoting.
    Arrays are 0-based numpy views; k is 1-based as in the reference."""
    k0 = k - 1
    junkL, jjL = _cauchy_max(D[k0:M], F[k0], u[k0:M])
    junkU, jjU = _cauchy_max(F[k0:N], D[k0], v[k0:N])
    junkL *= abs(v[k0])
    junkU *= abs(u[k0])
    piv = abs(u[k0] * v[k0] / (D[k0] - F[k0]))
    if junkL <= piv and junkU <= piv:
        return
    flg = 1 if junkL > junkU else 0
    while True:
        if flg == 1:
            jj = jjL
            a, b = k0, jj + k0 - 1
            D[a], D[b] = D[b], D[a]
            u[a], u[b] = u[b], u[a]
            A[a], A[b] = A[b], A[a]
            PL[a], PL[b] = PL[b], PL[a]
            junkU, jjU = _cauchy_max(F[k0:N], D[k0], v[k0:N])
            if jjU == 1:
                return
            flg = 0
        jj = jjU
        a, b = k0, jj + k0 - 1
        F[a], F[b] = F[b], F[a]
        v[a], v[b] = v[b], v[a]
        PU[a], PU[b] = PU[b], PU[a]
        junkL, jjL = _cauchy_max(D[k0:M], F[k0], u[k0:M])
        if jjL == 1:
            return
        flg = 1


def _cauchy_pivt_g_cp(D, F, u, v, PL, PU, k, A, M, N):
    """CauchyPivtG_CP (Cauchylowrank.f90:246-296): complete pivoting on the Schur complement."""
    k0 = k - 1
    best, ii, jj = -1.0, 1, 1
    for j in range(1, N - k + 2):
        junk, i1 = _cauchy_max(D[k0:M], F[k0 + j - 1], u[k0:M])
        junk = abs(junk * v[k0 + j - 1])
        if j == 1 or junk > best:
            best, ii, jj = junk, i1, j
    a, b = k0, ii + k0 - 1
    D[a], D[b] = D[b], D[a]
    u[a], u[b] = u[b], u[a]
    A[a], A[b] = A[b], A[a]
    PL[a], PL[b] = PL[b], PL[a]
    a, b = k0, jj + k0 - 1
    F[a], F[b] = F[b], F[a]
    v[a], v[b] = v[b], v[a]
    PU[a], PU[b] = PU[b], PU[a]


def _search_max2(U, W, D2, D1, ldu, ldw):
    """searchMax2 (Cauchylowrank.f90:137-163): returns (ii, jj, Nmax), 1-based."""
    nmax, ii, jj = None, 1, 1
    for j in range(1, ldw + 1):
        junk, jjl = _cauchy_max(D2[:ldu], D1[j - 1], U[:ldu])
        junk *= abs(W[j - 1])
        if j == 1 or junk > nmax:
            nmax, ii, jj = junk, j, jjl
    return ii, jj, nmax


def rrlu_cauchy(D, F, A, V, tol, M, N):
    """rrluCauchy (Cauchylowrank.f90:7-134): rank-revealing LU in generator space.

    Returns (D, U, W, PL, PU, Rk) with the reference's conventions: the first Rk entries
    of the permuted D are the chosen rows, U(Rk+1:M) and W(1:Rk) are the generators of the
    interpolation matrix, PL/PU are 1-based permutations."""
    D = np.array(D, dtype=np.float64)
    F = np.array(F, dtype=np.float64)
    A = np.array(A, dtype=np.float64)
    V = np.array(V, dtype=np.float64)
    U = A.copy()
    W = np.zeros(min(M, N))
    Rk = min(M, N)
    mn = Rk
    PL = np.arange(1, M + 1)
    PU = np.arange(1, N + 1)
    amax = 0.0
    rho = 1.12
    prd = 10
    for k in range(1, mn + 1):
        k0 = k - 1
        _cauchy_pivt_g(D, F, U, V, PL, PU, k, A, M, N)
        ukk = U[k0] * V[k0] / (D[k0] - F[k0])
        amax = max(amax, abs(ukk))
        if abs(ukk) < tol * amax:
            _cauchy_pivt_g_cp(D, F, U, V, PL, PU, k, A, M, N)
            ukk = U[k0] * V[k0] / (D[k0] - F[k0])
            amax = max(amax, abs(ukk))
            if abs(ukk) < tol * amax:
                Rk = k - 1
                break
        U[k:M] = U[k:M] * (D[k:M] - D[k0]) / (D[k:M] - F[k0])
        V[k:N] = V[k:N] * (F[k:N] - F[k0]) / (F[k:N] - D[k0])
        for j in range(k - 1):
            W[j] = W[j] * ((F[k0] - D[j]) / (D[k0] - D[j]))
        W[k0] = (D[k0] - F[k0]) / A[k0]
        for j in range(k - 1):
            W[k0] = W[k0] * (F[j] - D[k0]) / (D[j] - D[k0])
        flgl = k % prd
        while flgl < 1:
            flgl = 1
            ii, jj, nmax = _search_max2(U[k:], W, D[k:], D, M - k, k)
            if nmax > rho:
                flgl = 0
                jj = jj + k
                i0, j0 = ii - 1, jj - 1
                V[k:N] = V[k:N] * ((F[k:N] - D[i0]) / (F[k:N] - D[j0]))
                U[k:j0] = U[k:j0] * ((D[k:j0] - D[j0]) / (D[k:j0] - D[i0]))
                U[jj:M] = U[jj:M] * ((D[jj:M] - D[j0]) / (D[jj:M] - D[i0]))
                W[:i0] = W[:i0] * ((D[:i0] - D[i0]) / (D[:i0] - D[j0]))
                W[ii:k] = W[ii:k] * ((D[ii:k] - D[i0]) / (D[ii:k] - D[j0]))
                U[j0] = A[i0] * ((D[i0] - D[j0]) / (D[i0] - F[i0]))
                W[i0] = (D[j0] - F[i0]) / A[j0]
                for j in list(range(ii - 1)) + list(range(ii, k)):
                    U[j0] = U[j0] * ((D[i0] - D[j]) / (D[i0] - F[j]))
                    W[i0] = W[i0] * ((F[j] - D[j0]) / (D[j] - D[j0]))
                PL[i0], PL[j0] = PL[j0], PL[i0]
                D[i0], D[j0] = D[j0], D[i0]
                A[i0], A[j0] = A[j0], A[i0]
    return D, F, U, V, W, PL, PU, Rk, A


def cauchy_like2(D, F, u, v, M, N) -> np.ndarray:
    """Cauchylike2 (Cauchylowrank.f90:524-559) for the M >= N branch used by
    compress_cauchy: [I; Z] with Z(i,j) = u(i)v(j)/(D(i)-F(j))."""
    out = np.zeros((M, N))
    rk = M - N
    if rk == 0:
        np.fill_diagonal(out, 1.0)
    elif rk > 0:
        out[:N, :N] = np.eye(N)
        out[N:, :] = cauchy_like(D[:M - N], F[:N], u[:M - N], v[:N])
    else:
        out[:, :M] = np.eye(M)
        out[:, M:] = (v[:M][:, None] * u[:N - M][None, :]) / (D[:N - M][None, :] - F[:M][:, None])
    return out


def compress_cauchy_rows(D, F, U, V, tol, M, N):
    """compress_cauchy('R', ...) (Cauchylowrank.f90:387-491).

    rrluCauchy is called on copies (LD, LF, LU, LV) with Z as its working row generator;
    it permutes LD and LU together with PL.  For Rk < M the factors are
    X = [I; Z(i)W(j)/(LD(i)-LD(j))] with rows put back by the inverse of PL (Cauchylike2 +
    invp, :448-451) and Y(i,j) = LU(i)V(j)/(LD(i)-F(j)), i <= Rk, with the caller's
    unpermuted F and V (:452).  Returns (X, Y, Rk) with the tile ~= X @ Y; X and Y are None
    when Rk == M (the reference then prints a warning and writes nothing, :455-464)."""
    LD, _LF, Z, _LV, W, PL, _PU, Rk, LU = rrlu_cauchy(D, F, U, V, tol, M, N)
    if Rk < M:
        inv = np.empty(M, dtype=np.int64)
        inv[PL - 1] = np.arange(1, M + 1)        # invp (Cauchylowrank.f90:494-506)
        Q = cauchy_like2(LD[Rk:], LD, Z[Rk:], W, M, Rk)
        X = Q[inv - 1, :]
        Y = cauchy_like(LD[:Rk], np.asarray(F, float), LU[:Rk], np.asarray(V, float))
        return X, Y, Rk
    return None, None, Rk


# ---------------------------------------------------------------------------------------
# RRQR compression (Auxil_2p5D.f90:1063-1189 + mdgeqp3.f)
# ---------------------------------------------------------------------------------------
def compress_rrqr(T: np.ndarray, tol: float = TOL_RRQR):
    """Compress_RRQR: pivoted QR T P = Q R, rank = first i with |R_ii| <= tol |R_11|, minus 1
    (:1150-1156; MDGEQP3's early exit at a panel boundary does not change it).  Returns
    (Qk, RkPt, Rk) with T ~= Qk @ RkPt; (None, None, min(M,N)) when full rank."""
    M, N = T.shape
    Q, R, P = sla.qr(T, mode="economic", pivoting=True)
    mn = min(M, N)
    diag = np.abs(np.diag(R))
    rk = mn
    for i in range(mn):
        if diag[i] <= tol * abs(R[0, 0]):
            rk = i
            break
    if rk == mn:
        return None, None, rk
    Y = np.zeros((rk, N))
    Y[:, P] = R[:rk, :]                         # DLAPMT(.FALSE.) : R * P^T
    return Q[:, :rk].copy(), Y, rk


# ---------------------------------------------------------------------------------------
# The SPMMA ring (PS*_COMPUTE) on an emulated NPROW x NPCOL grid
# ---------------------------------------------------------------------------------------
def ps_compute(kind: str, n: int, k: int, alpha: float, A: np.ndarray, gen, beta: float,
               Q: np.ndarray, nprow: int = 2, npcol: int = 2, nb: int = 64,
               lowrank: bool = True, stats: dict | None = None) -> np.ndarray:
    """Restatement of PSCAUCHY_COMPUTE / PSTOEPLITZ_COMPUTE / PSHANKEL_COMPUTE
    (pscauchy_compute.f90:298-423; pstoeplitz_compute.f90:198-310;
    pshankel_compute.f90:225-265) for every process of an nprow x npcol grid, block nb,
    IMROW = IMCOL = 0.  A (n x k) and Q (n x k) are global arrays; the result is the global
    Q the processes would hold.  The ring shift of A (DGESD2D/DGERV2D, :414-423) is the
    permutation "after K1 shifts, process column c holds panel (c + K1) mod npcol".

    Each process keeps its own flat WORK(IPB) buffer so that the reference's handling of a
    full-rank Cauchy off-diagonal tile is reproduced: compress_cauchy writes nothing when
    Rk == M (Cauchylowrank.f90:455-464) and the caller then multiplies whatever WORK(IPB)
    holds (pscauchy_compute.f90:379-381)."""
    gen = np.asarray(gen, dtype=np.float64)
    out = np.array(Q, dtype=np.float64, copy=True)
    if n == 0 or ((alpha == 0.0 or k == 0) and beta == 1.0):
        return out
    stats = stats if stats is not None else {}
    stats.setdefault("lowrank_steps", 0)
    stats.setdefault("fullrank_offdiag", 0)
    stats.setdefault("ranks", [])
    for myrow in range(nprow):
        rows = const_index(n, nb, myrow, nprow) - 1
        mp = numroc(n, nb, myrow, 0, nprow)
        assert mp == len(rows)
        if mp == 0:
            continue
        for mycol in range(npcol):
            cidx = const_index(k, nb, mycol, npcol)
            nq = len(cidx)
            Cloc = out[np.ix_(rows, cidx - 1)] if nq else np.zeros((mp, 0))
            # Flat WORK from IPB on (pscauchy_compute.f90:327-331): the tile/factor region of
            # (NQ+NB)*NQ doubles, then IPDW where the low-rank GEMM writes A*X.
            ipdw = (nq + nb) * nq
            work = np.zeros(ipdw + mp * (nq + nb) + (nq + nb) * (nq + nb))
            tbeta = beta
            for k1 in range(npcol):
                nroll = (mycol + k1) % npcol
                ridx = const_index(k, nb, nroll, npcol)
                kbp = len(ridx)
                if nq == 0 or kbp == 0:
                    continue
                Apan = A[np.ix_(rows, ridx - 1)]
                low = lowrank and kind != "hankel" and is_intersect(cidx, ridx)
                if low and kind == "cauchy":
                    stats["lowrank_steps"] += 1
                    X, Y, rk = compress_cauchy_rows(gen[ridx - 1, 0], gen[cidx - 1, 1],
                                                    gen[ridx - 1, 2], gen[cidx - 1, 3],
                                                    TOL_RRLU, kbp, nq)
                    stats["ranks"].append(rk)
                    if X is not None:
                        work[:kbp * rk] = X.ravel(order="F")
                        work[kbp * rk:kbp * rk + rk * nq] = Y.ravel(order="F")
                        if kbp * rk + rk * nq > ipdw:
                            stats["factor_overflow"] = stats.get("factor_overflow", 0) + 1
                    if rk == min(kbp, nq):
                        stats["fullrank_offdiag"] += 1
                        Hs = work[:kbp * nq].reshape((kbp, nq), order="F")
                        Cloc = alpha * (Apan @ Hs) + tbeta * Cloc
                    else:
                        Xs = work[:kbp * rk].reshape((kbp, rk), order="F")
                        work[ipdw:ipdw + mp * rk] = (Apan @ Xs).ravel(order="F")   # DGEMM 1
                        Wd = work[ipdw:ipdw + mp * rk].reshape((mp, rk), order="F")
                        Ys = work[kbp * rk:kbp * rk + rk * nq].reshape((rk, nq), order="F")
                        Cloc = alpha * (Wd @ Ys) + tbeta * Cloc                     # DGEMM 2
                    tbeta = 1.0
                elif low and kind == "toeplitz":
                    stats["lowrank_steps"] += 1
                    T = const_toeplitz(gen, k, ridx, cidx)
                    Qk, Y, rk = compress_rrqr(T)
                    stats["ranks"].append(rk)
                    if Qk is None:
                        Cloc = alpha * (Apan @ T) + tbeta * Cloc
                    else:
                        Cloc = alpha * ((Apan @ Qk) @ Y) + tbeta * Cloc
                    tbeta = 1.0
                else:
                    if kind == "cauchy":
                        T = const_cauchy(gen, ridx, cidx)
                    elif kind == "toeplitz":
                        T = const_toeplitz(gen, k, ridx, cidx)
                    else:
                        T = const_hankel(gen, k, ridx, cidx)
                    work[:kbp * nq] = T.ravel(order="F")
                    Cloc = alpha * (Apan @ T) + tbeta * Cloc
                    tbeta = 1.0
            if nq:
                out[np.ix_(rows, cidx - 1)] = Cloc
    return out


# ---------------------------------------------------------------------------------------
# DFT multiply (PZMDFTL / PZMDFTL1)
# ---------------------------------------------------------------------------------------
def _fortran_cpow(z: complex, e: int) -> complex:
    """Complex ** integer by repeated squaring, the usual Fortran runtime evaluation of
    ``Wn**PowK`` (pzmdftL.f90:332)."""
    if e == 0:
        return complex(1.0, 0.0)
    neg = e < 0
    e = abs(e)
    result = complex(1.0, 0.0)
    base = complex(z)
    while e:
        if e & 1:
            result *= base
        e >>= 1
        if e:
            base *= base
    return 1.0 / result if neg else result


def pzmdftl_compute(n: int, k: int, alpha: float, B: np.ndarray, beta: float, Cm: np.ndarray,
                    nprow: int = 2, variant: str = "svd", stats: dict | None = None) -> np.ndarray:
    """Restatement of PZMDFTL (variant "svd", pzmdftL.f90:296-493) and PZMDFTL1 (variant
    "rrqr", pzmdftL1.f90:318-514) on an nprow x nprow grid with N = NB*nprow (SRC/Readme.txt:5)
    and K = N columns split the same way.  Global arrays in and out."""
    assert n % nprow == 0, "PZMDFTL assumes N = NB * NPROW (SRC/Readme.txt:5)"
    assert k == n, "PZMDFTL distributes B's columns with NUMROC(N, NB, ...) and offsets with KP: K = N"
    P = nprow
    mp = n // P
    kp = mp
    out = np.array(Cm, dtype=np.complex128, copy=True)
    if n == 0 or ((alpha == 0.0 or k == 0) and beta == 1.0):
        return out
    pi = 4.0 * math.atan(1.0)
    wn = complex(math.cos(-2.0 * pi / n), math.sin(-2.0 * pi / n))  # EXP(NEONE*TWO*PI*CI/N)
    F11 = np.empty((mp, mp), dtype=np.complex128)
    for i2 in range(mp):
        for j2 in range(mp):
            F11[j2, i2] = _fortran_cpow(wn, i2 * j2)
    if variant == "svd":
        Uu, s, Vh = np.linalg.svd(F11, full_matrices=False)     # ZGESVD('A','S')
        rk = int(np.count_nonzero(s > TOL_DFT))
        Ul = Uu[:, :rk] * s[:rk][None, :]                      # ZLASCL column scaling
        Vt = Vh[:rk, :]
    else:
        Qf, R, piv = sla.qr(F11, mode="economic", pivoting=True)  # ZGEQP3
        diag = np.abs(np.diag(R))
        rk = mp
        for ii in range(mp):
            if diag[ii] <= TOL_DFT * abs(R[0, 0]):
                rk = ii
                break
        Ul = Qf[:, :rk]                                          # ZUNMQR on an identity
        Vt = np.zeros((rk, mp), dtype=np.complex128)
        Vt[:, piv] = R[:rk, :]                                   # ZLAPMT(.FALSE.)
    if stats is not None:
        stats["rank"] = rk
    nq = n // P
    for myrow in range(P):
        gapc = mp * myrow
        DR = np.array([_fortran_cpow(wn, gapc * i2) for i2 in range(mp)])
        for mycol in range(P):
            cols = slice(mycol * nq, min((mycol + 1) * nq, k))
            Cloc = out[myrow * mp:(myrow + 1) * mp, cols]
            tbeta = beta
            for k1 in range(P):
                icol = (myrow + k1) % P
                ipr = (myrow * mp) * (icol * kp)
                gapr = mp * icol
                DL = np.array([_fortran_cpow(wn, ipr + gapr * i2) for i2 in range(mp)])
                Ua = Ul.copy()
                Va = Vt.copy()
                if myrow == 0:
                    Ua = DL[:, None] * Ua
                elif icol == 0:
                    Va = Va * DR[None, :]
                else:
                    Ua = DL[:, None] * Ua
                    Va = Va * DR[None, :]
                Bblk = B[icol * mp:(icol + 1) * mp, cols]
                tmp = alpha * (Va @ Bblk)
                Cloc = Ua @ tmp + tbeta * Cloc
                tbeta = 1.0
            out[myrow * mp:(myrow + 1) * mp, cols] = Cloc
    return out


# ---------------------------------------------------------------------------------------
# Exact-math products (the build's checkers)
# ---------------------------------------------------------------------------------------
def dense_product(kind: str, alpha, A, gen, beta, Q, k: int) -> np.ndarray:
    """alpha*A@H + beta*Q with H formed explicitly (FP64 BLAS), as the reference tests do
    with PDGEMM (psmma_testcauchy.f90:127)."""
    H = dense_h(kind, gen, k)
    out = alpha * (np.asarray(A) @ H)
    if beta != 0.0:
        out = out + beta * np.asarray(Q)
    return out


def dft_product(alpha, B, beta, Cm) -> np.ndarray:
    """alpha*F@B + beta*C via the FFT: np.fft.fft(B, axis=0) == F @ B with w = exp(-2*pi*i/n)."""
    out = alpha * np.fft.fft(np.asarray(B), axis=0)
    if beta != 0.0:
        out = out + beta * np.asarray(Cm)
    return out


def toeplitz_product_fft(A: np.ndarray, g: np.ndarray, k: int) -> np.ndarray:
    """A @ T for T(i,j) = G(K+j-i) via FFT convolution, O(n k log k): (A T)(r, j) =
    sum_i A(r,i) G(K+j-i), a correlation of each row of A with G."""
    n = A.shape[0]
    L = 1 << int(math.ceil(math.log2(3 * k)))
    # (A T)(r, j) = sum_i A(r, i) g[k-1 + j - i] = (A_r * g)(k-1+j) (full convolution)
    fa = np.fft.rfft(A, n=L, axis=1)
    fg = np.fft.rfft(np.asarray(g, dtype=np.float64), n=L)
    conv = np.fft.irfft(fa * fg[None, :], n=L, axis=1)
    return conv[:, k - 1:2 * k - 1][:n]


def hankel_product_fft(A: np.ndarray, g: np.ndarray, k: int) -> np.ndarray:
    """A @ H for H(i,j) = G(i+j-1): (A H)(r, j) = sum_i A(r,i) g[i+j], a correlation."""
    L = 1 << int(math.ceil(math.log2(3 * k)))
    fa = np.fft.rfft(A[:, ::-1], n=L, axis=1)   # reversed rows turn correlation into convolution
    fg = np.fft.rfft(np.asarray(g, dtype=np.float64), n=L)
    conv = np.fft.irfft(fa * fg[None, :], n=L, axis=1)
    return conv[:, k - 1:2 * k - 1]


def exact_cauchy_product(A, gen, k: int):
    """A @ H in exact rational arithmetic on the FP64 inputs (small sizes only)."""
    gen = np.asarray(gen, dtype=np.float64)
    D = [Fraction(float(x)) for x in gen[:k, 0]]
    F = [Fraction(float(x)) for x in gen[:k, 1]]
    U = [Fraction(float(x)) for x in gen[:k, 2]]
    V = [Fraction(float(x)) for x in gen[:k, 3]]
    H = [[U[i] * V[j] / (D[i] - F[j]) for j in range(k)] for i in range(k)]
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    out = np.empty((n, k))
    for r in range(n):
        ar = [Fraction(float(x)) for x in A[r]]
        for j in range(k):
            out[r, j] = float(sum(ar[i] * H[i][j] for i in range(k)))
    return out


def decimal_cauchy_product(A_rows, gen, cols, k: int, digits: int = 40) -> np.ndarray:
    """(A_rows @ H)[:, cols] with every operation in ``decimal`` arithmetic at ``digits``
    significant digits on the exact values of the FP64 inputs (Decimal(float) is exact), for
    samples of products too large for Fraction: relative error ~k * 10^-digits."""
    import decimal
    ctx = decimal.Context(prec=digits)
    Dd = decimal.Decimal
    gen = np.asarray(gen, dtype=np.float64)
    D = [Dd(float(x)) for x in gen[:k, 0]]
    U = [Dd(float(x)) for x in gen[:k, 2]]
    cols = list(cols)
    Hc = []
    for j in cols:
        fj, vj = Dd(float(gen[j, 1])), Dd(float(gen[j, 3]))
        Hc.append([ctx.divide(ctx.multiply(U[i], vj), ctx.subtract(D[i], fj)) for i in range(k)])
    A_rows = np.asarray(A_rows, dtype=np.float64)
    out = np.empty((A_rows.shape[0], len(cols)))
    for r in range(A_rows.shape[0]):
        ar = [Dd(float(x)) for x in A_rows[r, :k]]
        for c, h in enumerate(Hc):
            s = Dd(0)
            for i in range(k):
                s = ctx.fma(ar[i], h[i], s)
            out[r, c] = float(s)
    return out


def col_max_rel(x, ref) -> float:
    """Largest per-column relative 2-norm error max_j ||x_j - ref_j|| / ||ref_j|| (columns
    of zero norm count their absolute error)."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    num = np.linalg.norm(x - ref, axis=0)
    den = np.linalg.norm(ref, axis=0)
    return float(np.max(num / np.where(den > 0, den, 1.0)))


def rel_fro(x, ref) -> float:
    """Relative Frobenius error ||x - ref||_F / ||ref||_F."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (den if den > 0 else 1.0))


def col1_error(x, ref) -> float:
    """The reference tests' own metric: ||X1(:,1) - X(:,1)||_2 / ||X(:,1)||_2, first column
    only (psmma_testcauchy.f90:155-163)."""
    x = np.asarray(x)[:, 0]
    ref = np.asarray(ref)[:, 0]
    return float(np.linalg.norm(ref - x) / np.linalg.norm(x))


# ---------------------------------------------------------------------------------------
# Inputs: the reference tests' fixtures and the seeded workloads
# ---------------------------------------------------------------------------------------
def reference_cauchy_generators(n: int, U: np.ndarray, V: np.ndarray) -> np.ndarray:
    """Test/psmma_testcauchy.f90:37-53: F(i) = 0.1 + (2i-1)*gap, D(i) = F(i) + gap,
    gap = (9-0.1)/(2N); U, V supplied (the reference draws them unseeded from U(0,1)).
    Returns [D | F | U | V] as an (n x 4) array."""
    sa, bb = 0.1, 9.0
    gap = (bb - sa) / (2 * n)
    i = np.arange(1, n + 1, dtype=np.float64)
    F = sa + (2 * i - 1) * gap
    D = F + gap
    return np.column_stack([D, F, np.asarray(U, float), np.asarray(V, float)])


def reference_toeplitz_generator(n: int) -> np.ndarray:
    """Test/psmma_testtoeplitz.f90:38-46: G(i) = N - i for i != N, G(N) = N*N (1-based).
    The matrix is H(i,j) = G(N+j-i) = N^2 delta_ij + (i - j)."""
    g = np.empty(2 * n - 1)
    for i in range(1, n):
        g[i - 1] = 1.0 * ((n - i + 1) - 1)
    g[n - 1] = float(n * n)
    for i in range(n + 1, 2 * n):
        g[i - 1] = 1.0 * (1 - (i - n + 1))
    return g


def toeplitz_reference_known_answer(A: np.ndarray) -> np.ndarray:
    """Closed form of A @ H for reference_toeplitz_generator: H = N^2 I + r 1^T - 1 r^T with
    r_i = i, so A H = N^2 A + (A r) 1^T - (A 1) r^T.  Exact in integers for integer A."""
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[1]
    r = np.arange(1, n + 1, dtype=np.float64)
    return float(n * n) * A + np.outer(A @ r, np.ones(n)) - np.outer(A @ np.ones(n), r)


def cfg_cauchy_generators(n: int, seed: int = 0, clustered: float = 0.0, cluster_gap: float = 1e-10):
    """Seeded Cauchy generators of the benchmark workloads: d = sort(U(0,1)); w_j uniform in
    (d_j, d_{j+1}), w_n in (d_n, d_n + 1); u, v ~ N(0,1).  With clustered > 0, that fraction
    of the d_j is moved to within cluster_gap of its left neighbour, keeping strict
    interlacing.  Returns [D | F | U | V] (n x 4), D = d (row poles), F = w (column poles)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = np.sort(rng.uniform(0.0, 1.0, n))
    if clustered > 0:
        m = int(round(clustered * n))
        idx = rng.choice(np.arange(1, n), size=m, replace=False)
        for j in np.sort(idx):
            d[j] = d[j - 1] + cluster_gap * rng.uniform(0.5, 1.0)
        d = np.maximum.accumulate(d)
        # re-establish strict increase
        for j in range(1, n):
            if d[j] <= d[j - 1]:
                d[j] = np.nextafter(d[j - 1], np.inf) + cluster_gap * 0.5
    w = np.empty(n)
    t = rng.uniform(0.0, 1.0, n)
    w[:-1] = d[:-1] + t[:-1] * (d[1:] - d[:-1])
    w[-1] = d[-1] + t[-1]
    for j in range(n - 1):  # keep d_j < w_j < d_{j+1} strictly
        if not (d[j] < w[j] < d[j + 1]):
            w[j] = 0.5 * (d[j] + d[j + 1])
    u = rng.standard_normal(n)
    v = rng.standard_normal(n)
    return np.column_stack([d, w, u, v])


def cfg_matrix(n: int, k: int, seed: int = 1, dist: str = "uniform", complex_: bool = False):
    """Seeded A (n x k): uniform[-1,1] or N(0,1); complex128 with both parts uniform[-1,1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if complex_:
        return np.asfortranarray(rng.uniform(-1, 1, (n, k)) + 1j * rng.uniform(-1, 1, (n, k)))
    if dist == "normal":
        return np.asfortranarray(rng.standard_normal((n, k)))
    return np.asfortranarray(rng.uniform(-1.0, 1.0, (n, k)))


def cfg_vector(m: int, seed: int = 2) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-1.0, 1.0, m)


# ---------------------------------------------------------------------------------------
# Batched merge level with compressed off-diagonal blocks
# ---------------------------------------------------------------------------------------
def merge_level_product(A, gen, beta_Q, alpha: float, beta: float, compressor: str = "rrqr",
                        tol: float = 1e-14, kind: str = "cauchy"):
    """One problem of the batched merge level: Q = alpha*A*H + beta*Q with H the Cauchy-like
    matrix of gen = [D|F|U|V], split 2 x 2 at h = n // 2.  The diagonal blocks are multiplied
    as dense tiles (ConstCauchy + DGEMM, pscauchy_compute.f90:395-407); each off-diagonal
    tile is compressed as the reference's low-rank branch does (pscauchy_compute.f90:371-391):
    "rrqr" -> Compress_RRQR (X = Q_k, Y = R_k P^T), "rrlu" -> compress_cauchy('R') (X, Y from
    rrluCauchy), then Q(:,C) += alpha * (A(:,R) X) Y.  A tile that does not compress is
    multiplied as the dense tile (the mathematical A*H; the reference would reuse a stale
    buffer there, Cauchylowrank.f90:455-464).  Returns (Q, [rank of H(R1,C2), rank of
    H(R2,C1)]) -- ranks as the compressor reports them (min(M,N) or M when uncompressed).
    kind="toeplitz": gen is G (2n - 1) and the tiles are ConstToeplitzlowrank's explicit tiles
    compressed by Compress_RRQR (pstoeplitz_compute.f90:262-294, Auxil_2p5D.f90:968-1060); a
    full-rank tile is multiplied dense, as the reference does there."""
    A = np.asarray(A, dtype=np.float64)
    gen = np.asarray(gen, dtype=np.float64)
    n = A.shape[0]
    Q = (beta * np.asarray(beta_Q, dtype=np.float64)) if beta != 0.0 else np.zeros((n, n))
    if n == 0:
        return Q, []
    h = n // 2
    H = cauchy_like(gen[:n, 0], gen[:n, 1], gen[:n, 2], gen[:n, 3]) if kind == "cauchy" else dense_h(kind, gen, n)
    if kind != "cauchy" and compressor != "rrqr":
        raise ValueError("only RRQR compresses Toeplitz / Hankel tiles")
    Q[:, :h] += alpha * (A[:, :h] @ H[:h, :h])
    Q[:, h:] += alpha * (A[:, h:] @ H[h:, h:])
    ranks = []
    if h == 0:
        return Q, ranks
    for (r0, r1, c0, c1) in [(0, h, h, n), (h, n, 0, h)]:
        T = H[r0:r1, c0:c1]
        M, N = T.shape
        if compressor == "rrqr":
            X, Y, rk = compress_rrqr(T, tol)
        else:
            X, Y, rk = compress_cauchy_rows(gen[r0:r1, 0].copy(), gen[c0:c1, 1].copy(), gen[r0:r1, 2].copy(),
                                            gen[c0:c1, 3].copy(), tol, M, N)
        ranks.append(rk)
        if X is None or rk >= min(M, N):
            Q[:, c0:c1] += alpha * (A[:, r0:r1] @ T)
        elif rk > 0:
            Q[:, c0:c1] += alpha * ((A[:, r0:r1] @ X) @ Y)
    return Q, ranks


def cfg_batch_sizes(count: int = 64, lo: int = 256, hi: int = 8192, seed: int = 7) -> list[int]:
    """Seeded sizes of the batched merge level: n log-uniform in [lo, hi]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return [int(round(math.exp(x))) for x in rng.uniform(math.log(lo), math.log(hi), count)]


# ---------------------------------------------------------------------------------------
# Accurate-denominator Cauchy (PSMMA_CAUCHYEIG)
# ---------------------------------------------------------------------------------------
def cauchy_like_eig(F, U, V, DIFL, DIFR, rindex=None, cindex=None) -> np.ndarray:
    """CauchylikeEig (CauchyHssEig.f90:1693-1774) as ConstCauchyEig calls it
    (Auxil_2p5D.f90:532-637): T(i,j) = U(PL(i)) V(PU(j)) / den with, for PL(i) <= PU(j),
    den = (F(PL(i)) - F(PU(j))) - DIFL(PU(j)), else (F(PL(i)) - F(PU(j)+1)) - DIFR(PU(j))
    (1-based global indices PL = rindex, PU = cindex; default the whole k x k matrix)."""
    F = np.asarray(F, dtype=np.float64)
    k = len(U)
    r = np.arange(1, k + 1) if rindex is None else np.asarray(rindex)
    c = np.arange(1, k + 1) if cindex is None else np.asarray(cindex)
    Fr = F[r - 1][:, None]
    Fj = F[c - 1][None, :]
    cj1 = np.minimum(c, len(F) - 1)          # F(PU(j)+1); not read when PU(j) = k
    Fj1 = F[cj1][None, :]
    upper = r[:, None] <= c[None, :]
    dl = np.asarray(DIFL, dtype=np.float64)[c - 1][None, :]
    dr = np.asarray(DIFR, dtype=np.float64)[np.minimum(c, len(DIFR)) - 1][None, :]
    den = np.where(upper, (Fr - Fj) - dl, (Fr - Fj1) - dr)
    return (np.asarray(U, dtype=np.float64)[r - 1][:, None] * np.asarray(V, dtype=np.float64)[c - 1][None, :]) / den


def eig_generators(k: int, seed: int = 0, tiny: int = 0):
    """Seeded generators of a secular-equation shaped Cauchy matrix: F sorted uniform(0,1) (old
    eigenvalues), D(j) = F(j) + t_j (F(j+1) - F(j)) with t_j uniform(0.05, 0.95) (the last:
    F(k) + t_k), except `tiny` roots placed 2^-70 relative above their pole (D(j) equal to F(j)
    in FP64); DIFL(j) = D(j) - F(j) >= 0, DIFR(j) = D(j) - F(j+1) < 0 (exact from the gap
    rounded once); U, V ~ N(0,1).  Returns F, U, V, DIFL, DIFR (length k each)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    F = np.sort(rng.uniform(0.0, 1.0, k))
    gap = np.empty(k)
    gap[:-1] = F[1:] - F[:-1]
    gap[-1] = 1.0
    t = rng.uniform(0.05, 0.95, k)
    if tiny:
        idx = rng.choice(np.arange(k - 1), size=min(tiny, k - 1), replace=False)
        t[idx] = 2.0 ** -70
    DIFL = t * gap
    DIFR = DIFL - gap
    DIFR[-1] = 0.0
    return F, rng.standard_normal(k), rng.standard_normal(k), DIFL, DIFR


def exact_cauchy_eig_product(A, F, U, V, DIFL, DIFR):
    """A @ H in exact rational arithmetic on the FP64 inputs, H from cauchy_like_eig's rule
    (small sizes only)."""
    k = len(U)
    Fq = [Fraction(float(x)) for x in F]
    H = [[None] * k for _ in range(k)]
    for i in range(k):
        for j in range(k):
            if i <= j:
                den = (Fq[i] - Fq[j]) - Fraction(float(DIFL[j]))
            else:
                den = (Fq[i] - Fq[j + 1]) - Fraction(float(DIFR[j]))
            H[i][j] = Fraction(float(U[i])) * Fraction(float(V[j])) / den
    A = np.asarray(A)
    out = np.empty((A.shape[0], k))
    for r in range(A.shape[0]):
        ar = [Fraction(float(x)) for x in A[r]]
        for j in range(k):
            out[r, j] = float(sum(ar[i] * H[i][j] for i in range(k)))
    return out


def merge_level_eig_product(A, F, U, V, DIFL, DIFR, beta_Q, alpha: float, beta: float, tol: float = 1e-14,
                            compressor: str = "rrqr"):
    """The merge level of merge_level_product for the eigensolver's matrix H =
    cauchy_like_eig(F, U, V, DIFL, DIFR): diagonal blocks dense, off-diagonal tiles
    compressed by Compress_RRQR on the tile built by ConstCauchyEig's rule ("rrqr") or by the
    structured Compress_cauchyEig2 (rrluCauchyEigrow, CauchyHssEig.f90:2640-2829; "rrlu",
    the reference's own choice), then Q(:,C) += alpha (A(:,R) X) Y.  Returns (Q, ranks)."""
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    Q = (beta * np.asarray(beta_Q, dtype=np.float64)) if beta != 0.0 else np.zeros((n, n))
    if n == 0:
        return Q, []
    h = n // 2
    H = cauchy_like_eig(F, U, V, DIFL, DIFR)
    Q[:, :h] += alpha * (A[:, :h] @ H[:h, :h])
    Q[:, h:] += alpha * (A[:, h:] @ H[h:, h:])
    ranks = []
    if h == 0:
        return Q, ranks
    for (r0, r1, c0, c1) in [(0, h, h, n), (h, n, 0, h)]:
        T = H[r0:r1, c0:c1]
        if compressor == "rrqr":
            X, Y, rk = compress_rrqr(T, tol)
        else:
            X, Y, rk = compress_cauchy_eig(F, U, V, DIFL, DIFR, np.arange(r0 + 1, r1 + 1),
                                           np.arange(c0 + 1, c1 + 1), tol)
        ranks.append(rk)
        if X is None:
            Q[:, c0:c1] += alpha * (A[:, r0:r1] @ T)
        elif rk > 0:
            Q[:, c0:c1] += alpha * ((A[:, r0:r1] @ X) @ Y)
    return Q, ranks


# ---------------------------------------------------------------------------------------
# Structured RRLU of accurate-denominator Cauchy blocks (CauchyHssEig.f90)
# ---------------------------------------------------------------------------------------
def _fd(FF, DL, DR, pl, pu):
    """computfd (CauchyHssEig.f90:519-568): F(pl) - D(pu) with 1-based global indices,
    (FF(pl) - FF(pu)) - DIFL(pu) for pl <= pu, else (FF(pl) - FF(pu+1)) - DIFR(pu).  Arrays."""
    pl = np.asarray(pl)
    pu = np.asarray(pu)
    pu1 = np.minimum(pu, len(FF) - 1)  # FF(pu+1), not used when pu = n
    return np.where(pl <= pu, (FF[pl - 1] - FF[pu - 1]) - DL[pu - 1], (FF[pl - 1] - FF[pu1]) - DR[pu - 1])


def _dd(FF, DL, DR, pj, pk):
    """computdd (CauchyHssEig.f90:470-516): D(pj) - D(pk), 1-based global indices.  Arrays."""
    pj = np.asarray(pj)
    pk = np.asarray(pk)
    a = np.minimum(pj, len(FF) - 1)
    b = np.minimum(pk, len(FF) - 1)
    return np.where(pj < pk, (FF[a] - FF[pk - 1]) + DR[pj - 1] - DL[pk - 1],
                    (FF[pj - 1] - FF[b]) + DL[pj - 1] - DR[pk - 1])


def _argmax1(v):
    j = int(np.argmax(v))  # MAXLOC: the first maximum
    return float(v[j]), j + 1


def _pivt_eig(F, U, V, PL, PU, PQ, A, k, M, N, FF, DL, DR):
    """CauchyPivtEig (CauchyHssEig.f90:571-717), with CauchyMaxEigmc / CauchyMaxEigm
    (:1506-1589, :1418-1503).  The pivot magnitude uses FF(PL(k)) (the reference reads the
    local row-pole array F at the global index PL(k), :676-678, which equals it only for an
    unpermuted block starting at row 1)."""
    k0 = k - 1
    col = lambda: _argmax1(np.abs(U[k0:M] / _fd(FF, DL, DR, PL[k0:M], PU[k0])))
    row = lambda: _argmax1(np.abs(V[k0:N] / _fd(FF, DL, DR, PL[k0], PU[k0:N])))
    junkL, jjL = col()
    junkU, jjU = row()
    junkL *= abs(V[k0])
    junkU *= abs(U[k0])
    piv = abs(U[k0] * V[k0] / _fd(FF, DL, DR, PL[k0], PU[k0]))
    if junkL <= piv and junkU <= piv:
        return
    flg = 1 if junkL > junkU else 0
    while True:
        if flg == 1:
            a, b = k0, jjL + k0 - 1
            for arr in (F, U, A, PL, PQ):
                arr[a], arr[b] = arr[b], arr[a]
            junkU, jjU = row()
            if jjU == 1:
                return
            flg = 0
        a, b = k0, jjU + k0 - 1
        for arr in (V, PU):
            arr[a], arr[b] = arr[b], arr[a]
        junkL, jjL = col()
        if jjL == 1:
            return
        flg = 1


def _pivt_eig_cp(F, U, V, PL, PU, PQ, A, k, M, N, FF, DL, DR):
    """CauchyPivtEig_CP (CauchyHssEig.f90:1004-1134): complete pivoting, strict '>' over
    columns after the first, MAXLOC within a column."""
    k0 = k - 1
    best, ii, jj = -1.0, 1, 1
    for j in range(1, N - k + 2):
        junk, i1 = _argmax1(np.abs(U[k0:M] / _fd(FF, DL, DR, PL[k0:M], PU[k0 + j - 1])))
        junk = abs(junk * V[k0 + j - 1])
        if j == 1 or junk > best:
            best, ii, jj = junk, i1, j
    a, b = k0, ii + k0 - 1
    for arr in (F, U, A, PL, PQ):
        arr[a], arr[b] = arr[b], arr[a]
    a, b = k0, jj + k0 - 1
    for arr in (V, PU):
        arr[a], arr[b] = arr[b], arr[a]


def rrlu_cauchy_eig_row(F, A, V, PL, PU, tol, M, N, FF, DL, DR):
    """rrluCauchyEigrow (CauchyHssEig.f90:7-212): the structured RRLU of a block of the
    eigensolver's Cauchy matrix, rows with old eigenvalues F = FF(PL) and weights A, columns
    PU (new eigenvalues, through DIFL/DIFR) with weights V.  rho = 1.2, swap check every 5
    steps.  Returns (F, A, Z, V, W, PL, PU, PQ, Rk): permuted row poles and weights, the
    Schur weights Z, interpolation weights W and the local row permutation PQ (1-based)."""
    F = np.array(F, dtype=np.float64)
    A = np.array(A, dtype=np.float64)
    V = np.array(V, dtype=np.float64)
    PL = np.array(PL)
    PU = np.array(PU)
    FF = np.asarray(FF, dtype=np.float64)
    DL = np.asarray(DL, dtype=np.float64)
    DR = np.asarray(DR, dtype=np.float64)
    U = A.copy()
    PQ = np.arange(1, M + 1)
    mn = min(M, N)
    W = np.zeros(mn)
    Rk = mn
    amax = 0.0
    rho, prd = 1.2, 5
    fd = lambda pl, pu: _fd(FF, DL, DR, pl, pu)
    for k in range(1, mn + 1):
        k0 = k - 1
        _pivt_eig(F, U, V, PL, PU, PQ, A, k, M, N, FF, DL, DR)
        ukk = U[k0] * V[k0] / fd(PL[k0], PU[k0])
        amax = max(amax, abs(ukk))
        if abs(ukk) < tol * amax:
            _pivt_eig_cp(F, U, V, PL, PU, PQ, A, k, M, N, FF, DL, DR)
            ukk = U[k0] * V[k0] / fd(PL[k0], PU[k0])
            amax = max(amax, abs(ukk))
            if abs(ukk) < tol * amax:
                Rk = k - 1
                break
        U[k:M] = U[k:M] * ((F[k:M] - F[k0]) / fd(PL[k:M], PU[k0]))
        V[k:N] = V[k:N] * (_dd(FF, DL, DR, PU[k:N], PU[k0]) / (-fd(PL[k0], PU[k:N])))
        for j in range(k - 1):
            W[j] = W[j] * ((-fd(PL[j], PU[k0])) / (F[k0] - F[j]))
        W[k0] = fd(PL[k0], PU[k0]) / A[k0]
        for j in range(k - 1):
            W[k0] = W[k0] * ((-fd(PL[k0], PU[j])) / (F[j] - F[k0]))
        flgl = k % prd
        while flgl < 1:
            flgl = 1
            ii, jj, nmax = _search_max2(U[k:], W, F[k:], F, M - k, k)   # searchMax2Eig, :1137-1203
            if nmax > rho:
                flgl = 0
                jj = jj + k
                i0, j0 = ii - 1, jj - 1
                V[k:N] = V[k:N] * ((-fd(PL[i0], PU[k:N])) / (-fd(PL[j0], PU[k:N])))
                U[k:j0] = U[k:j0] * ((F[k:j0] - F[j0]) / (F[k:j0] - F[i0]))
                U[jj:M] = U[jj:M] * ((F[jj:M] - F[j0]) / (F[jj:M] - F[i0]))
                W[:i0] = W[:i0] * ((F[:i0] - F[i0]) / (F[:i0] - F[j0]))
                W[ii:k] = W[ii:k] * ((F[ii:k] - F[i0]) / (F[ii:k] - F[j0]))
                U[j0] = A[i0] * ((F[i0] - F[j0]) / fd(PL[i0], PU[i0]))
                W[i0] = fd(PL[j0], PU[i0]) / A[j0]
                for j in list(range(ii - 1)) + list(range(ii, k)):
                    U[j0] = U[j0] * ((F[i0] - F[j]) / fd(PL[i0], PU[j]))
                    W[i0] = W[i0] * ((-fd(PL[j0], PU[j])) / (F[j] - F[j0]))
                for arr in (PL, PQ, F, A):
                    arr[i0], arr[j0] = arr[j0], arr[i0]
    return F, A, U, V, W, PL, PU, PQ, Rk


def compress_cauchy_eig(FF, U, V, DL, DR, rows, cols, tol):
    """Compress_cauchyEig2 (CauchyHssEig.f90:2640-2829) on the block rows x cols (1-based
    global index arrays) of the eigensolver's matrix: rrluCauchyEigrow, then
    X = P^-1 [I; Z'], Z'(t,j) = Z(Rk+t) W(j) / (F(Rk+t) - F(j)) (CauchylikeEigQ, :1882-1905)
    and Y = CauchylikeEig rows PL(1:Rk) with the unpermuted columns.  Returns (X, Y, Rk);
    (None, None, Rk) when Rk = min(M, N) (the tile is used as is)."""
    FF = np.asarray(FF, dtype=np.float64)
    rows = np.asarray(rows)
    cols = np.asarray(cols)
    M, N = len(rows), len(cols)
    F0 = FF[rows - 1]
    LF, LA, Z, _V, W, PL, _PU, PQ, Rk = rrlu_cauchy_eig_row(F0, np.asarray(U)[rows - 1], np.asarray(V)[cols - 1],
                                                            rows.copy(), cols.copy(), tol, M, N, FF, DL, DR)
    if Rk >= min(M, N):
        return None, None, Rk
    inv = np.empty(M, dtype=np.int64)
    inv[PQ - 1] = np.arange(1, M + 1)
    Q = cauchy_like2(LF[Rk:], LF, Z[Rk:], W, M, Rk)
    X = Q[inv - 1, :]
    den = _fd(FF, DL, DR, PL[:Rk, None], cols[None, :])
    Y = (LA[:Rk, None] * np.asarray(V)[cols - 1][None, :]) / den
    return X, Y, Rk
