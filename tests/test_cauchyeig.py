"""PSMMA_CAUCHYEIG: the eigensolver's Cauchy multiply with accurate denominators
(CauchylikeEig, CauchyHssEig.f90:1693-1774).  Pins: exact rational products on the FP64
inputs, including roots 2^-70 (relative) above their pole, where F(i) - D(j) formed from D
in FP64 is 0."""
import ctypes as C

import numpy as np
import pytest

from oracle import psmma_oracle as O
from psmma_git_gb300 import _lib


def test_oracle_restatement_is_exact_to_rounding_and_naive_form_fails():
    k = 24
    F, U, V, dl, dr = O.eig_generators(k, seed=1, tiny=3)
    A = O.cfg_matrix(5, k, seed=2)
    exact = O.exact_cauchy_eig_product(A, F, U, V, dl, dr)
    got = A @ O.cauchy_like_eig(F, U, V, dl, dr)
    assert O.rel_fro(got, exact) < 1e-15
    # the naive denominator F(i) - D(j) with D(j) = F(j) + DIFL(j) rounded to FP64 is zero
    D = F + dl
    with np.errstate(divide="ignore", invalid="ignore"):
        naive = A @ (U[:, None] * V[None, :] / (F[:, None] - D[None, :]))
    assert not np.all(np.isfinite(naive))


def test_argument_checks_use_pscauchyeig_info_numbers(lib):
    buf = np.zeros(64)
    p = C.c_void_p(buf.ctypes.data)
    f = lib.psmma_cauchyeig
    assert f(-1, 4, 1.0, p, 4, p, None, p, p, p, p, 0.0, p, 4, None, None) == -1
    assert f(4, -1, 1.0, p, 4, p, None, p, p, p, p, 0.0, p, 4, None, None) == -2
    assert f(4, 4, 1.0, p, 3, p, None, p, p, p, p, 0.0, p, 4, None, None) == -7
    assert f(4, 4, 1.0, p, 4, p, None, p, p, p, p, 0.0, p, 3, None, None) == -17
    assert f(4, 4, 1.0, p, 4, None, None, p, p, p, p, 0.0, p, 4, None, None) == _lib.PSMMA_EGEN
    assert f(0, 4, 1.0, p, 1, p, None, p, p, p, p, 0.0, p, 1, None, None) == 0       # quick return
    i = lambda v: C.byref(C.c_int(v))
    d = lambda v: C.byref(C.c_double(v))
    desc = (C.c_int * 9)(1, 0, 4, 4, 4, 4, 0, 0, 4)
    lib.psmma_cauchyeig_(i(-1), i(4), i(1), d(1.0), p, i(1), i(1), desc, p, p, p, p, p, p, d(0.0), p, i(1), i(1),
                         desc, p, i(0))
    assert lib.psmma_last_status() == -1


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("split", 1e-12)])
def test_cauchyeig_matches_exact_rational_product(prec, tol):
    import torch
    import psmma_git_gb300 as P
    k, n = 40, 7
    F, U, V, dl, dr = O.eig_generators(k, seed=3, tiny=4)
    A = O.cfg_matrix(n, k, seed=4)
    Q0 = O.cfg_matrix(n, k, seed=5)
    exact = 0.5 * O.exact_cauchy_eig_product(A, F, U, V, dl, dr) - 2.0 * Q0
    dA = P.fortran_empty(n, k)
    dA.copy_(torch.from_numpy(A))
    dQ = P.fortran_empty(n, k)
    dQ.copy_(torch.from_numpy(Q0))
    P.psmma_cauchyeig(n, k, 0.5, dA, _dev(F), _dev(U), _dev(V), _dev(dl), _dev(dr), -2.0, dQ, precision=prec)
    torch.cuda.synchronize()
    got = dQ.cpu().numpy()
    assert O.rel_fro(got, exact) < tol
    # per column too: every column of H carries one huge entry (the root next to its pole)
    cols = [O.rel_fro(got[:, j], exact[:, j]) for j in range(k)]
    assert max(cols) < 50 * tol


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(1, 1), (3, 2), (257, 300), (1000, 1031)])
def test_cauchyeig_fp64_and_split_match_oracle(n, k):
    import torch
    import psmma_git_gb300 as P
    F, U, V, dl, dr = O.eig_generators(k, seed=k, tiny=k // 50)
    A = O.cfg_matrix(n, k, seed=n)
    ref = A @ O.cauchy_like_eig(F, U, V, dl, dr)
    for prec, tol in [("fp64", 1e-13), ("split", 1e-12)]:
        dA = P.fortran_empty(n, k, ld=n + 2)
        dA.copy_(torch.from_numpy(A))
        dQ = P.fortran_empty(n, k)
        P.psmma_cauchyeig(n, k, 1.0, dA, _dev(F), _dev(U), _dev(V), _dev(dl), _dev(dr), 0.0, dQ, precision=prec)
        torch.cuda.synchronize()
        assert O.rel_fro(dQ.cpu().numpy(), ref) < tol, prec


@pytest.mark.gpu
def test_cauchyeig_host_and_fortran_abi():
    import psmma_git_gb300 as P
    lib = _lib.load()
    k, n = 64, 33
    F, U, V, dl, dr = O.eig_generators(k, seed=9, tiny=2)
    A = O.cfg_matrix(n, k, seed=10)
    ref = A @ O.cauchy_like_eig(F, U, V, dl, dr)
    Qh = np.zeros((n, k), order="F")
    P.psmma_cauchyeig(n, k, 1.0, A, F, U, V, dl, dr, 0.0, Qh)
    assert O.rel_fro(Qh, ref) < 1e-13
    i = lambda v: C.byref(C.c_int(v))
    d = lambda v: C.byref(C.c_double(v))
    desc = (C.c_int * 9)(1, 0, n, k, 64, 64, 0, 0, n)
    Qf = np.zeros((n, k), order="F")
    vp = lambda a: C.c_void_p(np.ascontiguousarray(a).ctypes.data)
    keep = [np.ascontiguousarray(x) for x in (F, U, V, dl, dr)]
    lib.psmma_cauchyeig_(i(n), i(k), i(1), d(1.0), C.c_void_p(A.ctypes.data), i(1), i(1), desc,
                         vp(keep[0]), None, vp(keep[1]), vp(keep[2]), vp(keep[3]), vp(keep[4]), d(0.0),
                         C.c_void_p(Qf.ctypes.data), i(1), i(1), desc, None, i(0))
    assert lib.psmma_last_status() == 0
    assert O.rel_fro(Qf, ref) < 1e-13


def test_oracle_eig_rrlu_factorises_the_tile():
    # rrluCauchyEigrow restated: X Y reproduces the off-diagonal tile at the truncation level and
    # the rank matches the pivoted QR's
    for n in [64, 300, 1031]:
        F, U, V, dl, dr = O.eig_generators(n, seed=n, tiny=n // 100)
        H = O.cauchy_like_eig(F, U, V, dl, dr)
        h = n // 2
        for (r0, r1, c0, c1) in [(0, h, h, n), (h, n, 0, h)]:
            X, Y, rk = O.compress_cauchy_eig(F, U, V, dl, dr, np.arange(r0 + 1, r1 + 1),
                                             np.arange(c0 + 1, c1 + 1), 1e-14)
            T = H[r0:r1, c0:c1]
            assert X is not None
            assert np.linalg.norm(X @ Y - T) / np.linalg.norm(T) < 1e-13
            assert abs(rk - O.compress_rrqr(T, 1e-14)[2]) <= 1


@pytest.mark.gpu
@pytest.mark.parametrize("comp", ["rrqr", "rrlu"])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("split", 1e-12)])
def test_cauchyeig_merge_level(prec, tol, comp):
    import torch
    import psmma_git_gb300 as P
    sizes = [1, 2, 37, 300, 1031]
    probs, dev = [], []
    for i, n in enumerate(sizes):
        F, U, V, dl, dr = O.eig_generators(n, seed=40 + i, tiny=n // 50)
        A = O.cfg_matrix(n, n, seed=50 + i)
        Q0 = O.cfg_matrix(n, n, seed=60 + i)
        probs.append((A, (F, U, V, dl, dr), Q0))
        dA = P.fortran_empty(n, n)
        dA.copy_(torch.from_numpy(A))
        g = torch.from_numpy(np.stack([F, U, V, dl, dr], axis=1)).cuda().t().contiguous().t()  # n x 5
        dQ = P.fortran_empty(n, n)
        dQ.copy_(torch.from_numpy(Q0))
        dev.append((dA, g, dQ))
    ranks, info = P.cauchy_batch_lowrank(dev, 0.5, -1.0, compressor=comp, tol=1e-14, precision=prec, eig=True)
    torch.cuda.synchronize()
    k = 0
    for (A, gens, Q0), (_, _, dQ) in zip(probs, dev):
        Qo, ro = O.merge_level_eig_product(A, *gens, Q0, 0.5, -1.0, 1e-14, comp)
        exact = 0.5 * A @ O.cauchy_like_eig(*gens) - Q0
        got = dQ.cpu().numpy()
        for a, b in zip(ranks[k:k + len(ro)], ro):
            assert abs(a - b) <= 1
        k += len(ro)
        assert O.rel_fro(got, Qo) < tol
        assert O.rel_fro(got, exact) < tol
    assert info["n_blocks"] == k


def test_cauchyeig_batch_argument_checks(lib):
    items = (_lib.PsmmaBatchItem * 1)()
    buf = np.zeros(64)
    p = buf.ctypes.data
    items[0].n, items[0].A, items[0].lda, items[0].gen, items[0].ldgen = 4, p, 4, p, 3
    items[0].Q, items[0].ldq = p, 4
    assert lib.psmma_cauchyeig_batch_lowrank(1, items, 1.0, 0.0, _lib.COMPRESS_RRLU, 1e-14, None, None, None,
                                             None) == _lib.PSMMA_EGEN
    assert lib.psmma_cauchyeig_batch_lowrank(0, items, 1.0, 0.0, _lib.COMPRESS_RRLU, 1e-14, None, None, None,
                                             None) == 0
