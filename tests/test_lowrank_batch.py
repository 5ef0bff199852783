"""Batched merge level (psmma_cauchy_batch_lowrank): off-diagonal blocks compressed by RRQR
(Compress_RRQR, Auxil_2p5D.f90:1063-1189) or the structured RRLU (compress_cauchy,
Cauchylowrank.f90:387-491), products through the FP64 and split paths.  GPU results are
compared with the oracle's restatement of the same merge level (ranks and result) and with
the exact dense product."""
import ctypes as C

import numpy as np
import pytest

from oracle import psmma_oracle as O
from psmma_git_gb300 import _lib

SIZES = [1, 2, 3, 37, 128, 300, 515, 1031]


def _problems(sizes, seed=0):
    out = []
    for i, n in enumerate(sizes):
        g = O.cfg_cauchy_generators(n, seed=seed + 10 * i)
        A = O.cfg_matrix(n, n, seed=seed + 10 * i + 1)
        Q0 = O.cfg_matrix(n, n, seed=seed + 10 * i + 2)
        out.append((A, g, Q0))
    return out


def _to_dev(problems, ld_pad=0):
    import torch
    from psmma_git_gb300 import fortran_empty
    dev = []
    for A, g, Q0 in problems:
        n = A.shape[0]
        Ad = fortran_empty(n, n, ld=n + ld_pad)
        Ad.copy_(torch.from_numpy(A))
        gd = torch.from_numpy(np.asfortranarray(g)).cuda()
        gd = gd.t().contiguous().t()  # column-major n x 4
        Qd = fortran_empty(n, n, ld=n + ld_pad)
        Qd.copy_(torch.from_numpy(Q0))
        dev.append((Ad, gd, Qd))
    return dev


def test_batch_argument_checks(lib):
    items = (_lib.PsmmaBatchItem * 1)()
    buf = np.zeros(16)
    p = buf.ctypes.data
    items[0].n, items[0].A, items[0].lda, items[0].gen, items[0].ldgen = 4, p, 4, p, 4
    items[0].Q, items[0].ldq = p, 4
    f = lib.psmma_cauchy_batch_lowrank
    assert f(0, items, 1.0, 0.0, 0, 1e-14, None, None, None, None) == 0          # empty batch
    items[0].n = -1
    assert f(1, items, 1.0, 0.0, 0, 1e-14, None, None, None, None) == -2
    items[0].n, items[0].lda = 4, 3
    assert f(1, items, 1.0, 0.0, 0, 1e-14, None, None, None, None) == -9
    items[0].lda, items[0].ldq = 4, 3
    assert f(1, items, 1.0, 0.0, 0, 1e-14, None, None, None, None) == -14
    items[0].ldq, items[0].ldgen = 4, 3
    assert f(1, items, 1.0, 0.0, 0, 1e-14, None, None, None, None) == _lib.PSMMA_EGEN
    items[0].ldgen = 4
    assert f(1, items, 1.0, 0.0, 7, 1e-14, None, None, None, None) == _lib.PSMMA_EUNSUPPORTED  # compressor
    assert f(1, items, 1.0, 0.0, 0, 0.0, None, None, None, None) == _lib.PSMMA_EUNSUPPORTED    # tol


def test_oracle_merge_level_matches_exact_product():
    for comp in ["rrqr", "rrlu"]:
        for (A, g, Q0) in _problems([2, 37, 300]):
            n = A.shape[0]
            Q, ranks = O.merge_level_product(A, g, Q0, 0.75, -0.5, comp, 1e-14)
            ref = 0.75 * A @ O.dense_h("cauchy", g, n) - 0.5 * Q0
            assert O.rel_fro(Q, ref) < 1e-14
            assert len(ranks) == 2 and all(0 <= r <= n for r in ranks)


def _run(problems, comp, precision, alpha, beta, ld_pad=0, n_moduli=0):
    import torch
    from psmma_git_gb300 import cauchy_batch_lowrank
    dev = _to_dev(problems, ld_pad)
    ranks, info = cauchy_batch_lowrank(dev, alpha, beta, compressor=comp, tol=1e-14, precision=precision,
                                       n_moduli=n_moduli)
    torch.cuda.synchronize()
    return [Qd.cpu().numpy() for (_, _, Qd) in dev], ranks, info


@pytest.mark.gpu
@pytest.mark.parametrize("comp", ["rrqr", "rrlu"])
def test_batch_fp64_matches_oracle(comp):
    problems = _problems(SIZES, seed=3)
    alpha, beta = 0.75, -0.5
    Qs, ranks, info = _run(problems, comp, "fp64", alpha, beta, ld_pad=3)
    k = 0
    for (A, g, Q0), Qg in zip(problems, Qs):
        n = A.shape[0]
        Qo, ro = O.merge_level_product(A, g, Q0, alpha, beta, comp, 1e-14)
        exact = alpha * A @ O.dense_h("cauchy", g, n) + beta * Q0
        rg = ranks[k:k + len(ro)]
        k += len(ro)
        for a, b in zip(rg, ro):  # QR pivots can differ at rounding-level near-ties
            assert abs(a - b) <= 1, (n, rg, ro)
        assert O.rel_fro(Qg, Qo) < 1e-13, n
        assert O.rel_fro(Qg, exact) < 1e-13, n
    assert k == len(ranks) == info["n_blocks"]
    eff = sum(2.0 * n ** 3 for n in SIZES)
    assert info["effective_flops"] == pytest.approx(eff)
    assert 0 < info["executed_flops"] < eff


@pytest.mark.gpu
@pytest.mark.parametrize("comp", ["rrqr", "rrlu"])
def test_batch_split_matches_exact(comp):
    problems = _problems([64, 300, 1031, 2048], seed=5)
    Qs, ranks, info = _run(problems, comp, "split", 1.0, 0.0)
    for (A, g, Q0), Qg in zip(problems, Qs):
        n = A.shape[0]
        exact = A @ O.dense_h("cauchy", g, n)
        assert O.rel_fro(Qg, exact) < 1e-12, n


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["split", "fp64"])
def test_repeated_batches_reuse_the_stream_graph(prec):
    # the product rounds' CUDA graph of a stream is updated in place on later calls (new
    # operands and buffers, alpha, beta; the same generators, hence the same ranks and
    # topology), and the results stay those of a fresh call
    import torch
    from psmma_git_gb300 import cauchy_batch_lowrank
    sizes = [64, 300, 515, 1031]
    base = _problems(sizes, seed=21)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        first = _to_dev(base)
        _, info0 = cauchy_batch_lowrank(first, 1.0, 0.0, compressor="rrlu", tol=1e-14, precision=prec, stream=s)
        for seed, (alpha, beta) in [(22, (0.5, 0.0)), (23, (-1.25, 0.75))]:
            other = _problems(sizes, seed=seed)
            problems = [(A, g, Q0) for (_, g, _), (A, _, Q0) in zip(base, other)]
            dev = _to_dev(problems)
            _, info = cauchy_batch_lowrank(dev, alpha, beta, compressor="rrlu", tol=1e-14, precision=prec, stream=s)
            s.synchronize()
            assert info["graph_reused"], "the second and later calls of the same shape update the graph"
            for (A, g, Q0), (_, _, Qd) in zip(problems, dev):
                exact = alpha * A @ O.dense_h("cauchy", g, A.shape[0]) + beta * Q0
                assert O.rel_fro(Qd.cpu().numpy(), exact) < (1e-12 if prec == "split" else 1e-13)
    assert info0["graph_reused"] in (True, False)


@pytest.mark.gpu
def test_batch_ranks_match_reference_scan_on_larger_blocks():
    # off-diagonal blocks of 2048 x 2048: the RRQR rank is the first |R_kk| <= tol |R_11|
    problems = _problems([4096], seed=11)
    _, ranks, _ = _run(problems, "rrqr", "fp64", 1.0, 0.0)
    A, g, _ = problems[0]
    _, ro = O.merge_level_product(A, g, np.zeros((4096, 4096)), 1.0, 0.0, "rrqr", 1e-14)
    assert all(abs(a - b) <= 1 for a, b in zip(ranks, ro)), (ranks, ro)


@pytest.mark.gpu
def test_batch_workspace_and_caller_buffer():
    import torch
    from psmma_git_gb300 import batch_workspace_size, cauchy_batch_lowrank
    problems = _problems([300, 515], seed=9)
    dev = _to_dev(problems)
    need = batch_workspace_size(dev, compressor="rrqr")
    assert need > 0
    work = torch.empty(need, dtype=torch.uint8, device="cuda")
    cauchy_batch_lowrank(dev, 1.0, 0.0, compressor="rrqr", work=work)
    torch.cuda.synchronize()
    for (A, g, _), (_, _, Qd) in zip(problems, dev):
        exact = A @ O.dense_h("cauchy", g, A.shape[0])
        assert O.rel_fro(Qd.cpu().numpy(), exact) < 1e-13
    small = torch.empty(need // 2, dtype=torch.uint8, device="cuda")
    from psmma_git_gb300 import PsmmaError
    with pytest.raises(PsmmaError) as e:
        cauchy_batch_lowrank(dev, 1.0, 0.0, compressor="rrqr", work=small)
    assert e.value.status == _lib.PSMMA_EWORKSPACE


@pytest.mark.gpu
@pytest.mark.parametrize("comp", ["rrqr", "rrlu"])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_batch_uncompressed_blocks_use_the_generated_tile(comp, prec):
    # tol so small that no block truncates: every off-diagonal block is multiplied as the
    # generated tile (the reference would multiply a stale buffer there)
    import torch
    from psmma_git_gb300 import cauchy_batch_lowrank
    problems = _problems([3, 37, 129], seed=21)
    dev = _to_dev(problems)
    ranks, info = cauchy_batch_lowrank(dev, 0.5, 2.0, compressor=comp, tol=1e-300, precision=prec)
    torch.cuda.synchronize()
    assert info["full_rank_blocks"] == len(ranks) == 6
    tol = 1e-13 if prec == "fp64" else 1e-12
    for (A, g, Q0), (_, _, Qd) in zip(problems, dev):
        exact = 0.5 * A @ O.dense_h("cauchy", g, A.shape[0]) + 2.0 * Q0
        assert O.rel_fro(Qd.cpu().numpy(), exact) < tol


def test_tuner_fp64_and_empty_batches_return_at_once(lib):
    # no tunables on the FP64 path and nothing to do for an empty batch: no GPU work
    items = (_lib.PsmmaBatchItem * 1)()
    res = _lib.PsmmaTuneResult()
    assert lib.psmma_tune_batch(0, items, 1.0, 0.0, 0, 1e-14, None, C.byref(res), None) == 0
    o = _lib.PsmmaOpts()
    o.precision = _lib.PREC_FP64
    assert lib.psmma_tune_batch(0, items, 1.0, 0.0, 1, 1e-14, C.byref(o), C.byref(res), None) == 0
    assert res.candidates == 0 and res.group_m > 0


@pytest.mark.gpu
def test_tuner_picks_a_configuration_and_results_stay_exact():
    import torch
    from psmma_git_gb300 import cauchy_batch_lowrank, tune_batch
    problems = _problems([200, 700, 1500], seed=31)
    dev = _to_dev(problems)
    t = tune_batch(dev, compressor="rrlu", precision="split")
    assert t["candidates"] >= 10 and t["ms_best"] > 0 and t["ms_best"] <= t["ms_default"] * 1.05
    assert t["group_m"] in (4, 8, 12, 16)
    dev = _to_dev(problems)
    cauchy_batch_lowrank(dev, 1.0, 0.0, compressor="rrlu", precision="split")
    torch.cuda.synchronize()
    for (A, g, _), (_, _, Qd) in zip(problems, dev):
        exact = A @ O.dense_h("cauchy", g, A.shape[0])
        assert O.rel_fro(Qd.cpu().numpy(), exact) < 1e-12


# ---- Toeplitz merge level (PSTOEPLITZ_COMPUTE's low-rank branch, RRQR) ---------------------
def _toeplitz_problems(sizes, seed=0, smooth=True):
    out = []
    for i, n in enumerate(sizes):
        if smooth:  # H(i, j) = 1 / (j - i + 0.5 + s): Cauchy-like, numerically low-rank off the diagonal
            s = 0.1 * ((seed + i) % 3)
            g = 1.0 / (np.arange(2 * n - 1) - (n - 1) + 0.5 + s)
        else:
            g = O.cfg_vector(2 * n - 1, seed=seed + 10 * i)
        A = O.cfg_matrix(n, n, seed=seed + 10 * i + 1)
        Q0 = O.cfg_matrix(n, n, seed=seed + 10 * i + 2)
        out.append((A, g, Q0))
    return out


def test_toeplitz_batch_argument_checks(lib):
    items = (_lib.PsmmaBatchItem * 1)()
    buf = np.zeros(16)
    p = buf.ctypes.data
    items[0].n, items[0].A, items[0].lda, items[0].gen, items[0].ldgen = 4, p, 4, p, 6  # G needs 2n - 1 = 7
    items[0].Q, items[0].ldq = p, 4
    f = lib.psmma_toeplitz_batch_lowrank
    assert f(1, items, 1.0, 0.0, 1e-14, None, None, None, None) == _lib.PSMMA_EGEN
    assert f(0, items, 1.0, 0.0, 1e-14, None, None, None, None) == 0


def test_oracle_toeplitz_merge_level_matches_exact_product():
    for smooth in [True, False]:
        for (A, g, Q0) in _toeplitz_problems([2, 37, 300], seed=4, smooth=smooth):
            n = A.shape[0]
            Q, ranks = O.merge_level_product(A, g, Q0, 0.75, -0.5, "rrqr", 1e-14, kind="toeplitz")
            ref = 0.75 * A @ O.dense_h("toeplitz", g, n) - 0.5 * Q0
            assert O.rel_fro(Q, ref) < 1e-14


def _run_toeplitz(problems, precision, alpha, beta, ld_pad=0):
    import torch
    from psmma_git_gb300 import fortran_empty, toeplitz_batch_lowrank
    dev = []
    for A, g, Q0 in problems:
        n = A.shape[0]
        Ad = fortran_empty(n, n, ld=n + ld_pad)
        Ad.copy_(torch.from_numpy(A))
        Qd = fortran_empty(n, n, ld=n + ld_pad)
        Qd.copy_(torch.from_numpy(Q0))
        dev.append((Ad, torch.from_numpy(np.ascontiguousarray(g)).cuda(), Qd))
    ranks, info = toeplitz_batch_lowrank(dev, alpha, beta, tol=1e-14, precision=precision)
    torch.cuda.synchronize()
    return [Qd.cpu().numpy() for (_, _, Qd) in dev], ranks, info


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_toeplitz_batch_matches_oracle_and_exact(prec):
    problems = _toeplitz_problems([1, 2, 3, 37, 300, 515, 1031], seed=7) + _toeplitz_problems([200, 333], seed=9,
                                                                                              smooth=False)
    alpha, beta = 0.75, -0.5
    Qs, ranks, info = _run_toeplitz(problems, prec, alpha, beta, ld_pad=2)
    tol = 1e-13 if prec == "fp64" else 1e-12
    k = 0
    for (A, g, Q0), Qg in zip(problems, Qs):
        n = A.shape[0]
        Qo, ro = O.merge_level_product(A, g, Q0, alpha, beta, "rrqr", 1e-14, kind="toeplitz")
        exact = alpha * A @ O.dense_h("toeplitz", g, n) + beta * Q0
        rg = ranks[k:k + len(ro)]
        k += len(ro)
        for a, b in zip(rg, ro):
            assert abs(a - b) <= 1 or min(a, b) >= 64, (n, rg, ro)  # full-rank tiles stop at the QR cap
        assert O.rel_fro(Qg, exact) < tol, n
        assert O.rel_fro(Qg, Qo) < tol, n
    assert k == len(ranks) == info["n_blocks"]
    assert info["full_rank_blocks"] >= 4  # the random generators do not compress
