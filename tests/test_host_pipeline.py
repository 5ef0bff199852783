"""Host-pointer split multiply with the copies overlapped (psmma_*_host with precision split):
A goes up in column chunks while H is generated, the GEMM and the CRT run in row panels and
each panel of Q comes back while the next multiplies.  Results are compared with the device
path and the exact product on ragged sizes (partial chunks and panels, one panel, padded
leading dimensions, beta != 0), on pageable and pinned host memory."""
import numpy as np
import pytest

from oracle import psmma_oracle as O


def _gen(kind, k, seed):
    return O.cfg_cauchy_generators(k, seed=seed) if kind == "cauchy" else O.cfg_vector(2 * k - 1, seed=seed)


def _fortran_view(x, pad):
    """x as a column-major view with leading dimension rows + pad."""
    n, k = x.shape
    base = np.zeros((n + pad, k), order="F")
    base[:n] = x
    return base[:n]


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
@pytest.mark.parametrize("n,k,beta,pad", [(1000, 2500, 0.0, 0), (1000, 2500, -0.75, 5), (100, 700, 0.5, 0),
                                          (513, 129, 0.0, 3)])
def test_host_split_matches_device_and_exact(kind, n, k, beta, pad):
    import torch
    import psmma_git_gb300 as P
    A = O.cfg_matrix(n, k, seed=1)
    gen = np.asfortranarray(_gen(kind, k, 2))
    Q0 = O.cfg_matrix(n, k, seed=3)
    exact = O.dense_product(kind, 0.5, A, gen, beta, Q0, k)
    Ah = _fortran_view(A, pad)
    Qh = _fortran_view(Q0, pad)
    getattr(P, "psmma_" + kind)(n, k, 0.5, Ah, gen, beta, Qh, precision="split")
    assert O.rel_fro(Qh, exact) < 1e-12
    # the device path on the same inputs
    dev = torch.device("cuda")
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    dg = col(gen) if kind == "cauchy" else torch.from_numpy(gen).to(dev)
    dQ = P.fortran_empty(n, k, torch.float64, dev)
    dQ.copy_(torch.from_numpy(Q0))
    getattr(P, "psmma_" + kind)(n, k, 0.5, col(A), dg, beta, dQ, precision="split")
    torch.cuda.synchronize()
    assert O.rel_fro(Qh, dQ.cpu().numpy()) < 1e-13


@pytest.mark.gpu
def test_host_split_pinned_memory_and_repeat():
    import torch
    import psmma_git_gb300 as P
    n, k = 2048, 3000
    A = O.cfg_matrix(n, k, seed=4)
    gen = np.asfortranarray(O.cfg_cauchy_generators(k, seed=5))
    exact = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    Ap = torch.empty((k, n), dtype=torch.float64, pin_memory=True)
    Qp = torch.empty((k, n), dtype=torch.float64, pin_memory=True)
    Ah = Ap.numpy().T
    Qh = Qp.numpy().T
    Ah[:] = A
    for _ in range(3):  # the arena, streams and events are reused across calls
        Qh[:] = np.nan
        P.psmma_cauchy(n, k, 1.0, Ah, gen, 0.0, Qh, precision="split")
        assert O.rel_fro(Qh, exact) < 1e-12


@pytest.mark.gpu
def test_host_split_cauchyeig():
    import psmma_git_gb300 as P
    k, n = 1500, 700
    F, U, V, dl, dr = O.eig_generators(k, seed=6, tiny=3)
    A = O.cfg_matrix(n, k, seed=7)
    Q0 = O.cfg_matrix(n, k, seed=8)
    ref = 2.0 * (A @ O.cauchy_like_eig(F, U, V, dl, dr)) + 0.25 * Q0
    Qh = np.asfortranarray(Q0.copy())
    P.psmma_cauchyeig(n, k, 2.0, A, F, U, V, dl, dr, 0.25, Qh, precision="split")
    assert O.rel_fro(Qh, ref) < 1e-12


@pytest.mark.gpu
def test_host_split_speculation_survives_changing_inputs():
    # the H residues are computed for the PH of the previous call of the same shape while A is
    # uploaded; inputs whose statistics move PH (flat rows, then one-hot rows, then flat rows
    # again) must still give the exact product and the device path's result
    import torch
    import psmma_git_gb300 as P
    n, k = 600, 700
    gen = np.asfortranarray(O.cfg_cauchy_generators(k, seed=51))
    rng = np.random.default_rng(52)
    flat = O.cfg_matrix(n, k, seed=53)
    spiky = 1e-3 * O.cfg_matrix(n, k, seed=54)
    spiky[np.arange(n), rng.integers(0, k, n)] = 10.0
    dev = torch.device("cuda")
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    for A in [flat, spiky, flat, spiky]:
        Qh = np.zeros((n, k), order="F")
        P.psmma_cauchy(n, k, 1.0, np.asfortranarray(A), gen, 0.0, Qh, precision="split")
        exact = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
        assert O.rel_fro(Qh, exact) < 1e-12
        dQ = P.fortran_empty(n, k, torch.float64, dev)
        P.psmma_cauchy(n, k, 1.0, col(A), col(gen), 0.0, dQ, precision="split")
        torch.cuda.synchronize()
        assert O.rel_fro(Qh, dQ.cpu().numpy()) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
def test_host_split_row_panels_repeat_ragged(kind):
    # repeated calls of one shape upload A in row panels and scale with the previous call's
    # PA / PH (ragged last panel: 1000 rows = 7 full 128-row tiles + 104 rows); fresh operands
    # of the same statistics each call, plus one call with a different scale of A
    import psmma_git_gb300 as P
    n, k = 1000, 777
    gen = np.asfortranarray(_gen(kind, k, 61))
    for seed, scale in [(62, 1.0), (63, 1.0), (64, 1.0), (65, 2.0 ** 40), (66, 2.0 ** 40)]:
        A = scale * O.cfg_matrix(n, k, seed=seed)
        Qh = np.full((n, k), np.nan, order="F")
        getattr(P, "psmma_" + kind)(n, k, 1.0, np.asfortranarray(A), gen, 0.0, Qh, precision="split")
        exact = O.dense_product(kind, 1.0, A, gen, 0.0, None, k)
        assert O.rel_fro(Qh, exact) < 1e-12


@pytest.mark.gpu
def test_host_split_panel_cuts():
    # 4300 rows = 34 row tiles (the last one ragged): the speculative calls cut the first
    # eighth to two tiles and halve the last one three times (panels 2, 3, 5 x 5, 2, 1, 1)
    import psmma_git_gb300 as P
    n, k = 4300, 300
    gen = np.asfortranarray(O.cfg_cauchy_generators(k, seed=71, clustered=0.1))
    for seed in (72, 73, 74):
        A = O.cfg_matrix(n, k, seed=seed, dist="normal")
        Qh = np.full((n, k), np.nan, order="F")
        P.psmma_cauchy(n, k, 1.0, np.asfortranarray(A), gen, 0.0, Qh, precision="split")
        assert O.rel_fro(Qh, O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("kind,n,k,levels,pad", [("cauchy", 1000, 2500, 0, 3), ("toeplitz", 700, 2000, 1, 0),
                                                 ("hankel", 300, 4096, 2, 5)])
def test_host_split_pinned_panels_match_pageable_and_device(kind, n, k, levels, pad):
    # pinned host buffers with padded leading dimensions through the speculative row-panel
    # pipeline (pitched copies of whole rows, rows past n untouched).  The repeated calls agree
    # bit for bit, and with the pageable host call and the device call (whose row statistics
    # are summed in other partitions) to rounding
    import torch
    import psmma_git_gb300 as P
    A = O.cfg_matrix(n, k, seed=n + 71)
    gen = np.asfortranarray(_gen(kind, k, 72))
    fn = getattr(P, "psmma_" + kind)
    Ap = torch.zeros((k, n + pad), dtype=torch.float64, pin_memory=True)
    Qp = torch.zeros((k, n + pad), dtype=torch.float64, pin_memory=True)
    Ah, Qh = Ap.numpy().T[:n], Qp.numpy().T[:n]
    Ah[:] = A
    Qp.numpy().T[n:] = 7.0  # rows past n must stay untouched
    pageable = np.zeros((n, k), order="F")
    fn(n, k, 1.25, np.asfortranarray(A), gen, 0.0, pageable, precision="split", block_levels=levels)
    first = None
    for _ in range(3):  # speculative calls (the pageable call was the shape's first)
        Qh[:] = np.nan
        fn(n, k, 1.25, Ah, gen, 0.0, Qh, precision="split", block_levels=levels)
        if first is None:
            first = Qh.copy()
        np.testing.assert_array_equal(Qh, first)
    assert O.rel_fro(Qh, pageable) < 1e-13
    assert (Qp.numpy().T[n:] == 7.0).all()
    dev = torch.device("cuda")
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    dg = col(gen) if kind == "cauchy" else torch.from_numpy(gen).to(dev)
    dQ = P.fortran_empty(n, k, torch.float64, dev)
    fn(n, k, 1.25, col(A), dg, 0.0, dQ, precision="split", block_levels=levels)
    torch.cuda.synchronize()
    assert O.rel_fro(Qh, dQ.cpu().numpy()) < 1e-13
    assert O.rel_fro(Qh, O.dense_product(kind, 1.25, A, gen, 0.0, None, k)) < 1e-12
