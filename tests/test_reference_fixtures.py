"""The reference tests' own configurations at their own sizes, on the GPU.

Each of the reference's test programs fixes a size, a block size, a generator recipe and a
REDIST flag; none stores an answer.  These tests run the same recipes at those sizes and
check them against answers that need no BLAS:

* Test/psmma_testtoeplitz.f90:30,38-46,74,132 -- n = 1024, G(i) = N - i, G(N) = N^2, block
  16, REDIST = .true.: H = N^2 I + (i - j), A H = N^2 A + (A r)1^T - (A 1)r^T, exact for an
  integer A (bit for bit on both paths, locally and through the block-cyclic REDIST path on
  a 2 x 2 grid with 16 x 16 blocks);
* Test/pzfox_fft2.f90:14,37,75,100 -- n = 4800, B = 1, PZMDFTL1 with nb = n / nprow: F*1 is
  N in row 1 and 0 elsewhere (within 1e-12 N);
* Test/psmma_testcauchy.f90:33-53 -- n = 768, poles interlaced on [0.1, 9], U, V, A from
  U(0,1): a 64 x 64 sample of A*H evaluated in 40-digit decimal arithmetic;
* Test/psmma_testhankel.f90:31,38,110 -- n = 16384, G and A from U(0,1): 256 sampled rows
  against the FFT correlation.
Plus the FP64 path at n = 16384 (the split path's headline inputs, clustered poles) on a
sampled block against the oracle at the plain path's 1e-13."""
import numpy as np
import pytest

from oracle import psmma_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-13, "split": 1e-12}


def _t(x, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(cuda).t()


def _np(t):
    return t.t().contiguous().cpu().numpy().T


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_toeplitz_reference_test_n1024_bit_exact(prec, cuda):
    import torch
    import psmma_git_gb300 as P
    n = 1024
    g = O.reference_toeplitz_generator(n)
    rng = np.random.Generator(np.random.PCG64(1024))
    A = rng.integers(-4, 5, size=(n, n)).astype(np.float64)
    X = O.toeplitz_reference_known_answer(A)
    dQ = P.fortran_empty(n, n, torch.float64, cuda)
    P.psmma_toeplitz(n, n, 1.0, _t(A, cuda), torch.from_numpy(g).to(cuda), 0.0, dQ, precision=prec)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_np(dQ), X)
    # the test's own A ~ U(0,1) (random_number): the closed form to rounding
    A = rng.uniform(0.0, 1.0, size=(n, n))
    P.psmma_toeplitz(n, n, 1.0, _t(A, cuda), torch.from_numpy(g).to(cuda), 0.0, dQ, precision=prec)
    torch.cuda.synchronize()
    assert O.rel_fro(_np(dQ), O.toeplitz_reference_known_answer(A)) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_toeplitz_reference_test_redist_2x2_nb16(prec):
    # the reference test's call: psmma_toeplitz(n, n, one, B, 1, 1, desca, TA, ldta, zero, X, 1, 1,
    # desca, WORK, REDIST = .true.) on a 2 x 2 grid ('R'), 16 x 16 blocks, ranks as threads
    import torch
    from psmma_git_gb300.redist import Grid, descinit, pstructured
    from tests.test_redist import ThreadExchange, _dev_local, _run_threads
    n, nb = 1024, 16
    g = Grid(2, 2, "R")
    gen = O.reference_toeplitz_generator(n)
    rng = np.random.Generator(np.random.PCG64(1025))
    GA = rng.integers(-4, 5, size=(n, n)).astype(np.float64)
    X = O.toeplitz_reference_known_answer(GA)
    dgen = torch.from_numpy(gen).cuda()
    ex = ThreadExchange(g.nprocs)

    def rank_fn(r):
        pr, pc = g.coords(r)
        da = descinit(n, n, nb, nb, 0, 0, g, r)
        A = _dev_local(O.bc_local(GA, da, 2, 2, pr, pc), da[8])
        Q = _dev_local(np.zeros_like(O.bc_local(GA, da, 2, 2, pr, pc)), da[8])
        pstructured("toeplitz", n, n, 1.0, A, da, dgen, 0.0, Q, da, g, r, redist=True, precision=prec,
                    exchange=ex(r))
        torch.cuda.synchronize()
        return Q.cpu().numpy(), da

    res = _run_threads(g.nprocs, rank_fn)
    Qg = O.bc_global({r: res[r][0] for r in res}, res[0][1], 2, 2, "R")
    np.testing.assert_array_equal(Qg, X)


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_dft_ones_reference_test_n4800(prec, cuda):
    import torch
    import psmma_git_gb300 as P
    n = 4800
    B = torch.ones((n, n), dtype=torch.complex128, device=cuda).t()  # column-major view
    dC = P.fortran_empty(n, n, torch.complex128, cuda)
    P.pzmdftl1(n, n, 1.0, B, 0.0, dC, precision=prec)
    torch.cuda.synchronize()
    want = torch.zeros((n, n), dtype=torch.complex128, device=cuda)
    want[0, :] = n
    assert float((dC - want).abs().max()) < 1e-12 * n


def test_dft_ones_reference_test_n4800_on_2x2_grid():
    # PZMDFTL1 as the test calls it: nb = kb = n / nprow on a 2 x 2 grid, B = 1
    import torch
    from psmma_git_gb300.redist import Grid, pzmdftl_distributed
    from tests.test_redist import ThreadExchange, _dev_local, _run_threads
    n = 4800
    g = Grid(2, 2, "R")
    nb = n // 2
    ex = ThreadExchange(g.nprocs)

    def rank_fn(r):
        pr, pc = g.coords(r)
        lr, lc = O.numroc(n, nb, pr, 0, 2), O.numroc(n, nb, pc, 0, 2)
        d = (1, 0, n, n, nb, nb, 0, 0, max(1, lr))
        B = _dev_local(np.ones((lr, lc), dtype=np.complex128), d[8])
        Cm = _dev_local(np.zeros((lr, lc), dtype=np.complex128), d[8])
        pzmdftl_distributed(n, n, nb, nb, 1.0, B, 0.0, Cm, 0, 0, g, r, precision="split", exchange=ex(r))
        torch.cuda.synchronize()
        return Cm.cpu().numpy(), d

    res = _run_threads(g.nprocs, rank_fn)
    Cg = O.bc_global({r: res[r][0] for r in res}, res[0][1], 2, 2, "R")
    want = np.zeros((n, n), dtype=np.complex128)
    want[0, :] = n
    assert np.abs(Cg - want).max() < 1e-12 * n


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_cauchy_reference_test_n768_decimal_sample(prec, cuda):
    import torch
    import psmma_git_gb300 as P
    n = 768
    rng = np.random.Generator(np.random.PCG64(768))
    gen = O.reference_cauchy_generators(n, rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 1.0, n))
    A = rng.uniform(0.0, 1.0, (n, n))
    dQ = P.fortran_empty(n, n, torch.float64, cuda)
    P.psmma_cauchy(n, n, 1.0, _t(A, cuda), _t(gen, cuda), 0.0, dQ, precision=prec)
    torch.cuda.synchronize()
    rows, cols = np.arange(5, n, 12), np.arange(0, n, 12)
    ref = O.decimal_cauchy_product(A[rows], gen, cols, n)
    got = _np(dQ)[np.ix_(rows, cols)]
    assert O.rel_fro(got, ref) < TOL[prec]
    assert O.col_max_rel(got, ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_hankel_reference_test_n16384_sampled_rows(prec, cuda):
    import torch
    import psmma_git_gb300 as P
    n = 16384
    g = torch.Generator(device=cuda)
    g.manual_seed(16384)
    G = torch.rand(2 * n - 1, generator=g, device=cuda, dtype=torch.float64)
    A = P.fortran_empty(n, n, torch.float64, cuda)
    A.copy_(torch.rand(n, n, generator=g, device=cuda, dtype=torch.float64))
    Q = P.fortran_empty(n, n, torch.float64, cuda)
    P.psmma_hankel(n, n, 1.0, A, G, 0.0, Q, precision=prec)
    torch.cuda.synchronize()
    rows = torch.arange(0, n, n // 256, device=cuda) + 7
    ref = O.hankel_product_fft(A[rows].cpu().numpy(), G.cpu().numpy(), n)
    assert O.rel_fro(Q[rows].cpu().numpy(), ref) < TOL[prec]
    del A, Q
    torch.cuda.empty_cache()


def test_fp64_path_n16384_clustered_cauchy_sampled_block(cuda):
    # the headline's inputs (10 % of the poles within 1e-10 of a neighbour, A ~ N(0,1)) on the
    # plain FP64 path, checked on a 256 x 512 block of Q at the plain path's bound
    import torch
    import psmma_git_gb300 as P
    n = 16384
    gen = O.cfg_cauchy_generators(n, seed=0, clustered=0.1)
    g = torch.Generator(device=cuda)
    g.manual_seed(1)
    A = P.fortran_empty(n, n, torch.float64, cuda)
    A.copy_(torch.randn(n, n, generator=g, device=cuda, dtype=torch.float64))
    Q = P.fortran_empty(n, n, torch.float64, cuda)
    P.psmma_cauchy(n, n, 1.0, A, _t(gen, cuda), 0.0, Q, precision="fp64")
    torch.cuda.synchronize()
    rows = np.arange(3, n, n // 256)
    cols = np.concatenate([np.arange(0, n, n // 448), np.arange(n - 64, n)])
    Ar = A[torch.from_numpy(rows).to(cuda)].cpu().numpy()
    H = O.const_cauchy(gen, np.arange(1, n + 1), cols + 1)
    ref = Ar @ H
    got = Q[torch.from_numpy(rows).to(cuda)][:, torch.from_numpy(cols).to(cuda)].cpu().numpy()
    assert O.rel_fro(got, ref) < TOL["fp64"]
    assert O.col_max_rel(got, ref) < TOL["fp64"]
    del A, Q
    torch.cuda.empty_cache()
