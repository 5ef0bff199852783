"""GPU parity of the FP64 plain path against the oracle (tolerance: 1e-13 relative
Frobenius, the plain-path bound; integer known answers must match bit for bit)."""
import numpy as np
import pytest

from oracle import psmma_oracle as O
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _t(x, cuda):
    """A numpy array as a column-major CUDA tensor."""
    import torch
    x = np.asfortranarray(x)
    return torch.from_numpy(np.ascontiguousarray(x.T)).to(cuda).t()


def _np(t):
    return t.t().contiguous().cpu().numpy().T


def _run(kind, n, k, alpha, A, gen, beta, Q0, cuda, ld_pad=0, **kw):
    import psmma_git_gb300 as P
    import torch
    dA = P.fortran_empty(n, k, torch.float64, cuda, ld=n + ld_pad)
    dA.copy_(_t(A, cuda))
    dQ = P.fortran_empty(n, k, torch.float64, cuda, ld=n + ld_pad)
    dQ.copy_(_t(Q0, cuda))
    if kind == "cauchy":
        dg = _t(np.asfortranarray(gen), cuda)
    else:
        dg = torch.from_numpy(np.asarray(gen)).to(cuda)
    getattr(P, "psmma_" + kind)(n, k, alpha, dA, dg, beta, dQ, **kw)
    torch.cuda.synchronize()
    return _np(dQ)


def _gen(kind, k, seed=3):
    return O.cfg_cauchy_generators(k, seed=seed) if kind == "cauchy" else O.cfg_vector(2 * k - 1, seed=seed)


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
@pytest.mark.parametrize("n,k", [(1, 1), (7, 5), (128, 128), (200, 333), (513, 130), (1024, 1024)])
def test_real_kinds_match_dense_oracle(kind, n, k, cuda):
    A = O.cfg_matrix(n, k, seed=n + k)
    gen = _gen(kind, k)
    Q0 = O.cfg_matrix(n, k, seed=7)
    got = _run(kind, n, k, 1.25, A, gen, -0.5, Q0, cuda)
    ref = O.dense_product(kind, 1.25, A, gen, -0.5, Q0, k)
    assert O.rel_fro(got, ref) < TOL


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
def test_leading_dimension_and_beta_zero_ignores_q(kind, cuda):
    n, k = 300, 260
    A = O.cfg_matrix(n, k, seed=1)
    gen = _gen(kind, k)
    Q0 = np.full((n, k), np.nan)            # beta == 0: Q must not be read (BLAS semantics)
    got = _run(kind, n, k, 2.0, A, gen, 0.0, Q0, cuda, ld_pad=37)
    ref = O.dense_product(kind, 2.0, A, gen, 0.0, None, k)
    assert np.isfinite(got).all()
    assert O.rel_fro(got, ref) < TOL


def test_alpha_zero_scales_q(cuda):
    n, k = 50, 40
    Q0 = O.cfg_matrix(n, k, seed=2)
    got = _run("cauchy", n, k, 0.0, np.zeros((n, k)), _gen("cauchy", k), 3.0, Q0, cuda)
    np.testing.assert_array_equal(got, 3.0 * Q0)


def test_toeplitz_reference_fixture_bit_exact(cuda):
    z = np.load(GOLDEN / "toeplitz_kat.npz")
    n = int(z["n"])
    got = _run("toeplitz", n, n, 1.0, z["A"], z["g"], 0.0, np.zeros((n, n)), cuda)
    np.testing.assert_array_equal(got, z["X"])


def test_hankel_fixture_bit_exact(cuda):
    z = np.load(GOLDEN / "hankel_exact.npz")
    n = int(z["n"])
    got = _run("hankel", n, n, 1.0, z["A"], z["g"], 0.0, np.zeros((n, n)), cuda)
    np.testing.assert_array_equal(got, z["X"])


def test_cauchy_reference_recipe_exact(cuda):
    z = np.load(GOLDEN / "cauchy_exact.npz")
    n = int(z["n"])
    got = _run("cauchy", n, n, 1.0, z["A"], z["gen"], 0.0, np.zeros((n, n)), cuda)
    assert O.rel_fro(got, z["X"]) < 1e-14


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
def test_matches_ring_restatement(kind, cuda):
    # the reference's ring on a 2x2 grid, block 64 (its defect-free configuration)
    n = 512
    A = O.cfg_matrix(n, n, seed=9)
    gen = _gen(kind, n, seed=10)
    Q0 = O.cfg_matrix(n, n, seed=11)
    ref = O.ps_compute(kind, n, n, 1.0, A, gen, 1.0, Q0, 2, 2, 64)
    got = _run(kind, n, n, 1.0, A, gen, 1.0, Q0, cuda)
    assert O.rel_fro(got, ref) < TOL


def _dft(n, k, alpha, B, beta, C0, cuda, variant="pzmdftl"):
    import psmma_git_gb300 as P
    import torch
    dB = _t(B.astype(np.complex128), cuda)
    dC = _t(C0.astype(np.complex128), cuda)
    getattr(P, variant)(n, k, alpha, dB, beta, dC)
    torch.cuda.synchronize()
    return _np(dC)


@pytest.mark.parametrize("n,k", [(1, 3), (8, 8), (96, 40), (250, 300), (1024, 512)])
def test_dft_matches_fft(n, k, cuda):
    B = O.cfg_matrix(n, k, seed=n, complex_=True)
    C0 = O.cfg_matrix(n, k, seed=k + 1, complex_=True)
    got = _dft(n, k, 0.5, B, -2.0, C0, cuda)
    ref = O.dft_product(0.5, B, -2.0, C0)
    assert O.rel_fro(got, ref) < TOL


@pytest.mark.parametrize("n,k,pad,beta", [(2050, 33, 2, -2.0), (4100, 17, 0, 0.0), (8192, 40, 3, 0.5)])
def test_dft_radix_steps_match_fft(n, k, pad, beta, cuda):
    # the FP64 path takes the split path's radix step (2, 4, 8 at these n): F_(n/R) on R k
    # columns, then the twiddles and butterflies; padded leading dimensions, rows past n untouched
    import psmma_git_gb300 as P
    import torch
    B = O.cfg_matrix(n, k, seed=n + 5, complex_=True)
    C0 = O.cfg_matrix(n, k, seed=k + 6, complex_=True)
    Bbig = np.zeros((n + pad, k), np.complex128)
    Bbig[:n] = B
    Cbig = np.full((n + pad, k), 3.0 - 1.0j)
    Cbig[:n] = C0
    dB = _t(Bbig, cuda)[:n]
    dC = _t(Cbig, cuda)
    P.pzmdftl(n, k, 0.5, dB, beta, dC[:n])
    torch.cuda.synchronize()
    got = _np(dC)
    assert O.rel_fro(got[:n], O.dft_product(0.5, B, beta, C0)) < TOL
    assert np.all(got[n:] == 3.0 - 1.0j)


def test_dft_ones_fixture_and_variant(cuda):
    z = np.load(GOLDEN / "dft_ones_kat.npz")
    n = int(z["n"])
    for variant in ["pzmdftl", "pzmdftl1"]:
        got = _dft(n, n, 1.0, z["B"], 0.0, np.zeros((n, n), complex), cuda, variant)
        assert np.abs(got - z["X"]).max() < 1e-12


def test_dft_matches_reference_restatement(cuda):
    # the reference truncates its seed block at 1e-13; the GPU path is exact
    n = 128
    B = O.cfg_matrix(n, n, seed=3, complex_=True)
    ref = O.pzmdftl_compute(n, n, 1.0, B, 0.0, np.zeros((n, n), complex), 2, "rrqr")
    got = _dft(n, n, 1.0, B, 0.0, np.zeros((n, n), complex), cuda)
    assert O.rel_fro(got, ref) < 1e-12
    assert O.rel_fro(got, O.dft_product(1.0, B, 0.0, None)) < TOL


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
def test_host_pointer_entry_points(kind, cuda):
    import psmma_git_gb300 as P
    n, k = 130, 90
    A = O.cfg_matrix(n, k, seed=4)
    gen = np.asfortranarray(_gen(kind, k))
    Q = np.asfortranarray(O.cfg_matrix(n, k, seed=5))
    ref = O.dense_product(kind, 1.0, A, gen, 0.5, Q, k)
    getattr(P, "psmma_" + kind)(n, k, 1.0, A, gen, 0.5, Q)
    assert O.rel_fro(Q, ref) < TOL


def test_fortran_abi_matches(lib, cuda):
    import ctypes as C
    n, k = 70, 70
    A = O.cfg_matrix(n, k, seed=12)
    gen = np.asfortranarray(O.cfg_cauchy_generators(k, seed=13))
    Q = np.asfortranarray(np.zeros((n, k)))
    i = lambda v: C.byref(C.c_int(v))
    d = lambda v: C.byref(C.c_double(v))
    desc = (C.c_int * 9)(1, 0, n, k, 16, 16, 0, 0, n)
    lib.psmma_cauchy_(i(n), i(k), d(1.0), C.c_void_p(A.ctypes.data), i(1), i(1), desc,
                      C.c_void_p(gen.ctypes.data), i(k), d(0.0), C.c_void_p(Q.ctypes.data), i(1), i(1),
                      desc, None, i(0))
    assert lib.psmma_last_status() == 0
    assert O.rel_fro(Q, O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)) < TOL
    B = np.asfortranarray(O.cfg_matrix(64, 64, seed=1, complex_=True))
    Cm = np.asfortranarray(np.zeros((64, 64), complex))
    lib.pzmdftl1_(i(64), i(64), i(32), i(32), d(1.0), C.c_void_p(B.ctypes.data), i(64), d(0.0),
                  C.c_void_p(Cm.ctypes.data), i(64), i(0), i(0), None, None)
    assert lib.psmma_last_status() == 0
    assert O.rel_fro(Cm, O.dft_product(1.0, B, 0.0, None)) < TOL


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
@pytest.mark.parametrize("n,k,beta", [(300, 1500, 0.0), (257, 2048, -0.5), (2048, 2048, 1.25)])
def test_split_k_products_match_oracle(kind, n, k, beta, cuda):
    # few output tiles and a long K: the FP64 path splits K into partial sums (pool workspace)
    import torch
    import psmma_git_gb300 as P
    A = O.cfg_matrix(n, k, seed=21)
    gen = _gen(kind, k)
    Q0 = O.cfg_matrix(n, k, seed=22)
    ref = O.dense_product(kind, 0.75, A, gen, beta, Q0, k)
    dev = torch.device("cuda")
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    dg = col(gen) if kind == "cauchy" else torch.from_numpy(np.asarray(gen)).to(dev)
    dQ = P.fortran_empty(n, k, torch.float64, dev, ld=n + 3)
    dQ.copy_(torch.from_numpy(Q0))
    getattr(P, "psmma_" + kind)(n, k, 0.75, col(A), dg, beta, dQ)
    torch.cuda.synchronize()
    assert O.rel_fro(dQ.cpu().numpy(), ref) < TOL


def test_split_k_with_caller_workspace_and_short_buffer(cuda):
    import torch
    import psmma_git_gb300 as P
    from psmma_git_gb300 import _lib
    n, k = 200, 1800
    A = O.cfg_matrix(n, k, seed=31)
    gen = O.cfg_cauchy_generators(k, seed=32)
    ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    dev = torch.device("cuda")
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    need = P.workspace_size(_lib.KIND_CAUCHY, n, k)
    assert need > 0
    for size in [need, need // 2]:  # the short buffer runs without split-K
        work = torch.empty(size, dtype=torch.uint8, device=dev)
        dQ = P.fortran_empty(n, k, torch.float64, dev)
        P.psmma_cauchy(n, k, 1.0, col(A), col(gen), 0.0, dQ, work=work)
        torch.cuda.synchronize()
        assert O.rel_fro(dQ.cpu().numpy(), ref) < TOL
