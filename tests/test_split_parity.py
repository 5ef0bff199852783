"""GPU parity of the split path (modular BF16 tensor-core slices, FP64 recombination).

Stated bound: relative Frobenius error <= 1e-12 against the FP64 oracle; integer fixtures
whose products are exactly representable must match bit for bit."""
import numpy as np
import pytest

from oracle import psmma_oracle as O
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _t(x, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(cuda).t()


def _np(t):
    return t.t().contiguous().cpu().numpy().T


def _split(kind, n, k, alpha, A, gen, beta, Q0, cuda, n_moduli=0, ld_pad=0, **kw):
    import psmma_git_gb300 as P
    import torch
    dA = P.fortran_empty(n, k, torch.float64, cuda, ld=n + ld_pad)
    dA.copy_(_t(A, cuda))
    dQ = P.fortran_empty(n, k, torch.float64, cuda, ld=n + ld_pad)
    dQ.copy_(_t(Q0, cuda))
    dg = _t(gen, cuda) if kind == "cauchy" else torch.from_numpy(np.asarray(gen)).to(cuda)
    getattr(P, "psmma_" + kind)(n, k, alpha, dA, dg, beta, dQ, precision="split", n_moduli=n_moduli, **kw)
    torch.cuda.synchronize()
    return _np(dQ)


def _gen(kind, k, seed=3, clustered=0.0):
    if kind == "cauchy":
        return O.cfg_cauchy_generators(k, seed=seed, clustered=clustered)
    return O.cfg_vector(2 * k - 1, seed=seed)


def test_split_smoke_small(cuda):
    n = k = 256
    A = O.cfg_matrix(n, k, seed=1)
    gen = _gen("cauchy", k)
    got = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda)
    ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    assert O.rel_fro(got, ref) < TOL


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
@pytest.mark.parametrize("n,k", [(1, 1), (5, 7), (256, 256), (300, 200), (129, 513), (1024, 1024)])
def test_split_matches_dense_oracle(kind, n, k, cuda):
    A = O.cfg_matrix(n, k, seed=n * 7 + k)
    gen = _gen(kind, k)
    Q0 = O.cfg_matrix(n, k, seed=2)
    got = _split(kind, n, k, 0.75, A, gen, -1.5, Q0, cuda)
    ref = O.dense_product(kind, 0.75, A, gen, -1.5, Q0, k)
    assert O.rel_fro(got, ref) < TOL


def test_split_clustered_cauchy(cuda):
    # the split workload's distribution: 10% of the poles within 1e-10 of a neighbour, A ~ N(0,1)
    n = k = 2048
    A = O.cfg_matrix(n, k, seed=5, dist="normal")
    gen = O.cfg_cauchy_generators(k, seed=6, clustered=0.1)
    got = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda)
    ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    assert O.rel_fro(got, ref) < TOL


def test_split_toeplitz_fixture_bit_exact(cuda):
    z = np.load(GOLDEN / "toeplitz_kat.npz")
    n = int(z["n"])
    got = _split("toeplitz", n, n, 1.0, z["A"], z["g"], 0.0, np.zeros((n, n)), cuda)
    np.testing.assert_array_equal(got, z["X"])


def test_split_hankel_fixture_bit_exact(cuda):
    z = np.load(GOLDEN / "hankel_exact.npz")
    n = int(z["n"])
    got = _split("hankel", n, n, 1.0, z["A"], z["g"], 0.0, np.zeros((n, n)), cuda)
    np.testing.assert_array_equal(got, z["X"])


def test_split_cauchy_reference_recipe(cuda):
    z = np.load(GOLDEN / "cauchy_exact.npz")
    n = int(z["n"])
    got = _split("cauchy", n, n, 1.0, z["A"], z["gen"], 0.0, np.zeros((n, n)), cuda)
    assert O.rel_fro(got, z["X"]) < TOL


def test_split_beta_zero_ignores_q_and_ld(cuda):
    n, k = 333, 270
    A = O.cfg_matrix(n, k, seed=8)
    gen = _gen("hankel", k)
    got = _split("hankel", n, k, 2.0, A, gen, 0.0, np.full((n, k), np.nan), cuda, ld_pad=19)
    assert np.isfinite(got).all()
    assert O.rel_fro(got, O.dense_product("hankel", 2.0, A, gen, 0.0, None, k)) < TOL


def test_split_nonfinite_row_gives_nan_row(cuda):
    n = k = 64
    A = O.cfg_matrix(n, k, seed=9)
    A[5, 7] = np.inf
    gen = _gen("toeplitz", k)
    got = _split("toeplitz", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda)
    assert np.isnan(got[5]).all()
    mask = np.ones(n, bool)
    mask[5] = False
    ref = O.dense_product("toeplitz", 1.0, A[mask], gen, 0.0, None, k)
    assert O.rel_fro(got[mask], ref) < TOL


def test_split_zero_rows_and_columns(cuda):
    n = k = 96
    A = O.cfg_matrix(n, k, seed=10)
    A[3] = 0.0
    g = _gen("hankel", k)
    got = _split("hankel", n, k, 1.0, A, g, 0.0, np.zeros((n, k)), cuda)
    assert (got[3] == 0.0).all()
    assert O.rel_fro(got, O.dense_product("hankel", 1.0, A, g, 0.0, None, k)) < TOL


@pytest.mark.parametrize("nmod", [10, 12, 16])
def test_split_moduli_count_accuracy(nmod, cuda):
    # fewer moduli -> fewer bits; the error must follow 2^-P and stay bounded
    n = k = 512
    A = O.cfg_matrix(n, k, seed=11)
    gen = _gen("cauchy", k)
    got = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, n_moduli=nmod)
    err = O.rel_fro(got, O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k))
    bound = {10: 1e-6, 12: 1e-9, 16: 1e-14}[nmod]
    assert err < bound


def test_split_is_deterministic_and_matches_fp64_path(cuda):
    import psmma_git_gb300 as P
    import torch
    n = k = 4096
    A = O.cfg_matrix(n, k, seed=12)
    gen = _gen("cauchy", k, seed=13)
    dA = _t(A, cuda)
    dg = _t(gen, cuda)
    outs = []
    for prec in ["split", "split", "fp64"]:
        dQ = P.fortran_empty(n, k, torch.float64, cuda)
        P.psmma_cauchy(n, k, 1.0, dA, dg, 0.0, dQ, precision=prec)
        torch.cuda.synchronize()
        outs.append(dQ)
    assert torch.equal(outs[0], outs[1])
    err = (torch.linalg.norm(outs[0] - outs[2]) / torch.linalg.norm(outs[2])).item()
    assert err < TOL


def test_split_no_cancellation_hits_the_range_bound_exactly(cuda):
    # all-positive operands: |A'H'| reaches the bound the moduli must cover; the exact
    # answer (k in every entry) must come back bit for bit
    n, k = 200, 1500
    A = np.ones((n, k))
    g = np.ones(2 * k - 1)
    for kind in ["toeplitz", "hankel"]:
        got = _split(kind, n, k, 1.0, A, g, 0.0, np.zeros((n, k)), cuda)
        np.testing.assert_array_equal(got, np.full((n, k), float(k)))


def test_split_wide_exponent_range_rows(cuda):
    # rows scaled by 2^+-400: per-row exponents keep every row at full relative accuracy
    n = k = 256
    A = O.cfg_matrix(n, k, seed=14)
    scale = np.where(np.arange(n) % 2 == 0, 2.0 ** 400, 2.0 ** -400)
    gen = _gen("toeplitz", k, seed=15)
    got = _split("toeplitz", n, k, 1.0, A * scale[:, None], gen, 0.0, np.zeros((n, k)), cuda)
    ref = O.dense_product("toeplitz", 1.0, A, gen, 0.0, None, k) * scale[:, None]
    for i in [0, 1, 100, 255]:
        assert np.linalg.norm(got[i] - ref[i]) / np.linalg.norm(ref[i]) < TOL


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
@pytest.mark.parametrize("n,k,levels,pad", [(1000, 2048, 1, 3), (2048, 4096, 2, 0), (333, 6144, 2, 5),
                                            (70, 3072, 1, 1), (130, 1536, 3, 2), (257, 8192, 0, 4),
                                            (300, 2000, 1, 2), (129, 3000, 2, 0), (200, 1000, 3, 1),
                                            (65, 8100, 0, 3)])
def test_split_block_step_matches_dense_oracle(kind, n, k, levels, pad, cuda):
    # the block step (3^L products of width k / 2^L on sums and differences of blocks), asked
    # for by opts->block_levels (0: the automatic choice, one level at k = 8192 and at 8100,
    # padded to 8192): ragged row counts, padded leading dimensions, alpha and beta, leaves
    # narrower than a GEMM tile (k = 1536 or 1000 at L = 3: 192 or 128 columns), orders that
    # 64 * 2^L does not divide (2000, 3000, 1000, 8100: the generator zero-extended, A with zero
    # columns), against the dense oracle on the whole product and column by column
    import psmma_git_gb300 as P
    if levels == 0:
        assert P.load().psmma_split_block_levels({"toeplitz": 1, "hankel": 2}[kind], n, k) == 1
    A = O.cfg_matrix(n, k, seed=n + k)
    gen = _gen(kind, k, seed=k + 1)
    Q0 = O.cfg_matrix(n, k, seed=n + 2)
    got = _split(kind, n, k, 0.75, A, gen, -1.5, Q0, cuda, ld_pad=pad, block_levels=levels)
    ref = O.dense_product(kind, 0.75, A, gen, -1.5, Q0, k)
    assert O.rel_fro(got, ref) < TOL
    assert O.col_max_rel(got, ref) < 10 * TOL


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
@pytest.mark.parametrize("n,k,levels,beta", [(1000, 8192, 0, 0.0), (700, 2000, 1, 0.0), (1300, 3000, 2, -1.5),
                                             (300, 4096, 2, 0.5)])
def test_split_block_step_host_pointer_path(kind, n, k, levels, beta, cuda):
    # host arrays through the overlapped host pipeline (row panels; the second call of a shape
    # scales with the bit counts cached from the first, the speculative panels): the same
    # result bit for bit as the device-pointer call, which the dense oracle checks
    import psmma_git_gb300 as P
    A = O.cfg_matrix(n, k, seed=n + 3 * k)
    gen = _gen(kind, k, seed=k + 13)
    Q0 = O.cfg_matrix(n, k, seed=n + 17)
    fn = getattr(P, "psmma_" + kind)
    outs = []
    for _ in range(2):
        Qh = np.asfortranarray(Q0.copy())
        fn(n, k, 0.75, np.asfortranarray(A), gen, beta, Qh, precision="split", block_levels=levels)
        outs.append(Qh)
    dev = _split(kind, n, k, 0.75, A, gen, beta, Q0, cuda, block_levels=levels)
    np.testing.assert_array_equal(outs[0], dev)
    np.testing.assert_array_equal(outs[1], dev)
    if k <= 4096:
        assert O.rel_fro(dev, O.dense_product(kind, 0.75, A, gen, beta, Q0, k)) < TOL


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
@pytest.mark.parametrize("n,k,levels", [(1, 128, 1), (3, 256, 2), (2, 512, 3), (5, 130, 1), (1, 200, 2)])
def test_split_block_step_tiny_shapes(kind, n, k, levels, cuda):
    # one to five rows, leaves of 64 columns (narrower than a GEMM tile), orders padded from
    # 130 and 200: against the dense oracle
    A = O.cfg_matrix(n, k, seed=n * 31 + k)
    gen = _gen(kind, k, seed=k + 9)
    Q0 = O.cfg_matrix(n, k, seed=n + 77)
    got = _split(kind, n, k, -0.5, A, gen, 2.0, Q0, cuda, block_levels=levels)
    ref = O.dense_product(kind, -0.5, A, gen, 2.0, Q0, k)
    assert O.rel_fro(got, ref) < TOL


@pytest.mark.parametrize("n,levels", [(2048, 2), (4096, 3), (8192, 0), (2000, 1), (3000, 2)])
def test_split_block_step_toeplitz_known_answer_bit_exact(n, levels, cuda):
    # the reference test's generator (G(i) = N - i, G(N) = N^2) with integer A: the block
    # step's sums and differences are exact, so the closed form comes back bit for bit
    g = O.reference_toeplitz_generator(n)
    rng = np.random.Generator(np.random.PCG64(n))
    A = rng.integers(-4, 5, size=(300, n)).astype(np.float64)
    got = _split("toeplitz", 300, n, 1.0, A, g, 0.0, np.zeros((300, n)), cuda, block_levels=levels)
    np.testing.assert_array_equal(got, O.toeplitz_reference_known_answer(A))


@pytest.mark.parametrize("k,levels", [(2048, 1), (4096, 2), (4096, 3)])
def test_split_block_step_range_bound_exact(k, levels, cuda):
    # all-positive operands at the moduli's range bound, through the block step
    n = 130
    A = np.ones((n, k))
    g = np.ones(2 * k - 1)
    for kind in ["toeplitz", "hankel"]:
        got = _split(kind, n, k, 1.0, A, g, 0.0, np.zeros((n, k)), cuda, block_levels=levels)
        np.testing.assert_array_equal(got, np.full((n, k), float(k)))


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
def test_split_block_step_same_result_as_single_product(kind, cuda):
    # generators whose column groups share their exponent: the block step computes the same
    # integer product as the single one, so the results are identical bit for bit
    n, k = 300, 4096
    A = O.cfg_matrix(n, k, seed=41)
    gen = _gen(kind, k, seed=42)
    one = _split(kind, n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, block_levels=-1)
    for levels in (1, 2, 3):
        got = _split(kind, n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, block_levels=levels)
        np.testing.assert_array_equal(got, one)


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
@pytest.mark.parametrize("k", [4096, 4000])
def test_split_block_step_nonfinite_generator_takes_single_product(kind, k, cuda):
    # a NaN and an Inf in the generator: the call falls back (on the device) to the single
    # product, which returns NaN in exactly the columns that hold them and the oracle's
    # values elsewhere (k = 4000: the padded order 4096)
    n = 200
    A = O.cfg_matrix(n, k, seed=31)
    gen = _gen(kind, k, seed=32)
    gen[k // 3] = np.nan
    gen[2 * k - 900] = np.inf
    got = _split(kind, n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, block_levels=2)
    H = O.const_toeplitz(gen, k, np.arange(1, k + 1), np.arange(1, k + 1)) if kind == "toeplitz" else \
        O.const_hankel(gen, k, np.arange(1, k + 1), np.arange(1, k + 1))
    bad = ~np.isfinite(H).all(axis=0)
    assert bad.any() and not bad.all()
    assert np.isnan(got[:, bad]).all()
    gen_f = np.where(np.isfinite(gen), gen, 0.0)
    ref = O.dense_product(kind, 1.0, A, gen_f, 0.0, None, k)
    assert O.rel_fro(got[:, ~bad], ref[:, ~bad]) < TOL


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
def test_split_block_step_graded_generator_keeps_column_accuracy(kind, cuda):
    # g(x) = 2^(-x/64): columns j and j + w differ by w/64 binades, more than the block step
    # lets a group share; the call takes the single product and every column keeps its own
    # relative accuracy
    n, k = 128, 4096
    A = O.cfg_matrix(n, k, seed=33)
    gen = 2.0 ** (-np.arange(2 * k - 1) / 64.0)
    got = _split(kind, n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, block_levels=2)
    ref = O.dense_product(kind, 1.0, A, gen, 0.0, None, k)
    assert O.col_max_rel(got, ref) < TOL


@pytest.mark.parametrize("n,k,levels,pad", [(1000, 2048, 1, 3), (4096, 4096, 1, 0), (258, 1536, 1, 7),
                                            (8192, 8192, 1, 0)])
def test_split_strassen_step_same_result_as_single_product(n, k, levels, pad, cuda):
    # Strassen's step on the residue planes (opts->block_levels = 1) computes the same integer
    # product, so the result is the single product's bit for bit: half-row counts that are not
    # whole tiles (500, 129), padded leading dimensions, alpha and beta
    A = O.cfg_matrix(n, k, seed=n + 5)
    gen = _gen("cauchy", k, seed=k + 6, clustered=0.05)
    Q0 = O.cfg_matrix(n, k, seed=n + 7)
    one = _split("cauchy", n, k, 0.75, A, gen, -1.5, Q0, cuda, ld_pad=pad, block_levels=-1)
    got = _split("cauchy", n, k, 0.75, A, gen, -1.5, Q0, cuda, ld_pad=pad, block_levels=levels)
    np.testing.assert_array_equal(got, one)
    if n <= 1000:
        assert O.rel_fro(got, O.dense_product("cauchy", 0.75, A, gen, -1.5, Q0, k)) < TOL


def test_split_strassen_step_nonfinite_row_and_eig_kind(cuda):
    # a non-finite row of A stays a NaN row (the others match the single product), and the
    # accurate-denominator kind takes the same step
    import psmma_git_gb300 as P
    import torch
    n, k = 2048, 2048
    A = O.cfg_matrix(n, k, seed=51)
    A[1500, 3] = np.inf
    gen = _gen("cauchy", k, seed=52)
    one = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, block_levels=-1)
    got = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda, block_levels=1)
    assert np.isnan(got[1500]).all()
    np.testing.assert_array_equal(np.delete(got, 1500, axis=0), np.delete(one, 1500, axis=0))
    eig = [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in O.eig_generators(k, seed=53, tiny=k // 100)]
    dA = _t(O.cfg_matrix(n, k, seed=54), cuda)
    outs = []
    for lv in (-1, 1):
        dQ = P.fortran_empty(n, k, torch.float64, cuda)
        P.psmma_cauchyeig(n, k, 1.0, dA, *eig, 0.0, dQ, precision="split", block_levels=lv)
        torch.cuda.synchronize()
        outs.append(dQ)
    assert torch.equal(outs[0], outs[1])


def _split_dft(n, k, alpha, B, beta, C0, cuda, n_moduli=0, variant="pzmdftl"):
    import psmma_git_gb300 as P
    import torch
    dB = _t(B.astype(np.complex128), cuda)
    dC = _t(C0.astype(np.complex128), cuda)
    getattr(P, variant)(n, k, alpha, dB, beta, dC, precision="split", n_moduli=n_moduli)
    torch.cuda.synchronize()
    return _np(dC)


@pytest.mark.parametrize("n,k", [(1, 1), (3, 5), (96, 40), (250, 300), (1024, 512), (2048, 2048), (1500, 37),
                                 (2046, 20)])
def test_split_dft_matches_fft(n, k, cuda):
    # (1500, 37) and (2046, 20): no radix step and an inner length of two 1024-deep chunks
    B = O.cfg_matrix(n, k, seed=n + 3, complex_=True)
    C0 = O.cfg_matrix(n, k, seed=k + 4, complex_=True)
    got = _split_dft(n, k, 0.5, B, -2.0, C0, cuda)
    ref = O.dft_product(0.5, B, -2.0, C0)
    assert O.rel_fro(got, ref) < TOL


@pytest.mark.parametrize("n,k,pad", [(300, 7, 5), (513, 130, 3)])
def test_split_dft_padded_leading_dimensions(n, k, pad, cuda):
    # B and C as column blocks of larger complex arrays (ldb = ldc = n + pad); n is not a
    # multiple of 256, so the imaginary half of the residue planes starts after padding
    import psmma_git_gb300 as P
    import torch
    B = O.cfg_matrix(n, k, seed=n + 11, complex_=True)
    C0 = O.cfg_matrix(n, k, seed=k + 12, complex_=True)
    Bbig = np.zeros((n + pad, k), np.complex128)
    Bbig[:n] = B
    Cbig = np.full((n + pad, k), 7.0 + 7.0j)
    Cbig[:n] = C0
    dB = _t(Bbig, cuda)[:n]
    dC = _t(Cbig, cuda)
    P.pzmdftl(n, k, 0.5, dB, -2.0, dC[:n], precision="split")
    torch.cuda.synchronize()
    got = _np(dC)
    assert O.rel_fro(got[:n], O.dft_product(0.5, B, -2.0, C0)) < TOL
    assert np.all(got[n:] == 7.0 + 7.0j)  # rows past n untouched


@pytest.mark.parametrize("n,k,pad,beta", [(2050, 33, 2, 1.0), (4100, 77, 3, -0.5), (8192, 300, 5, 0.0),
                                         (8192, 129, 0, 1.5), (12288, 64, 1, 0.25)])
def test_split_dft_radix_steps_match_fft(n, k, pad, beta, cuda):
    # radix 2 (n = 2050: n / 2 = 1025), 4 (n = 4100: n / 4 = 1025, odd) and 8 (n = 8192, 12288):
    # the modular products run on F_(n/R) and R k columns, the twiddles and butterflies
    # afterwards; padded leading dimensions, beta on and off, rows past n untouched
    import psmma_git_gb300 as P
    import torch
    radix = {2050: 2, 4100: 4, 8192: 8, 12288: 8}[n]
    assert [P.load().psmma_split_dft_radix(m) for m in (n, 2046, 4094, 4096, 8190, 0)] == [radix, 1, 2, 4, 2, 0]
    B = O.cfg_matrix(n, k, seed=n + 21, complex_=True)
    C0 = O.cfg_matrix(n, k, seed=k + 22, complex_=True)
    Bbig = np.zeros((n + pad, k), np.complex128)
    Bbig[:n] = B
    Cbig = np.full((n + pad, k), 7.0 + 7.0j)
    Cbig[:n] = C0
    dB = _t(Bbig, cuda)[:n]
    dC = _t(Cbig, cuda)
    P.pzmdftl(n, k, 0.75, dB, beta, dC[:n], precision="split")
    torch.cuda.synchronize()
    got = _np(dC)
    ref = O.dft_product(0.75, B, beta, C0)
    assert O.rel_fro(got[:n], ref) < TOL
    assert O.col_max_rel(got[:n], ref) < TOL
    assert np.all(got[n:] == 7.0 + 7.0j)


def test_split_dft_radix_rows_past_the_grid_y_limit(cuda):
    # n = k = 8192 at radix 8: the modular products have R k = 65536 rows, one more than a grid's
    # y dimension holds, so the row-indexed passes must index rows along x
    import psmma_git_gb300 as P
    import torch
    n = k = 8192
    g = torch.Generator(device=cuda)
    g.manual_seed(8192)
    X = P.fortran_empty(n, k, torch.complex128, cuda)
    X.copy_(torch.complex(torch.rand(k, n, generator=g, device=cuda, dtype=torch.float64) * 2 - 1,
                          torch.rand(k, n, generator=g, device=cuda, dtype=torch.float64) * 2 - 1).t())
    Y = P.fortran_empty(n, k, torch.complex128, cuda)
    P.pzmdftl(n, k, 1.0, X, 0.0, Y, precision="split")
    torch.cuda.synchronize()
    cols = torch.tensor([0, 1, 4095, 8191], device=cuda)
    ref = np.fft.fft(X[:, cols].cpu().numpy(), axis=0)
    assert O.rel_fro(Y[:, cols].cpu().numpy(), ref) < TOL
    del X, Y
    torch.cuda.empty_cache()


@pytest.mark.parametrize("n,k", [(2050, 24), (4100, 33), (8192, 40)])
@pytest.mark.parametrize("nmod", [10, 16])
def test_split_dft_radix_moduli_count(n, k, nmod, cuda):
    # radix 2 / 4 (three products, inner length 1025) and 8 (the three products in one launch,
    # inner length 1024), each through the CRT that applies the twiddles and butterflies, with
    # the top CRT limb in 32 bits (10 moduli) and in 64 (16)
    B = O.cfg_matrix(n, k, seed=n + 31, complex_=True)
    C0 = O.cfg_matrix(n, k, seed=k + 32, complex_=True)
    got = _split_dft(n, k, 0.5, B, 1.25, C0, cuda, n_moduli=nmod)
    err = O.rel_fro(got, O.dft_product(0.5, B, 1.25, C0))
    assert err < {10: 1e-6, 16: 1e-14}[nmod]


@pytest.mark.parametrize("n,k", [(1000, 9), (4100, 9), (8192, 6)])
def test_split_dft_nonfinite_column_gives_nan_column(n, k, cuda):
    # an Inf in column 3 of B: that column of C is NaN (its product row, or with the radix
    # step one of the R rows that each output of the column combines), the others are exact
    B = O.cfg_matrix(n, k, seed=n + 51, complex_=True)
    B[17, 3] = np.inf
    C0 = O.cfg_matrix(n, k, seed=k + 52, complex_=True)
    got = _split_dft(n, k, 0.5, B, 1.5, C0, cuda)
    assert np.isnan(got[:, 3]).all()
    keep = [c for c in range(k) if c != 3]
    ref = O.dft_product(0.5, B[:, keep], 1.5, C0[:, keep])
    assert O.rel_fro(got[:, keep], ref) < TOL


@pytest.mark.parametrize("n,k", [(1000, 17), (4100, 9), (8192, 12)])
def test_split_dft_power_of_two_scaling_is_exact(n, k, cuda):
    # B scaled by 2^200 shifts the row exponents only: the residues, the CRT's integers, the
    # twiddle products and the butterflies are those of the unscaled call times 2^200, bit for bit
    B = O.cfg_matrix(n, k, seed=n + 41, complex_=True)
    zero = np.zeros((n, k), complex)
    base = _split_dft(n, k, 0.75, B, 0.0, zero, cuda)
    got = _split_dft(n, k, 0.75, B * 2.0 ** 200, 0.0, zero, cuda)
    np.testing.assert_array_equal(got, base * 2.0 ** 200)
    assert O.rel_fro(base, O.dft_product(0.75, B, 0.0, zero)) < TOL


def test_split_dft_ones_fixture(cuda):
    z = np.load(GOLDEN / "dft_ones_kat.npz")
    n = int(z["n"])
    for variant in ["pzmdftl", "pzmdftl1"]:
        got = _split_dft(n, n, 1.0, z["B"], 0.0, np.zeros((n, n), complex), cuda, variant=variant)
        assert np.abs(got - z["X"]).max() < 1e-10


def test_split_power_of_two_scaling_is_exact(cuda):
    # scaling A by 2^300 and U by 2^-200 scales every step exactly (row / column exponents,
    # the FP32 bound sums on their per-thread scales, the division, the CRT's exponent), so the
    # result is the unscaled one times 2^100, bit for bit
    n, k = 700, 900
    A = O.cfg_matrix(n, k, seed=41, dist="normal")
    gen = _gen("cauchy", k, seed=42, clustered=0.1)
    base = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda)
    g2 = gen.copy()
    g2[:, 2] *= 2.0 ** -200  # U
    got = _split("cauchy", n, k, 1.0, A * 2.0 ** 300, g2, 0.0, np.zeros((n, k)), cuda)
    np.testing.assert_array_equal(got, base * 2.0 ** 100)
    assert O.rel_fro(base, O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)) < TOL


def test_split_pole_gap_outside_the_fast_division_range(cuda):
    # D(11) = 1e-32, F(11) = 2.5e-32: |D(11) - F(11)| < 2^-100 takes the full division, and the
    # 1e32-sized entry is 2^100 times its column's others (the FP32 bound sums of that
    # thread fall back to FP64)
    n, k = 256, 512
    A = O.cfg_matrix(n, k, seed=43)
    gen = _gen("cauchy", k, seed=44)
    gen[10, 0], gen[10, 1] = 1e-32, 2.5e-32
    got = _split("cauchy", n, k, 1.0, A, gen, 0.0, np.zeros((n, k)), cuda)
    ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    assert np.isfinite(got).all()
    assert O.rel_fro(got, ref) < TOL
    others = np.arange(k) != 10  # the other columns keep their own accuracy
    assert O.rel_fro(got[:, others], ref[:, others]) < TOL
