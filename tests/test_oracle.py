"""CPU tests of the oracle: pinned against the golden fixtures and exact products."""
import numpy as np
import pytest

from oracle import psmma_oracle as O
from tests.conftest import GOLDEN


def test_numroc_and_const_index_agree():
    # ConstIndex must enumerate exactly NUMROC indices, the block-cyclic slice of 1..n.
    for n in [1, 7, 64, 100, 129, 768]:
        for nb in [1, 4, 16, 64]:
            for np_ in [1, 2, 3, 4]:
                allidx = []
                for p in range(np_):
                    idx = O.const_index(n, nb, p, np_)
                    assert len(idx) == O.numroc(n, nb, p, 0, np_)
                    for i in idx:  # block-cyclic owner of global index i
                        assert ((i - 1) // nb) % np_ == p
                    allidx.extend(idx.tolist())
                assert sorted(allidx) == list(range(1, n + 1))


def test_is_intersect_returns_true_when_disjoint():
    assert O.is_intersect(np.array([1, 2, 3]), np.array([4, 5])) is True
    assert O.is_intersect(np.array([1, 2, 3]), np.array([3, 5])) is False


def test_toeplitz_golden_known_answer():
    z = np.load(GOLDEN / "toeplitz_kat.npz")
    n = int(z["n"])
    H = O.dense_h("toeplitz", z["g"], n)
    assert H[0, 0] == n * n and H[3, 1] == 2 and H[1, 3] == -2
    np.testing.assert_array_equal(z["A"] @ H, z["X"])
    got = O.ps_compute("toeplitz", n, n, 1.0, z["A"], z["g"], 0.0, np.zeros((n, n)), 2, 2, 16)
    assert O.rel_fro(got, z["X"]) < 1e-15


def test_hankel_golden_exact():
    z = np.load(GOLDEN / "hankel_exact.npz")
    n = int(z["n"])
    np.testing.assert_array_equal(z["A"] @ O.dense_h("hankel", z["g"], n), z["X"])
    got = O.ps_compute("hankel", n, n, 1.0, z["A"], z["g"], 0.0, np.zeros((n, n)), 2, 2, 8)
    np.testing.assert_array_equal(got, z["X"])


def test_cauchy_golden_exact_rational():
    z = np.load(GOLDEN / "cauchy_exact.npz")
    n = int(z["n"])
    dense = O.dense_product("cauchy", 1.0, z["A"], z["gen"], 0.0, None, n)
    assert O.rel_fro(dense, z["X"]) < 1e-14
    for grid, nb in [((1, 1), 12), ((2, 2), 12), ((2, 3), 4), ((2, 2), 4)]:
        st = {}
        got = O.ps_compute("cauchy", n, n, 1.0, z["A"], z["gen"], 0.0, np.zeros((n, n)), *grid, nb=nb,
                           stats=st)
        defect = st.get("factor_overflow", 0) + st["fullrank_offdiag"]
        if defect == 0:
            assert O.rel_fro(got, z["X"]) < 1e-13
        else:  # the reference's own low-rank buffer defect: its result is wrong
            assert O.rel_fro(got, z["X"]) > 1e-6


def test_decimal_cauchy_sample_matches_exact_rational():
    # the 40-digit decimal product that checks the n = 768 reference recipe on the GPU agrees
    # with the exact rational fixture (rounded once to FP64) at n = 24
    z = np.load(GOLDEN / "cauchy_exact.npz")
    n = int(z["n"])
    got = O.decimal_cauchy_product(z["A"], z["gen"], range(n), n)
    assert O.rel_fro(got, z["X"]) < 1e-16
    assert O.col_max_rel(got, z["X"]) < 1e-16
    # and a sample of its columns is the same sample of the whole
    np.testing.assert_array_equal(O.decimal_cauchy_product(z["A"][3:9], z["gen"], [2, 7, 19], n),
                                  got[3:9][:, [2, 7, 19]])


def test_dft_ones_golden_and_restatement():
    z = np.load(GOLDEN / "dft_ones_kat.npz")
    n = int(z["n"])
    np.testing.assert_allclose(O.dft_product(1.0, z["B"], 0.0, None), z["X"], atol=1e-12)
    np.testing.assert_allclose(O.dft_matrix(n) @ z["B"], z["X"], atol=1e-11)
    for var in ["svd", "rrqr"]:
        got = O.pzmdftl_compute(n, n, 1.0, z["B"], 0.0, np.zeros((n, n), complex), 2, var)
        # the reference truncates its seed block at 1e-13: small but nonzero error
        assert np.abs(got - z["X"]).max() < 1e-10 * n


@pytest.mark.parametrize("kind", ["cauchy", "toeplitz", "hankel"])
def test_restatement_matches_dense_product(kind):
    rng = np.random.default_rng(5)
    n = 256
    A = O.cfg_matrix(n, n, seed=11)
    if kind == "cauchy":
        gen = O.cfg_cauchy_generators(n, seed=3)
    else:
        gen = O.cfg_vector(2 * n - 1, seed=4)
    Q0 = rng.uniform(-1, 1, (n, n))
    ref = O.dense_product(kind, 0.75, A, gen, -1.25, Q0, n)
    got = O.ps_compute(kind, n, n, 0.75, A, gen, -1.25, Q0, 2, 2, 64)
    assert O.rel_fro(got, ref) < 1e-13


def test_reference_cauchy_lowrank_overflow_is_reproduced():
    # With NB small the RRLU rank exceeds (NQ+NB)/2 and the reference's factors overflow
    # WORK(IPB) into WORK(IPDW), which the first DGEMM overwrites: the restatement shows it.
    rng = np.random.default_rng(0)
    n = 96
    gen = O.reference_cauchy_generators(n, rng.uniform(0, 1, n), rng.uniform(0, 1, n))
    A = O.cfg_matrix(n, n, seed=3)
    st = {}
    got = O.ps_compute("cauchy", n, n, 1.0, A, gen, 0.0, np.zeros((n, n)), 2, 2, 16, stats=st)
    assert st.get("factor_overflow", 0) > 0
    assert O.rel_fro(got, O.dense_product("cauchy", 1.0, A, gen, 0.0, None, n)) > 1e-3


def test_fft_products():
    A = O.cfg_matrix(33, 70, seed=5)
    g = O.cfg_vector(139, seed=6)
    assert O.rel_fro(O.toeplitz_product_fft(A, g, 70), O.dense_product("toeplitz", 1.0, A, g, 0, None, 70)) < 1e-14
    assert O.rel_fro(O.hankel_product_fft(A, g, 70), O.dense_product("hankel", 1.0, A, g, 0, None, 70)) < 1e-14


def test_seeded_cauchy_generators_interlace():
    for clustered in [0.0, 0.1]:
        gen = O.cfg_cauchy_generators(2000, seed=0, clustered=clustered)
        d, w = gen[:, 0], gen[:, 1]
        assert np.all(np.diff(d) > 0)
        assert np.all(d < w)
        assert np.all(w[:-1] < d[1:])
        if clustered:
            assert np.sum(np.diff(d) < 2e-10) >= 150
