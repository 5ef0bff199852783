"""The split path's Toeplitz / Hankel block step, restated in numpy (CPU) on integers.

With A = [X1 | X2] and H = [[Y00, Y01], [Y10, Y11]] (blocks of width w = K/2):
- Toeplitz (Y11 = Y00): P = (X1 + X2) Y00, Q1 = P + X2 (Y10 - Y00), Q2 = P + X1 (Y01 - Y00);
- Hankel (Y10 = Y01):   P = (X1 + X2) Y01, Q1 = P + X1 (Y00 - Y01), Q2 = P + X2 (Y11 - Y01);
and every right operand is Toeplitz (Hankel) again, so the step recurses: L levels give 3^L
products of width K/2^L.  The kernels (k_residues_A_blocks, k_residues_H_leaf, the leaf GEMMs'
multi-place epilogue in psmma_git_gb300/csrc/split_crt.cu) run these sums and differences on
residues, where they are exact; here they run on int64, where they are exact too, and the
result must be A H bit for bit.  Orders that 64 * 2^L does not divide are padded: the generator
zero-extended around its centre, A with zero columns.
"""
import numpy as np
import pytest

from oracle import psmma_oracle as O


def _is_toeplitz(T):
    return all(np.array_equal(np.diagonal(T, d)[1:], np.diagonal(T, d)[:-1]) for d in range(-T.shape[0] + 1, T.shape[1]))


def _is_hankel(T):
    return _is_toeplitz(T[::-1])


def _block_product(kind, X, H, levels):
    """X H by `levels` block steps (explicit integer matrices; asserts the structure kept)."""
    assert (_is_toeplitz if kind == "toeplitz" else _is_hankel)(H)
    if levels == 0:
        return X @ H
    w = H.shape[0] // 2
    X1, X2 = X[:, :w], X[:, w:]
    Y00, Y01, Y10, Y11 = H[:w, :w], H[:w, w:], H[w:, :w], H[w:, w:]
    if kind == "toeplitz":
        assert np.array_equal(Y11, Y00)
        P = _block_product(kind, X1 + X2, Y00, levels - 1)
        Q1 = P + _block_product(kind, X2, Y10 - Y00, levels - 1)
        Q2 = P + _block_product(kind, X1, Y01 - Y00, levels - 1)
    else:
        assert np.array_equal(Y10, Y01)
        P = _block_product(kind, X1 + X2, Y01, levels - 1)
        Q1 = P + _block_product(kind, X1, Y00 - Y01, levels - 1)
        Q2 = P + _block_product(kind, X2, Y11 - Y01, levels - 1)
    return np.hstack([Q1, Q2])


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
@pytest.mark.parametrize("levels", [1, 2, 3])
def test_block_step_is_exact_on_integers(kind, levels):
    rng = np.random.default_rng(levels + (7 if kind == "hankel" else 0))
    n, K = 11, 96
    A = rng.integers(-50, 51, (n, K)).astype(np.int64)
    g = rng.integers(-50, 51, 2 * K - 1).astype(np.int64)
    H = O.dense_h(kind, g.astype(float), K).astype(np.int64)
    assert np.array_equal(_block_product(kind, A, H, levels), A @ H)


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
def test_block_step_on_residues(kind):
    # the same steps modulo one of the split path's moduli: the residue of A H
    m = 251
    rng = np.random.default_rng(11)
    n, K = 9, 64
    A = rng.integers(-10 ** 6, 10 ** 6, (n, K)).astype(np.int64)
    g = rng.integers(-10 ** 6, 10 ** 6, 2 * K - 1).astype(np.int64)
    H = O.dense_h(kind, g.astype(float), K).astype(np.int64)
    got = _block_product(kind, A % m, H % m, 2) % m
    assert np.array_equal(got, (A @ H) % m)


@pytest.mark.parametrize("kind", ["toeplitz", "hankel"])
def test_padding_keeps_the_leading_block(kind):
    # order N padded to Np: the generator zero-extended around its centre (entries N - 1 .. 2N - 2
    # of the padded one's index range keep their offsets from the centre), A with zero columns;
    # the first N columns of the padded product are the product
    rng = np.random.default_rng(5)
    n, N, Np = 7, 50, 64
    A = rng.integers(-9, 10, (n, N)).astype(np.int64)
    g = rng.integers(-9, 10, 2 * N - 1).astype(np.int64)
    H = O.dense_h(kind, g.astype(float), N).astype(np.int64)
    if kind == "toeplitz":
        gp = np.zeros(2 * Np - 1, np.int64)
        gp[Np - N:Np + N - 1] = g  # T(i, j) = G(K + j - i): the centre G(K) stays the centre
    else:
        gp = np.zeros(2 * Np - 1, np.int64)
        gp[:2 * N - 1] = g  # H(i, j) = G(i + j): the leading entries stay in place
    Hp = O.dense_h(kind, gp.astype(float), Np).astype(np.int64)
    assert np.array_equal(Hp[:N, :N], H)
    Ap = np.zeros((n, Np), np.int64)
    Ap[:, :N] = A
    assert np.array_equal(_block_product(kind, Ap, Hp, 2)[:, :N], A @ H)
