"""The split DFT's radix step, restated in numpy (CPU): the index maps and butterflies that
k_dft_deinterleave_stats, the 3M core and k_crt_dft_radix (psmma_git_gb300/csrc/split_crt.cu)
implement, checked against np.fft.

With l = R m + r and j = j' + (n/R) s (r, s < R; m, j' < n/R):
    C(j' + (n/R) s, c) = sum_r w_R^(s r) w_n^(j' r) P(j', r k + c),
    P = F_(n/R) B',  B'(m, r k + c) = B(R m + r, c),
where w_n = exp(-2 pi i / n) and F_n(j, l) = w_n^(j l), so that np.fft.fft(B, axis=0) = F_n B.
The R-point butterflies: R = 2 and 4 by additions (w_4 = -i), R = 8 as two 4-point transforms
of a_r = X_r + X_(r+4) (the even outputs) and b_r = w_8^r (X_r - X_(r+4)) (the odd ones).
"""
import numpy as np
import pytest


def _dft4(x0, x1, x2, x3):
    """dft4 in split_crt.cu: t0 = x0 + x2, t1 = x0 - x2, t2 = x1 + x3, t3 = x1 - x3;
    y0 = t0 + t2, y2 = t0 - t2, y1 = t1 - i t3, y3 = t1 + i t3."""
    t0, t1, t2, t3 = x0 + x2, x0 - x2, x1 + x3, x1 - x3
    return t0 + t2, t1 - 1j * t3, t0 - t2, t1 + 1j * t3


def _butterfly(X):
    """radix_butterfly: Y = DFT_R X for R = 2, 4, 8 (X a list of R arrays)."""
    R = len(X)
    if R == 2:
        return [X[0] + X[1], X[0] - X[1]]
    if R == 4:
        return list(_dft4(*X))
    h = 1.0 / np.sqrt(2.0)
    a = [X[r] + X[r + 4] for r in range(4)]
    b = [X[r] - X[r + 4] for r in range(4)]
    b[1] = h * (b[1].real + b[1].imag) + 1j * h * (b[1].imag - b[1].real)   # (1 - i)/sqrt(2)
    b[2] = b[2].imag - 1j * b[2].real                                      # -i
    b[3] = h * (b[3].imag - b[3].real) - 1j * h * (b[3].real + b[3].imag)  # (-1 - i)/sqrt(2)
    ye, yo = _dft4(*a), _dft4(*b)
    Y = [None] * 8
    for t in range(4):
        Y[2 * t], Y[2 * t + 1] = ye[t], yo[t]
    return Y


@pytest.mark.parametrize("R", [2, 4, 8])
def test_butterflies_are_the_R_point_dft(R):
    rng = np.random.default_rng(R)
    X = rng.standard_normal((R, 64)) + 1j * rng.standard_normal((R, 64))
    Y = np.array(_butterfly([X[r] for r in range(R)]))
    np.testing.assert_allclose(Y, np.fft.fft(X, axis=0), rtol=0, atol=1e-13)


@pytest.mark.parametrize("n,k,R", [(64, 5, 2), (96, 3, 4), (256, 7, 8), (4100, 2, 4)])
def test_radix_step_index_maps(n, k, R):
    rng = np.random.default_rng(n + R)
    B = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
    nq = n // R
    # B' (nq x R k): column r k + c holds B(r::R, c)
    Bp = np.empty((nq, R * k), complex)
    for r in range(R):
        for c in range(k):
            Bp[:, r * k + c] = B[r::R, c]
    P = np.fft.fft(Bp, axis=0)  # F_(n/R) B'
    # the exact twiddle table w_n^t, t < n (j' r < n: no reduction)
    wn = np.exp(-2j * np.pi * np.arange(n) / n)
    jq = np.arange(nq)
    C = np.empty((n, k), complex)
    for c in range(k):
        X = [P[:, r * k + c] * (wn[jq * r] if r else 1.0) for r in range(R)]
        Y = _butterfly(X)
        for s in range(R):
            C[jq + nq * s, c] = Y[s]
    ref = np.fft.fft(B, axis=0)
    assert np.abs(C - ref).max() <= 1e-11 * np.abs(ref).max()
    assert int(np.max(jq) * (R - 1)) < n  # every twiddle index is inside the table


def test_deinterleave_thread_classes():
    # k_dft_deinterleave_stats: with 256 threads striding by 256 over a column, thread t meets
    # only entries l = t mod R, so its row statistics belong to row r k + c with r = t mod R
    for R in (2, 4, 8):
        assert 256 % R == 0
        for t in range(256):
            assert {l % R for l in range(t, 4096, 256)} == {t % R}
