"""Generates the golden fixtures in this directory (run from the repository root:
``python tests/golden/make_golden.py``).

The reference's tests store no answers and draw their random inputs unseeded, so the
fixtures are built from the reference tests' own recipes with seeded inputs and answers
that do not depend on any BLAS:

* toeplitz_kat.npz -- the deterministic generator of Test/psmma_testtoeplitz.f90:38-46
  (G(i) = N-i, G(N) = N^2) with an integer-valued A; the answer is the closed form
  N^2 A + (A r)1^T - (A 1)r^T, exact in FP64 (all values are small integers).
* dft_ones_kat.npz -- Test/pzfox_fft2.f90:99 multiplies the DFT matrix by B = 1; the
  answer is N in row 1 and 0 elsewhere.
* cauchy_exact.npz -- the generator recipe of Test/psmma_testcauchy.f90:37-53 (interlaced
  equispaced poles on [0.1, 9], U, V in U(0,1), seeded here) with A in U(0,1); the answer
  A*H is evaluated in exact rational arithmetic on the FP64 inputs, then rounded once.
* hankel_exact.npz -- a Hankel generator of small integers with an integer A; A*H is exact
  in FP64 integer arithmetic.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import psmma_oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def main() -> None:
    rng = np.random.Generator(np.random.PCG64(20220801))

    n = 64
    A = rng.integers(-4, 5, size=(n, n)).astype(np.float64)
    g = O.reference_toeplitz_generator(n)
    np.savez(OUT / "toeplitz_kat.npz", n=n, A=A, g=g, X=O.toeplitz_reference_known_answer(A))

    n = 48
    X = np.zeros((n, n), dtype=np.complex128)
    X[0, :] = n
    np.savez(OUT / "dft_ones_kat.npz", n=n, B=np.ones((n, n), dtype=np.complex128), X=X)

    n = 24
    U = rng.uniform(0.0, 1.0, n)
    V = rng.uniform(0.0, 1.0, n)
    gen = O.reference_cauchy_generators(n, U, V)
    A = rng.uniform(0.0, 1.0, (n, n))
    np.savez(OUT / "cauchy_exact.npz", n=n, A=A, gen=gen, X=O.exact_cauchy_product(A, gen, n))

    n = 40
    A = rng.integers(-3, 4, size=(n, n)).astype(np.float64)
    g = rng.integers(-5, 6, size=2 * n - 1).astype(np.float64)
    H = O.dense_h("hankel", g, n)
    Xh = np.array([[int(sum(int(A[r, i]) * int(H[i, j]) for i in range(n))) for j in range(n)]
                   for r in range(n)], dtype=np.float64)
    np.savez(OUT / "hankel_exact.npz", n=n, A=A, g=g, X=Xh)
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    main()
