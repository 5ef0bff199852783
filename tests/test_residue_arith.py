"""The split path's residue arithmetic, restated in numpy: exactness of the FP32 method.

The residue kernels (write_residue_quad / residue_f / residue_sum in
psmma_git_gb300/csrc/split_crt.cu) reduce a scaled integer x < 2^53 with sign s modulo each
modulus m <= 256 on the FP32 pipe.  The steps restated here:
- chunks of 23, 15 and 15 bits;
- t = s*x0 + g1*s*x1 + g2*s*x2 with the symmetric g1 = 2^23 mod m and g2 = 2^38 mod m;
- q = rint(t * fl(1/m)), from one FMA on the 1.5 * 2^23 magic number;
- r = t - q*m.
Each residue must be congruent to s*x and lie in [-128, 128]: that range is what the modular
GEMM's exact FP32 accumulation (1024 * 128 * 128 = 2^24) assumes.  The sum of two residues
(the 3M DFT's (Br + Bi) and (Fr + Fi) operands) is reduced the same way.
Every product here is exact in float64, as it is in the kernels' FP32 FMAs (|t| < 2^24).
"""
import numpy as np

MODULI = [256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 211, 199, 197, 193, 191]


def _sym(c, m):
    return c - m if c > m // 2 else c


def _residues(u, neg, m):
    s = np.where(neg, -1.0, 1.0)
    x0 = (u & np.uint64(0x7FFFFF)).astype(np.float64) * s
    x1 = ((u >> np.uint64(23)) & np.uint64(0x7FFF)).astype(np.float64) * s
    x2 = (u >> np.uint64(38)).astype(np.float64) * s
    g1, g2 = _sym((1 << 23) % m, m), _sym((1 << 38) % m, m)
    inv = np.float64(np.float32(1.0 / m))
    t = x2 * g2 + (x1 * g1 + x0)
    assert np.all(np.abs(t) < 2.0 ** 24)  # both FMAs exact in FP32
    q = np.rint(t * inv)  # the FMA's exact product, rounded once (ties to even)
    return t - q * m


def _values(rng, n):
    u = np.concatenate([
        rng.integers(0, 2 ** 53, n, dtype=np.uint64),
        rng.integers(0, 2 ** 24, n // 4, dtype=np.uint64),
        np.array([0, 1, 2 ** 23 - 1, 2 ** 23, 2 ** 38 - 1, 2 ** 38, 2 ** 52, 2 ** 53 - 1], dtype=np.uint64),
    ])
    return u, rng.integers(0, 2, u.size).astype(bool)


def test_fp32_residues_are_exact_and_in_range():
    rng = np.random.default_rng(2024)
    u, neg = _values(rng, 200_000)
    sign = np.where(neg, -1, 1)
    for m in MODULI:
        r = _residues(u, neg, m)
        assert np.all(r == np.rint(r))
        assert np.abs(r).max() <= 128, m
        ref = sign * (u % np.uint64(m)).astype(np.int64)
        assert np.all((r.astype(np.int64) - ref) % m == 0), m


def test_residue_sums_stay_in_range():
    # the 3M DFT's third operand: (a + b) mod m from two residues |a|, |b| <= 128
    grid = np.arange(-128, 129, dtype=np.float64)
    a, b = np.meshgrid(grid, grid)
    for m in MODULI:
        inv = np.float64(np.float32(1.0 / m))
        t = a + b
        r = t - np.rint(t * inv) * m
        assert np.abs(r).max() <= 128, m
        assert np.all(((r - t) % m) == 0), m
