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


# ---- the one-launch 3M products' drain (mod_sym_f_bits, mod_sym_f_bits_add, offset_byte_f,
# pack_low_bytes in split_crt.cu): residues of the exact FP32 chunk sums on the FP32 pipe ----
ROUND = np.float32(1.5 * 2 ** 23)


def _drain_residue(v, m, a=None):
    """The drain's steps on float32 chunk sums v (integers, |v| <= 2^24) and an optional
    integer addend a (|a| <= 256): q from the rounded sum and the rounded product plus and
    minus 1.5 * 2^23, the remainder exact (the kernel's FMA; exact in float64 here), one
    correction on each side.  Returns the float32 residue and the bits of x + 1.5 * 2^23."""
    inv = np.float32(1.0 / m)
    mf = np.float32(m)
    t = v if a is None else (v + a).astype(np.float32)
    q = ((t * inv).astype(np.float32) + ROUND).astype(np.float32) - ROUND
    x = v.astype(np.float64) - q.astype(np.float64) * m
    if a is not None:
        x = x + a.astype(np.float64)
    x = x.astype(np.float32)
    x = np.where(x > 127, x - mf, x)
    x = np.where(x < -128, x + mf, x)
    return x, (x + ROUND).astype(np.float32).view(np.uint32)


def _int_path_residue(v, m):
    """mod_sym, the integer epilogue's reduction of the same sum: q = rint(fl(v * fl(1/m)))."""
    inv = np.float32(1.0 / m)
    q = np.rint((v * inv).astype(np.float32)).astype(np.int64)
    x = v.astype(np.int64) - q * m
    x = np.where(x > 127, x - m, x)
    return np.where(x < -128, x + m, x)


def test_drain_residues_match_the_integer_path():
    # every sum |v| <= 2^24 for three moduli (the even one and the two ends of the odd ones),
    # sampled sums for the others: the residue is congruent, in [-128, 127], the integer
    # path's representative, and the low byte of its bits
    rng = np.random.default_rng(3)
    for m in MODULI:
        if m in (256, 255, 191):
            chunks = [np.arange(s, min(s + 2 ** 22, 2 ** 24 + 1), dtype=np.float32)
                      for s in range(-2 ** 24, 2 ** 24 + 1, 2 ** 22)]
        else:
            chunks = [np.concatenate([rng.integers(-2 ** 24, 2 ** 24 + 1, 400_000),
                                      np.arange(-4096, 4097), np.arange(2 ** 24 - 4096, 2 ** 24 + 1),
                                      np.arange(-2 ** 24, -2 ** 24 + 4097)]).astype(np.float32)]
        for v in chunks:
            x, bits = _drain_residue(v, m)
            xi = x.astype(np.int64)
            assert np.all((xi - v.astype(np.int64)) % m == 0), m
            assert xi.min() >= -128 and xi.max() <= 127, m
            assert np.array_equal(xi, _int_path_residue(v, m)), m
            assert np.array_equal((bits & 0xFF).astype(np.uint8).view(np.int8).astype(np.int64), xi), m


def test_drain_residues_with_an_addend():
    # x1 - T2, -x1 - T2 and s + T3 (the addends |a| <= 256 from kept residues): congruent to
    # v + a and in [-128, 127] for sums near +-2^24 and near 0
    rng = np.random.default_rng(4)
    v = np.concatenate([np.arange(-2 ** 24, -2 ** 24 + 2048), np.arange(2 ** 24 - 2048, 2 ** 24 + 1),
                        np.arange(-2048, 2049), rng.integers(-2 ** 24, 2 ** 24 + 1, 20_000)]).astype(np.float32)
    for m in MODULI:
        for a0 in range(-256, 257, 17):
            a = np.full(v.shape, a0, dtype=np.float32)
            x, _ = _drain_residue(v, m, a)
            xi = x.astype(np.int64)
            assert np.all((xi - v.astype(np.int64) - a0) % m == 0), (m, a0)
            assert xi.min() >= -128 and xi.max() <= 127, (m, a0)


def test_kept_residue_bytes_round_trip():
    # a kept residue is the byte x + 128; 0x4B4000uu is the float 1.5 * 2^23 + u, so
    # subtracting 1.5 * 2^23 + 128 gives x back
    x = np.arange(-128, 128, dtype=np.int64)
    u = ((x.astype(np.int8).view(np.uint8)) ^ 0x80).astype(np.uint32)
    back = (u | np.uint32(0x4B400000)).view(np.float32) - np.float32(1.5 * 2 ** 23 + 128)
    assert np.array_equal(back.astype(np.int64), x)
