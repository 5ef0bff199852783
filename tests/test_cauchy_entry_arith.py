"""The split path's double-float Cauchy entries u*v/(d - w), restated in numpy.

cauchy_entry (psmma_git_gb300/csrc/tcgen05_util.cuh) forms x = d - w in FP64 and then works
on the significands of u, v and x on the FP32 pipe.
- Each significand is split into hi (24 bits, rounded) + lo floats.
- y0 is the FP32 reciprocal of xh, and one Newton step against the whole x gives y1.
- e = 1 - x*y1 comes from two FMAs.
- a = u*v = ah + al is renormalised.
- q = a*(y1 + y1*e) = qh + ql is summed into a double.
- The exponents are added back from the bits.
The reciprocal approximation is modelled as the correctly rounded FP32 reciprocal, perturbed
by up to one ulp.  An FMA is modelled as a float64 product and sum rounded once to float32;
every product here is exact in float64.  The checks:
- the relative error is below 2^-45 (the kernel's self-test bound is 256 ulp);
- the result is exactly equivariant under power-of-two scalings of u, v and x.
"""
import numpy as np

F32 = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def _split_unit(x):
    """Significand of x (in [1, 2), with x's sign) as hi + lo floats, and x's exponent."""
    b = x.view(np.uint64)
    hx = (b >> np.uint64(32)).astype(np.uint32)
    lx = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    sgn = hx & np.uint32(0x80000000)
    up = (lx >> np.uint32(28)) & np.uint32(1)
    hi = ((sgn | np.uint32(127 << 23) | ((hx & np.uint32(0xFFFFF)) << np.uint32(3)) | (lx >> np.uint32(29)))
          + up).view(F32)
    rem = (lx & np.uint32(0x1FFFFFFF)).astype(np.int64) - (up.astype(np.int64) << 29)
    lo = (rem.astype(F32) * F32(2.0 ** -52)).astype(F32)
    lo = np.where(sgn != 0, -lo, lo).astype(F32)
    e = ((hx >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64) - 1023
    return hi, lo, e


def _entry(u, v, x, rng):
    us, ul, eu = _split_unit(u)
    vs, vl, ev = _split_unit(v)
    xs, xl, ex = _split_unit(x)
    one = np.ones_like(xs)
    y0 = (1.0 / xs.astype(np.float64)).astype(F32)
    y0 = (y0.view(np.int32) + rng.integers(-1, 2, y0.size).astype(np.int32)).view(F32)  # 1-ulp rcp
    y1 = _fma(y0, _fma(-xl, y0, _fma(-xs, y0, one)), y0)
    e = _fma(-xl, y1, _fma(-xs, y1, one))
    p = (us * vs).astype(F32)
    pl = _fma(ul, vl, _fma(us, vl, _fma(ul, vs, _fma(us, vs, -p))))
    ah = (p + pl).astype(F32)
    al = (pl - (ah - p)).astype(F32)
    qh = (ah * y1).astype(F32)
    ql = _fma(y1, _fma(al, e, _fma(ah, e, al)), _fma(ah, y1, -qh))
    q = qh.astype(np.float64) + ql.astype(np.float64)  # the kernel's single FP64 add
    return np.ldexp(q, (eu + ev - ex).astype(np.int32))


def _inputs(rng, n):
    u = rng.standard_normal(n)
    v = rng.standard_normal(n)
    d = rng.random(n)
    gap = np.exp2(-43.2 * rng.random(n))  # poles 1e-13 .. 1 apart
    w = np.where(rng.random(n) < 0.5, d - gap, d + gap)
    return u, v, d - w


def test_double_float_entries_within_bound():
    rng = np.random.default_rng(11)
    u, v, x = _inputs(rng, 400_000)
    q = _entry(u, v, x, rng)
    exact = np.longdouble(u) * np.longdouble(v) / np.longdouble(x)
    rel = np.abs((np.longdouble(q) - exact) / exact).astype(np.float64)
    assert rel.max() < 2.0 ** -45
    assert np.median(rel) < 2.0 ** -48


def test_double_float_entries_scale_exactly():
    rng = np.random.default_rng(12)
    u, v, x = _inputs(rng, 50_000)
    base = _entry(u, v, x, np.random.default_rng(5))
    scaled = _entry(u * 2.0 ** -200, v * 2.0 ** 150, x * 2.0 ** -30, np.random.default_rng(5))
    assert np.array_equal(scaled, base * 2.0 ** -20)
