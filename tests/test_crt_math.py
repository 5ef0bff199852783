"""The split path's CRT recombination, restated in Python integers (CPU).

crt_row4 (psmma_git_gb300/csrc/split_crt.cu) recovers Z from residues r_l in [-128, 127] of the
moduli m_l (make_consts: C_l = (M/m_l) * ((M/m_l)^-1 mod m_l) mod M in four 32-bit limbs,
ffix_l = round(2^19 C_l / M)):
- per limb t, acc_t = sum_l (r_l + 128) climb_l,t (unsigned), and qi = sum_l r_l ffix_l;
- q = (qi + 2^18) >> 19, the quotient estimate;
- z_t = acc_t - sum_l 128 climb_l,t - q Mlimb_t (signed 64-bit), carries z_(t+1) += z_t >> 32;
- Z = sum_t z_t 2^(32 t), the top limb carrying the sign.
Z is exact when |Z| < (1/2 - 0.002) M: the estimate's error is at most 16 * 128 * 0.5 * 2^-19.
For an odd modulus, 127 and -128 can both stand for a class (m = 255) or any r and r -+ m
inside [-128, 127] (m < 255); the result does not depend on which one a kernel stored, which
the one-launch 3M epilogue relies on (its FP32 residues pick by their own rounded quotient).
"""
import random

import pytest

MODULI = [256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 211, 199, 197, 193, 191]
MASK32 = (1 << 32) - 1


def _consts(nmod):
    ms = MODULI[:nmod]
    M = 1
    for m in ms:
        M *= m
    C = []
    for m in ms:
        Ml = M // m
        C.append(Ml * pow(Ml % m, -1, m) % M)
    climb = [[(c >> (32 * t)) & MASK32 for t in range(4)] for c in C]
    ffix = [(c * (1 << 19) + M // 2) // M for c in C]  # round(2^19 C_l / M), |error| <= 1/2
    biasl = [sum(128 * climb[l][t] for l in range(nmod)) for t in range(4)]
    Mlimb = [(M >> (32 * t)) & MASK32 for t in range(4)]
    return ms, M, C, climb, ffix, biasl, Mlimb


def _i64(x):
    x &= (1 << 64) - 1
    return x - (1 << 64) if x >> 63 else x


def _crt(res, consts):
    ms, M, C, climb, ffix, biasl, Mlimb = consts
    acc = [0, 0, 0, 0]
    qi = 0
    for l, r in enumerate(res):
        assert -128 <= r <= 127
        ur = r + 128
        qi += r * ffix[l]
        for t in range(4):
            acc[t] += ur * climb[l][t]
    assert all(a < 1 << 64 for a in acc) and -(1 << 31) <= qi < 1 << 31
    q = (qi + (1 << 18)) >> 19
    z = [_i64(acc[t] - biasl[t] - q * Mlimb[t]) for t in range(4)]
    for t in range(3):
        z[t + 1] = _i64(z[t + 1] + (z[t] >> 32))
    return sum((z[t] & MASK32) << (32 * t) for t in range(3)) + (z[3] << 96)


def _residue_choices(Z, ms, rng):
    """Each residue of Z as one of its representatives in [-128, 127], chosen at random."""
    out = []
    for m in ms:
        reps = [x for x in range(-128, 128) if (x - Z) % m == 0]
        out.append(rng.choice(reps))
    return out


@pytest.mark.parametrize("nmod", [8, 10, 13, 16])
def test_crt_recovers_z_from_any_representatives(nmod):
    consts = _consts(nmod)
    ms, M = consts[0], consts[1]
    rng = random.Random(nmod)
    lim = int(M * (0.5 - 0.002))
    zs = [rng.randrange(-lim, lim + 1) for _ in range(300)]
    zs += [lim, -lim, 0, 1, -1, M // 3, -(M // 3)]
    for Z in zs:
        for _ in range(3):
            assert _crt(_residue_choices(Z, ms, rng), consts) == Z


def test_crt_limb_bounds():
    # the top limb of the 13-moduli CRT fits the 32-bit sum the kernel keeps it in (top32), and
    # the 16-moduli one does not (it takes the 64-bit sum)
    for nmod, top32 in [(13, True), (16, False)]:
        ms, M, C, climb, ffix, biasl, Mlimb = _consts(nmod)
        assert (2 * biasl[3] < 1 << 32) == top32
        assert M < 1 << 128
