"""Division by a shared denominator in the FP64 path (gf_recip_y / gf_div in
geoflac_gb300/csrc/gf_kernels.cuh), restated with exact arithmetic and
checked against IEEE division.  For a denominator b:

    y  = RN(1/b)                  one IEEE division
    yl = RN(RN(1 - b y) y)        1 - b y is exact in an FMA

and for each numerator a:

    q  = RN(a y + RN(a yl))       faithful (within 0.5 ulp + 2^-104 |a/b|)
    r  = RN(a - b q)              exact because q is faithful
    RN(q + r y)                   = RN(a/b) by Markstein's theorem (a faithful
                                  quotient and the correctly rounded
                                  reciprocal; P. Markstein, IBM J. Res. Dev.
                                  34 (1990) 111-119)

Operands whose magnitude lies outside [2^-450, 2^451) take an IEEE division,
and a zero numerator gives a * y.  Python's float(Fraction) rounds correctly,
so fma(x, y, z) = float(Fraction(x) * y + z) is the fused multiply-add.  The
cases include quotients within r * 2^-106 (r = 1, 3, 5, ...) of a rounding
midpoint, the hardest cases for any division scheme.  Also here: the other
integer-pipe stand-in for an FP64 instruction, pre_plast's phase-ratio
cut-off taken on the bit pattern (gf_ratio_below_cut)."""
import math
import random
import struct
from fractions import Fraction

import pytest


def fma(x, y, z):
    return float(Fraction(x) * Fraction(y) + Fraction(z))


def dexp(x):
    """biased exponent field of a double"""
    return (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def dmid(x):
    return 573 <= dexp(x) <= 1473


def recip(b):
    y = 1.0 / b
    return b, y, fma(-y, b, 1.0) * y, dmid(b)


def div(a, r):
    b, y, yl, ok = r
    if not (ok and dmid(a)):
        return a * y if (ok and a == 0.0) else a / b
    q = fma(a, y, a * yl)
    return fma(fma(-q, b, a), y, q)


def same(x, y):
    """equal as bit patterns (signed zeros distinguished)"""
    return struct.pack("<d", x) == struct.pack("<d", y)


def near_midpoint_cases(rng, n):
    """(a, b) with a/b = u/2^54 - r/(2^54 B): u odd of 54 bits, so u/2^54 is
    the midpoint between two doubles, and a/b is r * 2^-106 away from it."""
    out = []
    while len(out) < n:
        B = rng.randrange(2 ** 52, 2 ** 53) | 1
        inv = pow(B, -1, 2 ** 54)
        r = rng.choice([1, -1, 3, -3, 5, -5, 7, -7, 101, -101])
        u = (r * inv) % 2 ** 54
        if u < 2 ** 53:
            continue
        A, rem = divmod(u * B - r, 2 ** 54)
        assert rem == 0
        if not 2 ** 52 <= A < 2 ** 53:
            continue
        ea, eb = rng.randint(-60, 60), rng.randint(-60, 60)
        sa, sb = rng.choice([1.0, -1.0]), rng.choice([1.0, -1.0])
        out.append((sa * math.ldexp(A, ea), sb * math.ldexp(B, eb)))
    return out


def test_reciprocal_pair_is_1_over_b_to_2_pow_minus_105():
    rng = random.Random(3)
    for _ in range(3000):
        b = rng.uniform(0.5, 1.0) * 10.0 ** rng.uniform(-100, 100) * rng.choice([1, -1])
        _, y, yl, ok = recip(b)
        assert ok
        exact = 1 / Fraction(b)
        assert abs(Fraction(y) + Fraction(yl) - exact) <= abs(exact) * Fraction(1, 2 ** 105)


def test_shared_denominator_quotients_are_correctly_rounded():
    rng = random.Random(5)
    cases = []
    for _ in range(6000):
        a = rng.uniform(-1.0, 1.0) * 10.0 ** rng.uniform(-12, 12)
        b = rng.uniform(0.5, 1.0) * 10.0 ** rng.uniform(-12, 12)
        cases.append((a, b))
    # denominators at and next to powers of two, numerators that are
    # multiples of the denominator and one ulp off
    for _ in range(2000):
        e = rng.randint(-40, 40)
        b = rng.choice([2.0 ** e, (2.0 ** e) * (1 + 2.0 ** -52), (2.0 ** e) * (2 - 2.0 ** -52),
                        (2.0 ** e) * (1 - 2.0 ** -53)])
        k = rng.uniform(1.0, 2.0) * 2.0 ** rng.randint(-20, 20)
        a = k * b
        for aa in (a, a * (1 + 2.0 ** -52), a * (1 - 2.0 ** -53), rng.uniform(-1, 1) * 2.0 ** rng.randint(-30, 30)):
            cases.append((aa, b))
    # the magnitudes of the FP64 callers: stresses over 2 mu, stresses over
    # inverse triangle areas
    for _ in range(2000):
        cases.append((rng.uniform(-1e10, 1e10), 2.0 * rng.uniform(1e9, 1e11)))
        cases.append((rng.uniform(-1e9, 1e9), rng.uniform(1e-10, 1e-6)))
    cases += near_midpoint_cases(rng, 6000)
    bad = [(a, b) for a, b in cases if not same(div(a, recip(b)), a / b)]
    assert not bad, bad[:5]


@pytest.mark.parametrize("b", [3.0, -3.0, 1e-200, 7e300, 2.0 ** -460, 2.0 ** 460])
def test_zeros_and_operands_outside_the_range_give_ieee_results(b):
    r = recip(b)
    for a in (0.0, -0.0, 1.5, -2.0 ** -470, 2.0 ** 470, 1e-300, 1e300, math.inf, -math.inf):
        try:
            want = a / b
        except OverflowError:
            continue
        assert same(div(a, r), want), (a, b)
    assert math.isnan(div(math.nan, r))


def ratio_below_cut(r):
    """gf_ratio_below_cut (geoflac_gb300/csrc/gf_kernels.cuh): r < 0.01 on the
    bit pattern of r"""
    b = struct.unpack("<Q", struct.pack("<d", r))[0]
    cut = struct.unpack("<Q", struct.pack("<d", 0.01))[0]
    if (b & 0x7FFFFFFFFFFFFFFF) > 0x7FF0000000000000:
        return False
    return True if (b >> 63) else b < cut


def test_phase_ratio_cut_off_on_the_bit_pattern_is_the_ieee_comparison():
    """pre_plast's `phase_ratio < 0.01` (rh_plastic.f90:250) taken on the
    integer pipe gives the IEEE comparison's answer on every class of value."""
    nxt = lambda x, d: struct.unpack("<d", struct.pack("<q", struct.unpack("<q", struct.pack("<d", x))[0] + d))[0]
    vals = [0.0, -0.0, 0.01, nxt(0.01, -1), nxt(0.01, 1), -0.01, 1.0, 0.5, 1e-300, -1e-300, 5e-324, -5e-324,
            math.inf, -math.inf, math.nan, -math.nan, 1 / 32, 1 / 3, 2.0, 1e300]
    rng = random.Random(9)
    vals += [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-20, 5) for _ in range(5000)]
    for v in vals:
        assert ratio_below_cut(v) == (v < 0.01), v
