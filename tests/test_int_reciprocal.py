"""The reciprocal and the division without the FP64 pipe (gf_rcp_sig,
gf_rcp and gf_ddiv in geoflac_gb300/csrc/gf_kernels.cuh), restated step for
step and checked against IEEE division (Python floats are IEEE doubles).

The FP32 steps (__frcp_rn, fmaf, __fmul_rn) are restated with exact rational
arithmetic rounded once to the nearest float32 (ties to even), the integer
steps on Python integers reduced to 64 bits as the device holds them.  The
bounds the device code relies on are asserted on every case: the Newton
residual R fits in a signed 64-bit integer, the corrected candidate lies
within 1.5 units of 2^105 / M, and the midpoint residuals are exact in 64
bits; for the division, the residual is below 2^55 and ends in [0, Mb)
without a tie.  The cases include significands next to both ends of
[2^52, 2^53), the significands whose top 24 bits are all zero or all one,
powers of two, exact quotients and one ulp beside them, signed zeros, and
the ends of the covered exponent range."""
import math
import random
import struct
from fractions import Fraction

M32 = 0xFFFFFFFF
M64 = (1 << 64) - 1


def f2u(f):
    return struct.unpack("<I", struct.pack("<f", f))[0]


def u2f(u):
    return struct.unpack("<f", struct.pack("<I", u & M32))[0]


def rn_f32(q):
    """an exact rational rounded to the nearest float32, ties to even
    (normal range)"""
    q = Fraction(q)
    if q == 0:
        return 0.0
    s = -1 if q < 0 else 1
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    scaled = a / Fraction(2) ** (e - 23)
    n = scaled.numerator // scaled.denominator
    rem = scaled - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n & 1):
        n += 1
    return s * float(Fraction(n) * Fraction(2) ** (e - 23))


def split(x):
    u = struct.unpack("<Q", struct.pack("<d", x))[0]
    return u & M32, u >> 32


def join(lo, hi):
    return struct.unpack("<d", struct.pack("<Q", (hi & M32) << 32 | (lo & M32)))[0]


def s64(x):
    x &= M64
    return x - (1 << 64) if x >> 63 else x


def rcp_sig(mhi, lo):
    """gf_rcp_sig: RN(2^105 / M) for M = 2^52 + mhi:lo"""
    Mh = u2f(0x3F800000 | (((mhi << 3) | (lo >> 29)) & 0x7FFFFF))
    Ml = rn_f32(Fraction((lo >> 5) & 0xFFFFFF, 2 ** 47))
    assert Fraction(Ml) == Fraction((lo >> 5) & 0xFFFFFF, 2 ** 47)
    r = rn_f32(1 / Fraction(Mh))                                   # __frcp_rn
    e2 = rn_f32(-Fraction(Ml) * Fraction(r) + Fraction(rn_f32(-Fraction(Mh) * Fraction(r) + 1)))  # fmaf x2
    rl = rn_f32(Fraction(r) * Fraction(e2))                        # __fmul_rn
    ur, ul = f2u(r), f2u(rl)
    er, el = (ur >> 23) & 0xFF, (ul >> 23) & 0xFF
    sh = el - 97
    Sl = (ul & 0x7FFFFF) | 0x800000
    v = 0 if el == 0 else (Sl << sh) & M32 if sh >= 0 else (Sl >> -sh) if sh > -32 else 0
    assert abs(rl) < 2.0 ** -22 and v < 1 << 31
    t = (((ur & 0x7FFFFF) | 0x800000) << (er - 97)) + (-v if ul >> 31 else v)
    M = ((mhi | 0x100000) << 32) | lo
    R = s64(-(M * t))
    assert R == 2 ** 105 - M * t and abs(R) < 2 ** 62
    t += s64((R * t) >> 64) >> 41                                  # __mul64hi (signed)
    assert abs(Fraction(2 ** 105, M) - t) < Fraction(3, 2)
    Dp = s64(-(M * (2 * t + 1)))
    assert Dp == 2 ** 106 - M * (2 * t + 1) and Dp != 0
    t += 1 if Dp > 0 else (-1 if Dp + 2 * M < 0 else 0)
    assert abs(Fraction(2 ** 105, M) - t) <= Fraction(1, 2)
    return t


def gf_rcp(b):
    lo, hi = split(b)
    E = (hi >> 20) & 0x7FF
    if ((E - 573) & M32) > 900:  # the IEEE division out of line (1/(+-0) = +-inf)
        return (math.copysign(math.inf, b) if b == 0.0 else 1.0 / b), False
    sign, mhi = hi & 0x80000000, hi & 0xFFFFF
    if (mhi | lo) == 0:
        return join(0, sign | ((2046 - E) << 20)), True
    bits = (((2044 - E) << 52) + rcp_sig(mhi, lo)) & M64
    return join(bits & M32, (bits >> 32) | sign), True


def gf_ddiv(a, b):
    la, ha = split(a)
    lb, hb = split(b)
    Ea, Eb = (ha >> 20) & 0x7FF, (hb >> 20) & 0x7FF
    za = ((ha << 1) & M32 | la) == 0
    if not ((((Ea - 573) & M32) <= 900 or za) and ((Eb - 573) & M32) <= 900):
        return a / b, False
    sign = (ha ^ hb) & 0x80000000
    if za:
        return join(0, sign), True
    Ma = (((ha & 0xFFFFF) | 0x100000) << 32) | la
    Mb = (((hb & 0xFFFFF) | 0x100000) << 32) | lb
    t = rcp_sig(hb & 0xFFFFF, lb)
    k = 52 if Ma >= Mb else 53
    q = ((((Ma * t) >> 64) << (k - 41)) | (((Ma * t) & M64) >> (105 - k))) & M64   # __umul64hi, low word
    res = s64((Ma << k) - Mb * q)
    assert res == Ma * 2 ** k - Mb * q and abs(res) < 2 * Mb
    for _ in range(2):
        if res < 0:
            q, res = q - 1, res + Mb
    for _ in range(2):
        if res >= Mb:
            q, res = q + 1, res - Mb
    assert 0 <= res < Mb and 2 * res != Mb
    q += 1 if 2 * res > Mb else 0
    bits = (((1074 - k + Ea - Eb) << 52) + q) & M64
    return join(bits & M32, (bits >> 32) | sign), True


def same(x, y):
    return struct.pack("<d", x) == struct.pack("<d", y)


def check(bs):
    bad = []
    for b in bs:
        got, _ = gf_rcp(b)
        if not same(got, 1.0 / b):
            bad.append((b, got, 1.0 / b))
    assert not bad, bad[:4]


def test_random_reciprocals_are_ieee_quotients():
    rng = random.Random(31)
    check([rng.uniform(0.5, 1.0) * 10.0 ** rng.uniform(-130, 130) * rng.choice([1, -1]) for _ in range(12000)])
    # the step's magnitudes: inverse areas, determinants, 1 + dt/tau
    check([rng.uniform(1e-12, 1e-4) for _ in range(3000)] + [rng.uniform(1e4, 1e12) for _ in range(3000)]
          + [1.0 + rng.uniform(0, 0.5) for _ in range(3000)])


def test_significand_edges():
    rng = random.Random(32)
    ms = []
    for _ in range(3000):
        ms.append((1 << 53) - 1 - rng.randrange(1 << 20))         # next to 2^53
        ms.append((1 << 52) + 1 + rng.randrange(1 << 20))         # next to 2^52: r = 1
        top = rng.choice([0, (1 << 23) - 1, rng.randrange(1 << 23)])
        ms.append((1 << 52) | (top << 29) | rng.randrange(1, 1 << 29))   # all-zero / all-one top bits
    check([math.ldexp(m, rng.randint(-400, 400) - 52) * rng.choice([1.0, -1.0]) for m in ms])


def test_powers_of_two_zero_and_range_ends():
    lo, hi = 2.0 ** -450, 2.0 ** 451 * (1 - 2.0 ** -53)
    vals = [2.0 ** k for k in range(-450, 451, 7)] + [-0.5, lo, hi, -lo, -hi, 3.0, 0.1, 1.0000000000000002]
    check(vals)
    for b in (0.0, -0.0, math.inf, -math.inf, 1e-300, 1e300, math.nextafter(lo, 0.0), 2.0 ** 451):
        got, fast = gf_rcp(b)
        assert not fast
        if not math.isnan(got) and b != 0.0:
            assert same(got, 1.0 / b)


def test_quotients_are_ieee_quotients():
    rng = random.Random(33)
    cases = [(rng.uniform(-1, 1) * 10.0 ** rng.uniform(-130, 130), rng.uniform(-1, 1) * 10.0 ** rng.uniform(-130, 130))
             for _ in range(8000)]
    for _ in range(4000):
        ma = rng.choice([(1 << 53) - 1 - rng.randrange(100), (1 << 52) + rng.randrange(100), rng.randrange(1 << 52, 1 << 53)])
        mb = rng.choice([(1 << 53) - 1 - rng.randrange(100), (1 << 52) + rng.randrange(100),
                         rng.randrange(1 << 52, 1 << 53), 1 << 52])
        cases.append((math.ldexp(ma, rng.randint(-200, 200)), math.ldexp(mb, rng.randint(-200, 200))))
    for _ in range(3000):  # exact quotients and one ulp beside them
        b = rng.uniform(1, 2) * 2.0 ** rng.randint(-100, 100)
        a = b * rng.uniform(1, 2) * 2.0 ** rng.randint(-100, 100)
        cases += [(a, b), (math.nextafter(a, 0.0), b), (math.nextafter(a, math.inf), b)]
    # the step's quotients: dt f / (m drat^2), rhs dt / area, the rotation / det
    for _ in range(2000):
        cases.append((rng.uniform(-1e12, 1e12), rng.uniform(1e10, 1e20)))
        cases.append((rng.uniform(-1e-3, 1e-3), rng.uniform(1e-7, 1e-5)))
    cases += [(0.0, 3.0), (-0.0, 3.0), (0.0, -3.0), (-0.0, -3.0), (1.0, 3.0), (2.0, 2.0), (1.0, 1.0000000000000002)]
    bad = [(a, b) for a, b in cases if not same(gf_ddiv(a, b)[0], a / b)]
    assert not bad, bad[:4]
    # outside the covered range: the IEEE division out of line
    for a, b in [(1.0, 1e-300), (1e300, 3.0), (5e-324, 1.0), (1.0, 2.0 ** 451)]:
        got, fast = gf_ddiv(a, b)
        assert not fast and same(got, a / b)
