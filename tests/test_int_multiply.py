"""FP64 products on the integer pipes (gf_mul and gf_scale in
geoflac_gb300/csrc/gf_kernels.cuh), restated step for step on 32-bit words
and checked against IEEE multiplication (Python floats are IEEE doubles,
round to nearest even).

gf_mul takes the 53-bit significands of two operands whose biased exponents
lie in 573 .. 1473 (or that are zero), forms the 106-bit product from four
32x32->64-bit multiplies, keeps 53 bits and rounds to nearest even from the
round bit, the dropped bits and the kept value's parity; other operands take
the FP64 multiply.  gf_scale multiplies by 0.25, 0.5, 2 or 4 by moving the
exponent field while operand and result are normal.  The cases include exact
ties and products within one unit of the last dropped bit of a tie (the
rounding decisions), significands whose rounding carries into the exponent,
signed zeros, and exponents at both ends of the covered range.  Also the
integer-pipe forms of additions and products with a +0 operand."""
import math
import random
import struct

M32 = 0xFFFFFFFF


def split(x):
    u = struct.unpack("<Q", struct.pack("<d", x))[0]
    return u & M32, u >> 32


def join(lo, hi):
    return struct.unpack("<d", struct.pack("<Q", (hi & M32) << 32 | (lo & M32)))[0]


def funnel_l(lo, hi, sh):
    """__funnelshift_l(lo, hi, sh): high word of (hi:lo) << sh"""
    return ((hi << 32 | lo) << sh >> 32) & M32


def gf_mul(a, b):
    la, ha = split(a)
    lb, hb = split(b)
    za = ((ha << 1) & M32 | la) == 0
    zb = ((hb << 1) & M32 | lb) == 0
    ia = (((ha >> 20) & 0x7FF) - 573) & M32 <= 900
    ib = (((hb >> 20) & 0x7FF) - 573) & M32 <= 900
    if not ((ia or za) and (ib or zb)):
        return a * b, False
    mh = (ha & 0xFFFFF) | 0x100000
    nh = (hb & 0xFFFFF) | 0x100000
    p0 = la * lb
    t = la * nh + (p0 >> 32)
    t += mh * lb
    u = mh * nh + (t >> 32)
    w2, w1, w0, wm = u >> 32, u & M32, t & M32, p0 & M32
    assert w2 < 1 << 10 and t < 1 << 64 and u < 1 << 64
    top = w2 >> 9
    sh = 12 - top
    mhi, mlo = funnel_l(w1, w2, sh), funnel_l(w0, w1, sh)
    rem = (w0 << sh) & M32
    x = min(wm, 1) | (mlo & 1)
    assert rem & 1 == 0
    up = 1 if rem + x > 0x80000000 else 0
    S = ((ha & 0xFFF00000) + (hb & 0xFFF00000) - (1024 << 20) + (top << 20)) & M32
    r = ((((mhi + S) & M32) << 32) | mlo) + up
    if za or zb:
        return join(0, (ha ^ hb) & 0x80000000), True
    return join(r & M32, (r >> 32) & M32), True


def gf_scale(x, k):
    lo, hi = split(x)
    e = (hi >> 20) & 0x7FF
    lo_e, hi_e = (1 - k, 2046) if k < 0 else (1, 2046 - k)
    if ((e - lo_e) & M32) <= hi_e - lo_e:
        return join(lo, (hi + k * (1 << 20)) & M32)
    if ((hi << 1) & M32 | lo) == 0:
        return x
    return x * 2.0 ** k


def same(x, y):
    return struct.pack("<d", x) == struct.pack("<d", y)


def check(cases):
    bad, fast = [], 0
    for a, b in cases:
        got, f = gf_mul(a, b)
        fast += f
        if not same(got, a * b):
            bad.append((a, b, got, a * b))
    assert not bad, bad[:4]
    return fast


def test_random_products_are_ieee_products():
    rng = random.Random(21)
    cases = []
    for _ in range(40000):
        a = rng.uniform(-1, 1) * 10.0 ** rng.uniform(-130, 130)
        b = rng.uniform(-1, 1) * 10.0 ** rng.uniform(-130, 130)
        cases.append((a, b))
    # the magnitudes of the FP64 step: coordinates x velocities, stresses x
    # strain increments, shape derivatives x areas
    for _ in range(20000):
        cases.append((rng.uniform(-1e6, 1e6), rng.uniform(-1e-9, 1e-9)))
        cases.append((rng.uniform(-1e10, 1e10), rng.uniform(-1e-3, 1e-3)))
    assert check(cases) == len(cases)


def test_ties_near_ties_and_carries():
    """Significands with low zero bits make the 106-bit product end exactly
    on a tie or one unit beside it; all-ones significands carry the rounding
    into the exponent."""
    rng = random.Random(22)
    cases = []
    for _ in range(60000):
        ma = rng.randrange(1 << 52, 1 << 53)
        mb = rng.randrange(1 << 52, 1 << 53)
        kind = rng.randrange(4)
        if kind == 0:   # product = odd * 2^k: an exact tie at the round bit
            ma = (ma >> 27 << 27) | (1 << 26)
            mb = mb >> 26 << 26 | (1 << 26)
        elif kind == 1:  # a tie plus or minus one unit of the sticky bits
            ma = (ma >> 27 << 27) | (1 << 26) | rng.choice([0, 1])
            mb = mb >> 27 << 27
        elif kind == 2:  # rounding carries out of the significand
            ma = (1 << 53) - 1 - rng.randrange(64)
            mb = (1 << 53) - 1 - rng.randrange(64)
        ea, eb = rng.randint(-300, 300), rng.randint(-300, 300)
        a = math.ldexp(ma, ea - 52) * rng.choice([1.0, -1.0])
        b = math.ldexp(mb, eb - 52) * rng.choice([1.0, -1.0])
        cases.append((a, b))
    assert check(cases) == len(cases)


def test_zeros_range_edges_and_other_operands():
    lo = 2.0 ** -450             # smallest magnitude on the integer path
    hi = 2.0 ** 451 * (1 - 2.0 ** -53)  # largest
    edge = [lo, hi, -lo, -hi, math.nextafter(lo, 0.0), math.nextafter(hi, math.inf), 1.0, -1.0,
            0.0, -0.0, 0.5, 3.0, 1e-300, 1e300, 5e-324, math.inf, -math.inf]
    cases = [(a, b) for a in edge for b in edge]
    check([(a, b) for a, b in cases if not (math.isinf(a) or math.isinf(b))])
    # the integer path takes zeros and the covered range, nothing else
    for a, b in cases:
        got, fast = gf_mul(a, b)
        want_fast = all(x == 0.0 or 2.0 ** -450 <= abs(x) < 2.0 ** 451 for x in (a, b))
        assert fast == want_fast, (a, b)
        if not math.isnan(a * b):
            assert same(got, a * b), (a, b)
    # signed zeros: the sign is the exclusive or
    for a in (0.0, -0.0):
        for b in (2.5, -2.5, 0.0, -0.0):
            assert same(gf_mul(a, b)[0], a * b) and same(gf_mul(b, a)[0], b * a)


def test_power_of_two_scaling():
    rng = random.Random(23)
    vals = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-307, 307) for _ in range(20000)]
    vals += [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 4.450147717014403e-308,
             8.900295434028806e-308, 1.7976931348623157e308, 4.49423283715579e307, 8.98846567431158e307,
             math.inf, -math.inf, 1.0, -3.0]
    for k in (-2, -1, 1, 2):
        for v in vals:
            got, want = gf_scale(v, k), v * 2.0 ** k
            assert same(got, want), (v, k, got, want)


def plus_pzero(x):
    """gf_plus_pzero: x + (+0) on the bit pattern"""
    lo, hi = split(x)
    return join(lo, 0 if (lo == 0 and hi == 0x80000000) else hi)


def zero_minus(x):
    """gf_zero_minus: +0 - x on the bit pattern"""
    lo, hi = split(x)
    return join(lo, 0 if (lo | hi) == 0 else hi ^ 0x80000000)


def mul_z_shortcut(z, y):
    """gf_mul_z's integer case: +0 * y for y in [+0, +max]"""
    zl, zh = split(z)
    yl, yh = split(y)
    return 0.0 if (zl | zh) == 0 and yh < 0x7FF00000 else None


def test_plus_zero_operand_shortcuts():
    """The +0 operands of the plane-strain step without dikes or thermal
    stress (gf_add_z, gf_sub_z, gf_zero_minus, gf_mul_z, and the Maxwell
    s33 of a plane-strain triangle) give the IEEE results."""
    rng = random.Random(24)
    vals = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-300, 300) for _ in range(5000)]
    vals += [0.0, -0.0, 5e-324, -5e-324, 1.7976931348623157e308, -1.7976931348623157e308, math.inf, -math.inf]
    for x in vals:
        assert same(plus_pzero(x), x + 0.0), x
        assert same(x, x - 0.0), x                    # gf_sub_z returns x
        assert same(zero_minus(x), 0.0 - x), x
        got = mul_z_shortcut(0.0, x)
        if got is not None:
            assert same(got, 0.0 * x) and x >= 0.0, x
        else:
            assert math.copysign(1.0, x) < 0 or not math.isfinite(x), x  # the FP64 multiply out of line
    # Maxwell, plane strain: s33d = de33d = +0 and s33 = (s33d vic1 +
    # 2 rmu de33d) vic2 + s0 is +0 + s0 for vic1, 2 rmu, vic2 in [+0, +max]
    pos = [0.0, 5e-324, 0.5, 1.0, 3e10, 1.7976931348623157e308]
    for vic1 in pos:
        for rmu2 in pos:
            for vic2 in pos:
                for s0 in (0.0, -0.0, -1e8, 2.5, 5e-324):
                    full = (0.0 * vic1 + rmu2 * 0.0) * vic2 + s0
                    assert same(full, plus_pzero(s0)), (vic1, rmu2, vic2, s0)
    # the plastic trial with de33 = +0: (de + de33) and s + de33 * e1
    for de in vals[:2000]:
        assert same(de + 0.0, plus_pzero(de))
        for e1 in (1e10, 5e-324, 0.0):
            assert same(de + 0.0 * e1, plus_pzero(de))


def test_magnitude_comparison_on_bits():
    """gf_abs_gt (the damping test |v| > 1e-13 of fl_node) on the bit
    patterns gives the FP64 comparison's answer."""
    c = 1.0e-13
    cb = struct.unpack("<Q", struct.pack("<d", c))[0]
    rng = random.Random(25)
    vals = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-20, 5) for _ in range(5000)]
    vals += [0.0, -0.0, c, -c, math.nextafter(c, 1.0), math.nextafter(c, 0.0), math.inf, -math.inf, math.nan]
    for v in vals:
        ax = struct.unpack("<Q", struct.pack("<d", v))[0] & 0x7FFFFFFFFFFFFFFF
        assert (ax > cb and ax <= 0x7FF0000000000000) == (abs(v) > c), v


def deq(a, b):
    """gf_deq: IEEE a == b on the bit patterns"""
    al, ah = split(a)
    bl, bh = split(b)
    nan = (ah & 0x7FFFFFFF) > 0x7FF00000 or ((ah & 0x7FFFFFFF) == 0x7FF00000 and al != 0)
    return (al == bl and ah == bh and not nan) or ((((ah | bh) << 1) & M32) == 0 and (al | bl) == 0)


def test_equality_on_bits():
    """gf_deq (the thermal sweeps' change test) is IEEE equality."""
    rng = random.Random(26)
    vals = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-300, 300) for _ in range(300)]
    vals += [0.0, -0.0, math.inf, -math.inf, math.nan, 5e-324, -5e-324, 1.0, math.nextafter(1.0, 2.0)]
    for a in vals:
        for b in vals[-12:] + [a, -a]:
            assert deq(a, b) == (a == b), (a, b)
