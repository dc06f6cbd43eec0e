"""Division by a shared denominator in the FP64 path: each quotient a / b
from y = RN(1/b) (one IEEE division per denominator) and FMA residual
corrections,

    q0 = RN(a y);  q1 = RN(q0 + RN(a - b q0) y);  q2 = RN(q1 + RN(a - b q1) y)

(device code: div_shared in geoflac_gb300/csrc/gf_kernels.cuh).  q0 is
within 1.5 ulp of a/b, q1 is faithful, and Markstein's theorem (a faithful
quotient q and the correctly rounded reciprocal y give RN(q + (a - b q) y) =
RN(a/b); P. Markstein, IBM J. Res. Dev. 34 (1990) 111-119) makes q2 the
correctly rounded quotient, the bits of an IEEE division.  Restated here with
an exact fused multiply-add (Python's int and Fraction arithmetic rounds
correctly) and checked against IEEE division on random and hard cases."""
import random
from fractions import Fraction


def fma(x, y, z):
    return float(Fraction(x) * Fraction(y) + Fraction(z))


def div_shared(a, b, y):
    q = a * y
    r = fma(-q, b, a)
    q = fma(r, y, q)
    r = fma(-q, b, a)
    return fma(r, y, q)


def test_shared_denominator_quotients_are_correctly_rounded():
    rng = random.Random(5)
    cases = []
    for _ in range(6000):
        a = rng.uniform(-1.0, 1.0) * 10.0 ** rng.uniform(-12, 12)
        b = rng.uniform(0.5, 1.0) * 10.0 ** rng.uniform(-12, 12)
        cases.append((a, b))
    # denominators at and next to powers of two, mantissas of all ones,
    # numerators that are multiples of the denominator and one ulp off
    for _ in range(2000):
        e = rng.randint(-40, 40)
        b = rng.choice([2.0 ** e, (2.0 ** e) * (1 + 2.0 ** -52), (2.0 ** e) * (2 - 2.0 ** -52),
                        (2.0 ** e) * (1 - 2.0 ** -53)])
        k = rng.uniform(1.0, 2.0) * 2.0 ** rng.randint(-20, 20)
        a = k * b
        for aa in (a, a * (1 + 2.0 ** -52), a * (1 - 2.0 ** -53), rng.uniform(-1, 1) * 2.0 ** rng.randint(-30, 30)):
            cases.append((aa, b))
    # the magnitudes of the shear-heating terms: stresses over 2 mu
    for _ in range(2000):
        cases.append((rng.uniform(-1e10, 1e10), 2.0 * rng.uniform(1e9, 1e11)))
    bad = []
    for a, b in cases:
        y = 1.0 / b
        if div_shared(a, b, y) != a / b:
            bad.append((a, b))
    assert not bad, bad[:5]
