"""The wall function's TE^1.5 (navier_bc.cpp:279): the oracle and the GPU compute it as x*sqrt(x)
with a Newton-corrected root and an exact two-product, which is the correctly rounded x^1.5.
This checks the construction against exact rational arithmetic (FMA emulated exactly), over the
range k takes; the GPU-vs-oracle stage tests check that both builds evaluate it identically."""
import math
import random
from decimal import Decimal, getcontext
from fractions import Fraction


def _fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _pow15(x):
    if x == 0.0:
        return 0.0
    s = math.sqrt(x)
    r = _fma(-s, s, x)
    d = r / (2.0 * s)
    p = x * s
    e = _fma(x, s, -p)
    return p + (e + x * d)


def test_pow15_is_correctly_rounded():
    getcontext().prec = 80
    rng = random.Random(5)
    xs = [10.0 ** rng.uniform(-12, 3) for _ in range(20000)] + [1e-9, 1.0, 4.0, 2.25, 0.25]
    for x in xs:
        exact = Decimal(x) * Decimal(x).sqrt()
        assert _pow15(x) == float(exact), x
    assert _pow15(0.0) == 0.0
