"""The force-density kernel divides face differences of phi by cell-centre
spacings as q0 = a y, r = fma(-b, q0, a), q = fma(r, y, q0) with y the
correctly rounded reciprocal of b (Markstein's correction step, IBM J. Res.
Dev. 34(1), 1990).  Here the same three roundings are emulated exactly in
double precision (fma through exact rational arithmetic) and compared with
IEEE division over random quotients of the ranges the densities see, and
over divisors at the edges of the significand."""
import random
from fractions import Fraction


def _fma(x, y, z):
    return float(Fraction(x) * Fraction(y) + Fraction(z))


def _div_step(a, b):
    y = 1.0 / b
    q0 = a * y
    return _fma(_fma(-b, q0, a), y, q0)


def test_division_step_matches_ieee_division():
    rng = random.Random(2026)
    for t in range(20000):
        b = rng.uniform(1e-3, 2.0) * rng.choice([1e-2, 1.0, 10.0])
        if t % 5 == 0:  # significands all ones / a power of two / random bits
            b = float.fromhex(rng.choice(["0x1.fffffffffffffp%d", "0x1.0000000000000p%d",
                                          "0x1.%013xp" % rng.getrandbits(52) + "%d"]) % rng.randint(-12, 4))
        a = rng.uniform(-1.0, 1.0) * 10.0 ** rng.randint(-14, 3)
        if t % 7 == 0:
            a = float.fromhex("0x1.%013xp%d" % (rng.getrandbits(52), rng.randint(-40, 8)))
        assert _div_step(a, b) == a / b, (a.hex(), b.hex())


def test_division_step_exact_cases():
    for a, b in ((0.0, 0.3), (1.0, 1.0), (3.0, 0.5), (-7.25, 2.0), (1.0, 3.0), (2.0, 3.0), (1e-300, 0.7)):
        assert _div_step(a, b) == a / b
