"""The interpolation's (ulp - vp) / dt without a division (div_dt in
csrc/ibm.cu): with y = RN(1/dt) and yl = RN(1/dt - y), q0 = RN(x*y + RN(x*yl)),
r = x - dt*q0 (exact, one FMA) and q = RN(q0 + r*y).  The FMA steps are
emulated here in exact rational arithmetic (Python's float(Fraction) rounds to
nearest even), and q must equal x / dt bit for bit over random x and time
steps: dt with an all-ones significand and just above a power of two, x next to
multiples of dt, and quotients just below a power of two, where a rounded 1/dt
errs the most."""
import random
import struct
from fractions import Fraction


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def div_dt(x, dt):
    y = 1.0 / dt
    e = Fraction(1) - Fraction(dt) * Fraction(y)
    assert Fraction(float(e)) == e, "the reciprocal's remainder must be exact"
    yl = float(e) / dt
    q0 = float(Fraction(x) * Fraction(y) + Fraction(x * yl))
    r = Fraction(x) - Fraction(dt) * Fraction(q0)
    assert Fraction(float(r)) == r, "the remainder must be exact"
    return float(Fraction(q0) + r * Fraction(y))


def random_double(rng, emin, emax):
    m = rng.getrandbits(52)
    e = rng.randint(emin, emax) + 1023
    return from_bits((rng.getrandbits(1) << 63) | (e << 52) | m)


def test_division_by_dt_is_correctly_rounded():
    rng = random.Random(7)
    dts = [1e-3, 5e-4, 1e-2, 1.0 / 3.0, 0.7, 3.0, 1e-5, 7.3e-4,
           from_bits(0x3F4FFFFFFFFFFFFF), from_bits(0x3F50000000000001)]
    dts += [abs(random_double(rng, -20, 2)) for _ in range(6)]
    n = 0
    for dt in dts:
        for i in range(4000):
            x = random_double(rng, -60, 10)
            if i % 4 == 0:
                # next to a multiple of dt, where rounding is closest to a tie
                x = dt * rng.randint(1, 100000)
                x = from_bits(struct.unpack("<Q", struct.pack("<d", x))[0] + rng.choice((-1, 1)))
            elif i % 4 == 1:
                # a quotient with a significand just below 2
                x = dt * 2.0 ** rng.randint(-8, 20) * (1.0 - rng.random() * 2.0 ** -rng.randint(20, 52))
            assert div_dt(x, dt) == x / dt, (x, dt)
            n += 1
    assert n == 4000 * len(dts)
