"""The exact-arithmetic methods the secant pass uses instead of IEEE divisions
and products, checked on the CPU against exact rational arithmetic
(fractions.Fraction; float(Fraction) rounds to nearest even, so an FMA is
float(a * b + c) over rationals). These tests restate each method from its
mathematics in Python; tests/test_gpu_parity.py checks the device code of
the same methods against IEEE results on millions of operands.

- quot_gt_pos (fpbits.cuh): RN(a / b) > c decided by the sign of the FMA
  residual RN(a - c b) against y = b ulp(c) / 2;
- shared_div (fpbits.cuh): a / b from the correctly rounded reciprocal
  y = RN(1 / b), one product and two Markstein corrections;
- twice_chain (fpbits.cuh): (((2a) b) c) d equals 2 (((a b) c) d) while the
  products stay normal;
- fp_half (fpbits.cuh): 0.5 x as an exponent decrement for exponent fields
  2..0x7fe.
"""
import math
import struct
from fractions import Fraction as F

import numpy as np

RNG = np.random.default_rng(2026)


def fma(a, b, c):
    return float(F(a) * F(b) + F(c))


def exp_field(x):
    return (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def quot_gt_pos_method(a, b, c):
    """Returns (decision, used_division)."""
    eb, ec = exp_field(b), exp_field(c)
    k = ec - 1023 - 53
    if 1 <= eb <= 0x7FE and 1 <= ec <= 0x7FE and 1 <= eb + k <= 0x7FE:
        y = math.ldexp(b, k)                 # exact: b 2^k stays normal
        e = fma(-c, b, a)                    # RN(a - c b)
        if e > y:
            return True, False
        if e < y:
            return False, False
    return (a / b) > c, True


def test_division_free_stop_test_is_exact():
    n_div = 0
    cases = 0
    for c in (1e-8, 0.01, 1e-6, 0.3, 2.0 ** -30, np.nextafter(1e-8, 1.0)):
        b = np.exp(RNG.uniform(np.log(1e-4), np.log(1e4), 3000))
        steps = RNG.integers(-6, 7, b.size)
        for bi, st in zip(b, steps):
            a = float(bi) * c
            for _ in range(abs(int(st))):
                a = float(np.nextafter(a, np.inf if st > 0 else -np.inf))
            got, used = quot_gt_pos_method(a, float(bi), c)
            assert got == (float(F(a) / F(float(bi))) > c), (a, bi, c)
            n_div += used
            cases += 1
        # random magnitudes
        for _ in range(1000):
            a = math.ldexp(RNG.uniform(1, 2), int(RNG.integers(-1000, 1000)))
            bb = math.ldexp(RNG.uniform(1, 2), int(RNG.integers(-1000, 1000)))
            got, used = quot_gt_pos_method(a, bb, c)
            assert got == ((a / bb) > c)
            n_div += used
            cases += 1
    # the division is needed only for operands outside the exact range
    assert n_div < 0.2 * cases


def test_shared_reciprocal_quotient_is_correctly_rounded():
    def shared_div(a, b):
        y = float(F(1) / F(b))               # RN(1 / b)
        q = a * y                            # RN(a y)
        r = fma(-b, q, a)
        q = fma(r, y, q)
        r = fma(-b, q, a)
        return fma(r, y, q)

    for _ in range(20000):
        a = math.ldexp(RNG.uniform(1, 2), int(RNG.integers(-480, 480))) * float(RNG.choice([-1, 1]))
        b = math.ldexp(RNG.uniform(1, 2), int(RNG.integers(-480, 480))) * float(RNG.choice([-1, 1]))
        assert shared_div(a, b) == a / b, (a, b)
    # significands of all ones and powers of two, the hardest quotients
    ones = 2.0 - 2.0 ** -52
    for e1 in range(-20, 21, 5):
        for e2 in range(-20, 21, 5):
            for a, b in ((ones, 1.0), (1.0, ones), (ones, ones), (1.0 + 2.0 ** -52, ones)):
                a, b = math.ldexp(a, e1), math.ldexp(b, e2)
                assert shared_div(a, b) == a / b


def test_doubled_chain_and_halving_are_exact():
    for _ in range(20000):
        a, b, c, d = (float(x) for x in np.exp(RNG.uniform(-20, 20, 4)))
        g = ((a * b) * c) * d
        assert (((2.0 * a) * b) * c) * d == 2.0 * g
    for _ in range(20000):
        x = math.ldexp(RNG.uniform(1, 2), int(RNG.integers(-1021, 1024))) * float(RNG.choice([-1, 1]))
        e = exp_field(x)
        if 2 <= e <= 0x7FE:
            bits = struct.unpack("<q", struct.pack("<d", x))[0] - (1 << 52)
            assert struct.unpack("<d", struct.pack("<q", bits))[0] == 0.5 * x
