"""Invariants of the 64-bit block-floating arithmetic of perceval_gb300/csrc/blockfloat.cuh
(the integer-pipe half of the FP64 permanents and of the sampler's FP64 mode), checked on
a restatement in Python integers that follows the device code operation by operation:

* bf_mul keeps its operands' invariant (|re|, |im| < 2^62, leading one at bit 61) and loses
  less than 2^-57 relative per product;
* bf_to_f64 rounds to nearest even and flushes below the normal FP64 range;
* the preparation's fixed-point scaling (row l1 nudged up by 2^-40 before its binade is
  taken) keeps every row sum below 2^62 even for rows whose l1 lies a rounding error below
  a power of two (rows of non-negative reals summing to 1, for one), where without the nudge
  the all-plus row sum reaches 2^62 and bf_norm's operand would overflow.
"""
import math
import random
import struct
from fractions import Fraction

import numpy as np

M64 = (1 << 64) - 1


def to_i64(x):
    x &= M64
    return x - (1 << 64) if x >> 63 else x


def clz64(x):
    x &= M64
    return 64 - x.bit_length()


def mul64hi(a, b):  # signed: the high 64 bits of the 128-bit product (floor)
    return to_i64((a * b) >> 64)


def bf_norm(re, im, e):
    ar, ai = abs(re), abs(im)
    sh = clz64(ar | ai) - 2
    assert sh >= 0, "operand at or above 2^62"
    return to_i64(re << sh), to_i64(im << sh), e - sh


def bf_mul(a, b):
    rr, ii = mul64hi(a[0], b[0]), mul64hi(a[1], b[1])
    ri, ir = mul64hi(a[0], b[1]), mul64hi(a[1], b[0])
    return bf_norm(rr - ii, ri + ir, a[2] + b[2] + 64)


def bf_to_f64(x, e):
    ax = abs(x)
    lz = clz64(ax)
    be = 1023 + 63 + e - lz
    if ax == 0 or be <= 0:
        return 0.0
    mn = (ax << (lz & 63)) & M64
    mant = mn >> 11
    rem = mn & 0x7FF
    mant += (rem + (mant & 1) + 0x3FF) >> 11
    bits = (1 << 63 if x < 0 else 0) | ((((be << 52) + mant - (1 << 52))) & M64)
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def value(z):
    return Fraction(z[0]) * Fraction(2) ** z[2], Fraction(z[1]) * Fraction(2) ** z[2]


def test_products_keep_the_invariant_and_62_bits():
    rng = random.Random(5)
    worst = 0.0
    for _ in range(3000):
        k = rng.randint(2, 27)
        F = 57
        rows = [(rng.randint(-(1 << 61), 1 << 61) >> rng.randint(0, 50),
                 rng.randint(-(1 << 61), 1 << 61) >> rng.randint(0, 50)) for _ in range(k)]
        z = bf_norm(rows[0][0], rows[0][1], -F)
        er, ei = value(z)
        for r in rows[1:]:
            w = bf_norm(r[0], r[1], -F)
            z = bf_mul(z, w)
            assert abs(z[0]) < 1 << 62 and abs(z[1]) < 1 << 62
            assert z == (0, 0, z[2]) or max(abs(z[0]), abs(z[1])).bit_length() == 62
            wr, wi = value(w)
            er, ei = er * wr - ei * wi, er * wi + ei * wr
        gr, gi = value(z)
        mag = math.sqrt(float(er * er + ei * ei))
        if mag > 0:
            err = math.sqrt(float((gr - er) ** 2 + (gi - ei) ** 2)) / mag
            worst = max(worst, err / (k - 1))
    assert worst < 2.0 ** -57, worst


def test_conversion_rounds_to_nearest_and_flushes():
    rng = random.Random(6)
    for _ in range(20000):
        x = rng.randint(-(1 << 62) + 1, (1 << 62) - 1) >> rng.randint(0, 61)
        e = rng.randint(-1150, 900)
        got = bf_to_f64(x, e)
        exact = Fraction(x) * Fraction(2) ** e
        want = float(exact)
        if abs(want) < 2.2250738585072014e-308:
            want = 0.0
        assert got == want or (got == 0.0 and want == 0.0), (x, e, got, want)


def _prepared_row_sums_fit(row, nudge=True):
    """The device preparation of one row: l1 by hypot sums (nudged up by 2^-40), the row
    scaled into [2^(c-1), 2^c) and stored as 64-bit fixed point with F = 62 - c; every
    signed row sum must stay below 2^62."""
    n = len(row)
    c = min(20, 120 // n)
    l1 = 0.0
    for v in row:
        l1 += math.hypot(v.real, v.imag)
    if nudge:
        l1 *= 1.0 + 2.0 ** -40
    _, x = math.frexp(l1)
    e = c - x
    F = 62 - c
    fx = [(round(math.ldexp(v.real, e + F)), round(math.ldexp(v.imag, e + F))) for v in row]
    # |re| and |im| of any signed sum are at most the sums of the parts' magnitudes
    return max(sum(abs(a) for a, _ in fx), sum(abs(b) for _, b in fx)) < 1 << 62


def test_fixed_point_headroom_at_power_of_two_l1():
    rng = np.random.default_rng(7)
    unnudged_overflows = 0
    for n in (8, 12, 16, 24, 32, 40):
        for _ in range(400):
            # non-negative real rows summing to a power of two up to rounding
            w = rng.random(n)
            w = w / w.sum() * 2.0 ** int(rng.integers(-5, 5))
            row = [complex(x, 0.0) for x in w]
            assert _prepared_row_sums_fit(row)
            unnudged_overflows += not _prepared_row_sums_fit(row, nudge=False)
            z = rng.normal(size=n) + 1j * rng.normal(size=n)
            assert _prepared_row_sums_fit(list(z))
    # the nudge is what keeps these rows inside: without it some reach 2^62
    assert unnudged_overflows > 0
