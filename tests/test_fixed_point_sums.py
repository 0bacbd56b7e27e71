"""The exact sums of the mixed path's coupled steps (kernels_step.cu,
phase_partials_fx / fx_warp_sum / fx_to_double), restated with Python
integers: a double x = m 2^(e-1075) goes onto its tile's grid (unit
2^(T - 1075 - 44), T the largest exponent in the tile) as an integer, tiles
then chunks then replicas are added after aligning to the larger grid (toward
zero), and the total is rounded to the nearest double.  Checked against the
exact rational sum: the error is below 2^-90 of the largest magnitude times
the count, for values spread over many binades and of both signs; and the
result does not depend on how the values are split into tiles."""
from __future__ import annotations

import math
import struct
from fractions import Fraction

import numpy as np

K = 44


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def fx_exp(x: float) -> int:
    e = (_bits(x) >> 52) & 0x7FF
    return e if e else 1


def fx_place(x: float, T: int) -> int:
    b = _bits(x)
    e = (b >> 52) & 0x7FF
    m = b & ((1 << 52) - 1)
    if e:
        m |= 1 << 52
    s = (e if e else 1) - T + K
    if s >= 0:
        v = m << s
    elif s > -64:
        v = m >> (-s)
    else:
        v = 0
    return -v if b >> 63 else v


def fx_align(v: int, T: int, Tmax: int) -> int:
    d = Tmax - T
    if d >= 127:
        return 0
    return -((-v) >> d) if v < 0 else v >> d


def fx_to_double(v: int, T: int) -> float:
    if v == 0:
        return 0.0
    neg = v < 0
    u = -v if neg else v
    p = u.bit_length() - 1
    sh = 0
    if p <= 52:
        mant = u
    else:
        sh = p - 52
        mant = u >> sh
        rem = u & ((1 << sh) - 1)
        half = 1 << (sh - 1)
        if rem > half or (rem == half and mant & 1):
            mant += 1
        if mant >> 53:
            mant >>= 1
            sh += 1
    r = math.ldexp(float(mant), sh + T - 1075 - K)
    return -r if neg else r


def level(rows):
    """rows: [(T, v)] -> (Tmax, sum) on the grid of the largest exponent."""
    Tm = max(T for T, _ in rows)
    return Tm, sum(fx_align(v, T, Tm) for T, v in rows)


def exact_fx_sum(xs, tile=128, chunk=256):
    tiles = []
    for i in range(0, len(xs), tile):
        t = xs[i:i + tile]
        T = max(fx_exp(x) for x in t)
        tiles.append((T, sum(fx_place(x, T) for x in t)))
    chunks = [level(tiles[i:i + chunk]) for i in range(0, len(tiles), chunk)]
    T, v = level(chunks)
    assert abs(v) < 2 ** 127
    return fx_to_double(v, T)


def _values(seed, n):
    rng = np.random.default_rng(seed)
    mags = 10.0 ** rng.uniform(-12, 6, n)
    return list(mags * rng.choice([-1.0, 1.0], n))


def test_sum_is_nearly_exact_over_many_binades():
    for seed in range(4):
        xs = _values(seed, 5000)
        got = exact_fx_sum(xs)
        want = sum(Fraction(x) for x in xs)
        bound = Fraction(max(abs(x) for x in xs)) * len(xs) * Fraction(1, 2 ** 90)
        # the final rounding to a double adds half an ulp of the result
        assert abs(Fraction(got) - want) <= bound + abs(want) * Fraction(1, 2 ** 53)


def test_sum_independent_of_tiling_and_order():
    xs = _values(7, 3000)
    a = exact_fx_sum(xs, tile=128, chunk=256)
    b = exact_fx_sum(list(reversed(xs)), tile=128, chunk=256)
    c = exact_fx_sum(xs, tile=64, chunk=3)
    # each tiling drops different bits far below 2^-90 of the largest value:
    # the rounded results agree to the last bit or one ulp
    for y in (b, c):
        assert abs(a - y) <= math.ulp(a)


def test_cancelling_sum_and_conversion_edges():
    xs = [1e6, 3.0e-9, -1e6, 5e-324, -5e-324, 2.0 ** -1000]
    got = exact_fx_sum(xs)
    assert got == 3.0e-9 or abs(got - 3.0e-9) <= 1e6 * 2 ** -90 * len(xs)
    assert exact_fx_sum([0.0] * 10) == 0.0
    for x in (1.0, -2.5, 1.0 / 3.0, 123456.789, 2.0 ** 52 + 1):
        assert exact_fx_sum([x]) == x
    # ties round to even (integers on the unit grid 2^0)
    assert fx_to_double((1 << 54) + 2, 1075 + K) == float(1 << 54)
    assert fx_to_double((1 << 54) + 6, 1075 + K) == float((1 << 54) + 8)
    assert fx_to_double(-((1 << 54) + 6), 1075 + K) == -float((1 << 54) + 8)
