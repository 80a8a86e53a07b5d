"""The exactness arguments of the tensor-core kernels, checked on CPU against
exact rational arithmetic (the kernels themselves are checked end to end by
the GPU parity tests):

* the FP64 emulation's fold turns W = T 2^28 + f into round-to-nearest-even
  FP64 with integer operations only (``fixed_to_double`` in dg_tc.cuh);
* the FP64 emulation's whole product (54-bit fixed point, seven balanced
  base-256 digits, level sums i + j <= 8, recombination) is accurate to
  FP64 rounding;
* the mixed kernel writes a row value as four balanced base-256 digits with
  FP32 arithmetic only (``digits4`` in dg_tcm.cuh), exactly;
* the level sums the tensor core accumulates stay exact integers in FP32.
"""

from __future__ import annotations

import math
import random
import struct
from fractions import Fraction

import numpy as np


def _fixed_to_double(T: int, f: int, s: int):
    """Restatement of fixed_to_double: RN(T 2^28 + f) 2^s, or None outside
    the normal range."""
    neg = T < 0
    A = (-T - (f != 0)) if neg else T
    B = ((1 << 28) - f) if (neg and f != 0) else f
    if A < (1 << 36):
        Z, zexp = (A << 28) | B, 0
    else:
        Z, zexp = ((A << 18) | (B >> 10) | (1 if (B & 1023) else 0)), 10
    if Z == 0:
        return 0.0
    n = Z.bit_length() - 1
    eb = n + zexp + s + 1023
    if eb < 1 or eb > 2045:
        return None
    up = 0
    if n <= 52:
        mant = Z << (52 - n)
    else:
        sh = n - 52
        mant, rem, half = Z >> sh, Z & ((1 << sh) - 1), 1 << (sh - 1)
        up = 1 if (rem > half or (rem == half and (mant & 1))) else 0
    bits = (eb << 52) + (mant - (1 << 52)) + up
    bits |= (1 << 63) if neg else 0
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def test_fixed_to_double_is_round_to_nearest_even():
    rng = random.Random(1)
    for _ in range(50000):
        kind = rng.random()
        if kind < 0.3:
            T = rng.randint(-(1 << 46) + 1, (1 << 46) - 1)
        elif kind < 0.6:
            T = rng.randint(-(1 << 36), 1 << 36)
        else:
            T = rng.randint(-1000, 1000)
        f = rng.randint(0, (1 << 28) - 1)
        s = rng.randint(-200, 200)
        got = _fixed_to_double(T, f, s)
        if got is None:
            continue
        assert got == float(Fraction(T * (1 << 28) + f) * Fraction(2) ** s)


def test_fixed_to_double_ties():
    rng = random.Random(2)
    for _ in range(3000):
        m = rng.randint(1 << 52, (1 << 53) - 1)
        for extra in range(1, 20):
            W = (m << extra) + (1 << (extra - 1))      # exactly halfway
            for w in (W, -W):
                T, f = w >> 28, w & ((1 << 28) - 1)
                assert _fixed_to_double(T, f, 0) == float(Fraction(w))


def _digits4(x: np.ndarray, e: int) -> np.ndarray:
    """Restatement of digits4 in FP32 (FMA as exact product + one rounding)."""
    f32 = np.float32
    scale = np.frombuffer(np.uint32((284 - e) << 23).tobytes(), np.float32)[0]

    def fma(a, b, c):
        return (a.astype(np.float64) * np.float64(b) + c.astype(np.float64)).astype(f32)

    v = np.rint(x * scale).astype(f32)
    d0 = np.rint(v * f32(2.0 ** -24)).astype(f32)
    r1 = fma(-d0, f32(2.0 ** 24), v)
    d1 = np.rint(r1 * f32(2.0 ** -16)).astype(f32)
    r2 = fma(-d1, f32(65536.0), r1)
    d2 = np.rint(r2 * f32(2.0 ** -8)).astype(f32)
    d3 = fma(-d2, f32(256.0), r2)
    return v, np.stack([d0, d1, d2, d3])


def test_four_digit_split_is_exact_and_fits_fp16():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(200000) * np.exp(rng.uniform(-20, 5, 200000))).astype(np.float32)
    e = max(int(np.frombuffer(np.abs(x).max().tobytes(), np.uint32)[0] >> 23), 30)
    v, d = _digits4(x, e)
    rec = (d[0].astype(np.float64) * 2.0 ** 24 + d[1] * 2.0 ** 16 + d[2] * 2.0 ** 8 + d[3])
    assert np.array_equal(rec, v.astype(np.float64))
    assert np.abs(d).max() <= 128 and np.abs(v).max() <= 2.0 ** 31
    assert np.array_equal(d.astype(np.float16).astype(np.float32), d)   # exact in FP16
    # the quantisation error relative to the row maximum: below 2^-31
    xs = v.astype(np.float64) * 2.0 ** (e - 157)
    assert np.max(np.abs(xs - x.astype(np.float64))) <= 2.0 ** (e - 127 - 31)


def test_level_sums_stay_exact_in_fp32():
    # mixed kernel: four digits (|d| <= 128), levels i + j <= 3 hold at most
    # four pairs, K <= 128 per phase: at most 2^23
    assert 4 * 128 * 128 * 128 <= 2 ** 23
    # FP64 emulation: seven base-256 digits (|d| <= 128), a level holds at
    # most seven pairs, K <= 146 per product
    assert 7 * 146 * 128 * 128 < 2 ** 24
    # integers below 2^24 are exact in FP32
    v = np.arange(2 ** 24 - 1000, 2 ** 24, dtype=np.int64)
    assert np.array_equal(v.astype(np.float32).astype(np.int64), v)
    assert math.isclose(float(np.float32(2 ** 24 + 1)), 2 ** 24)        # and no further


def _to_fixed(x: float, emax: int) -> int:
    """Restatement of to_fixed (dg_tc.cuh): round(x 2^(54 - e_n)), e_n = emax - 1022."""
    bits = struct.unpack("<q", struct.pack("<d", x))[0]
    ex = (bits >> 52) & 0x7FF
    m = bits & ((1 << 52) - 1)
    if ex:
        m |= 1 << 52
    else:
        ex = 1
    sh = emax - ex - 1
    if sh < 0:
        r = m << (-sh)
    elif sh == 0:
        r = m
    elif sh > 60:
        r = 0
    else:
        r = (m + (1 << (sh - 1))) >> sh
    return -r if bits < 0 else r


def _digits7(x: int) -> list:
    """Seven balanced base-256 digits, most significant first (digits7 and
    the host packing)."""
    d = [0] * 7
    for s in range(6, -1, -1):
        q = ((x + 128) & 255) - 128
        d[s] = q
        x = (x - q) >> 8
    assert x == 0
    return d


def _dexp(x: float) -> int:
    return (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def _emulated_dot(a: list, xs: list) -> float:
    """One output of the FP64 tensor-core emulation: row a (operator) times
    column xs (data), as the kernel computes it."""
    amax = max(abs(v) for v in a)
    e_m = math.frexp(amax)[1] if amax > 0 else 0              # |a| < 2^e_m
    emax = max(_dexp(v) for v in xs)
    da = [_digits7(int(round(math.ldexp(v, 54 - e_m)))) for v in a]
    dx = [_digits7(_to_fixed(v, emax)) for v in xs]
    lv = []
    for l in range(2, 9):                                     # levels 2..8
        tot = 0
        for i in range(max(1, l - 7), min(l - 1, 7) + 1):
            j = l - i
            tot += sum(p[i - 1] * q[j - 1] for p, q in zip(da, dx))
        assert abs(tot) < 2 ** 24
        lv.append(tot)
    hi = lv[0] * 65536 + lv[1] * 256 + lv[2]
    lo = lv[3] * 16777216 + lv[4] * 65536 + lv[5] * 256 + lv[6]
    T, f = hi * 16 + (lo >> 28), lo & ((1 << 28) - 1)
    s = e_m + (emax - 1022) - 60
    return _fixed_to_double(T, f, s)


def test_seven_digit_emulation_is_accurate_to_fp64():
    rng = random.Random(3)
    for K in (20, 35, 60, 105, 146):
        for _ in range(40):
            a = [rng.uniform(-1, 1) * 2.0 ** rng.randint(-3, 3) for _ in range(K)]
            xs = [rng.gauss(0, 1) * 2.0 ** rng.randint(-8, 8) for _ in range(K)]
            if rng.random() < 0.3:           # cancellation
                xs[-1] = -sum(p * q for p, q in zip(a[:-1], xs[:-1])) / a[-1]
            got = _emulated_dot(a, xs)
            exact = sum(Fraction(p) * Fraction(q) for p, q in zip(a, xs))
            scale = max(abs(v) for v in a) * max(abs(v) for v in xs)
            # input rounding 2^-55 per operand and the dropped pairs
            # (< 2^-51 K), on top of the final rounding
            bound = 2.0 ** -50 * K * scale + abs(float(exact)) * 2.0 ** -52
            assert abs(Fraction(got) - exact) <= Fraction(bound), (K, got, float(exact))


def test_digits_fit_fp16_and_the_fixed_point_range():
    for x in (2 ** 54, -(2 ** 54), 2 ** 54 - 1, 12345678901234567, -1, 0):
        d = _digits7(x)
        assert max(abs(v) for v in d) <= 128
        assert sum(v * 256 ** (6 - k) for k, v in enumerate(d)) == x
    # to_fixed never leaves |x| <= 2^54 for the column's largest exponent
    for v in (1.0, -1.9999999999999998, 0.75, 1e-300, -3.0):
        assert abs(_to_fixed(v, _dexp(v))) <= 2 ** 54


def _f32_exact_int24(v: np.float32) -> int:
    """Restatement of f32_exact_int24 (dg_tc.cuh) in FP32 arithmetic."""
    f32 = np.float32
    big_c = f32(3221225472.0)
    big = f32(v + big_c)
    lo = f32(v - f32(big - big_c))
    bits = lambda x: int(np.frombuffer(np.float32(x).tobytes(), np.int32)[0])  # noqa: E731
    return (bits(big) - bits(big_c)) * 256 + (bits(f32(lo + f32(12582912.0))) - 0x4B400000)


def test_level_sum_conversion_is_exact():
    rng = np.random.default_rng(5)
    vals = list(rng.integers(-(2 ** 24) + 1, 2 ** 24, 20000)) + [0, 1, -1, 127, 128, -128,
                                                                 129, 2 ** 24 - 1, -(2 ** 24) + 1]
    for v in vals:
        assert _f32_exact_int24(np.float32(v)) == int(v)
