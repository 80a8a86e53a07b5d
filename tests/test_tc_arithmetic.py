"""The exactness arguments of the tensor-core kernels, checked on CPU against
exact rational arithmetic (the kernels themselves are checked end to end by
the GPU parity tests):

* the FP64 emulation's fold turns W = T 2^28 + f into round-to-nearest-even
  FP64 with integer operations only (``fixed_to_double`` in dg_tc.cuh);
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
    # FP64 emulation: eight base-128 digits (|d| <= 64), a level holds at
    # most eight pairs, K <= 112 per product
    assert 8 * 112 * 64 * 64 < 2 ** 22
    # integers below 2^24 are exact in FP32
    v = np.arange(2 ** 24 - 1000, 2 ** 24, dtype=np.int64)
    assert np.array_equal(v.astype(np.float32).astype(np.int64), v)
    assert math.isclose(float(np.float32(2 ** 24 + 1)), 2 ** 24)        # and no further
