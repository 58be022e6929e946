"""The exact phase reduction of the tensor-core gridding (phase_pow2 and
i64_scaled in genfire_gb300/csrc/grid_mma.cu), restated on the CPU bit for
bit: for a power-of-two grid n = 2^t, integer a and an FP32 coordinate
w = m 2^e, the phase a w / n is reduced to [-1/2, 1/2) turns from the low bits
of the 64-bit product a m, and converted to FP32 with three exact 23-bit
chunks and FP32 fused multiply-adds.  Checked against exact rational
arithmetic: the reduced phase is within one FP32 unit in the last place of
the exact fraction (phases below 2^-83 turns are flushed to zero), over
random and adversarial coordinates (zeros, subnormals, integers, halves, the
largest grid coordinates)."""
import struct
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def fma32(a, b, c):
    # a * b is a power-of-two scaling of a 23-bit integer here, and the sum
    # spans fewer than 53 bits: the double sum is exact, one FP32 rounding
    return f32(float(a) * float(b) + float(c))


def i64_scaled(v, sh):
    a = abs(v)
    c0 = f32(a & 0x7FFFFF)
    c1 = f32((a >> 23) & 0x7FFFFF)
    c2 = f32((a >> 46) & 0x7FFFFF)
    p2 = lambda e: f32(2.0 ** e)
    f = f32(c0 * p2(-sh))
    f = fma32(c1, p2(23 - sh), f)
    f = fma32(c2, p2(46 - sh), f)
    return -f if v < 0 else f


def phase_pow2_fraction(a, w, t):
    bits = struct.unpack("<i", struct.pack("<f", w))[0]
    ex = (bits >> 23) & 0xFF
    if ex == 0:
        return f32(0)
    m = (bits & 0x7FFFFF) | 0x800000
    if bits < 0:
        m = -m
    sh = t - (ex - 150)
    P = a * m
    assert abs(P) < 2 ** 63
    if sh <= 0:
        return f32(0)
    if sh >= 62:
        return f32(0) if sh > 125 else i64_scaled(P, sh)
    low = P & ((1 << sh) - 1)
    if low >= (1 << (sh - 1)):
        low -= 1 << sh
    return i64_scaled(low, sh)


def exact_fraction(a, w, t):
    x = Fraction(a) * Fraction(float(w)) / (1 << t)
    return x - (x + Fraction(1, 2)).__floor__()          # in [-1/2, 1/2)


def ulp32(x):
    x = abs(float(x))
    if x == 0:
        return 2.0 ** -149
    return float(np.spacing(f32(x)))


def special_coordinates(n):
    h = n // 2
    vals = [0.0, -0.0, 1.0, -1.0, 0.5, -0.5, float(h), -float(h), float(h) - 0.5, 1e-30, -1e-38, 1e-45,
            float(np.nextafter(f32(h), f32(0))), float(np.nextafter(f32(0.5), f32(1)))]
    return [f32(v) for v in vals]


@pytest.mark.parametrize("t", [6, 8, 9, 10, 11, 12])
def test_phase_reduction_is_exact_to_one_ulp(t):
    n = 1 << t
    rng = np.random.default_rng(t)
    ws = [f32(v) for v in rng.uniform(-n / 2, n / 2, 300)] + special_coordinates(n)
    ws += [f32(v) for v in rng.standard_normal(50) * 1e-6]
    amax = (1 << 19) - 1
    As = [0, 1, -1, 32, -(n // 2), n // 2 - 1, amax, -amax] + [int(v) for v in rng.integers(-amax, amax + 1, 40)]
    for w in ws:
        for a in As:
            got = phase_pow2_fraction(a, w, t)
            want = exact_fraction(a, w, t)
            assert -0.5 <= float(got) <= 0.5
            if float(got) == 0.0 and abs(float(want)) < 2.0 ** -80:
                continue  # the kernel flushes phases below 2^-83 turns (shifts past 125 bits) to zero
            assert abs(float(got) - float(want)) <= ulp32(want), (a, float(w), t, float(got), float(want))


def test_reduction_wraps_to_the_half_open_interval():
    # a w / n = k + 1/2 exactly: the kernel maps it to -1/2 (low half bit set)
    t = 8
    for w in (f32(0.5), f32(1.5), f32(-2.5)):
        for a in (256, 768, -256):
            want = exact_fraction(a, w, t)
            got = phase_pow2_fraction(a, w, t)
            assert float(got) == float(want)
