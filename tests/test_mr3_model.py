"""The FP64 walk's m/r^3 (m_r3_from_seed, dev_internal.cuh), restated with
Python integers, against exact rational arithmetic: from an FP32 rsqrt seed of
r^-1 (up to a few ulp off), e = 1 - r2 y0^2 from one 128-bit product, the
series (1-e)^-3/2 in 62-bit fixed point and m y0^3 c by three high-word
multiplies, rounded once. Bar: within 1.01 x 2^-53 relative over the whole
accepted range (2^-99 <= r2 < 2^100, 2^-863 <= m < 2^865); the reference's
m / (r2 * sqrt(r2)) rounds three times (up to ~3 x 2^-53)."""
import math
import random
import struct
from fractions import Fraction

import numpy as np

M64 = 2**64 - 1
MANT = 2**52 - 1
HID = 1 << 52


def d2b(d):
    return struct.unpack("<Q", struct.pack("<d", d))[0]


def b2d(b):
    return struct.unpack("<d", struct.pack("<Q", b & M64))[0]


def f2b(f):
    return struct.unpack("<I", struct.pack("<f", f))[0]


def b2f(b):
    return struct.unpack("<f", struct.pack("<I", b & 0xFFFFFFFF))[0]


def hi64(a, b):
    return ((a & M64) * (b & M64)) >> 64


def s64(x):
    x &= M64
    return x - 2**64 if x >> 63 else x


def seed(r2b, rng, ulp):
    """rsqrtf of the truncated FP32 value of r2 (f32_from_f64_bits), moved by up to ulp."""
    r2f = b2f(((r2b >> 29) - (896 << 23)) & 0xFFFFFFFF)
    y = float(np.float32(1.0 / math.sqrt(r2f)))
    return b2f(f2b(y) + rng.randint(-ulp, ulp))


def m_r3(r2b, mb, y0):
    yb = f2b(y0)
    Y = (yb & 0x7FFFFF) | 0x800000
    ey = yb >> 23
    S = Y * Y
    Mr = (r2b & MANT) | HID
    P = Mr * S
    L, H = P & M64, P >> 64
    sh = 1375 - 64 - (r2b >> 52) - 2 * ey
    assert 34 <= sh <= 37
    Dhi = (1 << sh) - H - (1 if L else 0)
    Dlo = (-L) & M64
    E64 = s64(((Dhi & M64) << (64 - sh)) | (Dlo >> sh))
    aE = abs(E64)
    C = (1 << 62) + ((3 * E64) >> 3) + ((15 * hi64(aE, aE)) >> 5)
    hi3 = hi64(Y << 40, S << 16)
    Z = hi64(hi3, C << 1)
    Q = hi64((((mb & MANT) | HID) << 11), Z)
    lz = 32 - (Q >> 32).bit_length()
    s = 11 - lz
    M = (Q + (1 << (s - 1))) >> s
    return b2d((((mb >> 52) + 3 * ey - 378 - lz) << 52) + M)


def test_m_over_r3_is_within_one_rounding():
    rng = random.Random(21)
    worst = Fraction(0)
    for i in range(30000):
        r2 = math.ldexp(rng.uniform(1, 2), rng.randint(-99, 99))
        m = rng.choice((math.ldexp(rng.uniform(1, 2), rng.randint(-863, 864)), rng.uniform(1e-7, 1.0), 1.0))
        if i % 1000 == 0:
            r2 = rng.choice((2.0**-99, float(np.nextafter(2.0**100, 0)), 1.0, 4.0))
            m = rng.choice((2.0**-863, float(np.nextafter(2.0**865, 0)), 1.0))
        got = m_r3(d2b(r2), d2b(m), seed(d2b(r2), rng, 3))
        # compare got^2 r2^3 with m^2 (exact): |got / (m r2^-3/2) - 1| ~ |got^2 r2^3 / m^2 - 1| / 2
        rel = abs(Fraction(got) ** 2 * Fraction(r2) ** 3 / Fraction(m) ** 2 - 1) / 2
        worst = max(worst, rel)
    assert worst < Fraction(101, 100) * Fraction(1, 2**53), float(worst) / 2**-53
