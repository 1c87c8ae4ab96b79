"""The integer-pipe division and square root of dev_fpint.cuh, restated with
Python integers, against IEEE double division and sqrt (Python's `/` and
math.sqrt are correctly rounded): the method must give the same bits for every
operand it accepts, for FP32 seeds up to a few ulp off. The GPU code is
checked against the compiler's operators in test_fpint_gpu.py."""
import math
import random
import struct

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


class Seeds:
    """FP32 reciprocal / rsqrt seeds, rounded and then moved by up to `ulp`."""

    def __init__(self, rng, ulp):
        self.rng, self.ulp = rng, ulp

    def _move(self, f):
        return b2f(f2b(f) + self.rng.randint(-self.ulp, self.ulp))

    def rcp(self, x):
        return self._move(float(np.float32(1.0) / np.float32(x)))

    def rsqrt(self, x):
        return self._move(float(np.float32(1.0 / math.sqrt(x))))


def recip_word(Mb, seeds):
    D = Mb << 11
    rb = f2b(seeds.rcp(b2f((150 << 23) | ((Mb >> 29) & 0x7FFFFF))))
    e = (rb >> 23) - 103
    v = M64 if e >= 1 else (0 if e < 0 else (rb & 0x7FFFFF) << 41)
    for _ in range(2):
        E = s64(((1 << 64) - D) - hi64(D, v))
        d = abs(E) + hi64(v, abs(E))
        v = (v + d if v + d <= M64 else M64) if E >= 0 else (v - d if v >= d else 0)
    return v


def div_rn(a, b, seeds):
    """None where the device takes the compiler's operator."""
    ab, bb = d2b(a), d2b(b)
    ea, eb = (ab >> 52) & 0x7FF, (bb >> 52) & 0x7FF
    E = ea - eb + 1023
    sign = (ab ^ bb) & (1 << 63)
    bnorm = 1 <= eb <= 2046
    azero = (ab << 1) & M64 == 0
    if not (bnorm and (azero or (1 <= ea <= 2046 and 2 <= E <= 2045))):
        return None
    if azero:
        return b2d(sign)
    Ma, Mb = (ab & MANT) | HID, (bb & MANT) | HID
    u = Ma << 1
    Q = u + hi64(u, recip_word(Mb, seeds))
    rem = s64((Ma << 54) - Q * Mb)
    for _ in range(2):
        if rem < 0:
            Q, rem = Q - 1, rem + Mb
    for _ in range(2):
        if rem >= Mb:
            Q, rem = Q + 1, rem - Mb
    hi = Q >> 54
    M0 = Q >> (1 + hi)
    g = (Q >> hi) & 1
    st = (Q & 1 if hi else 0) | (rem != 0)
    M = M0 + (g & (st | (M0 & 1)))
    return b2d(sign | (((E - 2 + hi) << 52) + M))


def sqrt_rn(x, seeds):
    xb = d2b(x)
    ex = xb >> 52
    if not 1 <= ex <= 2046:
        return None
    Mx = (xb & MANT) | HID
    odd = (ex - 1075) & 1
    yb = f2b(seeds.rsqrt(b2f(((127 + odd) << 23) | ((Mx >> 29) & 0x7FFFFF))))
    ey = (yb >> 23) - 127
    Y = (1 << 63) if ey >= 0 else ((((yb & 0x7FFFFF) | 0x800000) << 39) if ey == -1 else (1 << 62))
    T = Mx << (10 + odd)
    for _ in range(2):
        Ee = s64((1 << 60) - hi64(T, hi64(Y, Y)))
        c = hi64(Y, abs(Ee)) << 3
        Y = Y + c if Ee >= 0 else Y - c
    S = hi64(T, Y) >> 7
    rem = s64((Mx << (56 + odd)) - S * S)
    for _ in range(2):
        if rem < 0:
            rem, S = rem + 2 * S - 1, S - 1
    for _ in range(2):
        if rem > 2 * S:
            S += 1
            rem -= 2 * S - 1
    M0 = S >> 2
    g = (S >> 1) & 1
    st = (S & 1) | (rem != 0)
    M = M0 + (g & (st | (M0 & 1)))
    E = ((ex - 1075 - 56 - odd) >> 1) + 1077
    return b2d(((E - 1) << 52) + M)


def operands(rng):
    k = rng.random()
    if k < 0.3:
        return rng.uniform(-1e3, 1e3), rng.uniform(-1e3, 1e3)
    if k < 0.5:
        return (math.ldexp(rng.uniform(1, 2), rng.randint(-1020, 1020)) * rng.choice((1, -1)),
                math.ldexp(rng.uniform(1, 2), rng.randint(-1020, 1020)) * rng.choice((1, -1)))
    if k < 0.7:  # exact quotients and ties
        return float(rng.getrandbits(53) | 1), float(rng.choice((3, 5, 7, 9, 1 << rng.randint(0, 60),
                                                                 rng.getrandbits(8) | 1)))
    if k < 0.8:
        return rng.choice((0.0, -0.0)), rng.uniform(-10, 10)
    return b2d(rng.getrandbits(64)), b2d(rng.getrandbits(64))


def test_division_is_correctly_rounded():
    rng = random.Random(11)
    done = 0
    for ulp in (0, 2, 8):
        seeds = Seeds(rng, ulp)
        for _ in range(8000):
            a, b = operands(rng)
            if b == 0 or any(math.isnan(v) or math.isinf(v) for v in (a, b)):
                continue
            q = div_rn(a, b, seeds)
            if q is None:
                continue
            done += 1
            assert d2b(q) == d2b(a / b), (a, b, ulp)
    assert done > 18000


def test_square_root_is_correctly_rounded():
    rng = random.Random(12)
    done = 0
    for ulp in (0, 2, 8):
        seeds = Seeds(rng, ulp)
        for _ in range(8000):
            k = rng.random()
            if k < 0.4:
                x = rng.uniform(0, 1e3)
            elif k < 0.7:
                x = math.ldexp(rng.uniform(1, 2), rng.randint(-1022, 1023))
            elif k < 0.85:
                x = float(rng.getrandbits(rng.randint(1, 53)))  # integers, perfect squares
            else:
                x = b2d(rng.getrandbits(63))
            if math.isinf(x) or math.isnan(x):
                continue
            s = sqrt_rn(x, seeds)
            if s is None:
                continue
            done += 1
            assert d2b(s) == d2b(math.sqrt(x)), (x, ulp)
    assert done > 20000
