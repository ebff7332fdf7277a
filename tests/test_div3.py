"""div3 (csrc/des_common.cuh): x / 3 as fma(x, YH, x * YL) is bit-identical
to the IEEE quotient for |x| >= 2^-900 and for +-0 (the kernels divide the
nonzero values below 2^-900).

The argument is in the kernel's comment; here the same two operations run
through the C library's fma, which is correctly rounded like the device's
DFMA, on random significands over the whole exponent range and on the inputs
closest to the cases that could round differently (multiples of 3 and their
neighbours, significands on either side of 3 * 2^52, powers of two)."""
import ctypes
import ctypes.util
import math
import struct
from fractions import Fraction

import numpy as np

YH = float.fromhex("0x1.5555555555555p-2")
YL = float.fromhex("0x1.5555555555555p-56")

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.fma.restype = ctypes.c_double
_libm.fma.argtypes = (ctypes.c_double, ctypes.c_double, ctypes.c_double)


def _bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def _div3(x):
    if abs(x) < 2.0 ** -900 and x != 0:   # +-0 takes the fma path
        return x / 3
    return _libm.fma(x, YH, x * YL)


def test_constants_are_the_two_term_reciprocal_of_3():
    assert YH == 1 / 3                                   # RN(1/3)
    assert YL == float(Fraction(1, 3) - Fraction(YH))    # RN(1/3 - YH)
    assert _libm.fma(2.0, 3.0, 1.0) == 7.0


def _inputs():
    rng = np.random.default_rng(12345)
    out = []
    # random significands over the exponent range the kernels can meet
    m = rng.integers(2 ** 52, 2 ** 53, size=60000, dtype=np.int64)
    e = rng.integers(-900, 1000, size=m.size)
    s = rng.choice([-1.0, 1.0], size=m.size)
    out += [float(sg) * math.ldexp(float(mm), int(ee) - 52) for mm, ee, sg in zip(m, e, s)]
    # significands that are multiples of 3 and their neighbours
    k = rng.integers(2 ** 52 // 3 + 1, (2 ** 53 - 1) // 3, size=20000, dtype=np.int64)
    for kk in k:
        for d in (-1, 0, 1):
            out.append(math.ldexp(float(3 * int(kk) + d), int(rng.integers(-60, 60))))
    # either side of the significand 3 * 2^52 (the quotient's exponent changes there)
    for d in range(-200, 201):
        out.append(math.ldexp(float(3 * 2 ** 51 + d), 0))
        out.append(math.ldexp(float(2 ** 53 - 1 - d), -30))
    # powers of two and small integers
    out += [math.ldexp(1.0, p) for p in range(-900, 1000)]
    out += [float(i) for i in range(-3000, 3001)]
    # stress-like magnitudes
    out += list(rng.normal(0, 1e9, size=20000)) + list(rng.normal(0, 1e-15, size=20000))
    return out


def test_div3_is_bit_identical_to_division():
    bad = [x for x in _inputs() if _bits(_div3(x)) != _bits(x / 3)]
    assert not bad, [x.hex() for x in bad[:10]]


def test_div3_special_values():
    for x in (0.0, -0.0, math.inf, -math.inf, 2.0 ** -1074, -(2.0 ** -1000), 1.7976931348623157e308):
        assert _bits(_div3(x)) == _bits(x / 3), x
    assert math.isnan(_div3(math.nan))


def _div6(x):
    if abs(x) < 2.0 ** -900:
        return x / 6
    return _div3(x * 0.5)


def test_div6_is_bit_identical_to_division():
    """div6 = div3(x / 2): halving is exact above the subnormal range."""
    xs = _inputs() + [math.ldexp(1.0, p) * 1.5 for p in range(-1074, -890)]
    bad = [x for x in xs if _bits(_div6(x)) != _bits(x / 6)]
    assert not bad, [x.hex() for x in bad[:10]]
