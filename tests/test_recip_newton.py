"""recip_newton (csrc/des_common.cuh): 1/x from an FP32 seed and one FP64
Newton step, r + r (1 - x r) as two fused multiply-adds.  The mixed step
and the reverse kernels use it for 1/viscosity, 1/(1 + tmp), 1/volume_old,
1/mass and other reciprocals; its comment claims ~1e-14 relative error for
|x| within the FP32 normal range.  Restated here with IEEE FP32 division
(the seed) and the C library's fma, which is correctly rounded like the
device's DFMA, and checked against exact rational reciprocals."""
import ctypes
import ctypes.util
from fractions import Fraction

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.fma.restype = ctypes.c_double
_libm.fma.argtypes = (ctypes.c_double,) * 3


def recip_newton(x: float) -> float:
    xf = np.float32(x)                       # f32_of: round to nearest (normal range)
    r = float(np.float32(1.0) / xf)          # the FP32 seed, f64_of exact
    return _libm.fma(r, _libm.fma(-x, r, 1.0), r)


def _rel_err(x, y):
    exact = 1 / Fraction(x)
    return abs(float((Fraction(y) - exact) / exact))


def test_relative_error_below_2e_minus_46_over_the_fp32_normal_range():
    rng = np.random.default_rng(5)
    xs = np.ldexp(rng.uniform(1, 2, 20_000), rng.integers(-125, 126, 20_000)) * rng.choice([-1.0, 1.0], 20_000)
    worst = max(_rel_err(float(x), recip_newton(float(x))) for x in xs)
    assert worst < 2.0 ** -46, worst


def test_values_the_kernels_divide_by():
    # viscosities 1e18..1e24, temperatures, volumes, masses, 1 + tmp near 1
    for x in (1e18, 1e21, 1e24, 273.0, 1603.0, 1.25e9, 3.7e15, 1.0, 1.0 + 2.5e-7, 1.0 + 0.25, 1e-30, 7.5e-8):
        assert _rel_err(x, recip_newton(x)) < 2.0 ** -46, x


def test_powers_of_two_are_exact():
    for k in range(-120, 121, 7):
        x = 2.0 ** k
        assert recip_newton(x) == 2.0 ** -k
