"""f32_of / f64_of (csrc/des_common.cuh): FP64 <-> FP32 conversions done with
integer instructions, because on GB300 the conversion instructions share the
FP64 pipe.

The device functions are a few lines of bit arithmetic on the two 32-bit
halves of a double.  This restates them step for step in numpy (uint32
arithmetic wraps as it does on the device) and checks them against IEEE
conversions:
- f32_of equals round-to-nearest-even except exactly halfway, where it rounds
  away from zero;
- magnitudes below 2^-126 become signed zeros;
- overflow gives inf, and NaN stays NaN;
- f64_of is exact for every normal float, and inf and NaN are kept.
"""
import numpy as np

U = np.uint32


def f32_of(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(U)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(U)
    mag = hi & U(0x7FFFFFFF)
    with np.errstate(over="ignore"):
        u = (((mag - U(896 << 20)) << U(3)) | (lo >> U(29))) + ((lo >> U(28)) & U(1))
    u = np.where(mag < U(897 << 20), U(0), u)
    special = np.where((mag > U(0x7FF00000)) | ((mag == U(0x7FF00000)) & (lo != 0)), U(0x7FC00000), U(0x7F800000))
    u = np.where(mag >= U(1151 << 20), special, u)
    return ((hi & U(0x80000000)) | u).astype(U).view(np.float32)


def f64_of(f):
    u = np.asarray(f, dtype=np.float32).view(U)
    mag = u & U(0x7FFFFFFF)
    hi = (mag >> U(3)) + (np.where(mag >= U(0x7F800000), U(1792), U(896)) << U(20))
    lo = mag << U(29)
    hi = np.where(mag < U(0x00800000), U(0), hi)
    lo = np.where(mag < U(0x00800000), U(0), lo)
    hi = (u & U(0x80000000)) | hi
    return ((hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)).view(np.float64)


def _doubles(n, rng):
    """Random significands over the float exponent range and a little beyond."""
    m = rng.integers(0, 2 ** 52, size=n, dtype=np.uint64)
    e = rng.integers(1023 - 140, 1023 + 140, size=n).astype(np.uint64)
    s = rng.integers(0, 2, size=n).astype(np.uint64)
    return ((s << np.uint64(63)) | (e << np.uint64(52)) | m).view(np.float64)


def test_f32_of_is_nearest_float():
    rng = np.random.default_rng(7)
    x = _doubles(400000, rng)
    got = f32_of(x)
    normal = (np.abs(x) >= 2.0 ** -126) & (np.abs(x) < 2.0 ** 128 * (1 - 2.0 ** -25))
    with np.errstate(over="ignore"):
        ref = x.astype(np.float32)
    tie = (x.view(np.uint64) & np.uint64((1 << 29) - 1)) == np.uint64(1 << 28)
    ok = normal & ~tie
    np.testing.assert_array_equal(got[ok].view(U), ref[ok].view(U))
    # halfway cases: away from zero, so the magnitude is never below the exact value
    t = normal & tie
    assert np.all(np.abs(got[t].astype(np.float64)) >= np.abs(x[t]))
    # below the float normal range: signed zero
    small = np.abs(x) < 2.0 ** -126
    assert np.all(got[small] == 0)
    np.testing.assert_array_equal(np.signbit(got[small]), np.signbit(x[small]))
    # beyond it: inf of the right sign
    big = np.abs(x) >= 2.0 ** 128
    assert np.all(np.isinf(got[big])) and np.all(np.sign(got[big]) == np.sign(x[big]))


def test_f32_of_specials_and_carries():
    x = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 2.0 ** -126, 2.0 ** 127,
                  np.nextafter(2.0, 0.0),                     # mantissa all ones: carries into the exponent
                  float(np.finfo(np.float32).max)])
    got = f32_of(x)
    assert got[0] == 0 and not np.signbit(got[0]) and got[1] == 0 and np.signbit(got[1])
    assert got[2] == np.inf and got[3] == -np.inf and np.isnan(got[4])
    np.testing.assert_array_equal(got[5:].view(U), x[5:].astype(np.float32).view(U))


def test_f64_of_is_exact():
    rng = np.random.default_rng(11)
    f = rng.integers(0, 2 ** 32, size=400000, dtype=np.uint64).astype(U).view(np.float32)
    got = f64_of(f)
    fin = np.isfinite(f) & (np.abs(f) >= np.float32(2.0 ** -126))
    np.testing.assert_array_equal(got[fin], f[fin].astype(np.float64))
    sub = np.isfinite(f) & (np.abs(f) < np.float32(2.0 ** -126))
    assert np.all(got[sub] == 0)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(f))
    inf = np.isinf(f)
    np.testing.assert_array_equal(got[inf], f[inf].astype(np.float64))


def test_round_trip():
    rng = np.random.default_rng(3)
    f = rng.standard_normal(100000).astype(np.float32) * np.float32(1e6)
    np.testing.assert_array_equal(f32_of(f64_of(f)).view(U), f.view(U))
