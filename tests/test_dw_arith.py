"""The double-word FP32 arithmetic of the mixed step (csrc/des_dw.cuh),
restated in numpy float32 (IEEE round-to-nearest, as the device's FP32
instructions) and held to its published error bounds against exact
rational arithmetic (fractions.Fraction), u = 2^-24:

* dw_split: the integer/FP32 split of an FP64 value, normalised:
  |x - (hi + lo)| <= 2^-47 |x| (|x| >= 2^-97) and |lo| <= ulp(hi) / 2;
* two_sum, two_prod: error-free (Knuth; the FMA product error);
* dw_add (Joldes-Muller-Popescu 2017, Algorithm 6): < 3u^2 + 13u^3 of the
  exact sum, with cancellation;
* dw_mul (Algorithm 12): < 4u^2;
* dw_dot3c, dw_diff2, dw_sum3 (Dot2 / Sum2 of Ogita-Rump-Oishi on
  double-word operands): a small multiple of u^2 of the terms' magnitudes;
* dw_recip: < 8u^2;
* the force terms of one element, T_i = (sigma . dN_i + b z) vol, as
  k_nmd_correct_ft3 forms them, within 2^-43 of the terms' magnitudes.

fmaf(a, b, c) is emulated as RN32(a b + c) with the product exact in FP64;
where it forms a product's exact error (two_prod) the emulation is exact.
"""
from fractions import Fraction as F

import numpy as np

U = 2.0 ** -24
f32 = np.float32


def fmaf(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    ap = f32(s - b)
    bp = f32(s - ap)
    return s, f32(f32(a - ap) + f32(b - bp))


def fast_two_sum(a, b):
    s = f32(a + b)
    z = f32(s - a)
    return s, f32(b - z)


def two_prod(a, b):
    p = f32(a * b)
    return p, fmaf(a, b, -p)


def dw_add(x, y):
    sh, sl = two_sum(x[0], y[0])
    th, tl = two_sum(x[1], y[1])
    c = f32(sl + th)
    vh, vl = fast_two_sum(sh, c)
    w = f32(tl + vl)
    return fast_two_sum(vh, w)


def dw_mul(x, y):
    ch, cl1 = two_prod(x[0], y[0])
    tl0 = f32(x[1] * y[1])
    tl1 = fmaf(x[0], y[1], tl0)
    cl2 = fmaf(x[1], y[0], tl1)
    cl3 = f32(cl1 + cl2)
    return fast_two_sum(ch, cl3)


def dw_neg(x):
    return (f32(-x[0]), f32(-x[1]))


def dw_dot3c(a0, b0, a1, b1, a2, b2):
    p0, p1, p2 = two_prod(a0[0], b0[0]), two_prod(a1[0], b1[0]), two_prod(a2[0], b2[0])
    s = f32(p0[1] + fmaf(a0[0], b0[1], f32(a0[1] * b0[0])))
    t1 = two_sum(p0[0], p1[0])
    s = f32(s + f32(t1[1] + f32(p1[1] + fmaf(a1[0], b1[1], f32(a1[1] * b1[0])))))
    t2 = two_sum(t1[0], p2[0])
    s = f32(s + f32(t2[1] + f32(p2[1] + fmaf(a2[0], b2[1], f32(a2[1] * b2[0])))))
    return two_sum(t2[0], s)


def dw_sum3(x, y, z):
    t1 = two_sum(x[0], y[0])
    c = f32(t1[1] + f32(x[1] + y[1]))
    t2 = two_sum(t1[0], z[0])
    c = f32(c + f32(t2[1] + z[1]))
    return two_sum(t2[0], c)


def dw_diff2(a, b, c, d):
    p, q = two_prod(a[0], b[0]), two_prod(c[0], d[0])
    t = two_sum(p[0], f32(-q[0]))
    s = f32(f32(f32(p[1] - q[1]) + f32(fmaf(a[0], b[1], f32(a[1] * b[0])) - fmaf(c[0], d[1], f32(c[1] * d[0]))))
            + t[1])
    return two_sum(t[0], s)


def dw_recip(x):
    r0 = f32(f32(1.0) / x[0])
    ph, pl = two_prod(x[0], r0)
    e = f32(f32(f32(f32(1.0) - ph) - pl) - f32(x[1] * r0))
    return fast_two_sum(r0, f32(r0 * e))


def dw_split(x):
    """des_dw.cuh dw_split on the bits of an FP64 value."""
    b = np.array([x], dtype=np.float64).view(np.uint64)[0]
    hw, lw = int(b >> np.uint64(32)), int(b & np.uint64(0xFFFFFFFF))
    mag, sg = hw & 0x7FFFFFFF, hw & 0x80000000
    hb = (((mag - (896 << 20)) << 3) & 0xFFFFFFFF) | (lw >> 29)
    L = lw & 0x1FFFFFFF
    fh = f32(np.array([0x4B000000 | (L >> 23)], dtype=np.uint32).view(np.float32)[0] - f32(8388608.0))
    fl = f32(np.array([0x4B000000 | (L & 0x7FFFFF)], dtype=np.uint32).view(np.float32)[0] - f32(8388608.0))
    fr = fmaf(fh, f32(8388608.0), fl)
    ef = (mag >> 20) - 948
    if mag < (897 << 20):
        hb, lo = 0, f32(0.0)
    elif ef >= 1:
        lo = f32(fr * np.array([ef << 23], dtype=np.uint32).view(np.float32)[0])
    else:
        lo = f32(f32(fr * np.array([(ef + 64) << 23], dtype=np.uint32).view(np.float32)[0]) * f32(2.0 ** -64))
    hi = np.array([sg | hb], dtype=np.uint32).view(np.float32)[0]
    lo = np.array([np.array([lo], dtype=np.float32).view(np.uint32)[0] ^ sg], dtype=np.uint32).view(np.float32)[0]
    return fast_two_sum(f32(hi), f32(lo))


def val(x):
    return F(float(x[0])) + F(float(x[1]))


def rel(got, exact, scale):
    return abs(val(got) - exact) / scale


def _dws(rng, n, spread=4):
    """n double-word values (hi, lo) of random sign and magnitude 10^[-spread, spread]."""
    out = []
    for _ in range(n):
        x = float(rng.standard_normal() * 10.0 ** rng.uniform(-spread, spread))
        out.append(dw_split(x))
    return out


def test_dw_split_bounds_and_special_values():
    rng = np.random.default_rng(1)
    xs = list(rng.standard_normal(3000) * 10.0 ** rng.uniform(-30, 30, 3000))
    xs += [1.0, -1.0, 2.0 ** -126, 3.4e38 * 0.99, 1e-300, 0.0, -0.0, np.nextafter(1.0, 2.0), 1.0 - 2.0 ** -53,
           2.0 ** -97, -(2.0 ** -98) * 3]
    for x in xs:
        hi, lo = dw_split(x)
        if abs(x) < 2.0 ** -126:
            assert hi == 0 and lo == 0
            continue
        err = abs(F(x) - val((hi, lo)))
        # lo is a normal float for |x| >= 2^-97, subnormal below
        assert err <= F(2) ** -47 * abs(F(x)) + (F(2) ** -149 if abs(x) < 2.0 ** -97 else 0), x
        assert abs(float(lo)) <= float(np.spacing(np.float32(abs(hi)))) / 2, x
        assert np.sign(hi) == np.sign(x)   # lo may take either sign once normalised


def test_error_free_transformations():
    rng = np.random.default_rng(2)
    a = (rng.standard_normal(4000) * 10.0 ** rng.uniform(-8, 8, 4000)).astype(np.float32)
    b = (rng.standard_normal(4000) * 10.0 ** rng.uniform(-8, 8, 4000)).astype(np.float32)
    for x, y in zip(a, b):
        s, e = two_sum(x, y)
        assert F(float(s)) + F(float(e)) == F(float(x)) + F(float(y))
        p, q = two_prod(x, y)
        assert F(float(p)) + F(float(q)) == F(float(x)) * F(float(y))


def test_dw_add_mul_recip_bounds():
    rng = np.random.default_rng(3)
    xs, ys = _dws(rng, 2000), _dws(rng, 2000)
    worst = {"add": 0.0, "mul": 0.0, "recip": 0.0}
    for i, (x, y) in enumerate(zip(xs, ys)):
        if i % 4 == 0:   # heavy cancellation: y ~ -x
            y = dw_add(dw_neg(x), dw_split(float(rng.standard_normal()) * 1e-6 * float(x[0])))
        ex = val(x) + val(y)
        if ex != 0:
            worst["add"] = max(worst["add"], float(rel(dw_add(x, y), ex, abs(ex))))
        ex = val(x) * val(y)
        if ex != 0:
            worst["mul"] = max(worst["mul"], float(rel(dw_mul(x, y), ex, abs(ex))))
        if val(x) != 0:
            ex = 1 / val(x)
            worst["recip"] = max(worst["recip"], float(rel(dw_recip(x), ex, abs(ex))))
    print({k: f"{v / U**2:.2f} u^2" for k, v in worst.items()})
    assert worst["add"] <= 3 * U ** 2 + 13 * U ** 3
    assert worst["mul"] <= 4 * U ** 2
    assert worst["recip"] <= 8 * U ** 2


def test_compensated_dot_diff_sum_bounds():
    rng = np.random.default_rng(4)
    worst = {"dot3": 0.0, "diff2": 0.0, "sum3": 0.0}
    for i in range(1500):
        a, b = _dws(rng, 3), _dws(rng, 3)
        if i % 3 == 0:   # a cancelling dot product
            p01 = val(a[0]) * val(b[0]) + val(a[1]) * val(b[1])
            a[2] = dw_split(float(-p01 / val(b[2])) * (1 + 1e-7 * float(rng.standard_normal())))
        terms = [val(a[k]) * val(b[k]) for k in range(3)]
        got = dw_dot3c(a[0], b[0], a[1], b[1], a[2], b[2])
        worst["dot3"] = max(worst["dot3"], float(rel(got, sum(terms), sum(abs(t) for t in terms))))
        got = dw_diff2(a[0], b[0], a[1], b[1])
        ex = terms[0] - terms[1]
        worst["diff2"] = max(worst["diff2"], float(rel(got, ex, abs(terms[0]) + abs(terms[1]))))
        x, y, z = _dws(rng, 3)
        if i % 3 == 0:
            z = dw_neg(dw_add(x, y))
        got = dw_sum3(x, y, z)
        worst["sum3"] = max(worst["sum3"], float(rel(got, val(x) + val(y) + val(z), abs(val(x)) + abs(val(y)) + abs(val(z)))))
    print({k: f"{v / U**2:.2f} u^2" for k, v in worst.items()})
    assert worst["dot3"] <= 16 * U ** 2
    assert worst["diff2"] <= 8 * U ** 2
    assert worst["sum3"] <= 6 * U ** 2


def test_element_force_terms_within_2_pow_minus_43():
    """T_i = (sigma . dN_i + b z) vol of one element as k_nmd_correct_ft3 forms
    them (sigma vol first, compensated dot products, T_0 = -(T_1 + T_2 + T_3),
    the buoyancy term added), against exact arithmetic on the FP64 inputs:
    lithostatic stresses ~1e8 Pa with small deviators, so the terms cancel."""
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(300):
        P = 10.0 ** rng.uniform(6, 9)
        sig = [-P + 1e-3 * P * rng.standard_normal() for _ in range(3)] + list(1e-3 * P * rng.standard_normal(3))
        shp = rng.standard_normal((3, 4)) * 10.0 ** rng.uniform(-5, -2)
        shp[:, 0] = -shp[:, 1:].sum(axis=1)
        vol = 10.0 ** rng.uniform(6, 11)
        b = 3300.0 * 10.0 / 4
        v = dw_split(vol)
        sv = [dw_mul(dw_split(x), v) for x in sig]
        rows = ((0, 3, 4), (3, 1, 5), (4, 5, 2))
        T = [[None] * 3 for _ in range(4)]
        for i in range(1, 4):
            sx, sy, sz = (dw_split(float(shp[k, i])) for k in range(3))
            for k, (p, q, r) in enumerate(rows):
                T[i][k] = dw_dot3c(sv[p], sx, sv[q], sy, sv[r], sz)
        for k in range(3):
            T[0][k] = dw_neg(dw_sum3(T[1][k], T[2][k], T[3][k]))
        bv = dw_mul(dw_split(b), v)
        for i in range(4):
            T[i][2] = dw_add(T[i][2], bv)
        for i in range(4):
            for k, (p, q, r) in enumerate(rows):
                # the exact term with dN_0 = -(dN_1 + dN_2 + dN_3) exactly
                sh = [F(float(shp[kk, i])) if i else -sum(F(float(shp[kk, j])) for j in (1, 2, 3)) for kk in range(3)]
                prods = [F(sig[p]) * sh[0], F(sig[q]) * sh[1], F(sig[r]) * sh[2]]
                ex = (sum(prods) + (F(b) if k == 2 else 0)) * F(vol)
                scale = (sum(abs(x) for x in prods) + (F(b) if k == 2 else 0)) * F(vol)
                if i == 0:   # node 0's scale: the other three nodes' terms
                    scale *= 4
                worst = max(worst, float(abs(val(T[i][k]) - ex) / scale))
    print(f"force terms: {worst:.2e} = 2^{np.log2(worst):.1f} of the terms' magnitudes")
    assert worst <= 2.0 ** -43
