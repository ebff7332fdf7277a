"""The FP32 screen of the EVP branch choice (j2_est3, j2_est_dev3, j2_less in
csrc/des_rheology.cuh), restated in numpy and checked against the FP64
comparison it stands for.

The device computes FP32 sums, products, quotients and square roots with
IEEE round-to-nearest, as numpy's float32 does; f32_of rounds to nearest
and flushes magnitudes below 2^-126 to zero; the kernels that use the
screen are compiled without FMA contraction.  The FP64 side is
second_invariant2_ (utils.hpp:110-128) in its expression order, the mean
divided by 3 with IEEE division (div3 equals it bit for bit).  Wherever
the screen decides, its answer must equal the FP64 comparison: on
near-lithostatic pairs (deviators down to 1e-17 of the pressure), ties and
near ties of every relative size, identical deviators under different
pressures, signed zeros, values near the FP32 range limits, infinities and
NaNs.
"""
import numpy as np

F = np.float32


def f32_of(x):
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(over="ignore"):
        y = x.astype(np.float32)
    return np.where(np.abs(x) < 2.0 ** -126, np.float32(0) * np.sign(x).astype(np.float32), y)


def second_invariant2(t):
    """(n, 6) FP64 -> FP64, the kernels' order of operations."""
    with np.errstate(all="ignore"):
        a = (t[:, 0] + t[:, 1] + t[:, 2]) / 3
        return (0.5 * ((t[:, 0] - a) * (t[:, 0] - a) + (t[:, 1] - a) * (t[:, 1] - a) + (t[:, 2] - a) * (t[:, 2] - a))
                + t[:, 3] * t[:, 3] + t[:, 4] * t[:, 4] + t[:, 5] * t[:, 5])


def screened_form(q, s):
    """The mixed kernel's FP64 J2 of a trial stress from its deviator q."""
    with np.errstate(all="ignore"):
        return (0.5 * (q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1] + q[:, 2] * q[:, 2])
                + s[:, 3] * s[:, 3] + s[:, 4] * s[:, 4] + s[:, 5] * s[:, 5])


def j2_est3(s):
    with np.errstate(all="ignore"):
        d01, d02, d12 = f32_of(s[:, 0] - s[:, 1]), f32_of(s[:, 0] - s[:, 2]), f32_of(s[:, 1] - s[:, 2])
        t3, t4, t5 = f32_of(s[:, 3]), f32_of(s[:, 4]), f32_of(s[:, 5])
        sixth = F(1) / F(6)
        j = (d01 * d01 + d02 * d02 + d12 * d12) * sixth + (t3 * t3 + t4 * t4 + t5 * t5)
        S = np.fmax(np.fmax(np.abs(f32_of(s[:, 0])), np.abs(f32_of(s[:, 1]))), np.abs(f32_of(s[:, 2])))
        h = F(2.0 ** -50) * S
        tol = F(2.0 ** -19) * j + F(2.0 ** -48) * S * np.sqrt(j) + h * h + F(2.0 ** -100)
    return j, tol


def j2_est_dev3(q, s):
    with np.errstate(all="ignore"):
        q0, q1, q2 = f32_of(q[:, 0]), f32_of(q[:, 1]), f32_of(q[:, 2])
        t3, t4, t5 = f32_of(s[:, 3]), f32_of(s[:, 4]), f32_of(s[:, 5])
        j = F(0.5) * (q0 * q0 + q1 * q1 + q2 * q2) + (t3 * t3 + t4 * t4 + t5 * t5)
        tol = F(2.0 ** -19) * j + F(2.0 ** -100)
    return j, tol


def j2_less(a, b):
    with np.errstate(all="ignore"):
        gap = b[0] - a[0]
        tol = a[1] + b[1]
        return np.where(gap > tol, 1, np.where(-gap > tol, 0, -1))


def _dev6(rng, n):
    d = rng.standard_normal((n, 6))
    d[:, :3] -= d[:, :3].mean(axis=1, keepdims=True)
    return d


def _pairs(seed, n=200_000):
    """Candidate pairs (a, b) of the kinds listed in the module docstring."""
    rng = np.random.default_rng(seed)
    P = 10 ** rng.uniform(-5, 12, n) * np.where(rng.random(n) < 0.8, -1, 1)
    d = _dev6(rng, n) * (np.abs(P) * 10 ** rng.uniform(-17, 0, n))[:, None]
    rel = np.where(rng.random(n) < 0.5, -1, 1) * 10 ** rng.uniform(-14, -2, n)
    rel[rng.random(n) < 0.1] = 0.0                      # equal deviators
    d2 = d * np.sqrt(1 + rel)[:, None]
    turn = _dev6(rng, n) * (np.sqrt((d * d).sum(axis=1)) * 10 ** rng.uniform(-16, -4, n))[:, None]
    d2 = d2 + np.where(rng.random(n) < 0.5, 0, 1)[:, None] * turn
    P2 = P * (1 + 10 ** rng.uniform(-12, -3, n) * rng.standard_normal(n))
    a = d.copy()
    a[:, :3] += P[:, None]
    b = d2.copy()
    b[:, :3] += P2[:, None]
    swap = rng.random(n) < 0.5
    a[swap], b[swap] = b[swap].copy(), a[swap].copy()
    return a, b


def _special(seed):
    rng = np.random.default_rng(seed)
    vals = np.array([0.0, -0.0, 1e-320, -1e-310, 1e-300, 2.0 ** -126, 2.0 ** -127, 1e-30, 1.0, 1e19, 1e20,
                     3.4e38, 3.5e38, 1e300, np.inf, -np.inf, np.nan])
    n = 20_000
    a = rng.choice(vals, (n, 6)) * np.where(rng.random((n, 6)) < 0.5, 1, rng.uniform(0.5, 2, (n, 6)))
    b = a.copy()
    mask = rng.random((n, 6)) < 0.3
    b[mask] = rng.choice(vals, mask.sum())
    return a, b


def _check(a, b):
    dec = j2_less(j2_est3(a), j2_est3(b))
    with np.errstate(invalid="ignore"):
        exact = (second_invariant2(a) < second_invariant2(b)).astype(int)
    wrong = (dec >= 0) & (dec != exact)
    assert not wrong.any(), (a[wrong][:3], b[wrong][:3])
    return dec


def test_screen_agrees_with_fp64_wherever_it_decides():
    for seed in range(3):
        a, b = _pairs(seed)
        dec = _check(a, b)
        assert (dec >= 0).mean() > 0.1 and (dec < 0).mean() > 0.05


def test_screen_on_special_values():
    a, b = _special(4)
    _check(a, b)
    nan = np.isnan(a).any(axis=1) | np.isnan(b).any(axis=1) | np.isinf(a).any(axis=1) | np.isinf(b).any(axis=1)
    assert (j2_less(j2_est3(a), j2_est3(b))[nan] == -1).all()


def test_screen_decides_clear_cases():
    """Pairs 1e-5 apart in J2 at moderate magnitudes are decided."""
    rng = np.random.default_rng(9)
    n = 50_000
    d = _dev6(rng, n) * 1e6
    P = -(10 ** rng.uniform(6, 9, n))
    a = d.copy()
    a[:, :3] += P[:, None]
    b = d * np.sqrt(1 + 1e-5)
    b[:, :3] += P[:, None] * 1.001
    dec = _check(a, b)
    assert (dec == 1).all()


def test_trial_deviator_form_agrees_with_fp64():
    """j2_est_dev3 against the mixed kernel's FP64 expression on the same q."""
    for seed in range(2):
        a, b = _pairs(10 + seed)
        with np.errstate(all="ignore"):
            am = (b[:, 0] + b[:, 1] + b[:, 2]) / 3
            q = b[:, :3] - am[:, None]
        dec = j2_less(j2_est3(a), j2_est_dev3(q, b))
        with np.errstate(invalid="ignore"):
            exact = (second_invariant2(a) < screened_form(q, b)).astype(int)
        assert np.array_equal(screened_form(q, b), second_invariant2(b))
        wrong = (dec >= 0) & (dec != exact)
        assert not wrong.any()
        assert (dec >= 0).mean() > 0.1


def test_pairs_reach_the_pressure_term():
    """Without its 2^-48 S sqrt(j) term (the FP64 mean's rounding under a
    large pressure) the bound decides some of these pairs wrongly: the
    generator reaches the regime that term is there for."""
    def no_pressure_term(s):
        j, _ = j2_est3(s)
        return j, F(2.0 ** -19) * j + F(2.0 ** -100)
    a, b = _pairs(1)
    dec = j2_less(no_pressure_term(a), no_pressure_term(b))
    with np.errstate(invalid="ignore"):
        exact = (second_invariant2(a) < second_invariant2(b)).astype(int)
    assert ((dec >= 0) & (dec != exact)).sum() > 100


# ---- the mixed EVP branch's trial deviator --------------------------------
# k_update_stress_mixed3 runs both screens on qt = x + y, x_i = s_i - s0 (the
# old normal deviator, s0 = div3 of the old trace) and y_i = 2G (de_i -
# div3(tr de)), instead of the deviator of the FP64 trial stress that
# elastic_mixed forms (s_i + fma(2G, de_i, lambda tr de)), whose mean and
# deviator second_invariant2_ then takes.  Its comment bounds the distance
# by 22 u S, S = |s0| + sum |x_i| + sum |y_i| + (2G + 2K) sum |de_i|.

def _fma_vec(a, b, c):
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.fma.restype = ctypes.c_double
    libm.fma.argtypes = (ctypes.c_double,) * 3
    return np.array([libm.fma(float(p), float(q), float(r)) for p, q, r in zip(a, b, c)])


def test_trial_deviator_from_shared_terms_is_within_22uS():
    rng = np.random.default_rng(21)
    n = 20_000
    u = 2.0 ** -53
    K = 10 ** rng.uniform(9, 11.5, n)
    G = K * rng.uniform(0.1, 1.5, n)   # Poisson's ratio from about 0.43 down to below zero
    P = np.where(rng.random(n) < 0.9, -1, 1) * 10 ** rng.uniform(0, 10, n)
    dev = rng.standard_normal((n, 3))
    dev -= dev.mean(axis=1, keepdims=True)
    s_old = P[:, None] + dev * (np.abs(P) * 10 ** rng.uniform(-12, 0, n))[:, None]
    # increments whose deviatoric part nearly cancels the old deviator (y ~ -x)
    # in a third of the cases, with a volumetric part up to the pressure's size
    c = np.where(rng.random(n) < 0.33, 1 + 10 ** rng.uniform(-12, -1, n), rng.uniform(-3, 3, n))
    de = -c[:, None] * (s_old - s_old.mean(axis=1, keepdims=True)) / (2 * G[:, None])
    de += (10 ** rng.uniform(-12, -2, n) * np.abs(P) / K * rng.standard_normal(n))[:, None]
    de *= 1 + 1e-3 * rng.standard_normal((n, 3))
    # the kernel's terms
    trde = (de[:, 0] + de[:, 1]) + de[:, 2]
    s0 = ((s_old[:, 0] + s_old[:, 1]) + s_old[:, 2]) / 3
    dv3 = trde / 3
    g2 = 2 * G
    x = s_old - s0[:, None]
    y = g2[:, None] * (de - dv3[:, None])
    qt = x + y
    S = np.abs(s0) + np.abs(x).sum(axis=1) + np.abs(y).sum(axis=1) + (2 * g2 + 2 * K) * np.abs(de).sum(axis=1)
    # the FP64 trial stress and the deviator second_invariant2_ forms from it
    lam = K - 2. / 3 * G
    ldev = lam * trde
    sp = np.stack([s_old[:, i] + _fma_vec(g2, de[:, i], ldev) for i in range(3)], axis=1)
    am = ((sp[:, 0] + sp[:, 1]) + sp[:, 2]) / 3
    q = sp - am[:, None]
    dist = np.abs(qt - q).max(axis=1)
    assert (dist <= 22 * u * S).all(), (dist / (u * S)).max()
    # and the bound is not loose by more than a few orders of magnitude
    assert (dist / (u * S)).max() > 0.05
