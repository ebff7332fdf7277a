"""The FP32 yield screen (clearly_elastic3_f / clearly_elastic3_dev in
csrc/des_rheology.cuh), restated in numpy and checked against the FP64
Mohr-Coulomb yield test it stands for (rheology.cxx:163-178: fs = p0 -
p2 anphi + amc > 0 and ft = p2 - ten_max < 0 on the principal stresses).

The restatement follows the kernel's operations: FP32 conversions that
round to nearest and flush magnitudes below 2^-126; twelve Rutishauser
rotations of a cyclic Jacobi (four sweeps); the principal stresses and
yield functions formed in FP32.  The kernel's approximate FP32 intrinsics
(the rotation's quotients and reciprocal square root) are restated with
IEEE operations: their few-ulp differences perturb the rotations by ~1e-7
of the deviator, against the screen's 2^-12 of it.  The FP64 side is
LAPACK's symmetric eigen-solve of the FP64 stress, whose eigenvalues carry
errors of a few eps64 of the stress, as the reference's dsyevh3 does.

Wherever the screen passes an element, the FP64 test must find it elastic:
on principal stresses 1e-10 to 1e-2 (relative) either side of the shear
yield surface and of the tension cutoff, near-lithostatic stresses (a
deviator down to 1e-15 of the pressure), two or three equal principal
stresses, random rotations, and special values.
"""
import numpy as np

F = np.float32


def f32_of(x):
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        y = x.astype(np.float32)
    return np.where(np.abs(x) < 2.0 ** -126, np.float32(0) * np.sign(x).astype(np.float32), y)


def _fmaf(a, b, c):
    # the product of two floats is exact in FP64; one rounding to FP32 after
    # the sum (a second one to FP64 first, immaterial here)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def _jrot(a, v, P, Q):
    R = 3 - P - Q
    apq = a[:, P, Q].copy()
    act = apq != 0
    with np.errstate(all="ignore"):
        theta = (a[:, Q, Q] - a[:, P, P]) / (F(2) * apq)
        at = np.abs(theta)
        t = np.copysign(F(1) / (at + np.sqrt(_fmaf(at, at, np.ones_like(at)))), theta)
        c = F(1) / np.sqrt(_fmaf(t, t, np.ones_like(t)))
        s = t * c
        tau = s / (F(1) + c)
        t = np.where(act, t, F(0))
        s = np.where(act, s, F(0))
        tau = np.where(act, tau, F(0))
        app, aqq = a[:, P, P].copy(), a[:, Q, Q].copy()
        a[:, P, P] = np.where(act, app - t * apq, app)
        a[:, Q, Q] = np.where(act, aqq + t * apq, aqq)
        a[:, P, Q] = a[:, Q, P] = np.where(act, F(0), apq)
        arp, arq = a[:, R, P].copy(), a[:, R, Q].copy()
        nrp = arp - s * (arq + tau * arp)
        nrq = arq + s * (arp - tau * arq)
        a[:, R, P] = a[:, P, R] = np.where(act, nrp, arp)
        a[:, R, Q] = a[:, Q, R] = np.where(act, nrq, arq)
        for k in range(3):
            vkp, vkq = v[:, k, P].copy(), v[:, k, Q].copy()
            v[:, k, P] = np.where(act, vkp - s * (vkq + tau * vkp), vkp)
            v[:, k, Q] = np.where(act, vkq + s * (vkp - tau * vkq), vkq)


def jacobi3f(d):
    """d: (n, 6) float32 (XX, YY, ZZ, XY, XZ, YZ) -> (n, 3) eigenvalues ascending."""
    n = d.shape[0]
    a = np.empty((n, 3, 3), dtype=np.float32)
    a[:, 0, 0], a[:, 1, 1], a[:, 2, 2] = d[:, 0], d[:, 1], d[:, 2]
    a[:, 0, 1] = a[:, 1, 0] = d[:, 3]
    a[:, 0, 2] = a[:, 2, 0] = d[:, 4]
    a[:, 1, 2] = a[:, 2, 1] = d[:, 5]
    v = np.broadcast_to(np.eye(3, dtype=np.float32), (n, 3, 3)).copy()
    for _ in range(4):
        _jrot(a, v, 0, 1)
        _jrot(a, v, 0, 2)
        _jrot(a, v, 1, 2)
    w = np.stack([a[:, 0, 0], a[:, 1, 1], a[:, 2, 2]], axis=1)
    return np.sort(w, axis=1)


def clearly_elastic3(amc, anphi, ten_max, s):
    """The FP64 path's screen on (n, 6) FP64 stresses (clearly_elastic3)."""
    with np.errstate(all="ignore"):
        m = (s[:, 0] + s[:, 1] + s[:, 2]) * (1.0 / 3)
        d = np.empty((s.shape[0], 6), dtype=np.float32)
        for i in range(3):
            d[:, i] = f32_of(s[:, i] - m)
        for i in range(3, 6):
            d[:, i] = f32_of(s[:, i])
        w = jacobi3f(d)
        nf = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
                     + F(2) * (d[:, 3] * d[:, 3] + d[:, 4] * d[:, 4] + d[:, 5] * d[:, 5]))
        mf = f32_of(m)
        af, cf, tf = f32_of(anphi), f32_of(amc), f32_of(ten_max)
        tol = F(2.0 ** -12) * nf + F(2.0 ** -19) * (np.abs(mf) + nf) + F(2.0 ** -100)
        p0, p2 = mf + w[:, 0], mf + w[:, 2]
        fs = p0 - p2 * af + cf
        ft = p2 - tf
        return (fs > (F(1) + af) * tol + F(2.0 ** -19) * np.abs(cf)) & (ft < -(tol + F(2.0 ** -19) * np.abs(tf)))


def fp64_elastic(amc, anphi, ten_max, s):
    A = np.empty((s.shape[0], 3, 3))
    A[:, 0, 0], A[:, 1, 1], A[:, 2, 2] = s[:, 0], s[:, 1], s[:, 2]
    A[:, 0, 1] = A[:, 1, 0] = s[:, 3]
    A[:, 0, 2] = A[:, 2, 0] = s[:, 4]
    A[:, 1, 2] = A[:, 2, 1] = s[:, 5]
    p = np.linalg.eigvalsh(A)
    return (p[:, 0] - p[:, 2] * anphi + amc > 0) & (p[:, 2] - ten_max < 0)


def _rotations(rng, n):
    q, r = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    return q * np.sign(np.diagonal(r, axis1=1, axis2=2))[:, None, :]


def _voigt(R, p):
    t = np.einsum("nij,nj,nkj->nik", R, p, R)
    return np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 2, 2], t[:, 0, 1], t[:, 0, 2], t[:, 1, 2]], axis=1)


def _material(phi=30.0, cohesion=44e6, tension_max=1e9):
    sp = np.sin(np.radians(phi))
    anphi = (1 + sp) / (1 - sp)
    amc = 2 * cohesion * np.sqrt(anphi)
    ten = min(tension_max, cohesion / np.tan(np.radians(phi)))
    return amc, anphi, ten


def _near_shear_surface(rng, n, amc, anphi):
    p2 = -(10 ** rng.uniform(5, 10, n))
    delta = np.where(rng.random(n) < 0.5, -1, 1) * 10 ** rng.uniform(-10, -2, n)
    p0 = anphi * p2 - amc + delta * (np.abs(p2) * (1 + anphi) + amc)
    kind = rng.integers(0, 3, n)   # 0: p1 between, 1: p1 = p0, 2: p1 = p2
    p1 = np.where(kind == 0, p0 + rng.random(n) * (p2 - p0), np.where(kind == 1, p0, p2))
    return _voigt(_rotations(rng, n), np.stack([p0, p1, p2], axis=1))


def _near_tension_cutoff(rng, n, ten):
    p2 = ten * (1 + np.where(rng.random(n) < 0.5, -1, 1) * 10 ** rng.uniform(-10, -2, n))
    p0 = p2 - 10 ** rng.uniform(-3, 0, n) * ten
    p1 = p0 + rng.random(n) * (p2 - p0)
    return _voigt(_rotations(rng, n), np.stack([p0, p1, p2], axis=1))


def _near_lithostatic(rng, n):
    P = -(10 ** rng.uniform(6, 10, n))
    dev = rng.standard_normal((n, 3))
    dev -= dev.mean(axis=1, keepdims=True)
    dev *= (np.abs(P) * 10 ** rng.uniform(-15, -2, n))[:, None]
    return _voigt(_rotations(rng, n), P[:, None] + dev)


def _check(s, mat):
    amc, anphi, ten = mat
    passed = clearly_elastic3(amc, anphi, ten, s)
    truth = fp64_elastic(amc, anphi, ten, s)
    wrong = passed & ~truth
    assert not wrong.any(), s[wrong][:3]
    return passed, truth


def test_screen_never_passes_a_yielding_element():
    rng = np.random.default_rng(1)
    for mat in (_material(), _material(phi=5.0, cohesion=4e6), _material(phi=45.0, cohesion=1e6, tension_max=1e5)):
        amc, anphi, ten = mat
        for gen in (lambda n: _near_shear_surface(rng, n, amc, anphi), lambda n: _near_tension_cutoff(rng, n, ten),
                    lambda n: _near_lithostatic(rng, n)):
            passed, truth = _check(gen(100_000), mat)
            assert passed.sum() > 0


def test_screen_passes_clearly_elastic_elements():
    """Principal stresses 3e-3 or more (relative) inside the surface pass.
    Closer ones fall back to the FP64 test: the margin's eigenvalue term,
    (1 + anphi) 2^-12 ||D||, is ~5e-4 of the yield function's scale here."""
    rng = np.random.default_rng(2)
    amc, anphi, ten = _material()
    n = 50_000
    p2 = -(10 ** rng.uniform(6, 9, n))
    delta = 10 ** rng.uniform(-2.5, -1, n)
    p0 = anphi * p2 - amc + delta * (np.abs(p2) * (1 + anphi) + amc)
    p1 = p0 + rng.random(n) * (p2 - p0)
    s = _voigt(_rotations(rng, n), np.stack([p0, p1, p2], axis=1))
    passed, truth = _check(s, (amc, anphi, ten))
    assert truth.all() and passed.all()


def test_screen_on_special_values():
    rng = np.random.default_rng(3)
    vals = np.array([0.0, -0.0, 1e-320, 1e-300, 2.0 ** -127, 1e-30, 1.0, -1e8, 1e20, 3.5e38, 1e300,
                     np.inf, -np.inf, np.nan])
    s = rng.choice(vals, (50_000, 6)) * np.where(rng.random((50_000, 6)) < 0.5, 1, -1)
    mat = _material()
    with np.errstate(all="ignore"):
        finite = np.isfinite(s).all(axis=1)
        passed = clearly_elastic3(*mat, s)
    assert not passed[~finite].any()
    _check(s[finite], mat)


def test_screen_bound_is_needed():
    """With the margin cut to 2^-30 of the stress the screen passes
    yielding elements of the near-surface set: the bound is doing work."""
    rng = np.random.default_rng(4)
    amc, anphi, ten = _material()
    s = _near_shear_surface(rng, 100_000, amc, anphi)
    with np.errstate(all="ignore"):
        m = (s[:, 0] + s[:, 1] + s[:, 2]) * (1.0 / 3)
        d = np.stack([f32_of(s[:, i] - m) for i in range(3)] + [f32_of(s[:, i]) for i in range(3, 6)], axis=1)
        w = jacobi3f(d)
        mf = f32_of(m)
        fs = (mf + w[:, 0]) - (mf + w[:, 2]) * f32_of(anphi) + f32_of(amc)
        weak = fs > F(2.0 ** -30) * np.abs(mf)
    truth = fp64_elastic(amc, anphi, ten, s)
    assert (weak & ~truth).sum() > 10
