"""The FP32 screens of update_stress, on elements built at their edges.

Two decisions of the 3D stress update are screened in FP32 and left to the
FP64 evaluation only where the FP32 estimate is too close to call:

* the Mohr-Coulomb yield test (rheology.cxx:163-178): clearly_elastic3
  passes an element as elastic only when both yield functions clear the
  surface by a bound on every FP32 and FP64 rounding;
* the EVP branch choice (rheology.cxx:594-634): j2_less compares the second
  invariants of the Maxwell and the elasto-plastic candidates from FP32
  estimates with bounds.

Here the elements sit at those edges: principal stresses within 1e-9 to
1e-3 (relative) of the yield surface, and Maxwell / elasto-plastic pairs
whose second invariants are ties to within 1e-12 to 1e-4.  The viscosity
is clamped (visc_min = visc_max) and the plastic properties come from
their tables, so no transcendental function enters: the FP64 device path
must match the oracle bit for bit wherever the yield decision is not
itself decided by an eigen-solve's last bits.
"""
from dataclasses import replace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from dynearthsol_gb300 import capi
    capi.load_library()


def _rotations(rng, n):
    q, r = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    return q * np.sign(np.diagonal(r, axis1=1, axis2=2))[:, None, :]


def _voigt(t):
    """3x3 symmetric tensors -> (XX, YY, ZZ, XY, XZ, YZ)."""
    return np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 2, 2], t[:, 0, 1], t[:, 0, 2], t[:, 1, 2]], axis=1)


def _dev(v):
    d = v.copy()
    d[:, :3] -= v[:, :3].mean(axis=1, keepdims=True)
    return d


def _j2_dev(d):
    return 0.5 * (d[:, :3] ** 2).sum(axis=1) + (d[:, 3:] ** 2).sum(axis=1)


def _base(rheol, **mat):
    """The 3D workload's mesh family at 8 x 8 x 4 cubes (1,536 tets), its
    initial fields from the oracle, plastic strain zero everywhere."""
    from dynearthsol_gb300.config import initial_state, make_workload
    from oracle.oracle import Oracle
    wl = make_workload("c1_3d_evp", cells=(8, 8, 4))
    wl.mat = replace(wl.mat, rheol_type=rheol, **mat)
    st, cp = initial_state(wl)
    o = Oracle(wl, st, cp)
    assert o.init_fields() == 0
    st["plstrain"][:] = 0
    return wl, st, cp


def _run_both(wl, st, cp, dt, precision=None):
    """update_stress once on the device and once in the oracle, from the
    same state; returns (device, oracle) states."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.solver import DeviceModel
    from oracle.oracle import Oracle, state_copy
    m = DeviceModel(wl, comp_pressure=cp, precision=capi.PREC_FP64 if precision is None else precision)
    m.upload(state_copy(st), (0.0, dt, 0))
    m.call("update_stress")
    out = m.download()
    ref = state_copy(st)
    o = Oracle(wl, ref, cp, 1, (0.0, dt, 0))
    assert o.call("update_stress") == 0
    return out, ref


def _evp_case(seed, dt):
    """EVP elements whose Maxwell and elasto-plastic candidates have nearly
    equal second invariants.  With s_dev = a and 2G dev(de) = b, the trial
    deviator is a + b and the Maxwell one f2 (f1 a + b); b = -c a + noise
    with c in [0, 3] puts ties near c = 1 and c = 2.  Cohesion is large, so
    every trial stress is elastic (the yield screen passes it)."""
    from dynearthsol_gb300 import capi
    wl, st, cp = _base(capi.RH_EVP, visc_min=1e24, visc_max=1e24, cohesion0=(1e12,), cohesion1=(1e12,),
                       tension_max=1e12)
    rng = np.random.default_rng(seed)
    ne = wl.mesh.nelem
    G = wl.mat.shear_modulus[0]
    P = 10 ** rng.uniform(6, 9, ne)
    a = _dev(rng.standard_normal((ne, 6)))
    a *= (10 ** rng.uniform(2, 7, ne) / np.sqrt(_j2_dev(a)))[:, None]
    c = rng.uniform(0, 3, ne)
    noise = _dev(rng.standard_normal((ne, 6))) * np.sqrt(_j2_dev(a))[:, None] * 10 ** rng.uniform(-6, -2, ne)[:, None]
    b = -c[:, None] * a + noise
    stress = a.copy()
    stress[:, :3] -= P[:, None]
    edot = b / (2 * G * dt)
    edot[:, :3] += (1e-15 * rng.standard_normal(ne))[:, None]
    edot[::97] = 0                       # no increment: sv and sp differ by the relaxation alone
    stress[::89, 3:] = 0                 # hydrostatic elements: both invariants vanish or nearly
    stress[::89, :3] = -P[::89, None]
    st["stress"][:] = stress
    st["strain_rate"][:] = edot
    st["edvoldt"][:] = edot[:, 0] + edot[:, 1] + edot[:, 2]
    st["volume_old"][:] = st["volume"] * (1 + 1e-9 * rng.standard_normal(ne))
    return wl, st, cp


@pytest.mark.parametrize("dt", [2e7, 2e8, 2e9])
def test_evp_choice_screen_bit_exact(dt):
    """FP64 device update_stress equals the oracle's bit for bit on EVP
    elements at and around ties of the two candidates' second invariants
    (tmp = dt G / (2 visc) = 2e-7, 2e-6, 2e-5: the larger tmp, the larger
    the share of elements that the FP32 estimates decide)."""
    wl, st, cp = _evp_case(7, dt)
    out, ref = _run_both(wl, st, cp, dt)
    for k in ("stress", "strain", "plstrain", "delta_plstrain", "dpressure"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    # both branches were taken: the elasto-plastic candidate moves the sum
    # of the normal stresses by 3 K tr(de), the Maxwell one by 3 K dv
    K = wl.mat.bulk_modulus[0]
    moved = out["stress"][:, :3].sum(axis=1) - st["stress"][:, :3].sum(axis=1)
    elastic_move = 3 * K * (st["strain_rate"][:, :3].sum(axis=1) * dt)
    took_maxwell = ~np.isclose(moved, elastic_move, rtol=1e-6, atol=0)
    assert 0 < took_maxwell.sum() < len(took_maxwell)


def test_evp_choice_mixed_follows_fp64_where_decided():
    """The mixed path's choice (the FP32 identity screen, or the FP64
    comparison of its FP64 candidates) equals the FP64 path's on every
    element whose two candidates differ by more than 1e-7 (relative) in J2.
    Its stress is then within the FP32 rounding of the step's increment of
    the FP64 stress (2^-20 of the increment, relative to the element's
    largest component, where the Maxwell update is taken as the old stress
    plus an FP32 increment), while a different choice would move the
    pressure by K (dv - tr de), ~1e-5 of it."""
    from dynearthsol_gb300 import capi
    dt = 2e8
    wl, st, cp = _evp_case(11, dt)
    f64, _ = _run_both(wl, st, cp, dt)
    mix, _ = _run_both(wl, st, cp, dt, precision=capi.PREC_MIXED)
    G = wl.mat.shear_modulus[0]
    visc = wl.mat.visc_max
    tmp = 0.5 * dt * G / visc
    a = _dev(st["stress"])
    b = 2 * G * _dev(st["strain_rate"] * dt)
    jp = _j2_dev(a + b)
    jv = _j2_dev((1 / (1 + tmp)) * ((1 - tmp) * a + b))
    clear = np.abs(jv - jp) > 1e-7 * (jv + jp)
    assert clear.sum() > 500 and (~clear).sum() > 20, (clear.sum(), (~clear).sum())
    scale = np.abs(f64["stress"]).max(axis=1)
    err = np.abs(mix["stress"] - f64["stress"]).max(axis=1) / scale
    # the FP32 increment's terms: f2 y (y from FP32 strain increments, within
    # 2^-22 (|y| + Y) of the FP64 y, Y = 2G sum |de_i|), the relaxation
    # -2 tmp f2 x and the volumetric K dv
    Kb = wl.mat.bulk_modulus[0]
    de = st["strain_rate"] * dt
    Y = 2 * G * np.abs(de[:, :3]).sum(axis=1)
    dv = st["volume"] / st["volume_old"] - 1
    inc = np.abs(b).max(axis=1) + Y + 2 * tmp * np.abs(a).max(axis=1) + Kb * np.abs(dv)
    bound = 1e-10 + 2.0 ** -20 * inc / scale
    r = np.where(clear, err / bound, 0.0)
    w = int(np.argmax(r))
    print(f"worst element {w}: err {err[w]:.3e} bound {bound[w]:.3e} |a| {np.abs(a[w]).max():.3e} "
          f"|b| {np.abs(b[w]).max():.3e} Y {Y[w]:.3e} tmp {tmp:.3e} K|dv| {Kb * abs(dv[w]):.3e} scale {scale[w]:.3e}")
    assert (err[clear] <= bound[clear]).all(), r.max()


def _ep_case(seed):
    """Mohr-Coulomb elements with principal stresses p0 <= p1 <= p2 at
    fs = p0 - anphi p2 + amc = delta (|p2| (1 + anphi) + amc), delta of
    either sign and magnitude 1e-9 .. 1e-3, randomly rotated; no strain
    increment, so the trial stress is the stress itself."""
    from dynearthsol_gb300 import capi
    wl, st, cp = _base(capi.RH_EP)
    rng = np.random.default_rng(seed)
    ne = wl.mesh.nelem
    phi = np.radians(wl.mat.friction_angle0[0])
    anphi = (1 + np.sin(phi)) / (1 - np.sin(phi))
    amc = 2 * wl.mat.cohesion0[0] * np.sqrt(anphi)
    p2 = -(10 ** rng.uniform(6.5, 9, ne))
    delta = np.where(rng.random(ne) < 0.5, -1, 1) * 10 ** rng.uniform(-9, -3, ne)
    p0 = anphi * p2 - amc + delta * (np.abs(p2) * (1 + anphi) + amc)
    p1 = p0 + rng.random(ne) * (p2 - p0)
    R = _rotations(rng, ne)
    t = np.einsum("nij,nj,nkj->nik", R, np.stack([p0, p1, p2], axis=1), R)
    st["stress"][:] = _voigt(t)
    st["strain_rate"][:] = 0
    st["edvoldt"][:] = 0
    return wl, st, cp, delta


def test_yield_screen_at_the_surface():
    """FP64 device update_stress on Mohr-Coulomb elements within 1e-9 to
    1e-3 of the yield surface: the same elements yield as in the oracle;
    elastic ones keep their stress bit for bit; yielded ones match to
    1e-12 (the eigen-solve's transcendental functions differ by ulps)."""
    wl, st, cp, delta = _ep_case(5)
    out, ref = _run_both(wl, st, cp, 1e6)
    yo, yr = out["plstrain"] > 0, ref["plstrain"] > 0
    np.testing.assert_array_equal(yo, yr)
    assert yr.sum() > 100 and (~yr).sum() > 100
    np.testing.assert_array_equal(out["stress"][~yr], ref["stress"][~yr])
    np.testing.assert_array_equal(out["stress"][~yr], st["stress"][~yr])
    scale = np.abs(ref["stress"]).max()
    assert np.abs(out["stress"] - ref["stress"]).max() <= 1e-12 * scale
    # elements closer than ~2^-19 of the surface are left to the FP64 test;
    # the sample reaches well inside that band on both sides
    assert np.sum(np.abs(delta) < 1e-7) > 100
