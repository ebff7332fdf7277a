"""Parity of the CUDA path (through the C ABI) with the reference's golden
fixtures and with the oracle.

Tolerances are normalised maximum errors (max|a-b| / max|b| per field).
The FP64 device path evaluates every expression in the reference's order
without FMA contraction, so differences come only from the last-ulp
differences of the transcendental functions (pow, exp, sin, tan, atan2, cos)
between CUDA's libdevice and glibc, amplified by the explicit dynamics.
The stated bound of the FP64 path is 1e-9 on velocity, stress, temperature
and plastic strain after 1000 steps.  Where the reference's own algorithm is
more sensitive than that to its libm -- 3D Mohr-Coulomb yielding through the
near-degenerate eigen-solve, measured per case by the fixture's
``envelope`` (the restatement rerun with every transcendental moved by +-1
ulp) -- the bound is 20x that envelope.  One step and ten steps from a
mid-run reference state are held to 1e-12 and 1e-10.
"""
import numpy as np
import pytest

from cases import CASES, FUNCTIONS, PERFN_CASES, build_case
from conftest import load_golden, rel_err, state_from

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-9          # vel, stress, temperature, plstrain after the run
TOL_FIELD = 1e-9         # every other field after the run
ENV_MARGIN = 20.0        # multiple of the libm-sensitivity envelope
TOL_FN = 1e-12           # one application of one function
KEY_FIELDS = ("vel", "stress", "temperature", "plstrain")
SKIP = {"stressyy"}      # uninitialised by the reference outside plane strain


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from dynearthsol_gb300 import capi
    capi.load_library()


def _model(wl, comp):
    from dynearthsol_gb300.solver import DeviceModel
    return DeviceModel(wl, comp_pressure=comp)


def _cmp(st, ref, fields, tol, label):
    errs = {}
    for k in fields:
        if k in SKIP or k not in ref:
            continue
        errs[k] = rel_err(st[k], ref[k])
    bad = {k: v for k, v in errs.items() if v > tol}
    assert not bad, f"{label}: " + ", ".join(f"{k}={v:.2e}" for k, v in bad.items())
    return errs


@pytest.mark.parametrize("name", CASES)
def test_gpu_init_matches_reference(name):
    from dynearthsol_gb300.config import initial_state
    g = load_golden(name)
    wl, _ = build_case(name)
    st, comp = initial_state(wl)
    m = _model(wl, comp)
    out = m.init_fields(st)
    fields = [k for k in g["init"] if k in out and not (wl.mesh.ndims == 2 and k == "shpdy")]
    _cmp(out, g["init"], fields, 1e-13, "init")
    t, dt, steps = m.clock()
    assert abs(dt / g["init"]["clock"][1] - 1) < 1e-13


@pytest.mark.parametrize("name", CASES)
def test_gpu_step_matches_reference(name):
    g = load_golden(name)
    wl, nsteps = build_case(name)
    m = _model(wl, float(g["init"]["compensation_pressure"]))
    c = g["init"]["clock"]
    m.upload(state_from(g["init"]), (c[0], c[1], int(c[2])))
    m.step(nsteps)
    out = m.download()
    assert m.device_status() == 0
    env = {k: float(v) for k, v in g["envelope"].items()}
    env_max = max(env.values())
    for k in KEY_FIELDS:
        _cmp(out, g["final"], [k], max(TOL_STEP, ENV_MARGIN * env[k]), "final")
    others = [k for k in g["final"] if k in out and k not in KEY_FIELDS
              and not (wl.mesh.ndims == 2 and k == "shpdy")]
    for k in others:
        _cmp(out, g["final"], [k], max(TOL_FIELD, ENV_MARGIN * env.get(k, env_max)), "final")
    t, dt, steps = m.clock()
    assert steps == int(g["final"]["clock"][2])
    assert abs(dt / g["final"]["clock"][1] - 1) < max(1e-9, ENV_MARGIN * env_max)


@pytest.mark.parametrize("name", PERFN_CASES)
@pytest.mark.parametrize("k_steps,tol", [(1, 1e-12), (10, 1e-10)])
def test_gpu_steps_from_mid_state(name, k_steps, tol):
    """Short runs from a mid-run reference state (plasticity active): one
    step agrees to 1e-12; ten steps to 1e-10 or the ten-step envelope."""
    g = load_golden(name)
    wl, _ = build_case(name)
    m = _model(wl, float(g["init"]["compensation_pressure"]))
    c = g["mid"]["clock"]
    m.upload(state_from(g["mid"]), (c[0], c[1], int(c[2])))
    m.step(k_steps)
    out = m.download()
    ref = g[f"mid{k_steps}"]
    env = {k: float(v) for k, v in g[f"envelope_mid{k_steps}"].items()}
    env_max = max(env.values())
    fields = [k for k in ref if k in out and k != "clock" and not (wl.mesh.ndims == 2 and k == "shpdy")]
    for k in fields:
        _cmp(out, ref, [k], max(tol, ENV_MARGIN * env.get(k, env_max)), f"mid+{k_steps}")


@pytest.mark.parametrize("name", PERFN_CASES)
@pytest.mark.parametrize("fn", list(FUNCTIONS))
def test_gpu_functions_match_reference(name, fn):
    g = load_golden(name)
    if f"fn_{fn}" not in g:
        pytest.skip(f"{name} keeps no {fn} output (full-horizon fixture)")
    wl, _ = build_case(name)
    m = _model(wl, float(g["init"]["compensation_pressure"]))
    c = g["mid"]["clock"]
    m.upload(state_from(g["mid"]), (c[0], c[1], int(c[2])))
    m.call(fn)
    out = m.download()
    fields = [f for f in FUNCTIONS[fn] if not (wl.mesh.ndims == 2 and f == "shpdy")]
    _cmp(out, g[f"fn_{fn}"], fields, TOL_FN, fn)


@pytest.mark.parametrize("name", PERFN_CASES)
def test_gpu_dt_and_quality_match_reference(name):
    g = load_golden(name)
    wl, _ = build_case(name)
    m = _model(wl, float(g["init"]["compensation_pressure"]))
    c = g["mid"]["clock"]
    m.upload(state_from(g["mid"]), (c[0], c[1], int(c[2])))
    dt = m.call("compute_dt")
    assert abs(dt / float(g["fn_compute_dt"]["dt"]) - 1) < 1e-14
    q, w = m.call("worst_elem_quality")
    ref = g["fn_worst_elem_quality"]["result"]
    assert w == int(ref[1])
    assert abs(q - ref[0]) <= 1e-14 * abs(ref[0])


def _perfn_step(m, thermal, elastic):
    """One step as the reference's main loop sequences the functions
    (dynearthsol.cxx:325-361), through the per-function entry points."""
    t, dt, steps = m.clock()
    m.set_clock(t + dt, dt, steps + 1)
    if thermal:
        m.call("update_temperature")
    for f in ("update_strain_rate", "compute_dvoldt", "compute_edvoldt", "update_stress",
              "NMD_stress", "update_force", "update_velocity", "apply_vbcs", "update_mesh"):
        m.call(f)
    if elastic:
        m.call("rotate_stress")
    if (steps + 1) % 10 == 0:
        m.call("compute_dt")


@pytest.mark.parametrize("name", ["3d_heat_jitter_multimat", "2d_evp_heat", "3d_percell"])
def test_gpu_fused_step_equals_function_sequence(name):
    """The fused, graph-replayed step gives bit-identical results to the
    per-function entry points run in the reference's order."""
    g = load_golden(name)
    wl, _ = build_case(name)
    cp = float(g["init"]["compensation_pressure"])
    c = g["init"]["clock"]
    a, b = _model(wl, cp), _model(wl, cp)
    a.upload(state_from(g["init"]), (c[0], c[1], int(c[2])))
    b.upload(state_from(g["init"]), (c[0], c[1], int(c[2])))
    a.step(25)
    for _ in range(25):
        _perfn_step(b, wl.params.has_thermal_diffusion, wl.mat.rheol_type & 1)
    sa, sb = a.download(), b.download()
    for k in sa:
        if k in ("ntmp", "shpdy") and (k == "ntmp" or wl.mesh.ndims == 2):
            continue
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    assert a.clock() == b.clock()


def test_gpu_deterministic_and_step_host():
    """Two runs give identical bits (no atomics in any sum); the host-buffer
    drop-in call equals upload + step + download."""
    g = load_golden("3d_heat_jitter_multimat")
    wl, _ = build_case("3d_heat_jitter_multimat")
    cp = float(g["init"]["compensation_pressure"])
    c = g["init"]["clock"]
    clk = (c[0], c[1], int(c[2]))
    m1, m2 = _model(wl, cp), _model(wl, cp)
    m1.upload(state_from(g["init"]), clk)
    m1.step(40)
    s1 = m1.download()
    st = state_from(g["init"])
    clk2 = m2.step_host(st, 40, clk)
    for k in s1:
        np.testing.assert_array_equal(s1[k], st[k], err_msg=k)
    assert clk2 == m1.clock()


def _long_run(wl, nsteps, perturb_seeds=()):
    """Device and oracle runs of nsteps from the same initial state; returns
    the normalised device errors and the perturbed-oracle envelope."""
    from dynearthsol_gb300.config import initial_state
    from oracle.oracle import Oracle, state_copy
    st, cp = initial_state(wl)
    o = Oracle(wl, st, cp)
    assert o.init_fields() == 0
    st0, clk0 = state_copy(st), o.clock
    m = _model(wl, cp)
    m.upload(state_copy(st0), clk0)
    m.step(nsteps)
    assert o.run(nsteps) == 0
    out = m.download()
    assert m.clock()[2] == o.clock[2]
    errs = {k: rel_err(out[k], st[k]) for k in KEY_FIELDS}
    env = {k: 0.0 for k in KEY_FIELDS}
    for seed in perturb_seeds:
        sp = state_copy(st0)
        op = Oracle(wl, sp, cp, 1, clk0, perturb_seed=seed)
        assert op.run(nsteps) == 0
        for k in KEY_FIELDS:
            env[k] = max(env[k], rel_err(sp[k], st[k]))
    return errs, env


def test_gpu_1000_steps_elastic_bit_exact_vs_oracle():
    """Elastic rheology with heat diffusion on the 3D workload's mesh family
    (12x12x4 cubes, 3,456 tets), 1000 steps.  This path calls no
    transcendental function, so the FP64 device (no FMA contraction,
    reference expression order, IEEE division and square root) must
    reproduce the oracle -- and with it the reference -- bit for bit."""
    from dataclasses import replace
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c1_3d_evp", cells=(12, 12, 4))
    wl.mat = replace(wl.mat, rheol_type=capi.RH_ELASTIC)
    errs, _ = _long_run(wl, 1000)
    print("normalised errors after 1000 steps:", errs)
    assert max(errs.values()) == 0.0, errs


def test_gpu_1000_steps_evp_damping2_vs_oracle():
    """The 3D visco-elasto-plastic workload physics (weak zone yields) at
    12x12x4 cubes with the continuous damping option 2: 1000 FP64 steps
    within 1e-9 of the oracle on velocity, stress, temperature and plastic
    strain.  With the default damping option 1 the reference's step is
    chaotic (next test); with option 2 it is not, so this is the strict
    long-run parity check of the whole path."""
    from dataclasses import replace
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c1_3d_evp", cells=(12, 12, 4))
    wl.params = replace(wl.params, damping_option=2)
    errs, _ = _long_run(wl, 1000)
    print("normalised errors after 1000 steps:", errs)
    assert max(errs.values()) <= 1e-9, errs


def test_gpu_1000_steps_evp_within_libm_envelope():
    """The 3D visco-elasto-plastic workload physics at 12x12x4 cubes, 1000
    steps with the default damping option 1.  That damping,
    f -= 0.8 copysign(f, v) for |v| > 1e-13 (fields.cxx:249-255), is
    discontinuous in the sign of near-zero velocities, which makes the
    reference's own run chaotic: a one-ulp change of its libm moves the
    stress by ~1e-4 after 1000 steps.  The device is held to 20x the drift
    the oracle shows under such a change (two seeds, same run)."""
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c1_3d_evp", cells=(12, 12, 4))
    errs, env = _long_run(wl, 1000, perturb_seeds=(1, 2))
    print("normalised errors:", errs, "envelope:", env)
    for k in KEY_FIELDS:
        assert errs[k] <= max(1e-9, ENV_MARGIN * env[k]), (k, errs[k], env[k])


def test_gpu_error_status_nan_and_negative_volume():
    """Faults injected on the host (a NaN coordinate; an inverted element)
    come back as device status bits, with the context still usable."""
    from dynearthsol_gb300 import capi
    g = load_golden("3d_evp_yield")
    wl, _ = build_case("3d_evp_yield")
    cp = float(g["init"]["compensation_pressure"])
    c = g["init"]["clock"]
    m = _model(wl, cp)
    st = state_from(g["init"])
    st["coord"][5, 2] = np.nan
    m.upload(st, (c[0], c[1], int(c[2])))
    m.step(1)
    bits = m.device_status()
    assert bits & capi.DES_DEV_NONFINITE
    # an element turned inside out
    st = state_from(g["init"])
    e = 7
    n0, n1 = wl.mesh.connectivity[e, 0], wl.mesh.connectivity[e, 1]
    st["coord"][[n0, n1]] = st["coord"][[n1, n0]]
    m.upload(st, (c[0], c[1], int(c[2])))
    m.call("compute_volume")
    assert m.device_status() & capi.DES_DEV_NEG_VOLUME
    # still usable
    m.upload(state_from(g["init"]), (c[0], c[1], int(c[2])))
    m.step(2)
    assert m.device_status() == 0


def test_gpu_dt_nonpositive_is_runtime_error():
    """compute_dt <= 0 maps to the reference's exit code 11 (geometry.cxx:304-308)."""
    from dataclasses import replace
    from dynearthsol_gb300 import capi
    g = load_golden("3d_evp")
    wl, _ = build_case("3d_evp")
    wl.params = replace(wl.params, characteristic_speed=-1e-9)
    m = _model(wl, float(g["init"]["compensation_pressure"]))
    c = g["init"]["clock"]
    m.upload(state_from(g["init"]), (c[0], c[1], int(c[2])))
    with pytest.raises(capi.DesError) as ei:
        m.call("compute_dt")
    assert ei.value.code == capi.DES_ERUNTIME


def test_gpu_create_rejects_bad_input():
    from dynearthsol_gb300 import capi
    wl, _ = build_case("3d_evp")
    wl.mesh.connectivity = wl.mesh.connectivity.copy()
    wl.mesh.connectivity[3, 2] = wl.mesh.nnode + 5
    with pytest.raises(capi.DesError) as ei:
        _model(wl, 0.0)
    assert ei.value.code == capi.DES_EINPUT


def test_gpu_full_size_properties():
    """The 998,400-tet workload: a few steps stay finite with a clean device
    status; nodal sums are consistent (sum of volume_n = 4 x total volume;
    sum of mass = pseudo-density x total volume); a rerun from the same state
    is bit-identical."""
    from dynearthsol_gb300.config import initial_state, make_workload
    wl = make_workload("c1_3d_evp")
    assert wl.mesh.nelem == 998_400 and wl.mesh.nnode == 177_147
    st, cp = initial_state(wl)
    m = _model(wl, cp)
    init = m.init_fields(st)
    c0 = m.clock()
    m.step(20)
    a = m.download()
    assert m.device_status() == 0
    for k in ("coord", "vel", "stress", "strain", "temperature", "plstrain", "force"):
        assert np.isfinite(a[k]).all(), k
    V = a["volume"].sum()
    assert abs(a["volume_n"].sum() / (4 * V) - 1) < 1e-12
    ps = wl.params.max_vbc_val() * wl.params.inertial_scaling
    rho = wl.mat.bulk_modulus[0] / (ps * ps)
    assert abs(a["mass"].sum() / (rho * V) - 1) < 1e-12
    m.upload(init, c0)
    m.step(20)
    b = m.download()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
