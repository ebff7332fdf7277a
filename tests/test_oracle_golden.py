"""The oracle (C restatement) and the workload set-up against the golden
fixtures produced by the reference's own code (tests/golden/gen_golden.py).

On the architecture the fixtures were generated on (x86-64, the same libm)
the restatement reproduces the reference bit for bit; elsewhere a 1e-12
normalised tolerance absorbs last-ulp differences of libm.
"""
import math
import platform

import numpy as np
import pytest

from cases import CASES, FUNCTIONS, PERFN_CASES, build_case
from conftest import load_golden, rel_err, state_from
from dynearthsol_gb300.config import initial_state
from oracle.oracle import Oracle, eigen3, state_copy

EXACT = platform.machine() in ("x86_64", "AMD64")
TOL = 0.0 if EXACT else 1e-12

# stressyy is uninitialised by the reference outside plane strain
# (rheology.cxx:611,632); it is not compared there.
SKIP = {"stressyy"}


def compare(st, ref, fields=None, tol=TOL, label=""):
    bad = []
    for k in fields or ref:
        if k in SKIP or k not in st:
            continue
        e = rel_err(st[k], ref[k])
        if e > tol:
            bad.append(f"{label}{k}: {e:.3e}")
    assert not bad, "; ".join(bad)


@pytest.mark.parametrize("name", CASES)
def test_initial_conditions_match_reference_init(name):
    """Workload set-up (ic.cxx restated) + oracle init == reference init."""
    g = load_golden(name)
    wl, _ = build_case(name)
    st, comp = initial_state(wl)
    assert comp == float(g["init"]["compensation_pressure"])
    np.testing.assert_array_equal(wl.mesh.bnormals, g["init"]["bnormals"])
    ev = g["init"]["edge_vectors"]
    np.testing.assert_array_equal(wl.mesh.edge_vectors, ev)
    for k in ("stress", "strain", "plstrain", "temperature", "coord", "coord0"):
        np.testing.assert_array_equal(st[k], g["init"][k], err_msg=k)
    o = Oracle(wl, st, comp)
    assert o.init_fields() == 0
    compare(st, g["init"], label="init ")
    assert o.clock[1] == pytest.approx(float(g["init"]["clock"][1]), rel=TOL or 0, abs=0)


@pytest.mark.parametrize("name", CASES)
def test_oracle_run_matches_reference(name):
    g = load_golden(name)
    wl, nsteps = build_case(name)
    st = state_from(g["init"])
    clk = tuple(g["init"]["clock"])
    o = Oracle(wl, st, float(g["init"]["compensation_pressure"]), clock=(clk[0], clk[1], int(clk[2])))
    assert o.run(nsteps) == 0
    compare(st, g["final"], label="final ")
    t, dt, steps = o.clock
    assert steps == int(g["final"]["clock"][2])
    assert dt == g["final"]["clock"][1] or abs(dt / g["final"]["clock"][1] - 1) <= TOL


@pytest.mark.parametrize("name", PERFN_CASES)
@pytest.mark.parametrize("fn", list(FUNCTIONS))
def test_oracle_functions_match_reference(name, fn):
    g = load_golden(name)
    if f"fn_{fn}" not in g:
        pytest.skip(f"{name} keeps no {fn} output (full-horizon fixture)")
    wl, _ = build_case(name)
    st = state_from(g["mid"])
    clk = tuple(g["mid"]["clock"])
    o = Oracle(wl, st, float(g["init"]["compensation_pressure"]), clock=(clk[0], clk[1], int(clk[2])))
    o.call(fn)
    fields = FUNCTIONS[fn]
    if wl.mesh.ndims == 2:
        fields = [f for f in fields if f != "shpdy"]
    compare(st, g[f"fn_{fn}"], fields=fields, label=f"{fn} ")


@pytest.mark.parametrize("name", PERFN_CASES)
def test_oracle_dt_and_quality_match_reference(name):
    g = load_golden(name)
    wl, _ = build_case(name)
    st = state_from(g["mid"])
    clk = tuple(g["mid"]["clock"])
    o = Oracle(wl, st, float(g["init"]["compensation_pressure"]), clock=(clk[0], clk[1], int(clk[2])))
    rc, dt = o.call("compute_dt")
    assert rc == 0
    assert abs(dt - float(g["fn_compute_dt"]["dt"])) <= TOL * abs(dt)
    q, w = o.call("worst_elem_quality")
    ref = g["fn_worst_elem_quality"]["result"]
    assert w == int(ref[1])
    assert abs(q - ref[0]) <= max(TOL, 0) * abs(q) + (0 if EXACT else 1e-15)


@pytest.mark.parametrize("name", PERFN_CASES)
def test_oracle_steps_from_mid_match_reference(name):
    g = load_golden(name)
    wl, _ = build_case(name)
    for k_steps in (1, 10):
        st = state_from(g["mid"])
        clk = tuple(g["mid"]["clock"])
        o = Oracle(wl, st, float(g["init"]["compensation_pressure"]), clock=(clk[0], clk[1], int(clk[2])))
        assert o.run(k_steps) == 0
        compare(st, g[f"mid{k_steps}"], fields=[k for k in g[f"mid{k_steps}"] if k != "clock"],
                label=f"mid+{k_steps} ")


def test_libm_envelope_recorded():
    """Every fixture records its libm-sensitivity envelope; plastic 3D runs
    are the chaotic ones."""
    for name in CASES:
        g = load_golden(name)
        assert set(g["envelope"]) >= {"vel", "stress", "temperature", "plstrain"}
    assert float(load_golden("3d_evp_yield")["envelope"]["stress"]) > 1e-9
    assert float(load_golden("2d_ep")["envelope"]["stress"]) < 1e-12


def test_plasticity_is_exercised():
    """The yield cases really go through the Mohr-Coulomb return map."""
    for name in ("2d_ep_yield", "3d_evp_yield", "3d_ep_yield", "3d_heat_jitter_multimat", "2d_ps_oedometer"):
        g = load_golden(name)
        assert (g["final"]["plstrain"] > g["init"]["plstrain"]).sum() > 0, name


def _oedometer_analytic(nsteps):
    """benchmarks/oedometer-2d-plot.py analytical(): Sxx vs displacement."""
    K = 200e6
    mu = 200e6
    coh = 1e6
    phi = psi = 10.0 * math.pi / 180
    vx = 1e-5
    e1, e2 = K + 4.0 * mu / 3.0, K - 2.0 * mu / 3.0
    nf = (1 + math.sin(phi)) / (1 - math.sin(phi))
    npsi = (1 + math.sin(psi)) / (1 - math.sin(psi))
    rl = (e1 - e2 * nf) / ((e1 + e2) * nf * npsi - 2.0 * e2 * (nf + npsi) + 2.0 * e1)
    step1 = 2.0 * coh * math.sqrt(nf) / ((e1 - e2 * nf) * vx)
    disp = vx * np.arange(nsteps + 1, dtype=float)
    S = np.zeros(nsteps + 1)
    for i in range(1, nsteps + 1):
        de = vx / (1 - disp[i])
        S[i] = S[i - 1] + (e1 * de if i < step1 else de * (e1 + 2.0 * rl * (e2 * npsi - e1)))
    return S


def test_oedometer_matches_analytic_solution():
    """Known-answer check of the plane-strain Mohr-Coulomb path against the
    reference's analytic oedometer benchmark (2000 steps, fixed dt = 1 s)."""
    g = load_golden("2d_ps_oedometer")
    sxx = -g["final"]["stress"][:, 0].mean()
    S = _oedometer_analytic(2000)
    assert abs(sxx / S[-1] - 1) < 1e-3
    assert (g["final"]["plstrain"] > 0).all()


def test_eigen_solver_known_matrix():
    """tests.cxx:79-127's matrix (diag 3e4,-1,3; off-diagonal 2,4,2): the
    eigenpairs reconstruct A, ascending after principal_stresses3's sort."""
    a6 = np.array([3e4, -1.0, 3.0, 2.0, 4.0, 2.0])
    rc, w, q, used_ql = eigen3(a6)
    assert rc == 0
    A = np.array([[a6[0], a6[3], a6[4]], [a6[3], a6[1], a6[5]], [a6[4], a6[5], a6[2]]])
    R = q @ np.diag(w) @ q.T
    assert np.abs(R - A).max() < 1e-10 * np.abs(A).max()
    np.testing.assert_allclose(np.sort(w), np.linalg.eigvalsh(A), rtol=1e-13, atol=1e-11)


def test_eigen_solver_degenerate_uses_ql():
    """Near-isotropic stress (the lithostatic state) takes the QL fallback."""
    rc, w, q, used_ql = eigen3(np.array([-1e8, -1e8, -1e8, 1.0, 0.0, 0.0]))
    assert rc == 0 and used_ql == 1
    np.testing.assert_allclose(np.sort(w), [-1e8 - 1, -1e8, -1e8 + 1], rtol=0, atol=1e-6)


def test_oracle_multithread_close_to_serial():
    """The OpenMP band schedule (CPU baseline) differs from the serial order
    only by summation order, on a mesh whose 2T element bands do not share
    nodes two bands apart (the condition create_elem_groups warns about,
    mesh.cxx:1764-1805)."""
    from dynearthsol_gb300.mesh import box3d
    wl, _ = build_case("3d_evp_yield")
    wl.mesh = box3d(16, 4, 3, 100e3, 100e3, 10e3)
    wl.resolution = 100e3 / 16
    st, cp = initial_state(wl)
    o1 = Oracle(wl, st, cp, 1)
    o1.init_fields()
    s4 = state_copy(st)
    clk = o1.clock
    o4 = Oracle(wl, s4, cp, 4, clk)
    o1.run(30)
    o4.run(30)
    for k in ("vel", "stress", "temperature", "plstrain"):
        assert rel_err(s4[k], st[k]) < 1e-9, k
