"""Full-horizon parity against the reference's own code.

* The 2D workload at its full size (200x20 cells x 2 = 8,000 triangles,
  4,221 nodes) over its full 10,000 steps, with the default damping and
  with damping option 2.  No transcendental of this elasto-plastic run
  reaches its state (the fixture's libm envelope is exactly 0), so the FP64
  device path is held to the 1e-9 bound on velocity, stress, temperature
  and plastic strain, with no envelope allowance.
* A yielding case of the 3D workload's physics (20x20x6 cubes x 6 =
  14,400 tets, Arrhenius Maxwell visco-elasto-plastic, +-1 cm/yr, 2000
  steps) whose band of weak material takes 9 % of the elements through the
  Mohr-Coulomb return map.  There the reference itself is chaotic: the
  restatement rerun with every transcendental moved by +-1 ulp ends 1.7e-2
  (velocity) and 1.8e-3 (stress) away with the default damping, 2.2e-3 and
  7.4e-5 with damping option 2 (the fixtures' envelopes).  The device run
  is held to 20x those envelopes over the full horizon, and tightly where
  the chaos has no time to act: one step (1e-12) and ten steps (1e-10 or
  20x the ten-step envelope) from the reference's state at step 1500, when
  1,158 elements yield in that step (test_gpu_parity's mid-state tests).
"""

import numpy as np
import pytest

from cases import build_case
from conftest import load_golden, rel_err, state_from

pytestmark = pytest.mark.gpu

NORTH_STAR = 1e-9
ENV_MARGIN = 20.0
KEY_FIELDS = ("vel", "stress", "temperature", "plstrain")


def _run(name, precision=None, group="init", nsteps=None):
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.solver import DeviceModel
    g = load_golden(name)
    wl, n = build_case(name)
    m = DeviceModel(wl, comp_pressure=float(g["init"]["compensation_pressure"]),
                    precision=capi.PREC_FP64 if precision is None else precision)
    c = g[group]["clock"]
    m.upload(state_from(g[group]), (c[0], c[1], int(c[2])))
    m.step(n if nsteps is None else nsteps)
    out = m.download()
    assert m.device_status() == 0
    return g, wl, out


@pytest.mark.parametrize("name", ["2d_c0_full", "2d_c0_full_damp2"])
def test_2d_workload_full_size_full_horizon(name):
    g, wl, out = _run(name)
    assert wl.mesh.nelem == 8000 and wl.mesh.nnode == 4221
    assert int(g["nsteps"]) == 10000
    assert all(float(v) == 0.0 for v in g["envelope"].values())
    errs = {k: rel_err(out[k], g["final"][k]) for k in KEY_FIELDS + ("coord", "strain", "force")}
    print(name, "FP64 device vs reference after 10,000 steps:", {k: f"{v:.2e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if v > NORTH_STAR}
    assert not bad, bad
    # the weak zone yields by the end, on the device as in the reference
    yielded = (g["final"]["plstrain"] > g["init"]["plstrain"]).sum()
    assert yielded > 0
    assert (out["plstrain"] > g["init"]["plstrain"]).sum() == yielded


@pytest.mark.parametrize("name", ["3d_c1_yield_band", "3d_c1_yield_band_damp2"])
def test_yielding_band_full_horizon(name):
    g, wl, out = _run(name)
    assert wl.mesh.nelem == 14400 and int(g["nsteps"]) == 2000
    ne = wl.mesh.nelem
    ref_y = int((g["final"]["plstrain"] > g["init"]["plstrain"]).sum())
    dev_y = int((out["plstrain"] > g["init"]["plstrain"]).sum())
    assert ref_y >= 0.05 * ne and dev_y >= 0.05 * ne, (ref_y, dev_y)
    env = {k: float(v) for k, v in g["envelope"].items()}
    errs = {k: rel_err(out[k], g["final"][k]) for k in KEY_FIELDS}
    print(name, f"yielded: reference {ref_y}, device {dev_y} of {ne};",
          "error", {k: f"{v:.2e}" for k, v in errs.items()}, "envelope", {k: f"{env[k]:.2e}" for k in KEY_FIELDS})
    bad = {k: v for k, v in errs.items() if v > max(NORTH_STAR, ENV_MARGIN * env[k])}
    assert not bad, bad


@pytest.mark.parametrize("nsteps,gate", [(1, 1e-6), (10, 1e-6)])
def test_mixed_step_on_the_yielding_band(nsteps, gate):
    """Mixed against FP64 from the reference's yielding state at step 1500
    (1,158 elements on the yield surface): the relative L2 stress error
    stays within the mixed step's gate, and as many elements yield."""
    from dynearthsol_gb300 import capi
    name = "3d_c1_yield_band_damp2"
    _, _, a = _run(name, capi.PREC_FP64, "mid", nsteps)
    g, _, b = _run(name, capi.PREC_MIXED, "mid", nsteps)
    assert (a["delta_plstrain"] > 0).sum() > 1000
    l2 = float(np.linalg.norm(b["stress"] - a["stress"]) / np.linalg.norm(a["stress"]))
    print(f"mixed vs FP64 from the yielding state, {nsteps} steps: L2 stress {l2:.2e}, yielding "
          f"{(a['delta_plstrain'] > 0).sum()} / {(b['delta_plstrain'] > 0).sum()}")
    assert l2 <= gate
    ya, yb = int((a["delta_plstrain"] > 0).sum()), int((b["delta_plstrain"] > 0).sum())
    assert abs(ya - yb) <= 0.005 * ya
