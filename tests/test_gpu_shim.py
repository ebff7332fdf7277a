"""The reference's own loop through the reference-signature shim.

``libref_shim{2,3}d.so`` (dynearthsol_gb300/shim) links the shim in place of
the reference's fields.o, geometry.o and rheology.o, next to the reference's
own bc.o, matprops.o, ic.o and binaryio.o and the reference harness
(oracle/ref_harness.cxx), which runs the reference's init sequence
(dynearthsol.cxx:82-98) and loop body (dynearthsol.cxx:325-361).  Every
hot-path call of that loop therefore lands in the shim and runs on the GPU
through libdesgpu.so, with the reference's own code around it (apply_vbcs's
host twin, surface_processes, the volume pointer swap of update_mesh, the
clock).

Both residency modes of the shim are run:
* sync: each call moves the Variables fields it reads and writes;
* resident (DESGPU_SHIM_RESIDENT=1): the state stays on the device; the
  harness uploads it once after setting it and downloads it once before
  reading it (desgpu_shim_sync_to_device / _to_host), as a host program does
  around output and remeshing.

The final states are held to the golden fixtures with the tolerances of
test_gpu_parity.py's step test.
"""
from dataclasses import replace

import numpy as np
import pytest

from cases import build_case, reference_material_for
from conftest import load_golden, rel_err, state_from

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-9
ENV_MARGIN = 20.0
KEY_FIELDS = ("vel", "stress", "temperature", "plstrain", "coord", "strain", "force")
SHIM_CASES = ["2d_evp_heat", "2d_ep_yield", "3d_evp_yield", "3d_heat_jitter_multimat", "3d_vbc_mix",
              "3d_elastic_damp3"]


def _shim(nd):
    from oracle.oracle import Reference
    try:
        return Reference(nd, flavour="shim")
    except OSError as e:
        pytest.fail(f"shim library not built: {e}")


@pytest.mark.parametrize("name", ["2d_evp_heat", "3d_heat_jitter_multimat", "3d_evp_yield"])
def test_reference_init_through_shim(name, monkeypatch):
    """The reference's init sequence with the shim's volume, mass and shape
    functions (sync mode: init reads the results on the host)."""
    from dynearthsol_gb300.config import initial_state
    monkeypatch.setenv("DESGPU_SHIM_RESIDENT", "0")
    g = load_golden(name)
    wl, _ = build_case(name)
    wl_ref = replace(wl, mat=reference_material_for(wl), elem_fields={})
    ref = _shim(wl.mesh.ndims)
    st, _ = initial_state(wl)
    bn, ev, cp, clk = ref.init(wl_ref, st)
    assert cp == float(g["init"]["compensation_pressure"])
    for k in ("volume", "mass", "tmass", "volume_n", "shpdx", "shpdz", "stress", "strain", "vel"):
        assert rel_err(st[k], g["init"][k]) <= 1e-13, k
    assert abs(clk[1] / g["init"]["clock"][1] - 1) < 1e-13


@pytest.mark.parametrize("resident", [0, 1])
@pytest.mark.parametrize("name", SHIM_CASES)
def test_reference_loop_through_shim_matches_golden(name, resident, monkeypatch):
    monkeypatch.setenv("DESGPU_SHIM_RESIDENT", str(resident))
    g = load_golden(name)
    wl, nsteps = build_case(name)
    wl_ref = replace(wl, mat=reference_material_for(wl), elem_fields={})
    ref = _shim(wl.mesh.ndims)
    st = state_from(g["init"])
    c = g["init"]["clock"]
    clk, _ = ref.run(wl_ref, st, float(g["init"]["compensation_pressure"]), (c[0], c[1], int(c[2])), nsteps)
    env = {k: float(v) for k, v in g["envelope"].items()}
    bad = {}
    for k in KEY_FIELDS:
        e = rel_err(st[k], g["final"][k])
        if e > max(TOL_STEP, ENV_MARGIN * env[k]):
            bad[k] = e
    assert not bad, f"{name} resident={resident}: " + ", ".join(f"{k}={v:.2e}" for k, v in bad.items())
    assert clk[2] == int(g["final"]["clock"][2])
    assert abs(clk[1] / g["final"]["clock"][1] - 1) < max(1e-9, ENV_MARGIN * max(env.values()))


def test_resident_mode_keeps_the_volume_swap(monkeypatch):
    """update_mesh swaps the host's volume and volume_old pointers
    (dynearthsol.cxx:226) and the shim mirrors that on the device: a resident
    run's volume_old after the loop is the volume one step before."""
    monkeypatch.setenv("DESGPU_SHIM_RESIDENT", "1")
    name = "3d_evp_yield"
    g = load_golden(name)
    wl, _ = build_case(name)
    wl_ref = replace(wl, mat=reference_material_for(wl), elem_fields={})
    ref = _shim(3)
    cp = float(g["init"]["compensation_pressure"])
    c = g["init"]["clock"]
    a = state_from(g["init"])
    clk, _ = ref.run(wl_ref, a, cp, (c[0], c[1], int(c[2])), 5)
    b = {k: v.copy() for k, v in a.items()}
    ref.run(wl_ref, b, cp, clk, 1)
    np.testing.assert_array_equal(b["volume_old"], a["volume"])
    assert not np.array_equal(b["volume"], a["volume"])
