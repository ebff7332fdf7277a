"""bad_mesh_quality (remeshing.cxx:1882-1935) on the device, against the
reference's own function (compiled from its sources into oracle/_ref) and
through the reference-signature shim.

Each check of the reference is tripped on purpose, on golden states of a 2D
and a 3D case: a tiny element (code 3), a drifted bottom node with a
remeshing option that checks it (code 2), a worst element quality below
min_quality (code 1), and a mesh that passes (code 0).  Code and index must
equal the reference's; the reported quality is bit for bit its value.
"""
from dataclasses import replace

import numpy as np
import pytest

from cases import build_case, reference_material_for
from conftest import load_golden, state_from

pytestmark = pytest.mark.gpu

SIZEFACTOR = {3: 0.118, 2: 0.433}   # remeshing.cxx:76-82


def _reference(nd, flavour="serial"):
    from oracle.oracle import Reference, reference_sources_available
    if not reference_sources_available():
        pytest.skip("reference sources not staged (make -C oracle stage REF=...)")
    return Reference(nd, flavour=flavour)


def _checks(wl, st):
    """(name, quality params, expected code) that trip each check on st."""
    nd = wl.mesh.ndims
    res = wl.resolution
    vol = st["volume"]
    bottom = -wl.mesh.lengths[2]
    zb = st["coord"][(wl.mesh.bcflag & 16) != 0, nd - 1]
    drift = np.abs(zb - bottom)
    # a threshold that some but not all elements / bottom nodes cross
    small = float(np.median(vol)) / (SIZEFACTOR[nd] * res ** nd)
    dmid = float(np.median(drift)) / res
    return [
        ("pass", (1e-6, res, 0.0, 1e9, 1), 0),
        ("tiny element", (small, res, 0.0, 1e9, 1), 3),
        ("bottom drift", (1e-6, res, 0.0, dmid, 1), 2),
        ("bottom drift unchecked", (1e-6, res, 0.0, dmid, 0), 0),
        ("bottom drift option 11", (1e-6, res, 0.0, dmid, 11), 2),
        ("quality", (1e-6, res, 0.99, 1e9, 1), 1),
    ]


def _ref_quality(ref, wl_ref, st, cp, clk, qp):
    from oracle.oracle import RefQuality
    rq = RefQuality(qp[0], qp[1], qp[2], qp[3], wl_ref.mesh.lengths[2], qp[4])
    return ref.bad_mesh_quality(wl_ref, {k: v.copy() for k, v in st.items()}, cp, clk, rq)


@pytest.mark.parametrize("name,group", [("3d_evp_yield", "final"), ("2d_evp_heat", "mid"),
                                        ("3d_heat_jitter_multimat", "final"), ("2d_ep", "final")])
def test_bad_mesh_quality_matches_reference(name, group):
    from dynearthsol_gb300.solver import DeviceModel
    g = load_golden(name)
    wl, _ = build_case(name)
    wl_ref = replace(wl, mat=reference_material_for(wl), elem_fields={})
    st = state_from(g[group])
    c = g[group]["clock"]
    clk = (c[0], c[1], int(c[2]))
    cp = float(g["init"]["compensation_pressure"])
    ref = _reference(wl.mesh.ndims)
    m = DeviceModel(wl, comp_pressure=cp)
    m.upload({k: v.copy() for k, v in st.items()}, clk)
    seen = set()
    for label, qp, want in _checks(wl, st):
        rcode, ridx = _ref_quality(ref, wl_ref, st, cp, clk, qp)
        code, idx, val = m.bad_mesh_quality(*qp)
        assert rcode == want, f"{label}: the reference returned {rcode}"
        assert code == rcode, f"{label}: device {code}, reference {rcode}"
        if code:
            assert idx == ridx, f"{label}: device index {idx}, reference {ridx}"
        if code == 3:
            assert val == st["volume"][idx]
        if code == 1:
            q, w = m.call("worst_elem_quality")
            assert w == idx and val == (q ** (1.0 / 3) if wl.mesh.ndims == 3 else q)
        seen.add(code)
    assert seen == {0, 1, 2, 3}


@pytest.mark.parametrize("resident", [0, 1])
def test_bad_mesh_quality_through_the_shim(resident, monkeypatch):
    """The shim's bad_mesh_quality (linked over remeshing.o's) runs the check
    on the device; in resident mode it reads the device's volume and
    coordinates without a download."""
    monkeypatch.setenv("DESGPU_SHIM_RESIDENT", str(resident))
    name = "3d_evp_yield"
    g = load_golden(name)
    wl, _ = build_case(name)
    wl_ref = replace(wl, mat=reference_material_for(wl), elem_fields={})
    st = state_from(g["final"])
    c = g["final"]["clock"]
    clk = (c[0], c[1], int(c[2]))
    cp = float(g["init"]["compensation_pressure"])
    ref = _reference(3)
    shim = _reference(3, "shim")
    for label, qp, want in _checks(wl, st):
        assert _ref_quality(shim, wl_ref, st, cp, clk, qp) == _ref_quality(ref, wl_ref, st, cp, clk, qp), label
