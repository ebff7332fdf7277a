"""Phase changes on the device (des_set_markers, des_phase_changes) against
the reference's own phase_changes (phasechanges.cxx:232-258, MarkerSet from
markerset.cxx), compiled from its sources into oracle/_ref.

The mesh is a 3D box 100 km deep (so that the SimpleSubduction transitions
-- basalt to eclogite, sediment to schist, serpentinite to mantle and
mantle to serpentinite -- all fire somewhere) with eight materials, random
markers (element, barycentric coordinates, material type) and random
hydrous-marker counts.  The new material types and per-element marker
counts must equal the reference's exactly, and the next steps must blend
the element properties from the new counts (the same state as a context
given the reference's counts by des_set_elemmarkers, bit for bit).
"""
from dataclasses import replace

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _reference(nd):
    from oracle.oracle import Reference, reference_sources_available
    if not reference_sources_available():
        pytest.skip("reference sources not staged (make -C oracle stage REF=...)")
    return Reference(nd)


def _deep_case(seed=5, nmark=6):
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import _evp_material, make_workload
    from dynearthsol_gb300.mesh import box3d
    wl = make_workload("c1_3d_evp", cells=(6, 4, 10))
    wl.mesh = box3d(6, 4, 10, 100e3, 60e3, 100e3)
    wl.t_bottom = 1600.0
    base = _evp_material()
    mats = {n: tuple(getattr(base, n)) * 8 for n in capi.MAT_ARRAYS}
    mats["rho0"] = (3300.0, 3000.0, 2900.0, 3400.0, 2500.0, 2700.0, 2700.0, 2900.0)
    wl.mat = replace(base, **mats)
    rng = np.random.default_rng(seed)
    ne = wl.mesh.nelem
    elem = np.repeat(np.arange(ne, dtype=np.int32), nmark)
    eta = rng.dirichlet(np.ones(4), size=elem.size)
    mt = rng.integers(0, 8, size=elem.size).astype(np.int32)
    em = np.zeros((ne, 8), np.int32)
    np.add.at(em, (elem, mt), 1)
    wl.mat.elemmarkers = em
    hyd = (rng.random(ne) < 0.5).astype(np.int32)
    return wl, elem, eta, mt, em, hyd


@pytest.mark.parametrize("option", [1, 101])
def test_phase_changes_match_reference(option):
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    wl, elem, eta, mt, em, hyd = _deep_case()
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp)
    init = m.init_fields(st)
    ref = _reference(3)
    ref_mt, ref_em = ref.phase_changes(wl, init, cp, option, elem, eta, mt, hyd, em)
    m.set_markers(elem, eta, mt)
    n = m.phase_changes(option, hyd)
    dev_mt, dev_em = m.get_markers()
    assert m.device_status() == 0
    np.testing.assert_array_equal(dev_mt, ref_mt)
    np.testing.assert_array_equal(dev_em, ref_em)
    assert n == int((ref_mt != mt).sum())
    if option == 1:
        moved = {(int(a), int(b)) for a, b in zip(mt[ref_mt != mt], ref_mt[ref_mt != mt])}
        assert {(2, 3), (4, 5), (1, 0), (0, 1)} <= moved, moved
    else:
        assert n == 0


def test_phase_changes_reach_the_next_steps():
    """After des_phase_changes the step blends from the new marker counts:
    ten steps equal those of a context given the reference's counts."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    wl, elem, eta, mt, em, hyd = _deep_case()
    st, cp = initial_state(wl)
    a = DeviceModel(wl, comp_pressure=cp)
    init = a.init_fields(st)
    clk = a.clock()
    ref_mt, ref_em = _reference(3).phase_changes(wl, init, cp, 1, elem, eta, mt, hyd, em)
    assert (ref_em != em).any()
    a.set_markers(elem, eta, mt)
    a.phase_changes(1, hyd)
    a.step(10)
    b = DeviceModel(wl, comp_pressure=cp)
    b.upload({k: v.copy() for k, v in init.items()}, clk)
    assert b.lib.des_set_elemmarkers(b.ctx, capi.iptr(np.ascontiguousarray(ref_em))) == 0
    b.step(10)
    sa, sb = a.download(), b.download()
    for k in ("vel", "stress", "temperature", "coord"):
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    # a context created with the new counts: the blended properties that
    # des_phase_changes and des_set_elemmarkers re-form are those of creation
    wl_new = replace(wl, mat=replace(wl.mat, elemmarkers=np.ascontiguousarray(ref_em)))
    d = DeviceModel(wl_new, comp_pressure=cp)
    d.upload({k: v.copy() for k, v in init.items()}, clk)
    d.step(10)
    sd = d.download()
    for k in ("vel", "stress", "temperature", "coord"):
        np.testing.assert_array_equal(sa[k], sd[k], err_msg="fresh context " + k)
    c = DeviceModel(wl, comp_pressure=cp)   # without the phase changes: another state
    c.upload({k: v.copy() for k, v in init.items()}, clk)
    c.step(10)
    assert rel_err(c.download()["stress"], sa["stress"]) > 0
