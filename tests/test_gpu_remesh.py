"""The remesh hand-off on the device.

* des_build_topology against the reference's own create_support and
  create_boundary_facets (mesh.cxx:1637-1721, compiled from its sources into
  oracle/_ref): jittered and permuted 3D meshes and a 2D mesh, boundary
  segments in a shuffled order with some interior segments (flag 0) among
  them; the lists must be equal, element by element and in order.
* des_remesh in a running context: steps on one mesh, then a different mesh
  of the same domain with the state carried over (interpolated on the host,
  with the derived fields -- volume, volume_old, masses, shape functions --
  formed on the new mesh, as remeshing.cxx:2009-2015 forms them), then
  steps on.  The device must continue exactly as the oracle does on the new
  mesh from the same state.
"""
import numpy as np
import pytest

from cases import build_case
from conftest import load_golden, rel_err, state_from

pytestmark = pytest.mark.gpu


def _reference(nd):
    from oracle.oracle import Reference, reference_sources_available
    if not reference_sources_available():
        pytest.skip("reference sources not staged (make -C oracle stage REF=...)")
    return Reference(nd)


def _meshes():
    from dynearthsol_gb300.mesh import box2d, box3d
    return [
        box3d(5, 4, 3, 100e3, 80e3, 10e3, jitter=0.2, permute=True, seed=3),
        box3d(20, 20, 6, 100e3, 100e3, 10e3),
        box3d(7, 3, 4, 60e3, 30e3, 20e3, jitter=0.1, permute=True, seed=9),
        box2d(30, 7, 100e3, 10e3),
    ]


@pytest.mark.parametrize("k", range(4))
def test_build_topology_matches_reference(k):
    from dynearthsol_gb300 import capi
    mesh = _meshes()[k]
    rng = np.random.default_rng(k)
    nb = int(mesh.bfacet_offsets[-1])
    seg, flag = capi.segments_of(mesh, rng.permutation(nb))
    # a few interior segments (flag 0), which both sides skip
    inner = mesh.connectivity[rng.integers(0, mesh.nelem, 5)][:, :mesh.ndims]
    seg = np.ascontiguousarray(np.concatenate([seg, inner]), dtype=np.int32)
    flag = np.ascontiguousarray(np.concatenate([flag, np.zeros(5, np.int32)]), dtype=np.int32)
    perm = rng.permutation(seg.shape[0])
    seg, flag = np.ascontiguousarray(seg[perm]), np.ascontiguousarray(flag[perm])
    topo = capi.Topology(mesh, seg, flag)
    off, elems, boff, fac = capi.build_topology(topo)
    ref = _reference(mesh.ndims)
    roff, relems = ref.create_support(mesh.nnode, mesh.connectivity)
    rboff, rfac = ref.create_boundary_facets(mesh.nnode, mesh.connectivity, mesh.bcflag, seg, flag)
    np.testing.assert_array_equal(off, roff)
    np.testing.assert_array_equal(elems, relems)
    np.testing.assert_array_equal(boff, rboff)
    np.testing.assert_array_equal(fac, rfac)
    assert boff[-1] == nb


def _carry_over(src_mesh, src: dict, dst_mesh) -> dict:
    """A stand-in for the reference's interpolation after remeshing: nodal
    fields from the nearest old node, element fields from the nearest old
    element centroid; the new mesh's own coordinates."""
    from scipy.spatial import cKDTree
    from dynearthsol_gb300.config import elem_center
    from oracle.oracle import empty_state
    nd = dst_mesh.ndims
    out = empty_state(nd, dst_mesh.nnode, dst_mesh.nelem)
    near_n = cKDTree(src_mesh.coord).query(dst_mesh.coord)[1]
    near_e = cKDTree(elem_center(src_mesh)).query(elem_center(dst_mesh))[1]
    for k in ("vel", "temperature"):
        out[k] = np.ascontiguousarray(src[k][near_n])
    for k in ("stress", "strain", "strain_rate", "plstrain", "delta_plstrain", "stressyy", "dpressure", "edvoldt"):
        out[k] = np.ascontiguousarray(src[k][near_e])
    out["coord"] = np.ascontiguousarray(dst_mesh.coord.copy())
    out["coord0"] = np.ascontiguousarray(dst_mesh.coord.copy())
    return out


# elastic: no transcendental, bit for bit; yielding: CUDA's and glibc's
# last-ulp differences (pow, exp, sin, ...) through the return map, which
# the yielding fixtures' ten-step envelopes put near 1e-10 after ten steps
@pytest.mark.parametrize("name,tol", [("3d_elastic_damp3", 0.0), ("3d_evp_yield", 1e-8)])
def test_remesh_handoff_continues_like_the_oracle(name, tol):
    from dataclasses import replace
    from dynearthsol_gb300.mesh import box3d
    from dynearthsol_gb300.solver import DeviceModel
    from oracle.oracle import Oracle
    g = load_golden(name)
    wl, _ = build_case(name)
    cp = float(g["init"]["compensation_pressure"])
    c = g["init"]["clock"]
    dev = DeviceModel(wl, comp_pressure=cp)
    dev.upload(state_from(g["init"]), (c[0], c[1], int(c[2])))
    dev.step(40)
    before = dev.download()
    clk = dev.clock()
    # another mesh of the same domain: one more cube along x, jittered and permuted
    mesh_b = box3d(4, 3, 2, *wl.mesh.lengths, jitter=0.15, permute=True, seed=21)
    mesh_b.bnormals, mesh_b.edge_vectors = wl.mesh.bnormals, wl.mesh.edge_vectors
    wl_b = replace(wl, mesh=mesh_b)
    st = _carry_over(wl.mesh, before, mesh_b)
    o = Oracle(wl_b, st, cp, clock=clk)
    o.call("compute_volume")
    st["volume_old"][:] = st["volume"]
    o.call("compute_mass")
    o.call("compute_shape_fn")
    dev.remesh(wl_b)
    dev.upload({k: v.copy() for k, v in st.items()}, clk)
    dev.step(20)
    out = dev.download()
    assert o.run(20) == 0
    assert dev.device_status() == 0
    for k in ("vel", "stress", "strain", "temperature", "plstrain", "coord", "volume"):
        e = rel_err(out[k], st[k])
        assert e <= tol, (k, e)
    assert out["stress"].shape == (mesh_b.nelem, 6) and mesh_b.nelem != wl.mesh.nelem
