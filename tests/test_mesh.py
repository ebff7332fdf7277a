"""Host-side mesh products the device step relies on (dynearthsol_gb300/mesh.py):
the box generators' element orientation, boundary flags and facets, the
node-to-element support lists, and the slab property of unpermuted boxes.

* Signed volumes (geometry.cxx:29-49) and 2D areas are positive: the shape
  function formulas (geometry.cxx:368-455) assume that orientation.
* Boundary flags use the reference's bits (constants.hpp:29-38); each
  boundary facet's nodes (NODE_OF_FACET, constants.hpp:59-71) carry its bit.
* Support lists (create_support, mesh.cxx:1707-1721) hold each (element,
  slot) once, ascending in element id: the order in which the device
  gathers sum, which makes the sums the reference's serial ones and the
  runs bit-reproducible.
* In an unpermuted box, x is the slowest index of both numberings, so an
  element's nodes lie in its x-layer or the next and a node's support
  elements in its x-layer or the previous one: the property the
  slab-pipelined host step checks before it overlaps transfers with the step.
"""
import numpy as np
import pytest

from dynearthsol_gb300.mesh import (BOUNDX0, BOUNDX1, BOUNDY0, BOUNDY1, BOUNDZ0, BOUNDZ1, NODE_OF_FACET_2D,
                                    NODE_OF_FACET_3D, box2d, box3d, support_csr)

BITS = (BOUNDX0, BOUNDX1, BOUNDY0, BOUNDY1, BOUNDZ0, BOUNDZ1)


def _tet_volumes(m):
    c = m.coord[m.connectivity.astype(np.int64)]
    a, b, d = c[:, 1] - c[:, 0], c[:, 2] - c[:, 0], c[:, 3] - c[:, 0]
    return np.einsum("ij,ij->i", a, np.cross(b, d)) / 6


def _tri_areas(m):
    c = m.coord[m.connectivity.astype(np.int64)]
    a, b = c[:, 1] - c[:, 0], c[:, 2] - c[:, 0]
    return 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])


@pytest.mark.parametrize("jitter,permute", [(0.0, False), (0.2, False), (0.2, True)])
def test_box3d_counts_orientation_and_volume(jitter, permute):
    nx, ny, nz = 7, 5, 4
    m = box3d(nx, ny, nz, 70e3, 50e3, 8e3, jitter=jitter, permute=permute, seed=3)
    assert m.nelem == 6 * nx * ny * nz and m.nnode == (nx + 1) * (ny + 1) * (nz + 1)
    v = _tet_volumes(m)
    assert (v > 0).all()
    assert v.sum() == pytest.approx(70e3 * 50e3 * 8e3, rel=1e-12)
    if not jitter:
        np.testing.assert_allclose(v, 70e3 / nx * 50e3 / ny * 8e3 / nz / 6, rtol=1e-12)
    assert m.coord[:, 2].min() == -8e3 and m.coord[:, 2].max() == 0.0


def test_box3d_permutation_keeps_the_elements():
    a = box3d(4, 3, 2, 1.0, 1.0, 1.0, jitter=0.1, seed=5)
    b = box3d(4, 3, 2, 1.0, 1.0, 1.0, jitter=0.1, permute=True, seed=5)
    np.testing.assert_array_equal(a.coord, b.coord)
    key = lambda c: sorted(map(tuple, c.tolist()))
    assert key(a.connectivity) == key(b.connectivity)
    assert not np.array_equal(a.connectivity, b.connectivity)


def test_box2d_counts_and_counter_clockwise():
    m = box2d(9, 4, 90e3, 10e3)
    assert m.nelem == 2 * 9 * 4 and m.nnode == 10 * 5
    area = _tri_areas(m)
    assert (area > 0).all()
    assert area.sum() == pytest.approx(90e3 * 10e3, rel=1e-12)


@pytest.mark.parametrize("nd", [2, 3])
def test_boundary_flags_and_facets(nd):
    m = box3d(5, 4, 3, 5.0, 4.0, 3.0) if nd == 3 else box2d(5, 3, 5.0, 3.0)
    x = m.coord
    lo, hi = x.min(axis=0), x.max(axis=0)
    axes = range(nd) if nd == 3 else (0, 1)
    bits = BITS if nd == 3 else (BOUNDX0, BOUNDX1, BOUNDZ0, BOUNDZ1)
    for k, ax in enumerate(axes):
        b0, b1 = bits[2 * k], bits[2 * k + 1]
        np.testing.assert_array_equal((m.bcflag & b0) != 0, x[:, ax] == lo[ax])
        np.testing.assert_array_equal((m.bcflag & b1) != 0, x[:, ax] == hi[ax])
    nof = NODE_OF_FACET_3D if nd == 3 else NODE_OF_FACET_2D
    cells = (5, 4, 3) if nd == 3 else (5, 3)
    for k, bit in enumerate(bits):
        ib = bit.bit_length() - 1   # facets are listed per boundary bit (z stays at 4, 5 in 2D)
        f = m.bfacets[m.bfacet_offsets[ib]:m.bfacet_offsets[ib + 1]]
        # one facet per boundary triangle (3D: 2 per face square) or segment (2D)
        ax = k // 2
        others = [c for a, c in enumerate(cells) if a != ax]
        assert len(f) == (2 if nd == 3 else 1) * int(np.prod(others))
        # ascending (element, local facet) order, every facet node on the boundary
        assert (np.diff(f[:, 0] * 4 + f[:, 1]) > 0).all()
        nodes = m.connectivity[f[:, 0][:, None], nof[f[:, 1]]]
        assert ((m.bcflag[nodes] & bit) != 0).all()


@pytest.mark.parametrize("permute", [False, True])
def test_support_lists_are_complete_and_ascending(permute):
    m = box3d(4, 3, 3, 1.0, 1.0, 1.0, jitter=0.15, permute=permute, seed=7)
    offs, ent = support_csr(m.connectivity, m.nnode)
    assert offs[0] == 0 and offs[-1] == m.nelem * 4
    e, slot = ent >> 2, ent & 3
    node_of_entry = np.repeat(np.arange(m.nnode), np.diff(offs))
    np.testing.assert_array_equal(m.connectivity[e, slot], node_of_entry)
    assert len(np.unique(ent)) == len(ent) == m.nelem * 4
    for n in range(m.nnode):
        es = e[offs[n]:offs[n + 1]]
        assert (np.diff(es) > 0).all(), n


def test_unpermuted_box_is_numbered_slab_by_slab():
    nx, ny, nz = 6, 4, 3
    m = box3d(nx, ny, nz, 6.0, 4.0, 3.0)
    elem_layer = np.arange(m.nelem) // (6 * ny * nz)
    node_layer = np.arange(m.nnode) // ((ny + 1) * (nz + 1))
    layers_of_elem = node_layer[m.connectivity]
    assert ((layers_of_elem == elem_layer[:, None]) | (layers_of_elem == elem_layer[:, None] + 1)).all()
    offs, ent = support_csr(m.connectivity, m.nnode)
    e_layer = elem_layer[ent >> 2]
    n_layer = np.repeat(node_layer, np.diff(offs))
    assert ((e_layer == n_layer) | (e_layer == n_layer - 1)).all()
    # both numberings are monotone in the layer
    assert (np.diff(elem_layer) >= 0).all() and (np.diff(node_layer) >= 0).all()


def test_edges_at_node0_give_the_reference_volume_and_shape_functions():
    """The mixed context's tet geometry (rel_volume, rel_shape_fn in
    csrc/des_kernels.cu) restated in numpy: from d_i = x_i - x_0 and the
    cross products c1 = d2 x d3, c2 = d3 x d1, c3 = d1 x d2, the volume
    d1 . c1 / 6 and the derivatives c_i / (6 vol), dN_0 = -(the others),
    agree with the reference's compute_volume and compute_shape_fn (the
    oracle) to a few ulps on a jittered, permuted mesh."""
    from dynearthsol_gb300.config import initial_state, make_workload
    from oracle.oracle import Oracle
    wl = make_workload("c1_3d_evp", cells=(4, 4, 3))
    wl.mesh = box3d(4, 4, 3, 100e3, 100e3, 10e3, jitter=0.2, permute=True, seed=3)
    st, cp = initial_state(wl)
    assert Oracle(wl, st, cp).init_fields() == 0
    x, c = wl.mesh.coord, wl.mesh.connectivity
    p = [x[c[:, i]] for i in range(4)]
    d1, d2, d3 = p[1] - p[0], p[2] - p[0], p[3] - p[0]
    c1, c2, c3 = np.cross(d2, d3), np.cross(d3, d1), np.cross(d1, d2)
    vol = np.einsum("ij,ij->i", d1, c1) / 6
    assert (vol > 0).all()
    assert np.abs(vol / st["volume"] - 1).max() < 1e-14
    g = [None] + [ci / (6 * vol)[:, None] for ci in (c1, c2, c3)]
    g[0] = -(g[1] + g[2] + g[3])
    for k, name in enumerate(("shpdx", "shpdy", "shpdz")):
        mine = np.stack([g[i][:, k] for i in range(4)], axis=1)
        assert np.abs(mine - st[name]).max() <= 1e-14 * np.abs(st[name]).max(), name
