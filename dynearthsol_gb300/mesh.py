"""Structured box meshes for the explicit-step workloads.

The reference meshes its box with Triangle/TetGen (mesh.cxx:338-516) and then
derives the boundary flags, boundary facets and node-to-element support lists
(mesh.cxx:1533-1721).  Remeshing and meshing stay on the host; this module
builds the same topology products directly for a structured box so that the
large synthetic workloads need no mesher:

* 3D: ``nx*ny*nz`` cubes, each split into 6 tetrahedra along its main
  diagonal (Kuhn/Freudenthal split), node order chosen so that the reference's
  signed volume (geometry.cxx:29-49) is positive;
* 2D: ``nx*nz`` rectangles, each split into 2 counter-clockwise triangles (the
  orientation ``compute_shape_fn``'s 2D formulas assume, geometry.cxx:440-448).

The box spans x in [0, xlength], y in [0, ylength], z in [-zlength, 0], as the
reference's box (mesh.cxx:355-375).  Boundary flags use the reference's bits
(constants.hpp:29-38); boundary facets are listed per boundary in ascending
(element, local facet) order, with the local facet numbering of
NODE_OF_FACET (constants.hpp:59-71).
"""
from __future__ import annotations

from dataclasses import dataclass, field
import itertools

import numpy as np

NBDRY = 10
BOUNDX0, BOUNDX1, BOUNDY0, BOUNDY1, BOUNDZ0, BOUNDZ1 = (1 << i for i in range(6))

NODE_OF_FACET_3D = np.array([[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]], dtype=np.int64)
NODE_OF_FACET_2D = np.array([[1, 2], [2, 0], [0, 1]], dtype=np.int64)


@dataclass
class Mesh:
    ndims: int
    coord: np.ndarray          # [nnode, ndims] float64
    connectivity: np.ndarray   # [nelem, ndims+1] int32
    bcflag: np.ndarray         # [nnode] uint32
    bfacet_offsets: np.ndarray  # [NBDRY+1] int32
    bfacets: np.ndarray        # [nbfacet, 2] int32 (element, facet)
    bnormals: np.ndarray = field(default_factory=lambda: np.zeros((NBDRY, 3)))
    edge_vectors: np.ndarray = field(default_factory=lambda: np.zeros((NBDRY, NBDRY, 3)))
    lengths: tuple = (0.0, 0.0, 0.0)
    cells: tuple = (0, 0, 0)

    @property
    def nnode(self) -> int:
        return self.coord.shape[0]

    @property
    def nelem(self) -> int:
        return self.connectivity.shape[0]


def _signed_tet_volume(c: np.ndarray, conn: np.ndarray) -> np.ndarray:
    """Signed volume with the reference's formula (geometry.cxx:29-49)."""
    d0, d1, d2, d3 = (c[conn[:, i]] for i in range(4))
    x01, x12, x23 = d0[:, 0] - d1[:, 0], d1[:, 0] - d2[:, 0], d2[:, 0] - d3[:, 0]
    y01, y12, y23 = d0[:, 1] - d1[:, 1], d1[:, 1] - d2[:, 1], d2[:, 1] - d3[:, 1]
    z01, z12, z23 = d0[:, 2] - d1[:, 2], d1[:, 2] - d2[:, 2], d2[:, 2] - d3[:, 2]
    return (x01 * (y23 * z12 - y12 * z23) + x12 * (y01 * z23 - y23 * z01)
            + x23 * (y12 * z01 - y01 * z12)) / 6


def _boundary_products(ndims, bcflag, conn):
    """bfacets per boundary (ascending element, facet) + offsets."""
    nof = NODE_OF_FACET_3D if ndims == 3 else NODE_OF_FACET_2D
    nfac = ndims + 1
    ne = conn.shape[0]
    lists = []
    for b in range(NBDRY):
        bit = np.uint32(1 << b)
        hits = []
        for f in range(nfac):
            on = np.ones(ne, dtype=bool)
            for j in range(ndims):
                on &= (bcflag[conn[:, nof[f, j]]] & bit) != 0
            e = np.nonzero(on)[0]
            hits.append(np.stack([e, np.full_like(e, f)], axis=1))
        h = np.concatenate(hits, axis=0)
        order = np.lexsort((h[:, 1], h[:, 0]))
        lists.append(h[order])
    offsets = np.zeros(NBDRY + 1, dtype=np.int32)
    for b in range(NBDRY):
        offsets[b + 1] = offsets[b] + lists[b].shape[0]
    bf = np.concatenate(lists, axis=0).astype(np.int32) if offsets[-1] else np.zeros((0, 2), np.int32)
    return offsets, np.ascontiguousarray(bf)


def boundary_normals(m: Mesh) -> None:
    """Unit outward normal of each boundary and the edge vectors of boundary
    pairs, as create_boundary_normals (bc.cxx:87-176) computes them."""
    nd = m.ndims
    nof = NODE_OF_FACET_3D if nd == 3 else NODE_OF_FACET_2D
    bn = np.zeros((NBDRY, 3))
    ev = np.zeros((NBDRY, NBDRY, 3))
    present = [m.bfacet_offsets[i + 1] > m.bfacet_offsets[i] for i in range(NBDRY)]
    for i in range(NBDRY):
        if not present[i]:
            continue
        rng = range(m.bfacet_offsets[i], m.bfacet_offsets[i + 1])
        for q in rng:
            e, f = m.bfacets[q]
            nodes = m.connectivity[e, nof[f]]
            c = m.coord
            if nd == 3:
                v01 = c[nodes[1]] - c[nodes[0]]
                v02 = c[nodes[2]] - c[nodes[0]]
                nrm = np.array([(v01[1] * v02[2] - v01[2] * v02[1]) / 2,
                                (v01[2] * v02[0] - v01[0] * v02[2]) / 2,
                                (v01[0] * v02[1] - v01[1] * v02[0]) / 2])
            else:
                v01 = c[nodes[1]] - c[nodes[0]]
                nrm = np.array([v01[1], -v01[0]])
            ln = np.sqrt(sum(nrm[d] * nrm[d] for d in range(nd)))
            nrm = nrm / ln
            if q == m.bfacet_offsets[i]:
                bn[i, :nd] = nrm
                if i < 6:
                    break
            else:
                diff2 = sum((bn[i, d] - nrm[d]) ** 2 for d in range(nd))
                if diff2 > 1e-12:
                    raise ValueError(f"boundary {i} is curved")
    for i in range(NBDRY):
        if not present[i]:
            continue
        for j in range(i + 1, NBDRY):
            if not present[j]:
                continue
            if nd == 3:
                if abs(bn[i, 2]) < 1e-15 and abs(bn[j, 2]) < 1e-15:
                    ev[i, j] = (0.0, 0.0, 1.0)
                else:
                    a, b = bn[i], bn[j]
                    ev[i, j] = (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                                a[0] * b[1] - a[1] * b[0])
            else:
                ev[i, j] = (0.0, 1.0, 0.0)
    m.bnormals = bn
    m.edge_vectors = ev


def box3d(nx: int, ny: int, nz: int, xlength: float, ylength: float, zlength: float,
          jitter: float = 0.0, permute: bool = False, seed: int = 0) -> Mesh:
    """3D box of nx*ny*nz cubes x 6 tetrahedra.

    jitter moves interior nodes uniformly by up to +-jitter cell spacings per
    axis; permute shuffles the element order (both seeded)."""
    dx, dy, dz = xlength / nx, ylength / ny, zlength / nz
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    coord = np.stack([i * dx, j * dy, -zlength + k * dz], axis=1).astype(np.float64)
    coord[i == nx, 0] = xlength
    coord[j == ny, 1] = ylength
    coord[k == nz, 2] = 0.0

    def nid(a, b, c):
        return (a * (ny + 1) + b) * (nz + 1) + c

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    tets = []
    for perm in itertools.permutations(range(3)):
        off = np.zeros(3, dtype=np.int64)
        verts = [off.copy()]
        for ax in perm:
            off = off.copy()
            off[ax] += 1
            verts.append(off)
        tets.append(np.stack([nid(ci + v[0], cj + v[1], ck + v[2]) for v in verts], axis=1))
    conn = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int64)

    bcflag = np.zeros(coord.shape[0], dtype=np.uint32)
    bcflag[i == 0] |= BOUNDX0
    bcflag[i == nx] |= BOUNDX1
    bcflag[j == 0] |= BOUNDY0
    bcflag[j == ny] |= BOUNDY1
    bcflag[k == 0] |= BOUNDZ0
    bcflag[k == nz] |= BOUNDZ1

    if jitter:
        rng = np.random.default_rng(seed)
        interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
        d = rng.uniform(-jitter, jitter, size=(interior.sum(), 3)) * np.array([dx, dy, dz])
        coord[interior] += d

    vol = _signed_tet_volume(coord, conn)
    neg = vol < 0
    conn[neg, 2], conn[neg, 3] = conn[neg, 3].copy(), conn[neg, 2].copy()
    vol = _signed_tet_volume(coord, conn)
    if not np.all(vol > 0):
        raise ValueError("non-positive tetrahedron volume in the generated mesh")
    if permute:
        rng = np.random.default_rng(seed + 1)
        conn = conn[rng.permutation(conn.shape[0])]
    conn = np.ascontiguousarray(conn.astype(np.int32))
    offs, bf = _boundary_products(3, bcflag, conn)
    m = Mesh(3, np.ascontiguousarray(coord), conn, bcflag, offs, bf,
             lengths=(xlength, ylength, zlength), cells=(nx, ny, nz))
    boundary_normals(m)
    return m


def box2d(nx: int, nz: int, xlength: float, zlength: float) -> Mesh:
    """2D box of nx*nz rectangles x 2 counter-clockwise triangles."""
    dx, dz = xlength / nx, zlength / nz
    i, k = np.meshgrid(np.arange(nx + 1), np.arange(nz + 1), indexing="ij")
    i, k = i.ravel(), k.ravel()
    coord = np.stack([i * dx, -zlength + k * dz], axis=1).astype(np.float64)
    coord[i == nx, 0] = xlength
    coord[k == nz, 1] = 0.0

    def nid(a, c):
        return a * (nz + 1) + c

    ci, ck = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    ci, ck = ci.ravel(), ck.ravel()
    n00, n10, n01, n11 = nid(ci, ck), nid(ci + 1, ck), nid(ci, ck + 1), nid(ci + 1, ck + 1)
    t0 = np.stack([n00, n10, n11], axis=1)   # counter-clockwise (x right, z up)
    t1 = np.stack([n00, n11, n01], axis=1)
    conn = np.stack([t0, t1], axis=1).reshape(-1, 3).astype(np.int32)
    bcflag = np.zeros(coord.shape[0], dtype=np.uint32)
    bcflag[i == 0] |= BOUNDX0
    bcflag[i == nx] |= BOUNDX1
    bcflag[k == 0] |= BOUNDZ0
    bcflag[k == nz] |= BOUNDZ1
    conn = np.ascontiguousarray(conn)
    offs, bf = _boundary_products(2, bcflag, conn)
    m = Mesh(2, np.ascontiguousarray(coord), conn, bcflag, offs, bf,
             lengths=(xlength, 0.0, zlength), cells=(nx, 0, nz))
    boundary_normals(m)
    return m


def support_csr(conn: np.ndarray, nnode: int):
    """Node-to-element support lists (create_support, mesh.cxx:1707-1721) in
    CSR form: offsets [nnode+1] and entries e*4 + local_slot, ascending in e."""
    ne, npe = conn.shape
    nodes = conn.ravel().astype(np.int64)
    ent = (np.repeat(np.arange(ne, dtype=np.int64), npe) * 4
           + np.tile(np.arange(npe, dtype=np.int64), ne))
    order = np.lexsort((ent, nodes))
    counts = np.bincount(nodes, minlength=nnode)
    offs = np.zeros(nnode + 1, dtype=np.int64)
    np.cumsum(counts, out=offs[1:])
    return offs, ent[order]
