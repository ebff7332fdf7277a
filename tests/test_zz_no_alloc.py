"""des_nmd_stress_noalloc: the nodal-mixed pressure smoothing for callers
that cannot allocate device memory (an application that owns every device
byte in its own pools, a process under a device-memory quota, code running
where cudaMalloc is not permitted).  The entry point takes only device
pointers the caller owns and keeps its per-node scratch in a fixed device
array, so this test owns the input and output arrays (torch tensors) and
checks the result against the context-based des_NMD_stress, bit for bit, on
three calls in a row: a larger 3D mesh first, then a smaller 2D mesh twice.
The 2D calls run on scratch that the 3D call left filled beyond their own
nodes, so a call that read a stale entry would show here.

This file is collected last on purpose, so that a run stopping at its first
failure has run every other test first."""
import ctypes as C

import numpy as np
import pytest

from cases import build_case
from conftest import load_golden, state_from

pytestmark = pytest.mark.gpu


def _context_nmd(wl, cp, st, clock):
    from dynearthsol_gb300.solver import DeviceModel
    m = DeviceModel(wl, comp_pressure=cp)
    m.upload({k: v.copy() for k, v in st.items()}, clock)
    m.call("NMD_stress")
    out = m.download()
    m.close()
    return out["stress"]


def _noalloc_nmd(lib, wl, st, stream):
    import torch
    from dynearthsol_gb300.mesh import support_csr
    mesh = wl.mesh
    nd, nn, ne = mesh.ndims, mesh.nnode, mesh.nelem
    dev = torch.device("cuda", 0)
    conn = torch.from_numpy(np.ascontiguousarray(mesh.connectivity.T.astype(np.int32))).to(dev)
    off, ent = support_csr(mesh.connectivity, nn)
    sup_off = torch.from_numpy(off.astype(np.int32)).to(dev)
    sup_ent = torch.from_numpy(ent.astype(np.int32)).to(dev)
    dp = torch.from_numpy(st["dpressure"].copy()).to(dev)
    vol = torch.from_numpy(st["volume"].copy()).to(dev)
    vol_n = torch.from_numpy(st["volume_n"].copy()).to(dev)
    stress = torch.from_numpy(np.ascontiguousarray(st["stress"].T)).to(dev)   # [nstr][nelem]
    torch.cuda.synchronize()
    rc = lib.des_nmd_stress_noalloc(nd, nn, ne, conn.data_ptr(), sup_off.data_ptr(), sup_ent.data_ptr(),
                                    dp.data_ptr(), vol.data_ptr(), vol_n.data_ptr(), stress.data_ptr(),
                                    C.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    return np.ascontiguousarray(stress.cpu().numpy().T)


def test_noalloc_nmd_matches_context_entry_point_twice():
    import torch
    from dynearthsol_gb300 import capi
    lib = capi.load_library()
    stream = torch.cuda.Stream()
    # the larger 3D case first, then the smaller 2D case twice
    for name, group in (("3d_heat_jitter_multimat", "mid"), ("2d_evp_heat", "mid"), ("2d_evp_heat", "mid")):
        g = load_golden(name)
        wl, _ = build_case(name)
        st = state_from(g[group])
        c = g[group]["clock"]
        ref = _context_nmd(wl, float(g["init"]["compensation_pressure"]), st, (c[0], c[1], int(c[2])))
        got = _noalloc_nmd(lib, wl, st, stream)
        # the same operations in the same order as des_NMD_stress: equal bits
        np.testing.assert_array_equal(got, ref, err_msg=name)
        # the first ndims components changed, the shear components did not
        assert not np.array_equal(got[:, :wl.mesh.ndims], st["stress"][:, :wl.mesh.ndims])
        np.testing.assert_array_equal(got[:, wl.mesh.ndims:], st["stress"][:, wl.mesh.ndims:])


def test_noalloc_rejects_meshes_beyond_the_scratch():
    from dynearthsol_gb300 import capi
    lib = capi.load_library()
    # rejected before any device work (pointers are never dereferenced)
    big = 2097152 + 1
    rc = lib.des_nmd_stress_noalloc(3, big, 10, 1, 1, 1, 1, 1, 1, 1, None)
    assert rc == capi.DES_EINPUT
