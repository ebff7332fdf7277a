"""The .save output writer (des_write_save_host) against the reference's own
BinaryOutput (binaryio.cxx, compiled from the reference sources into
oracle/_ref by oracle/Makefile): the same arrays give byte-identical files.
No GPU is needed: the host writer does no device work.  Skipped where the
reference sources were not available to build oracle/_ref."""
import ctypes as C
import os

import numpy as np
import pytest


def _frame(nd, nn, ne, rng):
    from dynearthsol_gb300 import capi
    nstr = nd * (nd + 1) // 2
    arrs = {
        "coord": rng.standard_normal((nn, nd)), "connectivity": rng.integers(0, nn, (ne, nd + 1)).astype(np.int32),
        "vel": rng.standard_normal((nn, nd)), "temperature": rng.standard_normal(nn),
        "plstrain": rng.random(ne), "delta_plstrain": rng.random(ne) * 1e-6,
        "strain_rate": rng.standard_normal((ne, nstr)), "strain": rng.standard_normal((ne, nstr)),
        "stress": rng.standard_normal((ne, nstr)) * 1e8, "density": 3000 + rng.random(ne),
        "mesh_quality": rng.random(ne), "viscosity": 10 ** (20 + rng.random(ne)),
        "material": rng.integers(0, 3, ne).astype(np.float64), "force": rng.standard_normal((nn, nd)),
        "coord0": rng.standard_normal((nn, nd)), "bcflag": rng.integers(0, 1024, nn).astype(np.uint32),
    }
    fr = capi.DesSaveFrame()
    fr.ndims, fr.nnode, fr.nelem = nd, nn, ne
    for k in capi.SAVE_FIELDS:
        a = arrs[k]
        ptr = capi.iptr(a) if k == "connectivity" else (capi.uptr(a) if k == "bcflag" else capi.dptr(a))
        setattr(fr, k, ptr)
    return fr, arrs


@pytest.mark.parametrize("nd", [2, 3])
def test_save_writer_matches_reference_binaryio(nd, tmp_path):
    from dynearthsol_gb300 import capi
    from oracle.oracle import REF_DIR
    path = os.path.join(REF_DIR, f"libref{nd}d.so")
    if not os.path.exists(path):
        pytest.skip("reference not built here (oracle/_ref)")
    ref = C.CDLL(path)
    ref.ref_write_save.argtypes = [C.c_char_p, C.POINTER(capi.DesSaveFrame)]
    ref.ref_write_save.restype = C.c_int
    lib = capi.load_library()
    rng = np.random.default_rng(nd)
    fr, arrs = _frame(nd, 37, 53, rng)
    a, b = tmp_path / "mine.save.000000", tmp_path / "ref.save.000000"
    assert lib.des_write_save_host(str(a).encode(), C.byref(fr)) == 0
    assert ref.ref_write_save(str(b).encode(), C.byref(fr)) == 0
    assert a.read_bytes() == b.read_bytes()
    got = capi.read_save(str(a))
    assert got["ndims"] == nd
    names = {"coord": "coordinate", "connectivity": "connectivity", "vel": "velocity",
             "temperature": "temperature", "plstrain": "plastic strain", "delta_plstrain": "plastic strain-rate",
             "strain_rate": "strain-rate", "strain": "strain", "stress": "stress", "density": "density",
             "mesh_quality": "mesh quality", "viscosity": "viscosity", "material": "material", "force": "force",
             "coord0": "coord0", "bcflag": "bcflag"}
    assert got["_order"] == [names[k] for k in capi.SAVE_FIELDS]
    for k, name in names.items():
        np.testing.assert_array_equal(got[name], arrs[k].ravel(), err_msg=k)


def test_save_writer_rejects_bad_input(tmp_path):
    from dynearthsol_gb300 import capi
    lib = capi.load_library()
    fr, _ = _frame(3, 5, 4, np.random.default_rng(0))
    fr.ndims = 4
    assert lib.des_write_save_host(str(tmp_path / "x").encode(), C.byref(fr)) == capi.DES_EINPUT
    fr.ndims = 3
    fr.stress = capi.dptr(None)
    assert lib.des_write_save_host(str(tmp_path / "x").encode(), C.byref(fr)) == capi.DES_EINPUT
