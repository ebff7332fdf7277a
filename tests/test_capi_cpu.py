"""Host-side checks of the C ABI library and the reference-signature shim
(no GPU needed: nothing here launches device work)."""
import os
import subprocess

import pytest

from dynearthsol_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from dynearthsol_gb300 import build
    build.build()
    return capi.load_library()


def test_library_exports_every_declared_symbol(lib):
    declared = capi.declared_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared) <= exported


def test_version_and_error_text_are_host_only(lib):
    assert b"sm_103a" in lib.des_version()
    import ctypes as C
    buf = C.create_string_buffer(64)
    assert lib.des_last_error(None, buf, 64) == 0


def test_ctypes_structs_match_header_layout():
    """The Python mirror of the C structs has the C layout: compile a probe
    that prints sizeof/offsetof of the header's structs and compare."""
    import ctypes as C
    import tempfile
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "desgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(des_mesh), sizeof(des_params), sizeof(des_material), sizeof(des_host_state));
  printf("%zu %zu %zu %zu\n", offsetof(des_mesh, bnormals), offsetof(des_params, vbc_values),
         offsetof(des_material, elemmarkers), offsetof(des_host_state, steps));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        exe = os.path.join(d, "p")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        sizes, offs = [list(map(int, ln.split())) for ln in subprocess.check_output([exe], text=True).split("\n")[:2]]
    assert sizes == [C.sizeof(capi.DesMesh), C.sizeof(capi.DesParams), C.sizeof(capi.DesMaterial),
                     C.sizeof(capi.DesHostState)]
    assert offs == [capi.DesMesh.bnormals.offset, capi.DesParams.vbc_values.offset,
                    capi.DesMaterial.elemmarkers.offset, capi.DesHostState.steps.offset]


def _defined_functions(obj):
    out = subprocess.run(["nm", "-C", "--defined-only", obj], capture_output=True, text=True).stdout
    names = set()
    for ln in out.splitlines():
        parts = ln.split(None, 2)
        if len(parts) == 3 and parts[1] == "T":
            names.add(parts[2])
    return names


def _reference_sources():
    from oracle.oracle import reference_sources_available
    return reference_sources_available()


@pytest.mark.skipif(not _reference_sources(), reason="reference sources not staged (make -C oracle stage REF=...)")
@pytest.mark.parametrize("nd", [2, 3])
def test_shim_replaces_fields_geometry_rheology(lib, nd):
    """The shim links in place of the reference's fields.o, geometry.o and
    rheology.o: it defines every function they define (same C++ signatures)
    and links with the rest of the reference with no undefined symbol."""
    from oracle.oracle import build_reference
    assert build_reference()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "dynearthsol_gb300", "shim"),
                           f"ND={nd}", "lib"])
    build = os.path.join(ROOT, "dynearthsol_gb300", "shim", "_build")
    shim = _defined_functions(os.path.join(build, f"des_shim{nd}d.o"))
    refobj = os.path.join(ROOT, "oracle", "_ref", f"obj{nd}d")
    needed = set()
    for o in ("fields.o", "geometry.o", "rheology.o"):
        needed |= {n for n in _defined_functions(os.path.join(refobj, o)) if "(anonymous namespace)" not in n}
    missing = sorted(needed - shim)
    assert not missing, missing
    assert os.path.exists(os.path.join(build, f"libref_shim{nd}d.so"))
