"""The slab-pipelined host step.

With a complete, page-locked host state, des_step_host of one step overlaps
the host transfers with the step: the mesh is cut into slabs of elements and
nodes, slab b is uploaded while earlier slabs compute, and downloaded as soon
as its last stage has run.  The step's stages run per slab in an order that
respects every read and write across neighbouring slabs, so the result must
equal upload + step + download bit for bit.  Meshes whose numbering is not
slab by slab (permuted elements) take the general path.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from dynearthsol_gb300 import capi
    capi.load_library()


def _pinned(st):
    import torch
    out, keep = {}, []
    for k, v in st.items():
        t = torch.empty(v.shape, dtype=torch.float64, pin_memory=True)
        a = t.numpy()
        a[...] = v
        out[k] = a
        keep.append(t)
    return out, keep


def _run(wl, precision, calls):
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    st0, cp = initial_state(wl)
    ref = DeviceModel(wl, comp_pressure=cp, precision=precision)
    init = ref.init_fields(st0)
    clk = ref.clock()
    ref.upload({k: v.copy() for k, v in init.items()}, clk)
    ref.step(calls)
    want = ref.download()
    m = DeviceModel(wl, comp_pressure=cp, precision=precision)
    st, keep = _pinned(init)
    c = clk
    per_call = []
    for _ in range(calls):
        n0 = m.launches()
        c = m.step_host(st, 1, c)
        per_call.append(m.launches() - n0)
    assert c == ref.clock()
    for k in want:
        np.testing.assert_array_equal(st[k], want[k], err_msg=k)
    return per_call


# kernel launches of one pipelined call: 8 stages per coarse slab, dt, and one
# upload and one download conversion per coarse slab; the general path
# launches 9 step kernels and about 20 conversions
def _pipelined(per_call, slabs):
    return min(per_call) >= 8 * slabs + 1 + 2 * slabs


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_pipelined_step_host_is_bit_identical(prec):
    """16 x 6 x 4 cubes: 16 fine slabs of one x-layer, 4 coarse slabs; 12
    calls cross the 10th step, where dt is recomputed."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c1_3d_evp", cells=(16, 6, 4))
    per_call = _run(wl, capi.PREC_FP64 if prec == "fp64" else capi.PREC_MIXED, 12)
    assert _pipelined(per_call, 4), per_call


def test_pipelined_wide_coarse_slabs():
    """32 x 4 x 3 cubes: 32 fine slabs, 4 coarse slabs of 8."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c1_3d_evp", cells=(32, 4, 3))
    per_call = _run(wl, capi.PREC_MIXED, 12)
    assert _pipelined(per_call, 4), per_call


def test_permuted_mesh_takes_the_general_path():
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c4_3d_heat_jitter", cells=(16, 4, 3))
    per_call = _run(wl, capi.PREC_MIXED, 3)
    assert max(per_call) < 33, per_call


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_pipelined_with_yielding(prec):
    """The weakened, fast-loaded material of the yielding golden cases on a
    16 x 4 x 3 box: the return map and the EVP branch choice run in the
    slabs; plastic strain must appear."""
    from cases import _fast, _weak
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import initial_state, make_workload
    from dynearthsol_gb300.solver import DeviceModel
    wl = make_workload("c1_3d_evp", cells=(16, 4, 3))
    wl.params = _fast(wl.params)
    wl.mat = _weak(wl.mat)
    precision = capi.PREC_FP64 if prec == "fp64" else capi.PREC_MIXED
    per_call = _run(wl, precision, 12)
    assert _pipelined(per_call, 4), per_call
    st0, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp, precision=precision)
    init = m.init_fields(st0)
    m.upload(init, m.clock())
    m.step(12)
    assert np.count_nonzero(m.download()["plstrain"]) > 0


def test_pipelined_2d():
    """2D box of 32 x 4 rectangles (plane strain elasto-plastic): 32 fine
    slabs of one column, 4 coarse slabs."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c0_2d_ep", cells=(32, 4))
    per_call = _run(wl, capi.PREC_FP64, 12)
    assert _pipelined(per_call, 4), per_call


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_pipelined_dynamic_mode(prec):
    """Not quasi-static, without heat diffusion: the mass is the density's
    (uploaded, like tmass, not formed on the device), 16 x 4 x 3 cubes."""
    from dataclasses import replace
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import make_workload
    wl = make_workload("c1_3d_evp", cells=(16, 4, 3))
    wl.params = replace(wl.params, is_quasi_static=False, has_thermal_diffusion=False)
    per_call = _run(wl, capi.PREC_FP64 if prec == "fp64" else capi.PREC_MIXED, 12)
    assert _pipelined(per_call, 4), per_call
