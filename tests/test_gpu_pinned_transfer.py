"""Pipelined state transfer and the host-buffer step call.

Every state transfer copies the host rows field after field on a copy
stream and converts the layout on the compute stream in between, and
des_step_host copies the fields that the step's tail no longer writes while
that tail runs.  None of this may change a bit: the tests compare against
upload + step + download issued as separate calls, for pinned, pageable and
mixed host memory, FP64 and mixed precision, 2D and 3D.
"""
import ctypes as C

import numpy as np
import pytest

from cases import build_case
from conftest import load_golden, state_from

pytestmark = pytest.mark.gpu

CASES = ("3d_heat_jitter_multimat", "2d_evp_heat", "3d_evp_yield")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from dynearthsol_gb300 import capi
    capi.load_library()


def _setup(name):
    from dynearthsol_gb300.solver import DeviceModel
    g = load_golden(name)
    wl, _ = build_case(name)
    cp = float(g["init"]["compensation_pressure"])
    c = g["init"]["clock"]
    mk = lambda prec=None: DeviceModel(wl, comp_pressure=cp) if prec is None else \
        DeviceModel(wl, comp_pressure=cp, precision=prec)
    return g, mk, (c[0], c[1], int(c[2]))


def _pinned(st, which=None):
    """Copies of the state's arrays, those in `which` (all when None) in
    pinned memory; returns the arrays and the tensors that own them."""
    import torch
    out, keep = {}, []
    for k, v in st.items():
        if which is not None and k not in which:
            out[k] = v.copy()
            continue
        t = torch.empty(v.shape, dtype=torch.float64, pin_memory=True)
        a = t.numpy()
        a[...] = v
        out[k] = a
        keep.append(t)
    return out, keep


def _same(a, b):
    for k in b:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("name", CASES)
def test_step_host_equals_separate_calls_pinned_and_pageable(name):
    g, mk, clk = _setup(name)
    ref = mk()
    ref.upload(state_from(g["init"]), clk)
    ref.step(7)
    want = ref.download()
    pageable = state_from(g["init"])
    pinned, keep = _pinned(state_from(g["init"]))
    half = [k for i, k in enumerate(sorted(pageable)) if i % 2 == 0]
    mixed, keep2 = _pinned(state_from(g["init"]), which=half)
    for st in (pageable, pinned, mixed):
        assert mk().step_host(st, 7, clk) == ref.clock()
        _same(st, want)


@pytest.mark.parametrize("name", ("3d_heat_jitter_multimat", "3d_evp_yield"))
def test_step_host_mixed_precision_equals_separate_calls(name):
    from dynearthsol_gb300 import capi
    g, mk, clk = _setup(name)
    ref = mk(capi.PREC_MIXED)
    ref.upload(state_from(g["init"]), clk)
    ref.step(5)
    want = ref.download()
    st, keep = _pinned(state_from(g["init"]))
    assert mk(capi.PREC_MIXED).step_host(st, 5, clk) == ref.clock()
    _same(st, want)


def test_one_step_calls_chain_like_one_run():
    """Ten one-step calls on the same host buffers equal one ten-step run:
    the staging regions and events are reused call after call."""
    g, mk, clk = _setup("3d_heat_jitter_multimat")
    ref = mk()
    ref.upload(state_from(g["init"]), clk)
    ref.step(10)
    want = ref.download()
    st, keep = _pinned(state_from(g["init"]))
    m = mk()
    c = clk
    for _ in range(10):
        c = m.step_host(st, 1, c)
    assert c == ref.clock()
    _same(st, want)


def test_zero_steps_and_per_field_calls():
    from dynearthsol_gb300 import capi
    g, mk, clk = _setup("3d_heat_jitter_multimat")
    st0 = state_from(g["init"])
    st, keep = _pinned(state_from(g["init"]))
    m = mk()
    assert m.step_host(st, 0, clk) == clk
    _same(st, st0)
    m.step(3)
    mask = capi.F_ALL & ~capi.F_CLOCK
    out_pin, keep2 = _pinned({k: np.zeros_like(v) for k, v in st.items()})
    out_pg = {k: np.zeros_like(v) for k, v in st.items()}
    for dst in (out_pin, out_pg):
        hs = capi.host_state_struct(dst)
        assert m.lib.des_download_fields(m.ctx, C.byref(hs), mask) == 0
    _same(out_pin, out_pg)
    ref = m.download()
    _same(out_pg, ref)
    # uploading the downloaded fields back leaves the state unchanged
    hs = capi.host_state_struct(out_pin)
    assert m.lib.des_upload_fields(m.ctx, C.byref(hs), mask) == 0
    _same(m.download(), ref)
