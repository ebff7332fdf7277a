"""Python handle on a device context of libdesgpu.so (the C ABI in
include/desgpu.h).  Used by the tests and the benchmark; a C++ host uses the
same entry points directly (see dynearthsol_gb300/shim).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .config import CStructs, Workload, initial_state, nstr_of

STATE_KEYS = capi.STATE_ARRAYS


def empty_state(nd: int, nn: int, ne: int) -> dict:
    nstr, npe = nstr_of(nd), nd + 1
    z = np.zeros
    return {
        "coord": z((nn, nd)), "coord0": z((nn, nd)), "vel": z((nn, nd)), "force": z((nn, nd)),
        "temperature": z(nn), "mass": z(nn), "tmass": z(nn), "volume_n": z(nn), "ntmp": z(nn),
        "volume": z(ne), "volume_old": z(ne), "stress": z((ne, nstr)), "strain": z((ne, nstr)),
        "strain_rate": z((ne, nstr)), "plstrain": z(ne), "delta_plstrain": z(ne),
        "stressyy": z(ne), "dpressure": z(ne), "edvoldt": z(ne),
        "shpdx": z((ne, npe)), "shpdy": z((ne, npe)), "shpdz": z((ne, npe)),
    }


class DeviceModel:
    """One device context for one workload."""

    def __init__(self, wl: Workload, comp_pressure: float | None = None,
                 precision: int = capi.PREC_FP64, stream: int | None = None):
        self.lib = capi.load_library()
        self.wl = wl
        if comp_pressure is None:
            comp_pressure = initial_state(wl)[1]
        self.comp_pressure = comp_pressure
        self.cs = CStructs(wl, comp_pressure)
        self.ctx = C.c_void_p()
        rc = self.lib.des_create(C.byref(self.cs.mesh), C.byref(self.cs.params),
                                 C.byref(self.cs.mat), precision,
                                 C.c_void_p(stream) if stream else None, C.byref(self.ctx))
        if rc:
            raise capi.DesError(rc, self._err(None))
        self._ef = {}
        for k, v in wl.elem_fields.items():
            a = np.ascontiguousarray(v, dtype=np.float64)
            self._ef[k] = a
            self._check(self.lib.des_set_elem_field(self.ctx, k, capi.dptr(a)))

    # -- errors --
    def _err(self, ctx) -> str:
        buf = C.create_string_buffer(512)
        self.lib.des_last_error(ctx, buf, 512)
        return buf.value.decode()

    def _check(self, rc: int):
        if rc:
            raise capi.DesError(rc, self._err(self.ctx))

    def close(self):
        if getattr(self, "ctx", None) and self.ctx.value:
            self.lib.des_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nd(self):
        return self.wl.mesh.ndims

    # -- state --
    def upload(self, st: dict, clock=(0.0, 0.0, 0)):
        hs = capi.host_state_struct(st, *clock)
        self._check(self.lib.des_upload_state(self.ctx, C.byref(hs)))

    def download(self, st: dict | None = None) -> dict:
        m = self.wl.mesh
        if st is None:
            st = empty_state(m.ndims, m.nnode, m.nelem)
        hs = capi.host_state_struct(st)
        self._check(self.lib.des_download_state(self.ctx, C.byref(hs)))
        return st

    def clock(self):
        t, dt, s = C.c_double(), C.c_double(), C.c_int()
        self._check(self.lib.des_get_clock(self.ctx, C.byref(t), C.byref(dt), C.byref(s)))
        return t.value, dt.value, s.value

    def set_clock(self, time, dt, steps):
        self._check(self.lib.des_set_clock(self.ctx, time, dt, steps))

    def init_fields(self, st: dict) -> dict:
        """The reference's init sequence (dynearthsol.cxx:86-94,316) on the
        device: volumes, volume_old = volume, masses (computed, as init()
        does, before the temperature is set), shape functions, velocity BCs,
        then dt.  Returns the initialised host state."""
        T = st["temperature"].copy()
        s0 = {k: v for k, v in st.items()
              if k not in ("volume", "mass", "tmass", "volume_n", "shpdx", "shpdy", "shpdz")}
        s0["temperature"] = np.zeros_like(T)
        self.upload(s0)
        self._check(self.lib.des_swap_volume(self.ctx))
        self._check(self.lib.des_apply_vbcs(self.ctx))
        out = self.download()
        out["temperature"] = T
        self.upload(out)
        dt = C.c_double()
        self._check(self.lib.des_compute_dt(self.ctx, C.byref(dt)))
        self.set_clock(0.0, dt.value, 0)
        return self.download()

    # -- compute --
    def step(self, n: int = 1):
        self._check(self.lib.des_step(self.ctx, n))

    def step_host(self, st: dict, n: int, clock) -> tuple:
        hs = capi.host_state_struct(st, *clock)
        self._check(self.lib.des_step_host(self.ctx, C.byref(hs), n))
        return hs.time, hs.dt, hs.steps

    def call(self, name: str):
        """One per-function entry point, e.g. call('update_stress')."""
        if name == "compute_dt":
            dt = C.c_double()
            self._check(self.lib.des_compute_dt(self.ctx, C.byref(dt)))
            return dt.value
        if name == "worst_elem_quality":
            q, w = C.c_double(), C.c_int()
            self._check(self.lib.des_worst_elem_quality(self.ctx, C.byref(q), C.byref(w)))
            return q.value, w.value
        self._check(getattr(self.lib, "des_" + name)(self.ctx))

    def sync(self):
        self._check(self.lib.des_synchronize(self.ctx))

    def device_status(self) -> int:
        bits = C.c_uint()
        self._check(self.lib.des_device_status(self.ctx, C.byref(bits)))
        return bits.value

    def launches(self) -> int:
        n = C.c_longlong()
        self._check(self.lib.des_launch_count(self.ctx, C.byref(n)))
        return n.value
