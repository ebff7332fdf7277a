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

    def download_fields(self, names) -> dict:
        """Only the named state arrays (des_download_fields)."""
        m = self.wl.mesh
        full = empty_state(m.ndims, m.nnode, m.nelem)
        st = {k: full[k] for k in names}
        mask = 0
        for k in names:
            mask |= capi.F_SHP if k.startswith("shp") else capi.F_BITS[k]
        hs = capi.host_state_struct(st)
        self._check(self.lib.des_download_fields(self.ctx, C.byref(hs), mask))
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

    def bad_mesh_quality(self, smallest_size, resolution, min_quality, max_boundary_distortion,
                         remeshing_option):
        """bad_mesh_quality (remeshing.cxx:1882-1935) on the device: (code,
        index, value); index and value are None when the code is 0."""
        qp = capi.DesQualityParams(smallest_size, resolution, min_quality, max_boundary_distortion,
                                   remeshing_option)
        code, idx, val = C.c_int(), C.c_int(-1), C.c_double()
        self._check(self.lib.des_bad_mesh_quality(self.ctx, C.byref(qp), C.byref(code), C.byref(idx),
                                                  C.byref(val)))
        if code.value == 0:
            return 0, None, None
        return code.value, idx.value, val.value

    # -- remeshing --
    def remesh(self, wl: Workload, topology=None):
        """des_remesh: the context's mesh becomes wl's (support lists and
        boundary facets built on the device from its segments); upload the
        state afterwards."""
        topo = topology or capi.Topology(wl.mesh)
        em = None if wl.mat.elemmarkers is None else np.ascontiguousarray(wl.mat.elemmarkers, dtype=np.int32)
        self._topo = topo
        self._check(self.lib.des_remesh(self.ctx, C.byref(topo.struct), capi.iptr(em)))
        self.wl = wl
        self.cs = CStructs(wl, self.comp_pressure)
        self._ef = {}

    # -- markers and phase changes --
    def set_markers(self, elem: np.ndarray, eta: np.ndarray, mattype: np.ndarray):
        """Markers (element, barycentric eta [n][ndims+1], material type) to the device."""
        self._markers = (np.ascontiguousarray(elem, dtype=np.int32), np.ascontiguousarray(eta, dtype=np.float64),
                         np.ascontiguousarray(mattype, dtype=np.int32))
        e, t, m = self._markers
        self._check(self.lib.des_set_markers(self.ctx, e.shape[0], capi.iptr(e), capi.dptr(t), capi.iptr(m)))

    def phase_changes(self, option: int, hydrous: np.ndarray | None = None) -> int:
        """phase_changes on the device; returns the number of markers changed."""
        h = None if hydrous is None else np.ascontiguousarray(hydrous, dtype=np.int32)
        n = C.c_int()
        self._check(self.lib.des_phase_changes(self.ctx, option, capi.iptr(h), C.byref(n)))
        return n.value

    def get_markers(self):
        """(material types [nmarkers], marker counts [nelem][nmat]) from the device."""
        nm = self._markers[0].shape[0] if getattr(self, "_markers", None) else 0
        mt = np.zeros(nm, np.int32)
        em = np.zeros((self.wl.mesh.nelem, self.wl.mat.nmat), np.int32)
        self._check(self.lib.des_get_markers(self.ctx, capi.iptr(mt), capi.iptr(em)))
        return mt, em

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

    # -- parameters --
    def set_elem_field(self, field: int, values: np.ndarray):
        """Per-element override (capi.EF_*) of a material property."""
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._ef[field] = a
        self._check(self.lib.des_set_elem_field(self.ctx, field, capi.dptr(a)))

    def set_params(self, **changes):
        """Change run-time parameters (des_params fields) of the context."""
        for k, v in changes.items():
            if k == "vbc_values":
                for i, x in enumerate(v):
                    self.cs.params.vbc_values[i] = float(x)
            else:
                setattr(self.cs.params, k, v)
        self._check(self.lib.des_set_params(self.ctx, C.byref(self.cs.params)))

    # -- reverse mode --
    ADJOINT_FIELDS = ("coord", "vel", "temperature", "stress", "plstrain", "volume_old")

    def adjoint_forward(self, nsteps: int, checkpoint_every: int):
        """Run a window of nsteps steps (dt held) recording a checkpoint every
        checkpoint_every steps and the last segment's tape (the whole
        window's when checkpoint_every >= nsteps)."""
        self._check(self.lib.des_adjoint_forward(self.ctx, nsteps, checkpoint_every))

    def adjoint_backward(self, seed: dict, want_start: bool = True):
        """Reverse sweep of the recorded window.  seed: adjoints of the final
        state (any of ADJOINT_FIELDS, reference layout).  Returns (start, grad):
        the adjoints of the window's start state and a dict with one [nelem]
        gradient per capi.EF_* field and 'vbc_values' [10]."""
        m = self.wl.mesh
        nd, nn, ne = m.ndims, m.nnode, m.nelem
        shapes = {"coord": (nn, nd), "vel": (nn, nd), "temperature": (nn,), "stress": (ne, nstr_of(nd)),
                  "plstrain": (ne,), "volume_old": (ne,)}
        sd = {k: np.ascontiguousarray(seed[k], dtype=np.float64) for k in self.ADJOINT_FIELDS if k in seed}
        for k, a in sd.items():
            if a.shape != shapes[k]:
                raise ValueError(f"seed {k}: shape {a.shape}, expected {shapes[k]}")
        hs_seed = capi.host_state_struct(sd)
        start = {k: np.zeros(shapes[k]) for k in self.ADJOINT_FIELDS} if want_start else {}
        hs_start = capi.host_state_struct(start)
        g = capi.DesAdjointGrad()
        garr = [np.zeros(ne) for _ in range(capi.EF_COUNT)]
        for k in range(capi.EF_COUNT):
            g.elem[k] = capi.dptr(garr[k])
        self._check(self.lib.des_adjoint_backward(self.ctx, C.byref(hs_seed),
                                                  C.byref(hs_start) if want_start else None, C.byref(g)))
        grad = {k: garr[k] for k in range(capi.EF_COUNT)}
        grad["vbc_values"] = np.array(list(g.vbc_values))
        return start, grad
