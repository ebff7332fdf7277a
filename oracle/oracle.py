"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

* ``Oracle``: the C restatement in des_oracle.c (liboracle.so), runnable on
  any host; tests, the smoke check and bench.py's CPU-baseline leg use it as
  the checker.
* ``Reference``: the reference's own hot-path sources compiled by
  ``make -C oracle ref`` (oracle/_ref/libref{2,3}d.so) from the staged copy
  of its sources (oracle/_ref/src); only where those are staged.  Used to
  pin the restatement, to generate the golden fixtures, as the CPU baseline
  (the OpenMP build) and, linked with the device shim, to run the
  reference's own loop body on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from dynearthsol_gb300 import capi
from dynearthsol_gb300.config import CStructs, Workload, nstr_of

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORACLE = os.path.join(HERE, "liboracle.so")
LIBORACLE_PERT = os.path.join(HERE, "liboracle_pert.so")
REF_DIR = os.path.join(HERE, "_ref")


def build_oracle(force: bool = False, perturbed: bool = False) -> str:
    src = os.path.join(HERE, "des_oracle.c")
    lib = LIBORACLE_PERT if perturbed else LIBORACLE
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return lib


def reference_sources_available() -> bool:
    """The reference's sources are staged under oracle/_ref/src, or the
    reference tree is named by DES_REFERENCE_DIR (make -C oracle stage)."""
    return bool(os.environ.get("DES_REFERENCE_DIR")) or os.path.isfile(os.path.join(REF_DIR, "src", "fields.cxx"))


def build_reference(targets=("ref",)) -> bool:
    """Compile the reference sources (make -C oracle ref), staging them first
    from DES_REFERENCE_DIR when that is set; False when neither the staged
    sources nor the tree are available."""
    if not reference_sources_available():
        return False
    ref = os.environ.get("DES_REFERENCE_DIR")
    subprocess.check_call(["make", "-s", "-j8", "-C", HERE, *targets] + ([f"REF={ref}"] if ref else []))
    return True


def state_copy(st: dict) -> dict:
    return {k: np.array(v, copy=True) for k, v in st.items()}


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


_FUNCS = ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
          "NMD_stress", "update_force", "update_velocity", "apply_vbcs", "update_coordinate",
          "swap_volume", "compute_volume", "compute_mass", "compute_shape_fn", "rotate_stress"]


class Oracle:
    """The C restatement bound to one workload and one state dict."""

    def __init__(self, wl: Workload, st: dict, comp_pressure: float, nthreads: int = 1,
                 clock=(0.0, 0.0, 0), perturb_seed: int | None = None):
        """perturb_seed selects the libm-sensitivity build (transcendental
        results moved by +-1 ulp, seeded)."""
        self.lib = C.CDLL(build_oracle(perturbed=perturb_seed is not None))
        if perturb_seed is not None:
            self.lib.oracle_perturb_seed.argtypes = [C.c_ulonglong]
            self.lib.oracle_perturb_seed(perturb_seed)
        L = self.lib
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                                    C.POINTER(capi.DesMaterial), C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_bind_state.argtypes = [C.c_void_p, C.POINTER(capi.DesHostState)]
        L.oracle_set_elem_field.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        L.oracle_run.argtypes = [C.c_void_p, C.c_int]
        L.oracle_threads.argtypes = [C.c_void_p]
        L.oracle_init_fields.argtypes = [C.c_void_p]
        L.oracle_update_stress.argtypes = [C.c_void_p]
        L.oracle_compute_dt.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_worst_elem_quality.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.oracle_worst_elem_quality.restype = C.c_double
        L.oracle_eigen3.argtypes = [C.POINTER(C.c_double)] * 3 + [C.POINTER(C.c_int)]
        for f in _FUNCS:
            getattr(L, "oracle_" + f).argtypes = [C.c_void_p]
        self.wl = wl
        self.cs = CStructs(wl, comp_pressure)
        self.st = st
        self.hs = capi.host_state_struct(st, *clock)
        self.ctx = L.oracle_create(C.byref(self.cs.mesh), C.byref(self.cs.params),
                                   C.byref(self.cs.mat), nthreads)
        L.oracle_bind_state(self.ctx, C.byref(self.hs))
        self._ef = {}
        for k, v in wl.elem_fields.items():
            a = np.ascontiguousarray(v, dtype=np.float64)
            self._ef[k] = a
            L.oracle_set_elem_field(self.ctx, k, capi.dptr(a))

    def __del__(self):
        if getattr(self, "ctx", None):
            self.lib.oracle_destroy(self.ctx)
            self.ctx = None

    @property
    def clock(self):
        return self.hs.time, self.hs.dt, self.hs.steps

    def init_fields(self) -> int:
        return self.lib.oracle_init_fields(self.ctx)

    def run(self, nsteps: int) -> int:
        return self.lib.oracle_run(self.ctx, nsteps)

    @property
    def threads(self) -> int:
        """Threads the element loops use (fewer than asked where the
        two-colour bands would share nodes)."""
        return self.lib.oracle_threads(self.ctx)

    def call(self, name: str):
        if name == "update_stress":
            return self.lib.oracle_update_stress(self.ctx)
        if name == "compute_dt":
            dt = C.c_double()
            rc = self.lib.oracle_compute_dt(self.ctx, C.byref(dt))
            self.hs.dt = dt.value
            return rc, dt.value
        if name == "worst_elem_quality":
            w = C.c_int()
            q = self.lib.oracle_worst_elem_quality(self.ctx, C.byref(w))
            return q, w.value
        return getattr(self.lib, "oracle_" + name)(self.ctx)


def eigen3(a6):
    lib = C.CDLL(build_oracle())
    lib.oracle_eigen3.argtypes = [C.POINTER(C.c_double)] * 3 + [C.POINTER(C.c_int)]
    a = np.ascontiguousarray(a6, dtype=np.float64)
    w = np.zeros(3)
    q = np.zeros(9)
    ql = C.c_int()
    rc = lib.oracle_eigen3(capi.dptr(a), capi.dptr(w), capi.dptr(q), C.byref(ql))
    return rc, w, q.reshape(3, 3), ql.value


class RefIC(C.Structure):
    _fields_ = [("weakzone_option", C.c_int)] + [(n, C.c_double) for n in (
        "weakzone_plstrain", "weakzone_azimuth", "weakzone_inclination", "weakzone_halfwidth",
        "weakzone_y_min", "weakzone_y_max", "weakzone_depth_min", "weakzone_depth_max",
        "weakzone_xcenter", "weakzone_ycenter", "weakzone_zcenter",
        "weakzone_xsemi_axis", "weakzone_ysemi_axis", "weakzone_zsemi_axis",
        "xlength", "ylength", "zlength", "resolution")]


class RefQuality(C.Structure):
    """The Param::mesh fields bad_mesh_quality reads (ref_quality in
    oracle/ref_harness.cxx)."""
    _fields_ = [(n, C.c_double) for n in ("smallest_size", "resolution", "min_quality",
                                          "max_boundary_distortion", "zlength")] + [("remeshing_option", C.c_int)]


SHIM_BUILD = os.path.join(os.path.dirname(HERE), "dynearthsol_gb300", "shim", "_build")


class Reference:
    """The reference's own functions (compiled from its sources).

    flavour "serial" is the 1-thread parity build (libref{2,3}d.so), "omp"
    the OpenMP build (libref3d_omp.so, the CPU baseline), and "shim" the
    reference harness and the reference's other objects linked with the
    device shim in place of fields.o, geometry.o and rheology.o
    (dynearthsol_gb300/shim: the reference's loop body on the GPU)."""

    def __init__(self, ndims: int, flavour: str = "serial"):
        if flavour == "serial":
            path = os.path.join(REF_DIR, f"libref{ndims}d.so")
        elif flavour == "omp":
            path = os.path.join(REF_DIR, f"libref{ndims}d_omp.so")
        elif flavour == "shim":
            path = os.path.join(SHIM_BUILD, f"libref_shim{ndims}d.so")
        else:
            raise ValueError(flavour)
        if not os.path.exists(path):
            raise OSError(f"{path} missing (make -C oracle ref refomp; make -C dynearthsol_gb300/shim lib)")
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_run_timed.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                                    C.POINTER(capi.DesMaterial), C.POINTER(capi.DesHostState), C.c_int,
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ref_bad_mesh_quality.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                                           C.POINTER(capi.DesMaterial), C.POINTER(RefQuality),
                                           C.POINTER(capi.DesHostState), C.POINTER(C.c_int)]
        L.ref_nthreads.restype = C.c_int
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_create_support.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]
        L.ref_create_boundary_facets.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_uint),
                                                 C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                 C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_phase_changes.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                                        C.POINTER(capi.DesMaterial), C.POINTER(capi.DesHostState), C.c_int,
                                        C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_init.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                               C.POINTER(capi.DesMaterial), C.POINTER(RefIC),
                               C.POINTER(capi.DesHostState), C.POINTER(C.c_double),
                               C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ref_run.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                              C.POINTER(capi.DesMaterial), C.POINTER(capi.DesHostState), C.c_int,
                              C.POINTER(C.c_double)]
        L.ref_call.argtypes = [C.POINTER(capi.DesMesh), C.POINTER(capi.DesParams),
                               C.POINTER(capi.DesMaterial), C.POINTER(capi.DesHostState),
                               C.c_char_p, C.POINTER(C.c_double)]
        assert L.ref_ndims() == ndims

    def init(self, wl: Workload, st: dict):
        """Reference init on st (temperature = input geotherm); returns
        (bnormals[10,3], edge_vectors[10,10,3], compensation_pressure, clock)."""
        cs = CStructs(wl, 0.0)
        wz = wl.weakzone
        ic = RefIC(wz.option, wz.plstrain, wz.azimuth, wz.inclination, wz.halfwidth,
                   wz.y_min, wz.y_max, wz.depth_min, wz.depth_max, wz.xcenter, wz.ycenter,
                   wz.zcenter, wz.xsemi_axis, wz.ysemi_axis, wz.zsemi_axis,
                   wl.mesh.lengths[0], wl.mesh.lengths[1], wl.mesh.lengths[2], wl.resolution)
        hs = capi.host_state_struct(st)
        bn = np.zeros(30)
        ev = np.zeros(300)
        cp = C.c_double()
        self.lib.ref_init(C.byref(cs.mesh), C.byref(cs.params), C.byref(cs.mat), C.byref(ic),
                          C.byref(hs), capi.dptr(bn), capi.dptr(ev), C.byref(cp))
        return bn.reshape(10, 3), ev.reshape(10, 10, 3), cp.value, (hs.time, hs.dt, hs.steps)

    def run(self, wl: Workload, st: dict, comp: float, clock, nsteps: int):
        cs = CStructs(wl, comp)
        hs = capi.host_state_struct(st, *clock)
        dts = np.zeros(max(nsteps, 1))
        self.lib.ref_run(C.byref(cs.mesh), C.byref(cs.params), C.byref(cs.mat), C.byref(hs),
                         nsteps, capi.dptr(dts))
        return (hs.time, hs.dt, hs.steps), dts[:nsteps]

    def run_timed(self, wl: Workload, st: dict, comp: float, clock, nsteps: int):
        """nsteps of the loop body; returns (clock, wall seconds of the loop alone)."""
        cs = CStructs(wl, comp)
        hs = capi.host_state_struct(st, *clock)
        sec = C.c_double()
        self.lib.ref_run_timed(C.byref(cs.mesh), C.byref(cs.params), C.byref(cs.mat), C.byref(hs),
                               nsteps, None, C.byref(sec))
        return (hs.time, hs.dt, hs.steps), sec.value

    def nthreads(self) -> int:
        return self.lib.ref_nthreads()

    def set_threads(self, n: int):
        """OpenMP threads of the following calls (the OpenMP build)."""
        self.lib.ref_set_threads(n)

    def bad_mesh_quality(self, wl: Workload, st: dict, comp: float, clock, rq: RefQuality):
        """bad_mesh_quality (remeshing.cxx:1882-1935): (code, index)."""
        cs = CStructs(wl, comp)
        hs = capi.host_state_struct(st, *clock)
        idx = C.c_int(-1)
        code = self.lib.ref_bad_mesh_quality(C.byref(cs.mesh), C.byref(cs.params), C.byref(cs.mat),
                                             C.byref(rq), C.byref(hs), C.byref(idx))
        return code, idx.value

    def create_support(self, nnode: int, conn: np.ndarray):
        """create_support (mesh.cxx:1707-1721) as CSR (off[nnode+1], elems)."""
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        off = np.zeros(nnode + 1, np.int32)
        elems = np.zeros(conn.size, np.int32)
        self.lib.ref_create_support(nnode, conn.shape[0], capi.iptr(conn), capi.iptr(off), capi.iptr(elems))
        return off, elems

    def create_boundary_facets(self, nnode: int, conn, bcflag, segment, segflag):
        """create_boundary_facets (mesh.cxx:1637-1704): (offsets[11], facets[n][2])."""
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        bcflag = np.ascontiguousarray(bcflag, dtype=np.uint32)
        segment = np.ascontiguousarray(segment, dtype=np.int32)
        segflag = np.ascontiguousarray(segflag, dtype=np.int32)
        off = np.zeros(capi.NBDRY + 1, np.int32)
        fac = np.zeros((segment.shape[0], 2), np.int32)
        self.lib.ref_create_boundary_facets(nnode, conn.shape[0], capi.iptr(conn), capi.uptr(bcflag),
                                            segment.shape[0], capi.iptr(segment), capi.iptr(segflag),
                                            capi.iptr(off), capi.iptr(fac))
        return off, fac[:off[-1]]

    def phase_changes(self, wl: Workload, st: dict, comp: float, option: int, elem, eta, mattype, hydem,
                      elemmarkers):
        """phase_changes (phasechanges.cxx:232-258): (new material types, new marker counts)."""
        cs = CStructs(wl, comp)
        hs = capi.host_state_struct(st)
        elem = np.ascontiguousarray(elem, dtype=np.int32)
        eta = np.ascontiguousarray(eta, dtype=np.float64)
        mt = np.array(mattype, dtype=np.int32)
        hyd = None if hydem is None else np.ascontiguousarray(hydem, dtype=np.int32)
        em = np.array(elemmarkers, dtype=np.int32)
        self.lib.ref_phase_changes(C.byref(cs.mesh), C.byref(cs.params), C.byref(cs.mat), C.byref(hs), option,
                                   elem.shape[0], capi.iptr(elem), capi.dptr(eta), capi.iptr(mt), capi.iptr(hyd),
                                   capi.iptr(em))
        return mt, em

    def call(self, wl: Workload, st: dict, comp: float, clock, name: str):
        cs = CStructs(wl, comp)
        hs = capi.host_state_struct(st, *clock)
        res = np.zeros(2)
        rc = self.lib.ref_call(C.byref(cs.mesh), C.byref(cs.params), C.byref(cs.mat), C.byref(hs),
                               name.encode(), capi.dptr(res))
        assert rc == 0, name
        return res, (hs.time, hs.dt, hs.steps)
