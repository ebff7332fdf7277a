"""ctypes mirror of ``include/desgpu.h`` and loader of the CUDA library.

The structs below are byte-for-byte the C structs of the header; the loader
finds ``libdesgpu.so`` next to this file (built in-tree by
``dynearthsol_gb300.build``) and raises when it is missing, so no caller can
silently run without the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

NBDRY = 10

DES_OK = 0
DES_EINPUT = 1
DES_ECUDA = 3
DES_ENOMEM = 4
DES_ERUNTIME = 11
DES_EASSERT = 12

DES_DEV_NONFINITE = 1
DES_DEV_NEG_VOLUME = 2
DES_DEV_QL_NOCONV = 4
DES_DEV_BAD_INDEX = 8

RH_ELASTIC = 1
RH_VISCOUS = 2
RH_PLASTIC = 4
RH_MAXWELL = RH_ELASTIC | RH_VISCOUS
RH_EP = RH_ELASTIC | RH_PLASTIC
RH_EVP = RH_ELASTIC | RH_VISCOUS | RH_PLASTIC

PREC_FP64 = 0
PREC_MIXED = 1

EF_COHESION0 = 0
EF_COHESION1 = 1
EF_LOG10_VISC = 2
EF_SHEAR_MODULUS = 3
EF_FRICTION0 = 4
EF_FRICTION1 = 5
EF_THERM_COND = 6
EF_COUNT = 7

F_BITS = {name: 1 << i for i, name in enumerate(
    ("coord", "coord0", "vel", "force", "temperature", "mass", "tmass", "volume_n", "ntmp", "volume",
     "volume_old", "stress", "strain", "strain_rate", "plstrain", "delta_plstrain", "stressyy",
     "dpressure", "edvoldt"))}
F_SHP = 1 << 19
F_CLOCK = 1 << 20
F_ALL = (1 << 21) - 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint)


class DesMesh(C.Structure):
    _fields_ = [
        ("ndims", C.c_int),
        ("nnode", C.c_int),
        ("nelem", C.c_int),
        ("connectivity", _ip),
        ("bcflag", _up),
        ("bfacet_offsets", _ip),
        ("bfacets", _ip),
        ("bnormals", (C.c_double * 3) * NBDRY),
        ("edge_vectors", ((C.c_double * 3) * NBDRY) * NBDRY),
    ]


class DesParams(C.Structure):
    _fields_ = [
        ("gravity", C.c_double),
        ("inertial_scaling", C.c_double),
        ("dt_fraction", C.c_double),
        ("fixed_dt", C.c_double),
        ("damping_factor", C.c_double),
        ("surface_diffusivity", C.c_double),
        ("max_vbc_val", C.c_double),
        ("damping_option", C.c_int),
        ("ref_pressure_option", C.c_int),
        ("surface_process_option", C.c_int),
        ("is_quasi_static", C.c_int),
        ("has_thermal_diffusion", C.c_int),
        ("surface_temperature", C.c_double),
        ("mantle_temperature", C.c_double),
        ("winkler_delta_rho", C.c_double),
        ("elastic_foundation_constant", C.c_double),
        ("has_fixed_bottom_temperature", C.c_int),
        ("has_winkler_foundation", C.c_int),
        ("has_elastic_foundation", C.c_int),
        ("has_water_loading", C.c_int),
        ("vbc_types", C.c_int * NBDRY),
        ("vbc_values", C.c_double * NBDRY),
        ("zlength", C.c_double),
        ("compensation_pressure", C.c_double),
    ]


MAT_ARRAYS = (
    "rho0", "alpha", "bulk_modulus", "shear_modulus", "visc_exponent",
    "visc_coefficient", "visc_activation_energy", "heat_capacity", "therm_cond",
    "radiogenic_heating", "pls0", "pls1", "cohesion0", "cohesion1",
    "friction_angle0", "friction_angle1", "dilation_angle0", "dilation_angle1",
)


class DesMaterial(C.Structure):
    _fields_ = [
        ("rheol_type", C.c_int),
        ("nmat", C.c_int),
        ("is_plane_strain", C.c_int),
        ("scalar_mask", C.c_uint),
        ("visc_min", C.c_double),
        ("visc_max", C.c_double),
        ("tension_max", C.c_double),
        ("therm_diff_max", C.c_double),
    ] + [(name, _dp) for name in MAT_ARRAYS] + [("elemmarkers", _ip)]


STATE_ARRAYS = (
    "coord", "coord0", "vel", "force", "temperature", "mass", "tmass", "volume_n",
    "ntmp", "volume", "volume_old", "stress", "strain", "strain_rate", "plstrain",
    "delta_plstrain", "stressyy", "dpressure", "edvoldt", "shpdx", "shpdy", "shpdz",
)


class DesHostState(C.Structure):
    _fields_ = [(name, _dp) for name in STATE_ARRAYS] + [
        ("time", C.c_double),
        ("dt", C.c_double),
        ("steps", C.c_int),
    ]


class DesQualityParams(C.Structure):
    """des_quality_params: the Param::mesh fields bad_mesh_quality reads."""
    _fields_ = [("smallest_size", C.c_double), ("resolution", C.c_double), ("min_quality", C.c_double),
                ("max_boundary_distortion", C.c_double), ("remeshing_option", C.c_int)]


class DesTopology(C.Structure):
    """des_topology: a mesh as remeshing leaves it (connectivity, boundary
    flags, boundary segments and their flags)."""
    _fields_ = [("ndims", C.c_int), ("nnode", C.c_int), ("nelem", C.c_int), ("connectivity", _ip),
                ("bcflag", _up), ("nseg", C.c_int), ("segment", _ip), ("segflag", _ip)]


class DesAdjointGrad(C.Structure):
    """des_adjoint_grad: per-element gradient arrays (NULL = skip) and the
    gradient with respect to each boundary's prescribed velocity value."""
    _fields_ = [("elem", _dp * EF_COUNT), ("vbc_values", C.c_double * NBDRY)]


SAVE_FIELDS = ("coord", "connectivity", "vel", "temperature", "plstrain", "delta_plstrain", "strain_rate",
               "strain", "stress", "density", "mesh_quality", "viscosity", "material", "force", "coord0",
               "bcflag")


class DesSaveFrame(C.Structure):
    """des_save_frame: host arrays of one .save output frame."""
    _fields_ = [("ndims", C.c_int), ("nnode", C.c_int), ("nelem", C.c_int)] + [
        (name, _ip if name == "connectivity" else (_up if name == "bcflag" else _dp)) for name in SAVE_FIELDS]


def dptr(a: np.ndarray | None):
    """double* of a C-contiguous float64 array (NULL for None)."""
    if a is None:
        return _dp()
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray | None):
    if a is None:
        return _ip()
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def uptr(a: np.ndarray | None):
    if a is None:
        return _up()
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_up)


# --------------------------------------------------------------------------
# CUDA library
# --------------------------------------------------------------------------
HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdesgpu.so")

_lib = None

# (name, argtypes); every entry point returns int
_SIGS = {
    "des_create": [C.POINTER(DesMesh), C.POINTER(DesParams), C.POINTER(DesMaterial), C.c_int,
                   C.c_void_p, C.POINTER(C.c_void_p)],
    "des_destroy": [C.c_void_p],
    "des_last_error": [C.c_void_p, C.c_char_p, C.c_size_t],
    "des_device_status": [C.c_void_p, _up],
    "des_upload_state": [C.c_void_p, C.POINTER(DesHostState)],
    "des_download_state": [C.c_void_p, C.POINTER(DesHostState)],
    "des_set_params": [C.c_void_p, C.POINTER(DesParams)],
    "des_upload_fields": [C.c_void_p, C.POINTER(DesHostState), C.c_uint],
    "des_download_fields": [C.c_void_p, C.POINTER(DesHostState), C.c_uint],
    "des_set_elemmarkers": [C.c_void_p, _ip],
    "des_set_elem_field": [C.c_void_p, C.c_int, _dp],
    "des_update_temperature": [C.c_void_p],
    "des_update_strain_rate": [C.c_void_p],
    "des_compute_dvoldt": [C.c_void_p],
    "des_compute_edvoldt": [C.c_void_p],
    "des_update_stress": [C.c_void_p],
    "des_NMD_stress": [C.c_void_p],
    "des_update_force": [C.c_void_p],
    "des_update_velocity": [C.c_void_p],
    "des_apply_vbcs": [C.c_void_p],
    "des_update_coordinate": [C.c_void_p],
    "des_swap_volume": [C.c_void_p],
    "des_compute_volume": [C.c_void_p],
    "des_compute_mass": [C.c_void_p],
    "des_compute_shape_fn": [C.c_void_p],
    "des_rotate_stress": [C.c_void_p],
    "des_compute_dt": [C.c_void_p, _dp],
    "des_update_mesh": [C.c_void_p],
    "des_worst_elem_quality": [C.c_void_p, _dp, _ip],
    "des_bad_mesh_quality": [C.c_void_p, C.POINTER(DesQualityParams), _ip, _ip, _dp],
    "des_set_markers": [C.c_void_p, C.c_int, _ip, _dp, _ip],
    "des_build_topology": [C.POINTER(DesTopology), _ip, _ip, _ip, _ip, C.c_void_p],
    "des_remesh": [C.c_void_p, C.POINTER(DesTopology), _ip],
    "des_phase_changes": [C.c_void_p, C.c_int, _ip, _ip],
    "des_get_markers": [C.c_void_p, _ip, _ip],
    "des_get_clock": [C.c_void_p, _dp, _dp, _ip],
    "des_set_clock": [C.c_void_p, C.c_double, C.c_double, C.c_int],
    "des_step": [C.c_void_p, C.c_int],
    "des_step_host": [C.c_void_p, C.POINTER(DesHostState), C.c_int],
    "des_synchronize": [C.c_void_p],
    "des_launch_count": [C.c_void_p, C.POINTER(C.c_longlong)],
    "des_nmd_stress_noalloc": [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 8,
    "des_write_save_host": [C.c_char_p, C.POINTER(DesSaveFrame)],
    "des_write_save": [C.c_void_p, C.c_char_p],
    "des_adjoint_forward": [C.c_void_p, C.c_int, C.c_int],
    "des_adjoint_backward": [C.c_void_p, C.POINTER(DesHostState), C.POINTER(DesHostState),
                             C.POINTER(DesAdjointGrad)],
}


def declared_symbols() -> list[str]:
    """Entry points declared in include/desgpu.h (parsed from the header)."""
    import re

    hdr = os.path.join(os.path.dirname(HERE), "include", "desgpu.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(des_\w+)\s*\(", text, re.M)))


def load_library(path: str | None = None):
    """Load libdesgpu.so (raises OSError when it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"libdesgpu.so not found at {p}; build it with "
                      "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.des_version.argtypes = []
    lib.des_version.restype = C.c_char_p
    if path is None:
        _lib = lib
    return lib


class DesError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"desgpu error {code}: {msg}")
        self.code = code


def host_state_struct(st: dict, time: float = 0.0, dt: float = 0.0, steps: int = 0) -> DesHostState:
    """DesHostState pointing into the float64 arrays of a state dict (keys of
    STATE_ARRAYS; missing keys become NULL).  The dict must outlive it."""
    s = DesHostState()
    for name in STATE_ARRAYS:
        a = st.get(name)
        if a is not None:
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"state array {name} must be C-contiguous float64")
            setattr(s, name, dptr(a))
    s.time = time
    s.dt = dt
    s.steps = steps
    return s


def read_save(path: str) -> dict:
    """Read a .save frame (BinaryOutput layout, binaryio.cxx:16-37): a 4096-byte
    header of "name<TAB>offset" lines after the revision line, then the arrays.
    Returns {"ndims": n, name: flat array}; connectivity int32, bcflag uint32,
    the rest float64."""
    raw = open(path, "rb").read()
    head = raw[:4096].split(b"\0", 1)[0].decode()
    lines = head.splitlines()
    ndims = int(lines[0].split("ndims=")[1].split()[0])
    items = [(ln.rsplit("\t", 1)[0], int(ln.rsplit("\t", 1)[1])) for ln in lines[1:] if "\t" in ln]
    out = {"ndims": ndims, "_order": [n for n, _ in items]}
    for k, (name, off) in enumerate(items):
        end = items[k + 1][1] if k + 1 < len(items) else len(raw)
        dt = np.int32 if name == "connectivity" else (np.uint32 if name == "bcflag" else np.float64)
        out[name] = np.frombuffer(raw[off:end], dtype=dt)
    return out


def segments_of(mesh, order=None):
    """Boundary segments of a mesh as a mesher lists them (Variables::segment,
    segflag): the nodes of each boundary facet (NODE_OF_FACET,
    constants.hpp:59-71) and its boundary's bit, in the mesh's boundary-facet
    order or in the given order of those facets."""
    from .mesh import NODE_OF_FACET_2D, NODE_OF_FACET_3D
    nd = mesh.ndims
    tab = NODE_OF_FACET_3D if nd == 3 else NODE_OF_FACET_2D
    off = np.asarray(mesh.bfacet_offsets)
    bdry = np.zeros(off[-1], dtype=np.int32)
    for b in range(NBDRY):
        bdry[off[b]:off[b + 1]] = b
    fac = np.asarray(mesh.bfacets)
    idx = np.arange(off[-1]) if order is None else np.asarray(order)
    e, f = fac[idx, 0], fac[idx, 1]
    seg = np.ascontiguousarray(np.asarray(mesh.connectivity)[e[:, None], tab[f]], dtype=np.int32)
    flag = np.ascontiguousarray((1 << bdry[idx]).astype(np.int32))
    return seg, flag


class Topology:
    """A DesTopology with the arrays it points to."""

    def __init__(self, mesh, segment=None, segflag=None):
        if segment is None:
            segment, segflag = segments_of(mesh)
        self.conn = np.ascontiguousarray(mesh.connectivity, dtype=np.int32)
        self.bcflag = np.ascontiguousarray(mesh.bcflag, dtype=np.uint32)
        self.segment = np.ascontiguousarray(segment, dtype=np.int32)
        self.segflag = np.ascontiguousarray(segflag, dtype=np.int32)
        self.struct = DesTopology(mesh.ndims, mesh.nnode, mesh.nelem, iptr(self.conn), uptr(self.bcflag),
                                  self.segment.shape[0], iptr(self.segment), iptr(self.segflag))


def build_topology(topo: "Topology", stream=None):
    """des_build_topology: (sup_off, sup_elem, bfacet_offsets, bfacets)."""
    lib = load_library()
    t = topo.struct
    off = np.zeros(t.nnode + 1, np.int32)
    elems = np.zeros(t.nelem * (t.ndims + 1), np.int32)
    boff = np.zeros(NBDRY + 1, np.int32)
    fac = np.zeros((max(t.nseg, 1), 2), np.int32)
    rc = lib.des_build_topology(C.byref(t), iptr(off), iptr(elems), iptr(boff), iptr(fac), stream)
    if rc:
        raise DesError(rc, "des_build_topology failed")
    return off, elems, boff, fac[:boff[-1]]
