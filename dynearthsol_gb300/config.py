"""Run parameters, material table, initial conditions and named workloads.

``Params``/``Material``/``WeakZone`` carry the subset of the reference's
``Param`` (parameters.hpp:36-221) that the explicit step reads, with the
reference's defaults (input.cxx:15-460).  ``initial_state`` restates the
reference's init-time initial conditions (ic.cxx:96-204) so that a workload
can be set up without the reference; the step itself runs on the GPU.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import capi
from .mesh import Mesh, box2d, box3d

YEAR2SEC = 365.2422 * 86400          # constants.hpp:73
DEG2RAD = math.pi / 180              # constants.hpp:74
CM_PER_YR = 0.01 / YEAR2SEC          # 1 cm/yr in m/s


@dataclass
class Params:
    gravity: float = 10.0
    characteristic_speed: float = 0.0
    inertial_scaling: float = 1e5
    dt_fraction: float = 1.0
    fixed_dt: float = 0.0
    damping_factor: float = 0.8
    damping_option: int = 1
    ref_pressure_option: int = 0
    surface_process_option: int = 0
    surface_diffusivity: float = 1e-6
    is_quasi_static: bool = True
    has_thermal_diffusion: bool = True
    surface_temperature: float = 273.0
    mantle_temperature: float = 1600.0
    has_fixed_bottom_temperature: bool = True
    has_winkler_foundation: bool = True
    winkler_delta_rho: float = 0.0
    has_elastic_foundation: bool = False
    elastic_foundation_constant: float = 1e11
    has_water_loading: bool = True
    # vbc x0, x1, y0, y1, z0, z1, n0..n3 (input.cxx:240-310)
    vbc_types: tuple = (1, 1, 0, 0, 0, 0, 1, 1, 1, 1)
    vbc_values: tuple = (-1e-9, 1e-9, 0, 0, 0, 0, 0, 0, 0, 0)

    def max_vbc_val(self) -> float:
        """Variables::max_vbc_val: characteristic_speed, or find_max_vbc
        (bc.cxx:59-84) over the boundaries whose type is odd."""
        if self.characteristic_speed != 0:
            return self.characteristic_speed
        m = 0.0
        for t, v in zip(self.vbc_types, self.vbc_values):
            if t % 2 == 1:
                m = max(m, abs(v))
        return m


@dataclass
class Material:
    rheol_type: int = capi.RH_EVP
    is_plane_strain: bool = False
    visc_min: float = 1e18
    visc_max: float = 1e24
    tension_max: float = 1e9
    therm_diff_max: float = 5e-6
    rho0: tuple = (3210.0,)
    alpha: tuple = (3e-5,)
    bulk_modulus: tuple = (128.2e9,)
    shear_modulus: tuple = (80.5e9,)
    visc_exponent: tuple = (3.05,)
    visc_coefficient: tuple = (1.25e-1,)
    visc_activation_energy: tuple = (3.76e5,)
    heat_capacity: tuple = (1e3,)
    therm_cond: tuple = (3.0,)
    radiogenic_heating: tuple = (0.0,)
    pls0: tuple = (0.0,)
    pls1: tuple = (0.1,)
    cohesion0: tuple = (4e7,)
    cohesion1: tuple = (4e6,)
    friction_angle0: tuple = (30.0,)
    friction_angle1: tuple = (5.0,)
    dilation_angle0: tuple = (0.0,)
    dilation_angle1: tuple = (0.0,)
    scalar_mask: int = 0
    elemmarkers: np.ndarray | None = None

    @property
    def nmat(self) -> int:
        return len(self.rho0)


@dataclass
class WeakZone:
    """initial_weak_zone parameters (input.cxx:325-360 defaults)."""
    option: int = 1
    plstrain: float = 0.1
    azimuth: float = 0.0
    inclination: float = 90.0
    halfwidth: float = 1.5
    y_min: float = 0.0
    y_max: float = 1.0
    depth_min: float = 0.0
    depth_max: float = 1.0
    xcenter: float = 0.5
    ycenter: float = 0.5
    zcenter: float = 0.5
    xsemi_axis: float = 1e3
    ysemi_axis: float = 1e3
    zsemi_axis: float = 1e3


@dataclass
class Workload:
    name: str
    mesh: Mesh
    params: Params
    mat: Material
    weakzone: WeakZone
    resolution: float
    t_top: float
    t_bottom: float
    steps: int
    elem_fields: dict = field(default_factory=dict)   # capi.EF_* -> [nelem] float64
    description: str = ""

    @property
    def lengths(self):
        return self.mesh.lengths


# --------------------------------------------------------------------------
# C structs
# --------------------------------------------------------------------------
class CStructs:
    """Holds the ctypes structs of a workload plus the arrays they point to."""

    def __init__(self, wl: Workload, compensation_pressure: float = 0.0):
        m, p, mt = wl.mesh, wl.params, wl.mat
        self._keep = []
        k = self._keep.append
        self.mesh = capi.DesMesh()
        self.mesh.ndims = m.ndims
        self.mesh.nnode = m.nnode
        self.mesh.nelem = m.nelem
        conn = np.ascontiguousarray(m.connectivity, dtype=np.int32); k(conn)
        bcf = np.ascontiguousarray(m.bcflag, dtype=np.uint32); k(bcf)
        offs = np.ascontiguousarray(m.bfacet_offsets, dtype=np.int32); k(offs)
        bf = np.ascontiguousarray(m.bfacets, dtype=np.int32); k(bf)
        self.mesh.connectivity = capi.iptr(conn)
        self.mesh.bcflag = capi.uptr(bcf)
        self.mesh.bfacet_offsets = capi.iptr(offs)
        self.mesh.bfacets = capi.iptr(bf)
        for i in range(capi.NBDRY):
            for d in range(3):
                self.mesh.bnormals[i][d] = float(m.bnormals[i, d])
                for j in range(capi.NBDRY):
                    self.mesh.edge_vectors[i][j][d] = float(m.edge_vectors[i, j, d])

        self.params = capi.DesParams()
        P = self.params
        P.gravity = p.gravity
        P.inertial_scaling = p.inertial_scaling
        P.dt_fraction = p.dt_fraction
        P.fixed_dt = p.fixed_dt
        P.damping_factor = p.damping_factor
        P.surface_diffusivity = p.surface_diffusivity
        P.max_vbc_val = p.max_vbc_val()
        P.damping_option = p.damping_option
        P.ref_pressure_option = p.ref_pressure_option
        P.surface_process_option = p.surface_process_option
        P.is_quasi_static = int(p.is_quasi_static)
        P.has_thermal_diffusion = int(p.has_thermal_diffusion)
        P.surface_temperature = p.surface_temperature
        P.mantle_temperature = p.mantle_temperature
        P.winkler_delta_rho = p.winkler_delta_rho
        P.elastic_foundation_constant = p.elastic_foundation_constant
        P.has_fixed_bottom_temperature = int(p.has_fixed_bottom_temperature)
        P.has_winkler_foundation = int(p.has_winkler_foundation)
        P.has_elastic_foundation = int(p.has_elastic_foundation)
        P.has_water_loading = int(p.has_water_loading)
        for i in range(capi.NBDRY):
            P.vbc_types[i] = int(p.vbc_types[i])
            P.vbc_values[i] = float(p.vbc_values[i])
        P.zlength = float(m.lengths[2])
        P.compensation_pressure = compensation_pressure

        self.mat = capi.DesMaterial()
        M = self.mat
        M.rheol_type = mt.rheol_type
        M.nmat = mt.nmat
        M.is_plane_strain = int(mt.is_plane_strain)
        M.scalar_mask = mt.scalar_mask
        M.visc_min = mt.visc_min
        M.visc_max = mt.visc_max
        M.tension_max = mt.tension_max
        M.therm_diff_max = mt.therm_diff_max
        for name in capi.MAT_ARRAYS:
            vals = np.ascontiguousarray(getattr(mt, name), dtype=np.float64)
            if vals.shape[0] != mt.nmat:
                vals = np.full(mt.nmat, vals[0])
            k(vals)
            setattr(M, name, capi.dptr(vals))
        if mt.elemmarkers is not None:
            em = np.ascontiguousarray(mt.elemmarkers, dtype=np.int32); k(em)
            M.elemmarkers = capi.iptr(em)


# --------------------------------------------------------------------------
# initial conditions (ic.cxx)
# --------------------------------------------------------------------------
def ref_pressure(wl: Workload, z):
    """ref_pressure option 0 (matprops.cxx:190-202): rho0[0]*g*depth."""
    if wl.params.ref_pressure_option != 0:
        raise NotImplementedError("only ref_pressure_option 0 is supported")
    depth = -np.asarray(z, dtype=np.float64)
    return wl.mat.rho0[0] * wl.params.gravity * depth


def elem_center(mesh: Mesh) -> np.ndarray:
    """Element centroids summed node by node, then divided (ic.cxx:183-193)."""
    c = mesh.coord[mesh.connectivity[:, 0]].copy()
    for i in range(1, mesh.connectivity.shape[1]):
        c += mesh.coord[mesh.connectivity[:, i]]
    return c / mesh.connectivity.shape[1]


def weak_zone_mask(wl: Workload) -> np.ndarray:
    """initial_weak_zone (ic.cxx:135-204) membership of each element."""
    m, wz = wl.mesh, wl.weakzone
    nd = m.ndims
    xl, yl, zl = m.lengths
    ctr = elem_center(m)
    if wz.option == 0:
        return np.zeros(m.nelem, dtype=bool)
    if wz.option == 1:
        c0 = wz.xcenter * xl
        c1 = wz.ycenter * yl
        cz = -wz.zcenter * zl
        az = math.tan(wz.azimuth * DEG2RAD)
        incl = 1 / math.tan(wz.inclination * DEG2RAD)
        hw = wz.halfwidth * wl.resolution
        zmin, zmax = -wz.depth_max * zl, -wz.depth_min * zl
        x, z = ctr[:, 0], ctr[:, nd - 1]
        ok = (z > zmin) & (z < zmax)
        if nd == 3:
            y = ctr[:, 1]
            ok &= (y > wz.y_min * yl) & (y < wz.y_max * yl)
            d = (x - c0) - az * (y - c1) + incl * (z - cz)
        else:
            d = (x - c0) + incl * (z - cz)
        return ok & (np.abs(d) < hw)
    if wz.option == 2:
        c0, c1, cz = wz.xcenter * xl, wz.ycenter * yl, -wz.zcenter * zl
        a2 = wz.xsemi_axis * wz.xsemi_axis
        b2 = wz.ysemi_axis * wz.ysemi_axis
        c2 = wz.zsemi_axis * wz.zsemi_axis
        r = (ctr[:, 0] - c0) * (ctr[:, 0] - c0) / a2
        if nd == 3:
            r = r + (ctr[:, 1] - c1) * (ctr[:, 1] - c1) / b2
        r = r + (ctr[:, nd - 1] - cz) * (ctr[:, nd - 1] - cz) / c2
        return r < 1
    raise ValueError(f"unknown weakzone option {wz.option}")


def linear_geotherm(wl: Workload) -> np.ndarray:
    """T(z) linear from t_top at z=0 to t_bottom at z=-zlength."""
    z = wl.mesh.coord[:, wl.mesh.ndims - 1]
    zl = wl.mesh.lengths[2]
    return wl.t_top + (wl.t_bottom - wl.t_top) * (-z / zl)


def nstr_of(nd):
    return 6 if nd == 3 else 3


def initial_state(wl: Workload) -> tuple[dict, float]:
    """Host state (reference AoS layout) after the initial conditions, and
    the compensation pressure.  Velocities start at zero; the boundary
    velocities, volumes, masses, shape functions and dt are computed by the
    library's init sequence (dynearthsol.cxx:82-94,316)."""
    m = wl.mesh
    nd, nn, ne = m.ndims, m.nnode, m.nelem
    nstr, npe = nstr_of(nd), nd + 1
    st = {
        "coord": m.coord.copy(),
        "coord0": m.coord.copy(),
        "vel": np.zeros((nn, nd)),
        "force": np.zeros((nn, nd)),
        "temperature": np.ascontiguousarray(linear_geotherm(wl)),
        "mass": np.zeros(nn), "tmass": np.zeros(nn), "volume_n": np.zeros(nn), "ntmp": np.zeros(nn),
        "volume": np.zeros(ne), "volume_old": np.zeros(ne),
        "stress": np.zeros((ne, nstr)), "strain": np.zeros((ne, nstr)),
        "strain_rate": np.zeros((ne, nstr)),
        "plstrain": np.zeros(ne), "delta_plstrain": np.zeros(ne), "stressyy": np.zeros(ne),
        "dpressure": np.zeros(ne), "edvoldt": np.zeros(ne),
        "shpdx": np.zeros((ne, npe)), "shpdy": np.zeros((ne, npe)), "shpdz": np.zeros((ne, npe)),
    }
    comp = 0.0
    if wl.params.gravity != 0:
        # initial_stress_state (ic.cxx:96-132): lithostatic stress and strain
        zc = m.coord[m.connectivity[:, 0], nd - 1].copy()
        for i in range(1, npe):
            zc += m.coord[m.connectivity[:, i], nd - 1]
        zc = zc / npe
        p = ref_pressure(wl, zc)
        ks = wl.mat.bulk_modulus[0]
        for i in range(nd):
            st["stress"][:, i] = -p
            st["strain"][:, i] = -p / ks / nd
        if wl.mat.is_plane_strain:
            st["stressyy"][:] = -p
        comp = float(ref_pressure(wl, -m.lengths[2]))
    mask = weak_zone_mask(wl)
    st["plstrain"][mask] = wl.weakzone.plstrain
    return st, comp


# --------------------------------------------------------------------------
# named workloads
# --------------------------------------------------------------------------
def _elastic_moduli(E: float, nu: float):
    K = E / (3 * (1 - 2 * nu))
    G = E / (2 * (1 + nu))
    return K, G


def _mc_material(rheol_type: int) -> Material:
    K, G = _elastic_moduli(50e9, 0.25)
    return Material(rheol_type=rheol_type, rho0=(2800.0,), bulk_modulus=(K,), shear_modulus=(G,),
                    cohesion0=(44e6,), cohesion1=(4e6,), friction_angle0=(30.0,),
                    friction_angle1=(15.0,), pls0=(0.0,), pls1=(0.1,),
                    dilation_angle0=(0.0,), dilation_angle1=(0.0,))


def _evp_material() -> Material:
    m = _mc_material(capi.RH_EVP)
    return replace(m, visc_exponent=(3.0,), visc_activation_energy=(2e5,), visc_coefficient=(1e-7,))


def make_workload(name: str, scale: float = 1.0, seed: int = 12345, cells: tuple | None = None) -> Workload:
    """Named workloads.  ``scale`` < 1 shrinks the cell counts (same physics)
    for tests; 1.0 gives the full sizes:

    * ``c0_2d_ep``: 2D 100x10 km, 200x20 cells x2 triangles (8,000 / 4,221),
      Mohr-Coulomb elasto-plastic, 0->600 C, +-0.5 cm/yr, 10,000 steps.
    * ``c1_3d_evp``: 3D 100x100x10 km, 80x80x26 cubes x6 (998,400 / 177,147),
      Maxwell visco-elasto-plastic with Arrhenius viscosity (A=1e-25 Pa^-3/s,
      n=3, Q=200 kJ/mol), 0->1330 C, +-1 cm/yr, 2000 steps.
    * ``c2_3d_evp_noise``: 160x160x52 x6 = 7,987,200 tets, C1 physics,
      per-element cohesion x (1 + 0.05 N(0,1)), 1000 steps.
    * ``c4_3d_heat_jitter``: 130x130x40 x6 = 4,056,000 tets, interior nodes
      jittered +-20 %, elements permuted, heat k=3.3, cp=1000, H=1e-6.

    ``cells`` overrides the cell counts ((nx, nz) in 2D, (nx, ny, nz) in 3D).
    """
    it = iter(cells) if cells else None

    def sc(n):
        if it is not None:
            return int(next(it))
        return max(2, int(round(n * scale)))

    vel = (-0.5 * CM_PER_YR, 0.5 * CM_PER_YR)
    if name == "c0_2d_ep":
        nx, nz = sc(200), sc(20)
        mesh = box2d(nx, nz, 100e3, 10e3)
        p = Params(vbc_values=(vel[0], vel[1], 0, 0, 0, 0, 0, 0, 0, 0))
        mat = _mc_material(capi.RH_EP)
        return Workload(name, mesh, p, mat, WeakZone(), 100e3 / nx, 273.0, 873.0, 10000,
                        description=f"2D EP {nx}x{nz}x2 tris")
    vel = (-1.0 * CM_PER_YR, 1.0 * CM_PER_YR)
    p3 = Params(vbc_values=(vel[0], vel[1], 0, 0, 0, 0, 0, 0, 0, 0))
    if name == "c1_3d_evp":
        nx, ny, nz = sc(80), sc(80), sc(26)
        mesh = box3d(nx, ny, nz, 100e3, 100e3, 10e3)
        return Workload(name, mesh, p3, _evp_material(), WeakZone(), 100e3 / nx, 273.0, 1603.0, 2000,
                        description=f"3D EVP {nx}x{ny}x{nz}x6 tets")
    if name == "c2_3d_evp_noise":
        nx, ny, nz = sc(160), sc(160), sc(52)
        mesh = box3d(nx, ny, nz, 100e3, 100e3, 10e3)
        wl = Workload(name, mesh, p3, _evp_material(), WeakZone(), 100e3 / nx, 273.0, 1603.0, 1000,
                      description=f"3D EVP + cohesion noise {nx}x{ny}x{nz}x6 tets")
        rng = np.random.default_rng(seed)
        noise = 1 + 0.05 * rng.standard_normal(mesh.nelem)
        wl.elem_fields[capi.EF_COHESION0] = np.ascontiguousarray(wl.mat.cohesion0[0] * noise)
        wl.elem_fields[capi.EF_COHESION1] = np.ascontiguousarray(wl.mat.cohesion1[0] * noise)
        return wl
    if name == "c4_3d_heat_jitter":
        nx, ny, nz = sc(130), sc(130), sc(40)
        mesh = box3d(nx, ny, nz, 100e3, 100e3, 10e3, jitter=0.2, permute=True, seed=seed)
        mat = replace(_evp_material(), therm_cond=(3.3,), heat_capacity=(1000.0,),
                      radiogenic_heating=(1e-6,))
        return Workload(name, mesh, p3, mat, WeakZone(), 100e3 / nx, 273.0, 1603.0, 1000,
                        description=f"3D EVP + heat, jittered/permuted {nx}x{ny}x{nz}x6 tets")
    raise KeyError(name)


def weak_band(wl: Workload, halfwidth: float = 15e3, cohesion=(1e6, 1e5), friction=(10.0, 5.0)) -> Workload:
    """Two materials: the workload's own outside the vertical band
    |x - xlength/2| < halfwidth (element centroids), and inside it the same
    material with low cohesion (cohesion0/1) and friction (friction_angle0/1),
    one marker per element (a marker-blended multi-material mesh,
    matprops.cxx:103-128).  At the workload's boundary speeds the band
    reaches the Mohr-Coulomb yield surface within a few hundred steps."""
    mt = wl.mat
    two = {n: tuple(getattr(mt, n)) * 2 for n in capi.MAT_ARRAYS}
    two["cohesion0"] = (mt.cohesion0[0], cohesion[0])
    two["cohesion1"] = (mt.cohesion1[0], cohesion[1])
    two["friction_angle0"] = (mt.friction_angle0[0], friction[0])
    two["friction_angle1"] = (mt.friction_angle1[0], friction[1])
    band = np.abs(elem_center(wl.mesh)[:, 0] - 0.5 * wl.mesh.lengths[0]) < halfwidth
    em = np.zeros((wl.mesh.nelem, 2), np.int32)
    em[~band, 0] = 1
    em[band, 1] = 1
    wl.mat = replace(mt, elemmarkers=em, **two)
    return wl
