"""Parity cases shared by the golden-fixture generator and the tests.

Each case is a small workload of the reference's physics with a parameter
set chosen to exercise one part of the hot path (plasticity in 2D/3D, plane
strain, Maxwell/viscous/elastic rheologies, heat with radiogenic source,
multi-material blending, per-element parameters, every velocity-BC family,
damping options, jittered/permuted meshes).  Sizes are small enough for the
reference and the oracle to run them in well under a second, except the
full-horizon cases (FULL_CASES: the 2D workload at its full size over its
10,000 steps, and a yielding case of the 3D workload's physics over its
2000 steps), which take tens of seconds.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np

from dynearthsol_gb300 import capi
from dynearthsol_gb300.config import (Params, Workload, WeakZone, make_workload, _mc_material,
                                      _evp_material, weak_band)
from dynearthsol_gb300.mesh import box2d, box3d, boundary_normals, BOUNDX1, _boundary_products

FAST = 3e-8            # boundary speed (m/s) that makes elements yield within ~100 steps


def _fast(p: Params, inertial=1e3, v=FAST):
    vals = list(p.vbc_values)
    vals[0], vals[1] = -v, v
    return replace(p, inertial_scaling=inertial, vbc_values=tuple(vals))


def _weak(mat):
    return replace(mat, cohesion0=(4e6,), cohesion1=(1e6,))


def _relabel_x1_as_n0(mesh):
    """Turn the x1 side into the slant boundary n0 (same plane, flag bit 6)."""
    bc = mesh.bcflag.copy()
    on = (bc & BOUNDX1) != 0
    bc[on] = (bc[on] & ~np.uint32(BOUNDX1)) | np.uint32(1 << 6)
    mesh.bcflag = bc
    mesh.bfacet_offsets, mesh.bfacets = _boundary_products(mesh.ndims, bc, mesh.connectivity)
    boundary_normals(mesh)
    return mesh


def build_case(name: str) -> tuple[Workload, int]:
    """(workload, nsteps) of a named parity case."""
    if name == "2d_ep":
        return make_workload("c0_2d_ep", cells=(8, 3)), 150
    if name == "2d_ep_yield":
        wl, n = build_case("2d_ep")
        wl.params = _fast(wl.params)
        wl.mat = _weak(wl.mat)
        return wl, n
    if name == "2d_evp_heat":
        wl, _ = build_case("2d_ep_yield")
        wl.mat = replace(_weak(_evp_material()), radiogenic_heating=(1e-6,), therm_cond=(3.3,))
        wl.params = replace(wl.params, damping_option=2, has_fixed_bottom_temperature=False,
                            mantle_temperature=900.0)
        return wl, 150
    if name == "2d_ps_oedometer":
        # benchmarks/oedometer-2d.cfg: plane-strain Mohr-Coulomb, fixed dt
        # one cell (two triangles, every node on the boundary), as the
        # benchmark's resolution-1 mesh of the unit square
        mesh = box2d(1, 1, 1.0, 1.0)
        p = Params(gravity=0.0, fixed_dt=1.0, inertial_scaling=1e5,
                   vbc_types=(1, 1, 1, 1, 1, 1, 1, 1, 1, 1),
                   vbc_values=(0, -1e-5, 0, 0, 0, 0, 0, 0, 0, 0),
                   surface_temperature=273.0, mantle_temperature=273.0)
        mat = replace(_mc_material(capi.RH_EP), is_plane_strain=True, rho0=(1.0,), alpha=(0.0,),
                      bulk_modulus=(200e6,), shear_modulus=(200e6,), cohesion0=(1e6,),
                      cohesion1=(1e6,), friction_angle0=(10.0,), friction_angle1=(10.0,),
                      dilation_angle0=(10.0,), dilation_angle1=(10.0,), tension_max=5.67e6)
        return Workload(name, mesh, p, mat, WeakZone(option=0), 1.0, 273.0, 273.0, 2000), 2000
    if name == "3d_evp":
        return make_workload("c1_3d_evp", cells=(3, 3, 2)), 150
    if name == "3d_evp_yield":
        wl, n = build_case("3d_evp")
        wl.params = _fast(wl.params)
        wl.mat = _weak(wl.mat)
        return wl, n
    if name == "3d_ep_yield":
        wl, n = build_case("3d_evp_yield")
        wl.mat = replace(wl.mat, rheol_type=capi.RH_EP)
        return wl, n
    if name == "3d_maxwell":
        wl, n = build_case("3d_evp_yield")
        wl.mat = replace(wl.mat, rheol_type=capi.RH_MAXWELL, visc_min=1e19)
        return wl, n
    if name == "3d_elastic_damp3":
        wl, n = build_case("3d_evp_yield")
        wl.mat = replace(wl.mat, rheol_type=capi.RH_ELASTIC)
        wl.params = replace(wl.params, damping_option=3, has_thermal_diffusion=False)
        return wl, n
    if name == "3d_viscous":
        wl, n = build_case("3d_evp")
        # the reference's viscous rheology is stable here only with a reduced dt
        wl.mat = replace(wl.mat, rheol_type=capi.RH_VISCOUS, visc_min=1e20)
        wl.params = replace(wl.params, dt_fraction=0.1, inertial_scaling=1e3)
        return wl, 100
    if name == "3d_heat_jitter_multimat":
        wl = make_workload("c1_3d_evp", cells=(3, 3, 2))
        wl.mesh = box3d(3, 3, 2, 100e3, 100e3, 10e3, jitter=0.2, permute=True, seed=7)
        wl.params = replace(_fast(wl.params), has_fixed_bottom_temperature=False,
                            mantle_temperature=1700.0, has_elastic_foundation=True,
                            elastic_foundation_constant=1e6)
        K1, K2 = 33.3e9, 40e9
        wl.mat = replace(_weak(_evp_material()), rho0=(2800.0, 3000.0), alpha=(3e-5, 2e-5),
                         bulk_modulus=(K1, K2), shear_modulus=(20e9, 25e9), visc_exponent=(3.0, 3.5),
                         visc_coefficient=(1e-7, 2e-7), visc_activation_energy=(2e5, 2.5e5),
                         heat_capacity=(1000.0, 1100.0), therm_cond=(3.3, 2.5),
                         radiogenic_heating=(1e-6, 2e-6), pls0=(0.0, 0.01), pls1=(0.1, 0.2),
                         cohesion0=(4e6, 6e6), cohesion1=(1e6, 2e6), friction_angle0=(30.0, 25.0),
                         friction_angle1=(15.0, 10.0), dilation_angle0=(0.0, 2.0),
                         dilation_angle1=(0.0, 1.0))
        rng = np.random.default_rng(3)
        em = rng.integers(0, 4, size=(wl.mesh.nelem, 2)).astype(np.int32)
        em[em.sum(axis=1) == 0, 0] = 1
        wl.mat.elemmarkers = em
        return wl, 150
    if name == "3d_vbc_mix":
        wl, n = build_case("3d_evp_yield")
        wl.params = replace(wl.params, vbc_types=(3, 7, 5, 4, 1, 2, 1, 1, 1, 1),
                            vbc_values=(-FAST, FAST, 0.5 * FAST, -0.5 * FAST, 0.0, 0.0, 0, 0, 0, 0),
                            damping_option=1)
        return wl, n
    if name == "3d_slant_n0_t1":
        wl, n = build_case("3d_evp_yield")
        wl.mesh = _relabel_x1_as_n0(wl.mesh)
        wl.params = replace(wl.params, vbc_types=(1, 0, 0, 0, 0, 0, 1, 1, 1, 1),
                            vbc_values=(-FAST, 0, 0, 0, 0, 0, FAST, 0, 0, 0))
        return wl, n
    if name == "3d_slant_n0_t11":
        wl, n = build_case("3d_slant_n0_t1")
        wl.params = replace(wl.params, vbc_types=(1, 0, 1, 0, 0, 0, 11, 1, 1, 1),
                            vbc_values=(-FAST, 0, 0, 0, 0, 0, FAST, 0, 0, 0))
        return wl, n
    if name == "3d_slant_n0_t13":
        wl, n = build_case("3d_slant_n0_t1")
        wl.params = replace(wl.params, vbc_types=(1, 0, 0, 0, 0, 0, 13, 1, 1, 1),
                            vbc_values=(-FAST, 0, 0, 0, 0, 0, FAST, 0, 0, 0))
        return wl, n
    if name == "2d_slant_n0_t3":
        wl, n = build_case("2d_ep_yield")
        wl.mesh = _relabel_x1_as_n0(wl.mesh)
        wl.params = replace(wl.params, vbc_types=(1, 0, 0, 0, 0, 0, 3, 1, 1, 1),
                            vbc_values=(-FAST, 0, 0, 0, 0, 0, FAST, 0, 0, 0))
        return wl, n
    if name == "3d_percell":
        wl, n = build_case("3d_evp_yield")
        rng = np.random.default_rng(11)
        ne = wl.mesh.nelem
        noise = 1 + 0.05 * rng.standard_normal(ne)
        wl.elem_fields = {
            capi.EF_COHESION0: np.ascontiguousarray(4e6 * noise),
            capi.EF_COHESION1: np.ascontiguousarray(1e6 * noise),
            capi.EF_FRICTION0: np.ascontiguousarray(30.0 + rng.uniform(-3, 3, ne)),
            capi.EF_FRICTION1: np.ascontiguousarray(15.0 + rng.uniform(-3, 3, ne)),
            capi.EF_THERM_COND: np.ascontiguousarray(3.0 + rng.uniform(-0.5, 0.5, ne)),
        }
        return wl, n
    if name == "2d_c0_full":
        # the 2D workload at its full size and horizon: 200x20 cells x 2
        # triangles (8,000 / 4,221 nodes), 10,000 steps, default damping
        return make_workload("c0_2d_ep"), 10000
    if name == "2d_c0_full_damp2":
        wl, n = build_case("2d_c0_full")
        wl.params = replace(wl.params, damping_option=2)
        return wl, n
    if name == "3d_c1_yield_band":
        # the 3D workload's physics and boundary speeds on 20x20x6 cubes
        # (14,400 tets) for the workload's 2000 steps, with a band of weak
        # material that yields (9 % of the elements by the end)
        wl = make_workload("c1_3d_evp", cells=(20, 20, 6))
        return weak_band(wl), 2000
    if name == "3d_c1_yield_band_damp2":
        wl, n = build_case("3d_c1_yield_band")
        wl.params = replace(wl.params, damping_option=2)
        return wl, n
    raise KeyError(name)


CASES = ["2d_ep", "2d_ep_yield", "2d_evp_heat", "2d_ps_oedometer", "3d_evp", "3d_evp_yield",
         "3d_ep_yield", "3d_maxwell", "3d_elastic_damp3", "3d_viscous", "3d_heat_jitter_multimat",
         "3d_vbc_mix", "3d_slant_n0_t1", "3d_slant_n0_t11", "3d_slant_n0_t13", "2d_slant_n0_t3",
         "3d_percell"] + ["2d_c0_full", "2d_c0_full_damp2", "3d_c1_yield_band", "3d_c1_yield_band_damp2"]

# the full-horizon cases: the 2D workload at full size over 10,000 steps and
# a yielding case of the 3D workload's physics over 2000 steps, each with a
# damping-option-2 twin (no copysign damping: not chaotic, see the tests)
FULL_CASES = ["2d_c0_full", "2d_c0_full_damp2", "3d_c1_yield_band", "3d_c1_yield_band_damp2"]

# cases whose fixture also holds a mid-run state and the output of every
# reference function applied to it
PERFN_CASES = ["2d_evp_heat", "3d_heat_jitter_multimat", "3d_evp_yield", "2d_ps_oedometer",
               "3d_c1_yield_band_damp2"]
PERFN_MID_STEPS = 60
# the yielding band's mid-run state comes later, once 7 % of its elements yield
MID_STEPS = {"3d_c1_yield_band_damp2": 1500}


def mid_steps(name: str) -> int:
    return MID_STEPS.get(name, PERFN_MID_STEPS)

FUNCTIONS = {
    "update_temperature": ["temperature", "ntmp"],
    "update_strain_rate": ["strain_rate"],
    "compute_dvoldt": ["ntmp"],
    "compute_edvoldt": ["edvoldt"],
    "update_stress": ["stress", "strain", "strain_rate", "plstrain", "delta_plstrain", "dpressure"],
    "NMD_stress": ["ntmp", "stress"],
    "update_force": ["force"],
    "update_velocity": ["vel"],
    "apply_vbcs": ["vel"],
    "update_coordinate": ["coord"],
    "compute_volume": ["volume"],
    "compute_mass": ["volume_n", "mass", "tmass"],
    "compute_shape_fn": ["shpdx", "shpdy", "shpdz"],
    "rotate_stress": ["stress", "strain"],
}


def reference_material_for(wl: Workload):
    """The reference has per-material (not per-element) properties.  A case
    with per-element overrides runs on the reference as nmat = nelem
    materials, one marker each, which reproduces the override exactly for
    cohesion, friction angle and conductivity (matprops.cxx:103-128,315-353)."""
    if not wl.elem_fields:
        return wl.mat
    ne = wl.mesh.nelem
    mt = wl.mat
    ef = wl.elem_fields
    rep = lambda v: tuple(float(v[0]) for _ in range(ne))
    kw = {name: rep(getattr(mt, name)) for name in capi.MAT_ARRAYS}
    if capi.EF_COHESION0 in ef:
        kw["cohesion0"] = tuple(ef[capi.EF_COHESION0])
    if capi.EF_COHESION1 in ef:
        kw["cohesion1"] = tuple(ef[capi.EF_COHESION1])
    if capi.EF_FRICTION0 in ef:
        kw["friction_angle0"] = tuple(ef[capi.EF_FRICTION0])
    if capi.EF_FRICTION1 in ef:
        kw["friction_angle1"] = tuple(ef[capi.EF_FRICTION1])
    if capi.EF_THERM_COND in ef:
        kw["therm_cond"] = tuple(ef[capi.EF_THERM_COND])
    mask = 1 | 2 | 4 | 8      # bulk, shear, cp, hr stay single values
    if capi.EF_THERM_COND not in ef:
        mask |= 16
    em = np.eye(ne, dtype=np.int32)
    return replace(mt, scalar_mask=mask, elemmarkers=em, **kw)
