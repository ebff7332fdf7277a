/*
 * ref_harness.cxx -- drives the REFERENCE's own hot-path functions, compiled
 * from the reference sources by oracle/Makefile into oracle/_ref/.  Test
 * infrastructure only: it pins the C restatement (des_oracle.c) and generates
 * the golden fixtures under tests/golden/.  Never shipped, never run on the
 * GPU host (the reference sources are not there).
 *
 * Built twice: with -DTHREED (3D) and without (2D), as the reference is.
 * It fills Param and Variables (parameters.hpp:212-279) from the plain C
 * structs of desgpu.h, runs the reference's init sequence
 * (dynearthsol.cxx:82-98) and the loop body (dynearthsol.cxx:325-361,
 * without phase changes, output and remeshing), and copies the fields back.
 */
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef USE_OMP
#include <omp.h>
#endif

#include "constants.hpp"
#include "parameters.hpp"
#include "matprops.hpp"
#include "fields.hpp"
#include "geometry.hpp"
#include "rheology.hpp"
#include "bc.hpp"
#include "ic.hpp"
#include "binaryio.hpp"
#include "remeshing.hpp"
#include "mesh.hpp"
#include "markerset.hpp"
#include "phasechanges.hpp"

#include "../include/desgpu.h"

/* ic.cxx references the COMSOL temperature reader (ic-read-temp.cxx), which
 * pulls in the marker/interpolation modules; the harness never selects that
 * option, so a stub satisfies the linker. */
void read_external_temperature_from_comsol(const Param &, const Variables &, double_vec &) {}

#ifndef THREED
/* The 2D mesh.cxx keeps a reference to Triangle's entry points after the
 * unused meshing code is dropped; the harness never meshes, so stubs that
 * stop the program satisfy the linker. */
struct triangulateio;
void triangulate(char *, triangulateio *, triangulateio *, triangulateio *) { std::abort(); }
void trifree(void *) { std::abort(); }
#endif

/* Hooks of a device shim linked in place of fields.o, geometry.o and
 * rheology.o (a library that keeps Variables on a device between calls):
 * the host program uploads Variables after changing them and downloads them
 * before reading them.  Weak, so that they are null in the plain reference
 * build. */
extern "C" void desgpu_shim_sync_to_host(void) __attribute__((weak));
extern "C" void desgpu_shim_sync_to_device(void) __attribute__((weak));

extern "C" {

/* The Param::mesh fields bad_mesh_quality reads (parameters.hpp:52-80). */
typedef struct ref_quality {
    double smallest_size, resolution, min_quality, max_boundary_distortion, zlength;
    int remeshing_option;
} ref_quality;

int ref_nthreads(void)
{
#ifdef USE_OMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* OpenMP threads of the following calls (the element bands follow them) */
void ref_set_threads(int n)
{
#ifdef USE_OMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

typedef struct ref_ic {
    int weakzone_option;
    double weakzone_plstrain, weakzone_azimuth, weakzone_inclination, weakzone_halfwidth;
    double weakzone_y_min, weakzone_y_max, weakzone_depth_min, weakzone_depth_max;
    double weakzone_xcenter, weakzone_ycenter, weakzone_zcenter;
    double weakzone_xsemi_axis, weakzone_ysemi_axis, weakzone_zsemi_axis;
    double xlength, ylength, zlength, resolution;
} ref_ic;

int ref_ndims(void) { return NDIMS; }
}

namespace {

void fill_vec(double_vec &v, const double *a, int n)
{
    v.assign(a, a + n);
}

void fill_param(Param &p, const des_params *dp, const des_material *dm, const ref_ic *ic)
{
    p.control.gravity = dp->gravity;
    p.control.characteristic_speed = dp->max_vbc_val;
    p.control.inertial_scaling = dp->inertial_scaling;
    p.control.dt_fraction = dp->dt_fraction;
    p.control.fixed_dt = dp->fixed_dt;
    p.control.damping_factor = dp->damping_factor;
    p.control.damping_option = dp->damping_option;
    p.control.ref_pressure_option = dp->ref_pressure_option;
    p.control.surface_process_option = dp->surface_process_option;
    p.control.surface_diffusivity = dp->surface_diffusivity;
    p.control.is_quasi_static = dp->is_quasi_static != 0;
    p.control.has_thermal_diffusion = dp->has_thermal_diffusion != 0;
    p.control.has_hydration_processes = false;
    p.control.hydration_migration_speed = 0;

    p.bc.surface_temperature = dp->surface_temperature;
    p.bc.mantle_temperature = dp->mantle_temperature;
    p.bc.has_fixed_bottom_temperature = dp->has_fixed_bottom_temperature != 0;
    p.bc.winkler_delta_rho = dp->winkler_delta_rho;
    p.bc.has_winkler_foundation = dp->has_winkler_foundation != 0;
    p.bc.elastic_foundation_constant = dp->elastic_foundation_constant;
    p.bc.has_elastic_foundation = dp->has_elastic_foundation != 0;
    p.bc.has_water_loading = dp->has_water_loading != 0;
    const int *t = dp->vbc_types;
    const double *v = dp->vbc_values;
    p.bc.vbc_x0 = t[0]; p.bc.vbc_x1 = t[1]; p.bc.vbc_y0 = t[2]; p.bc.vbc_y1 = t[3];
    p.bc.vbc_z0 = t[4]; p.bc.vbc_z1 = t[5]; p.bc.vbc_n0 = t[6]; p.bc.vbc_n1 = t[7];
    p.bc.vbc_n2 = t[8]; p.bc.vbc_n3 = t[9];
    p.bc.vbc_val_x0 = v[0]; p.bc.vbc_val_x1 = v[1]; p.bc.vbc_val_y0 = v[2]; p.bc.vbc_val_y1 = v[3];
    p.bc.vbc_val_z0 = v[4]; p.bc.vbc_val_z1 = v[5]; p.bc.vbc_val_n0 = v[6]; p.bc.vbc_val_n1 = v[7];
    p.bc.vbc_val_n2 = v[8]; p.bc.vbc_val_n3 = v[9];

    p.mesh.zlength = dp->zlength;
    if (ic) {
        p.mesh.xlength = ic->xlength;
        p.mesh.ylength = ic->ylength;
        p.mesh.zlength = ic->zlength;
        p.mesh.resolution = ic->resolution;
        p.ic.weakzone_option = ic->weakzone_option;
        p.ic.weakzone_plstrain = ic->weakzone_plstrain;
        p.ic.weakzone_azimuth = ic->weakzone_azimuth;
        p.ic.weakzone_inclination = ic->weakzone_inclination;
        p.ic.weakzone_halfwidth = ic->weakzone_halfwidth;
        p.ic.weakzone_y_min = ic->weakzone_y_min;
        p.ic.weakzone_y_max = ic->weakzone_y_max;
        p.ic.weakzone_depth_min = ic->weakzone_depth_min;
        p.ic.weakzone_depth_max = ic->weakzone_depth_max;
        p.ic.weakzone_xcenter = ic->weakzone_xcenter;
        p.ic.weakzone_ycenter = ic->weakzone_ycenter;
        p.ic.weakzone_zcenter = ic->weakzone_zcenter;
        p.ic.weakzone_xsemi_axis = ic->weakzone_xsemi_axis;
        p.ic.weakzone_ysemi_axis = ic->weakzone_ysemi_axis;
        p.ic.weakzone_zsemi_axis = ic->weakzone_zsemi_axis;
    }

    const int nm = dm->nmat;
    p.mat.rheol_type = dm->rheol_type;
    p.mat.nmat = nm;
    p.mat.is_plane_strain = dm->is_plane_strain != 0;
    p.mat.visc_min = dm->visc_min;
    p.mat.visc_max = dm->visc_max;
    p.mat.tension_max = dm->tension_max;
    p.mat.therm_diff_max = dm->therm_diff_max;
    /* a parameter flagged scalar is passed as a one-entry vector, which
     * VectorBase::create turns into Vector1 (matprops.cxx:176-187) */
    unsigned sm = dm->scalar_mask;
    fill_vec(p.mat.rho0, dm->rho0, nm);
    fill_vec(p.mat.alpha, dm->alpha, nm);
    fill_vec(p.mat.bulk_modulus, dm->bulk_modulus, (sm & 1u) ? 1 : nm);
    fill_vec(p.mat.shear_modulus, dm->shear_modulus, (sm & 2u) ? 1 : nm);
    fill_vec(p.mat.visc_exponent, dm->visc_exponent, nm);
    fill_vec(p.mat.visc_coefficient, dm->visc_coefficient, nm);
    fill_vec(p.mat.visc_activation_energy, dm->visc_activation_energy, nm);
    fill_vec(p.mat.heat_capacity, dm->heat_capacity, (sm & 4u) ? 1 : nm);
    fill_vec(p.mat.radiogenic_heating, dm->radiogenic_heating, (sm & 8u) ? 1 : nm);
    fill_vec(p.mat.therm_cond, dm->therm_cond, (sm & 16u) ? 1 : nm);
    fill_vec(p.mat.pls0, dm->pls0, nm);
    fill_vec(p.mat.pls1, dm->pls1, nm);
    fill_vec(p.mat.cohesion0, dm->cohesion0, nm);
    fill_vec(p.mat.cohesion1, dm->cohesion1, nm);
    fill_vec(p.mat.friction_angle0, dm->friction_angle0, nm);
    fill_vec(p.mat.friction_angle1, dm->friction_angle1, nm);
    fill_vec(p.mat.dilation_angle0, dm->dilation_angle0, nm);
    fill_vec(p.mat.dilation_angle1, dm->dilation_angle1, nm);
    p.debug.dt = false;
}

struct Model {
    Param param;
    Variables var;
};

void build_model(Model &md, const des_mesh *mesh, const des_params *dp, const des_material *dm,
                 const ref_ic *ic, const double *coord)
{
    Param &param = md.param;
    Variables &var = md.var;
    fill_param(param, dp, dm, ic);
    var.time = 0;
    var.steps = 0;
    var.dt = 0;
    var.nnode = mesh->nnode;
    var.nelem = mesh->nelem;
    var.nseg = 0;
    var.max_vbc_val = dp->max_vbc_val;
    var.compensation_pressure = dp->compensation_pressure;
    for (int i = 0; i < nbdrytypes; ++i) {
        var.vbc_types[i] = dp->vbc_types[i];
        var.vbc_values[i] = dp->vbc_values[i];
    }
    var.coord = new array_t(var.nnode);
    std::memcpy(var.coord->data(), coord, sizeof(double) * NDIMS * var.nnode);
    var.connectivity = new conn_t(var.nelem);
    std::memcpy(var.connectivity->data(), mesh->connectivity, sizeof(int) * NODES_PER_ELEM * var.nelem);
    var.segment = NULL;
    var.segflag = NULL;
    var.regattr = NULL;
    var.bcflag = new uint_vec(mesh->bcflag, mesh->bcflag + var.nnode);
    for (int n = 0; n < var.nnode; ++n)
        for (int j = 0; j < nbdrytypes; ++j)
            if ((*var.bcflag)[n] & (1u << j)) var.bnodes[j].push_back(n);
    for (int i = 0; i < nbdrytypes; ++i)
        for (int q = mesh->bfacet_offsets[i]; q < mesh->bfacet_offsets[i + 1]; ++q)
            var.bfacets[i].push_back(std::make_pair(mesh->bfacets[2 * q], mesh->bfacets[2 * q + 1]));
    var.support = NULL;
    var.egroups.clear();
#ifdef USE_OMP
    /* the element bands of the OpenMP build: 2T contiguous bands of equal
     * size, the last one taking the remainder, as create_elem_groups lays
     * them out (mesh.cxx:1724-1747); mesh.cxx itself needs TetGen and
     * Triangle, so the harness forms the bands */
    {
        const int ngroups = 2 * omp_get_max_threads();
        const int per = var.nelem / ngroups;
        for (int i = 0; i < ngroups; ++i) var.egroups.push_back(i * per);
    }
#else
    var.egroups.push_back(0);
#endif
    var.egroups.push_back(var.nelem);
    var.elemmarkers = new int_vec2D(var.nelem, std::vector<int>(dm->nmat, 0));
    for (int e = 0; e < var.nelem; ++e)
        for (int m = 0; m < dm->nmat; ++m)
            (*var.elemmarkers)[e][m] = dm->elemmarkers ? dm->elemmarkers[(size_t)e * dm->nmat + m] : (m == 0);
    var.hydrous_elemmarkers = NULL;
    var.phch = NULL;
    var.shpdy = NULL;
    allocate_variables(param, var);
    for (int i = 0; i < nbdrytypes; ++i)
        for (int d = 0; d < NDIMS; ++d) var.bnormals[i][d] = mesh->bnormals[i][d];
    for (int i = 0; i < nbdrytypes; ++i)
        for (int j = i + 1; j < nbdrytypes; ++j) {
            double *s = new double[NDIMS];
            for (int d = 0; d < NDIMS; ++d) s[d] = mesh->edge_vectors[i][j][d];
            var.edge_vectors[std::make_pair(i, j)] = s;
        }
}

template <class A>
void put(A &dst, const double *src)
{
    if (src) std::memcpy(dst.data(), src, sizeof(double) * dst.num_elements());
}
void putv(double_vec &dst, const double *src)
{
    if (src) std::memcpy(dst.data(), src, sizeof(double) * dst.size());
}
template <class A>
void get(const A &src, double *dst)
{
    if (dst) std::memcpy(dst, src.data(), sizeof(double) * src.num_elements());
}
void getv(const double_vec &src, double *dst)
{
    if (dst) std::memcpy(dst, src.data(), sizeof(double) * src.size());
}

void state_in(Variables &var, const des_host_state *st)
{
    put(*var.coord, st->coord);
    put(*var.coord0, st->coord0);
    put(*var.vel, st->vel);
    put(*var.force, st->force);
    putv(*var.temperature, st->temperature);
    putv(*var.mass, st->mass);
    putv(*var.tmass, st->tmass);
    putv(*var.volume_n, st->volume_n);
    putv(*var.ntmp, st->ntmp);
    putv(*var.volume, st->volume);
    putv(*var.volume_old, st->volume_old);
    put(*var.stress, st->stress);
    put(*var.strain, st->strain);
    put(*var.strain_rate, st->strain_rate);
    putv(*var.plstrain, st->plstrain);
    putv(*var.delta_plstrain, st->delta_plstrain);
    putv(*var.stressyy, st->stressyy);
    putv(*var.dpressure, st->dpressure);
    putv(*var.edvoldt, st->edvoldt);
    put(*var.shpdx, st->shpdx);
    if (NDIMS == 3) put(*var.shpdy, st->shpdy);
    put(*var.shpdz, st->shpdz);
    var.time = st->time;
    var.dt = st->dt;
    var.steps = st->steps;
}

void state_out(const Variables &var, des_host_state *st)
{
    get(*var.coord, st->coord);
    get(*var.coord0, st->coord0);
    get(*var.vel, st->vel);
    get(*var.force, st->force);
    getv(*var.temperature, st->temperature);
    getv(*var.mass, st->mass);
    getv(*var.tmass, st->tmass);
    getv(*var.volume_n, st->volume_n);
    getv(*var.ntmp, st->ntmp);
    getv(*var.volume, st->volume);
    getv(*var.volume_old, st->volume_old);
    get(*var.stress, st->stress);
    get(*var.strain, st->strain);
    get(*var.strain_rate, st->strain_rate);
    getv(*var.plstrain, st->plstrain);
    getv(*var.delta_plstrain, st->delta_plstrain);
    getv(*var.stressyy, st->stressyy);
    getv(*var.dpressure, st->dpressure);
    getv(*var.edvoldt, st->edvoldt);
    get(*var.shpdx, st->shpdx);
    if (NDIMS == 3) get(*var.shpdy, st->shpdy);
    get(*var.shpdz, st->shpdz);
    st->time = var.time;
    st->dt = var.dt;
    st->steps = var.steps;
}

void update_mesh_(const Param &param, Variables &var) /* dynearthsol.cxx:221-232 */
{
    update_coordinate(var, *var.coord);
    surface_processes(param, var, *var.coord);
    var.volume->swap(*var.volume_old);
    compute_volume(*var.coord, *var.connectivity, *var.volume);
    compute_mass(param, var.egroups, *var.connectivity, *var.volume, *var.mat,
                 var.max_vbc_val, *var.volume_n, *var.mass, *var.tmass);
    compute_shape_fn(*var.coord, *var.connectivity, *var.volume, var.egroups,
                     *var.shpdx, *var.shpdy, *var.shpdz);
}

}  // namespace

extern "C" {

/* The reference's init sequence (dynearthsol.cxx:82-98) on a given mesh and
 * initial temperature; writes the initialised state, the boundary normals
 * and the compensation pressure.  st->temperature is the input geotherm. */
int ref_init(const des_mesh *mesh, const des_params *dp, const des_material *dm, const ref_ic *ic,
             des_host_state *st, double *bnormals_out, double *edge_out, double *comp_pressure)
{
    Model md;
    build_model(md, mesh, dp, dm, ic, st->coord);
    Variables &var = md.var;
    const Param &param = md.param;
    for (int i = 0; i < var.nnode; i++)
        for (int d = 0; d < NDIMS; d++) (*var.coord0)[i][d] = (*var.coord)[i][d];
    compute_volume(*var.coord, *var.connectivity, *var.volume);
    *var.volume_old = *var.volume;
    compute_mass(param, var.egroups, *var.connectivity, *var.volume, *var.mat,
                 var.max_vbc_val, *var.volume_n, *var.mass, *var.tmass);
    compute_shape_fn(*var.coord, *var.connectivity, *var.volume, var.egroups,
                     *var.shpdx, *var.shpdy, *var.shpdz);
    create_boundary_normals(var, var.bnormals, var.edge_vectors);
    apply_vbcs(param, var, *var.vel);
    putv(*var.temperature, st->temperature);
    initial_stress_state(param, var, *var.stress, *var.stressyy, *var.strain, var.compensation_pressure);
    initial_weak_zone(param, var, *var.plstrain);
    var.dt = compute_dt(param, var);
    state_out(var, st);
    for (int i = 0; i < nbdrytypes; ++i)
        for (int d = 0; d < NDIMS; ++d) bnormals_out[i * 3 + d] = var.bnormals[i][d];
    for (auto &kv : var.edge_vectors)
        for (int d = 0; d < NDIMS; ++d)
            edge_out[(kv.first.first * nbdrytypes + kv.first.second) * 3 + d] = kv.second[d];
    *comp_pressure = var.compensation_pressure;
    return 0;
}

/* nsteps of the loop body (dynearthsol.cxx:325-361) on a given state.  When
 * record is not NULL, the (per-step) dt values are written there; when
 * seconds is not NULL, the wall time of the loop alone (no model set-up or
 * state copies). */
int ref_run_timed(const des_mesh *mesh, const des_params *dp, const des_material *dm, des_host_state *st,
                  int nsteps, double *record_dt, double *seconds)
{
    Model md;
    build_model(md, mesh, dp, dm, NULL, st->coord);
    Variables &var = md.var;
    const Param &param = md.param;
    state_in(var, st);
    if (desgpu_shim_sync_to_device) desgpu_shim_sync_to_device();
    const auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; it < nsteps; ++it) {
        var.steps++;
        var.time += var.dt;
        if (param.control.has_thermal_diffusion)
            update_temperature(param, var, *var.temperature, *var.ntmp);
        update_strain_rate(var, *var.strain_rate);
        compute_dvoldt(var, *var.ntmp);
        compute_edvoldt(var, *var.ntmp, *var.edvoldt);
        update_stress(var, *var.stress, *var.stressyy, *var.dpressure, *var.strain,
                      *var.plstrain, *var.delta_plstrain, *var.strain_rate);
        NMD_stress(var, *var.ntmp, *var.stress);
        update_force(param, var, *var.force);
        update_velocity(var, *var.vel);
        apply_vbcs(param, var, *var.vel);
        update_mesh_(param, var);
        if (var.mat->rheol_type & MatProps::rh_elastic)
            rotate_stress(var, *var.stress, *var.strain);
        if (var.steps % 10 == 0) var.dt = compute_dt(param, var);
        if (record_dt) record_dt[it] = var.dt;
    }
    if (desgpu_shim_sync_to_host) desgpu_shim_sync_to_host();
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    state_out(var, st);
    return 0;
}

int ref_run(const des_mesh *mesh, const des_params *dp, const des_material *dm, des_host_state *st,
            int nsteps, double *record_dt)
{
    return ref_run_timed(mesh, dp, dm, st, nsteps, record_dt, NULL);
}

/* The reference's bad_mesh_quality (remeshing.cxx:1882-1935) on a given
 * state: returns its code (0 good, 1 element quality, 2 bottom node drift,
 * 3 tiny element) and writes the index it reports. */
int ref_bad_mesh_quality(const des_mesh *mesh, const des_params *dp, const des_material *dm,
                         const ref_quality *rq, des_host_state *st, int *index)
{
    Model md;
    build_model(md, mesh, dp, dm, NULL, st->coord);
    Variables &var = md.var;
    Param &param = md.param;
    state_in(var, st);
    param.mesh.smallest_size = rq->smallest_size;
    param.mesh.resolution = rq->resolution;
    param.mesh.min_quality = rq->min_quality;
    param.mesh.max_boundary_distortion = rq->max_boundary_distortion;
    param.mesh.zlength = rq->zlength;
    param.mesh.remeshing_option = rq->remeshing_option;
    if (desgpu_shim_sync_to_device) desgpu_shim_sync_to_device();
    int idx = -1;
    int code = bad_mesh_quality(param, var, idx);
    *index = idx;
    return code;
}

/* One reference function on a given state, by name; used to pin the
 * per-function restatements. */
int ref_call(const des_mesh *mesh, const des_params *dp, const des_material *dm, des_host_state *st,
             const char *name, double *result)
{
    Model md;
    build_model(md, mesh, dp, dm, NULL, st->coord);
    Variables &var = md.var;
    const Param &param = md.param;
    state_in(var, st);
    std::string f(name);
    if (f == "update_temperature") update_temperature(param, var, *var.temperature, *var.ntmp);
    else if (f == "update_strain_rate") update_strain_rate(var, *var.strain_rate);
    else if (f == "compute_dvoldt") compute_dvoldt(var, *var.ntmp);
    else if (f == "compute_edvoldt") compute_edvoldt(var, *var.ntmp, *var.edvoldt);
    else if (f == "update_stress")
        update_stress(var, *var.stress, *var.stressyy, *var.dpressure, *var.strain,
                      *var.plstrain, *var.delta_plstrain, *var.strain_rate);
    else if (f == "NMD_stress") NMD_stress(var, *var.ntmp, *var.stress);
    else if (f == "update_force") update_force(param, var, *var.force);
    else if (f == "update_velocity") update_velocity(var, *var.vel);
    else if (f == "apply_vbcs") apply_vbcs(param, var, *var.vel);
    else if (f == "update_coordinate") update_coordinate(var, *var.coord);
    else if (f == "compute_volume") compute_volume(*var.coord, *var.connectivity, *var.volume);
    else if (f == "compute_mass")
        compute_mass(param, var.egroups, *var.connectivity, *var.volume, *var.mat,
                     var.max_vbc_val, *var.volume_n, *var.mass, *var.tmass);
    else if (f == "compute_shape_fn")
        compute_shape_fn(*var.coord, *var.connectivity, *var.volume, var.egroups,
                         *var.shpdx, *var.shpdy, *var.shpdz);
    else if (f == "rotate_stress") rotate_stress(var, *var.stress, *var.strain);
    else if (f == "compute_dt") *result = compute_dt(param, var);
    else if (f == "worst_elem_quality") {
        int worst;
        *result = worst_elem_quality(*var.coord, *var.connectivity, *var.volume, worst);
        result[1] = worst;
    } else return 1;
    state_out(var, st);
    return 0;
}

/* The reference's create_support (mesh.cxx:1707-1721) of a connectivity,
 * as CSR: off[nnode+1], elems[nelem*NODES_PER_ELEM]. */
int ref_create_support(int nnode, int nelem, const int *conn, int *off, int *elems)
{
    Variables var = Variables();
    var.nnode = nnode;
    var.nelem = nelem;
    var.connectivity = new conn_t(nelem);
    std::memcpy(var.connectivity->data(), conn, sizeof(int) * NODES_PER_ELEM * nelem);
    create_support(var);
    off[0] = 0;
    for (int n = 0; n < nnode; ++n) {
        const int_vec &s = (*var.support)[n];
        for (std::size_t k = 0; k < s.size(); ++k) elems[off[n] + k] = s[k];
        off[n + 1] = off[n] + (int)s.size();
    }
    delete var.support;
    delete var.connectivity;
    return 0;
}

/* The reference's create_boundary_facets (mesh.cxx:1637-1704) of a mesh and
 * its boundary segments (Variables::segment, segflag, as the mesher gives
 * them): offsets[nbdrytypes+1], facets[nfacets][2] = (element, facet). */
int ref_create_boundary_facets(int nnode, int nelem, const int *conn, const unsigned *bcflag, int nseg,
                               const int *segment, const int *segflag, int *offsets, int *facets)
{
    Variables var = Variables();
    var.nnode = nnode;
    var.nelem = nelem;
    var.nseg = nseg;
    var.connectivity = new conn_t(nelem);
    std::memcpy(var.connectivity->data(), conn, sizeof(int) * NODES_PER_ELEM * nelem);
    var.bcflag = new uint_vec(bcflag, bcflag + nnode);
    var.segment = new segment_t(nseg);
    std::memcpy(var.segment->data(), segment, sizeof(int) * NDIMS * nseg);
    var.segflag = new segflag_t(nseg);
    std::memcpy(var.segflag->data(), segflag, sizeof(int) * nseg);
    create_boundary_facets(var);
    offsets[0] = 0;
    for (int i = 0; i < nbdrytypes; ++i) {
        for (std::size_t k = 0; k < var.bfacets[i].size(); ++k) {
            facets[2 * (offsets[i] + k)] = var.bfacets[i][k].first;
            facets[2 * (offsets[i] + k) + 1] = var.bfacets[i][k].second;
        }
        offsets[i + 1] = offsets[i] + (int)var.bfacets[i].size();
    }
    delete var.connectivity;
    delete var.bcflag;
    delete var.segment;
    delete var.segflag;
    return 0;
}

/* The reference's phase_changes (phasechanges.cxx:232-258), option
 * phase_change_option, on a marker set given as arrays (element, barycentric
 * eta[NODES_PER_ELEM], material type) and a state; hydem[nelem] are the
 * hydrous-marker counts that SimpleSubduction reads.  Hydration processes
 * are off.  Writes the new material types and marker counts
 * (elemmarkers[nelem][nmat], in/out). */
int ref_phase_changes(const des_mesh *mesh, const des_params *dp, const des_material *dm, des_host_state *st,
                      int option, int nmarkers, const int *melem, const double *meta, int *mattype,
                      const int *hydem, int *elemmarkers)
{
    Model md;
    build_model(md, mesh, dp, dm, NULL, st->coord);
    Variables &var = md.var;
    Param &param = md.param;
    state_in(var, st);
    param.mat.phase_change_option = option;
    param.control.has_hydration_processes = false;
    const int nm = dm->nmat;
    for (int e = 0; e < var.nelem; ++e)
        for (int k = 0; k < nm; ++k) (*var.elemmarkers)[e][k] = elemmarkers[(size_t)e * nm + k];
    MarkerSet *ms = new MarkerSet("markerset");
    for (int m = 0; m < nmarkers; ++m) ms->append_marker(meta + (size_t)m * NODES_PER_ELEM, melem[m], mattype[m]);
    MarkerSet *hyd = new MarkerSet("hydrous-markerset");
    var.markersets.push_back(ms);
    var.markersets.push_back(hyd);
    var.hydrous_marker_index = 1;
    var.hydrous_elemmarkers = new Array2D<int, 1>(var.nelem);
    for (int e = 0; e < var.nelem; ++e) (*var.hydrous_elemmarkers)[e][0] = hydem ? hydem[e] : 0;
    var.phch = NULL;
    phase_changes_init(param, var);
    phase_changes(param, var);
    for (int m = 0; m < nmarkers; ++m) mattype[m] = ms->get_mattype(m);
    for (int e = 0; e < var.nelem; ++e)
        for (int k = 0; k < nm; ++k) elemmarkers[(size_t)e * nm + k] = (*var.elemmarkers)[e][k];
    delete var.phch;
    delete var.hydrous_elemmarkers;
    delete hyd;
    delete ms;
    return 0;
}

/* One output frame written by the reference's BinaryOutput (binaryio.cxx),
 * with the array names, types and order of Output::write
 * (output.cxx:93-179, not averaged, no markers): the pin of the library's
 * .save writer (des_write_save_host). */
int ref_write_save(const char *filename, const des_save_frame *fr)
{
    if (fr->ndims != NDIMS) return 1;
    const int nn = fr->nnode, ne = fr->nelem;
    BinaryOutput bin(filename);
    array_t coord(nn), vel(nn), force(nn), coord0(nn);
    conn_t conn(ne);
    tensor_t srate(ne), strain(ne), stress(ne);
    std::memcpy(coord.data(), fr->coord, sizeof(double) * nn * NDIMS);
    std::memcpy(vel.data(), fr->vel, sizeof(double) * nn * NDIMS);
    std::memcpy(force.data(), fr->force, sizeof(double) * nn * NDIMS);
    std::memcpy(coord0.data(), fr->coord0, sizeof(double) * nn * NDIMS);
    std::memcpy(conn.data(), fr->connectivity, sizeof(int) * ne * NODES_PER_ELEM);
    std::memcpy(srate.data(), fr->strain_rate, sizeof(double) * ne * NSTR);
    std::memcpy(strain.data(), fr->strain, sizeof(double) * ne * NSTR);
    std::memcpy(stress.data(), fr->stress, sizeof(double) * ne * NSTR);
    double_vec T(fr->temperature, fr->temperature + nn), pls(fr->plstrain, fr->plstrain + ne),
        dpls(fr->delta_plstrain, fr->delta_plstrain + ne), rho(fr->density, fr->density + ne),
        quality(fr->mesh_quality, fr->mesh_quality + ne), visc(fr->viscosity, fr->viscosity + ne),
        material(fr->material, fr->material + ne);
    uint_vec bcflag(fr->bcflag, fr->bcflag + nn);
    bin.write_array(coord, "coordinate", coord.size());
    bin.write_array(conn, "connectivity", conn.size());
    bin.write_array(vel, "velocity", vel.size());
    bin.write_array(T, "temperature", T.size());
    bin.write_array(pls, "plastic strain", pls.size());
    bin.write_array(dpls, "plastic strain-rate", dpls.size());
    bin.write_array(srate, "strain-rate", srate.size());
    bin.write_array(strain, "strain", strain.size());
    bin.write_array(stress, "stress", stress.size());
    bin.write_array(rho, "density", rho.size());
    bin.write_array(quality, "mesh quality", quality.size());
    bin.write_array(visc, "viscosity", visc.size());
    bin.write_array(material, "material", material.size());
    bin.write_array(force, "force", force.size());
    bin.write_array(coord0, "coord0", coord0.size());
    bin.write_array(bcflag, "bcflag", bcflag.size());
    bin.close();
    return 0;
}

}  // extern "C"
