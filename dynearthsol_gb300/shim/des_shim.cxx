// des_shim.cxx -- the reference's hot-path functions, with the reference's
// own C++ signatures, implemented over the C ABI of libdesgpu.so.
//
// Link-time substitution: compile this file against the reference's headers
// (-I<reference tree>, plus -DTHREED for the 3D build) and link it IN PLACE
// of fields.o, geometry.o and rheology.o.  Every symbol those three objects
// define is defined here (fields.hpp, geometry.hpp, rheology.hpp); the rest
// of the reference (dynearthsol.cxx's main loop, bc.o, matprops.o, mesh,
// remeshing, markers, output) is unchanged.
//
// Residency modes:
// * sync (default): each call uploads the Variables fields it reads and
//   downloads the fields it writes, so the host arrays stay authoritative
//   and any caller (init, restart, isostasy adjustment, remeshing, output)
//   sees exactly what the reference would leave there.
// * resident (environment DESGPU_SHIM_RESIDENT=1): state stays on the
//   device between calls; the host program calls desgpu_shim_sync_to_host()
//   before reading Variables (output, quality check, remesh) and
//   desgpu_shim_sync_to_device() after changing them.  update_velocity then
//   also applies the velocity BCs on the device, since the main loop always
//   calls apply_vbcs right after it (dynearthsol.cxx:341-342) and bc.o's
//   host apply_vbcs only sees the stale host copy.
//
// The context is (re)created when allocate_variables/reallocate_variables
// run (init, restart, after remeshing: fields.cxx:10-93) and when the
// boundary normals change (create_boundary_normals runs after
// allocate_variables in init, dynearthsol.cxx:93).  Errors print the
// library's message and exit with its code, as the reference exits
// (DEVELOPING:32-37).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <vector>

#include "constants.hpp"
#include "parameters.hpp"
#include "matprops.hpp"
#include "fields.hpp"
#include "geometry.hpp"
#include "rheology.hpp"
#include "remeshing.hpp"

#include "desgpu.h"

extern "C" {
void desgpu_shim_sync_to_host(void);
void desgpu_shim_sync_to_device(void);
}

namespace {

struct Shim {
    const Param *param = nullptr;
    Variables *var = nullptr;
    des_ctx *ctx = nullptr;
    bool resident = false;
    // host arrays of volume and volume_old as the device last saw them: the
    // main loop swaps the two pointers (dynearthsol.cxx:226) before
    // compute_volume, which the device mirrors in resident mode
    const double *vol_seen = nullptr, *vol_old_seen = nullptr;
    double bn_cache[nbdrytypes][NDIMS];
    // storage the C structs point into
    std::vector<int> bfacet_off, bfacets, emark;
    std::vector<double> mat_arrays[18];
    des_mesh mesh;
    des_params prm;
    des_material mat;
} g;

void die(int code)
{
    char buf[512];
    des_last_error(g.ctx, buf, sizeof buf);
    std::cerr << "Error (desgpu): " << buf << '\n';
    std::exit(code == DES_EINPUT ? 1 : code == DES_ERUNTIME ? 11 : 12);
}

void check(int rc)
{
    if (rc != DES_OK) die(rc);
}

void fill_params(const Param &p, const Variables &v, des_params &d)
{
    std::memset(&d, 0, sizeof d);
    d.gravity = p.control.gravity;
    d.inertial_scaling = p.control.inertial_scaling;
    d.dt_fraction = p.control.dt_fraction;
    d.fixed_dt = p.control.fixed_dt;
    d.damping_factor = p.control.damping_factor;
    d.surface_diffusivity = p.control.surface_diffusivity;
    d.max_vbc_val = v.max_vbc_val;
    d.damping_option = p.control.damping_option;
    d.ref_pressure_option = p.control.ref_pressure_option;
    d.surface_process_option = p.control.surface_process_option;
    d.is_quasi_static = p.control.is_quasi_static;
    d.has_thermal_diffusion = p.control.has_thermal_diffusion;
    d.surface_temperature = p.bc.surface_temperature;
    d.mantle_temperature = p.bc.mantle_temperature;
    d.winkler_delta_rho = p.bc.winkler_delta_rho;
    d.elastic_foundation_constant = p.bc.elastic_foundation_constant;
    d.has_fixed_bottom_temperature = p.bc.has_fixed_bottom_temperature;
    d.has_winkler_foundation = p.bc.has_winkler_foundation;
    d.has_elastic_foundation = p.bc.has_elastic_foundation;
    d.has_water_loading = p.bc.has_water_loading;
    for (int i = 0; i < nbdrytypes; ++i) {
        d.vbc_types[i] = v.vbc_types[i];
        d.vbc_values[i] = v.vbc_values[i];
    }
    d.zlength = p.mesh.zlength;
    d.compensation_pressure = v.compensation_pressure;
}

void fill_material(const Param &p, const Variables &v)
{
    const Mat &m = p.mat;
    const int nm = m.nmat;
    const double_vec *src[18] = {&m.rho0, &m.alpha, &m.bulk_modulus, &m.shear_modulus, &m.visc_exponent,
                                 &m.visc_coefficient, &m.visc_activation_energy, &m.heat_capacity,
                                 &m.therm_cond, &m.radiogenic_heating, &m.pls0, &m.pls1, &m.cohesion0,
                                 &m.cohesion1, &m.friction_angle0, &m.friction_angle1, &m.dilation_angle0,
                                 &m.dilation_angle1};
    const double **dst[18] = {&g.mat.rho0, &g.mat.alpha, &g.mat.bulk_modulus, &g.mat.shear_modulus,
                              &g.mat.visc_exponent, &g.mat.visc_coefficient, &g.mat.visc_activation_energy,
                              &g.mat.heat_capacity, &g.mat.therm_cond, &g.mat.radiogenic_heating, &g.mat.pls0,
                              &g.mat.pls1, &g.mat.cohesion0, &g.mat.cohesion1, &g.mat.friction_angle0,
                              &g.mat.friction_angle1, &g.mat.dilation_angle0, &g.mat.dilation_angle1};
    // a one-value parameter is VectorBase::create's Vector1 (matprops.cxx:176-187)
    const int scalar_bit[18] = {-1, -1, 0, 1, -1, -1, -1, 2, 4, 3, -1, -1, -1, -1, -1, -1, -1, -1};
    g.mat.scalar_mask = 0;
    for (int k = 0; k < 18; ++k) {
        std::vector<double> &a = g.mat_arrays[k];
        a.assign(nm, (*src[k])[0]);
        if ((int)src[k]->size() == nm)
            for (int i = 0; i < nm; ++i) a[i] = (*src[k])[i];
        else if (scalar_bit[k] >= 0 && nm > 1)
            g.mat.scalar_mask |= 1u << scalar_bit[k];
        *dst[k] = a.data();
    }
    g.mat.rheol_type = m.rheol_type;
    g.mat.nmat = nm;
    g.mat.is_plane_strain = m.is_plane_strain;
    g.mat.visc_min = m.visc_min;
    g.mat.visc_max = m.visc_max;
    g.mat.tension_max = m.tension_max;
    g.mat.therm_diff_max = m.therm_diff_max;
    g.mat.elemmarkers = nullptr;
    if (nm > 1 && v.elemmarkers) {
        g.emark.resize((size_t)v.nelem * nm);
        for (int e = 0; e < v.nelem; ++e)
            for (int i = 0; i < nm; ++i) g.emark[(size_t)e * nm + i] = (*v.elemmarkers)[e][i];
        g.mat.elemmarkers = g.emark.data();
    }
}

void destroy_ctx()
{
    if (g.ctx) des_destroy(g.ctx);
    g.ctx = nullptr;
}

void create_ctx()
{
    destroy_ctx();
    const Variables &v = *g.var;
    std::memset(&g.mesh, 0, sizeof g.mesh);
    g.mesh.ndims = NDIMS;
    g.mesh.nnode = v.nnode;
    g.mesh.nelem = v.nelem;
    g.mesh.connectivity = v.connectivity->data();
    g.mesh.bcflag = v.bcflag->data();
    g.bfacet_off.assign(nbdrytypes + 1, 0);
    g.bfacets.clear();
    for (int i = 0; i < nbdrytypes; ++i) {
        for (const auto &pr : v.bfacets[i]) {
            g.bfacets.push_back(pr.first);
            g.bfacets.push_back(pr.second);
        }
        g.bfacet_off[i + 1] = (int)g.bfacets.size() / 2;
    }
    g.mesh.bfacet_offsets = g.bfacet_off.data();
    g.mesh.bfacets = g.bfacets.empty() ? nullptr : g.bfacets.data();
    for (int i = 0; i < nbdrytypes; ++i)
        for (int d = 0; d < NDIMS; ++d) {
            g.mesh.bnormals[i][d] = v.bnormals[i][d];
            g.bn_cache[i][d] = v.bnormals[i][d];
        }
    for (const auto &kv : v.edge_vectors)
        for (int d = 0; d < NDIMS; ++d) g.mesh.edge_vectors[kv.first.first][kv.first.second][d] = kv.second[d];
    fill_params(*g.param, v, g.prm);
    fill_material(*g.param, v);
    int rc = des_create(&g.mesh, &g.prm, &g.mat, DES_PREC_FP64, nullptr, &g.ctx);
    if (rc) die(rc);
    g.vol_seen = v.volume->data();
    g.vol_old_seen = v.volume_old->data();
}

// host view of the current Variables arrays (pointers re-read every call:
// update_mesh swaps volume and volume_old, dynearthsol.cxx:226)
des_host_state view()
{
    Variables &v = *g.var;
    des_host_state s;
    std::memset(&s, 0, sizeof s);
    s.coord = v.coord->data();
    s.coord0 = v.coord0->data();
    s.vel = v.vel->data();
    s.force = v.force->data();
    s.temperature = v.temperature->data();
    s.mass = v.mass->data();
    s.tmass = v.tmass->data();
    s.volume_n = v.volume_n->data();
    s.ntmp = v.ntmp->data();
    s.volume = v.volume->data();
    s.volume_old = v.volume_old->data();
    s.stress = v.stress->data();
    s.strain = v.strain->data();
    s.strain_rate = v.strain_rate->data();
    s.plstrain = v.plstrain->data();
    s.delta_plstrain = v.delta_plstrain->data();
    s.stressyy = v.stressyy->data();
    s.dpressure = v.dpressure->data();
    s.edvoldt = v.edvoldt->data();
    s.shpdx = v.shpdx->data();
    s.shpdy = (NDIMS == 3) ? v.shpdy->data() : nullptr;
    s.shpdz = v.shpdz->data();
    s.time = v.time;
    s.dt = v.dt;
    s.steps = v.steps;
    return s;
}

// the context of the current Variables, refreshed where the host changed it
des_ctx *ctx()
{
    if (!g.var || !g.param) {
        std::cerr << "Error (desgpu): hot-path call before allocate_variables\n";
        std::exit(12);
    }
    bool normals_changed = false;
    for (int i = 0; i < nbdrytypes; ++i)
        for (int d = 0; d < NDIMS; ++d) normals_changed |= g.bn_cache[i][d] != g.var->bnormals[i][d];
    if (!g.ctx || normals_changed) {
        create_ctx();
        if (g.resident) desgpu_shim_sync_to_device();
    }
    des_params now;
    fill_params(*g.param, *g.var, now);
    if (std::memcmp(&now, &g.prm, sizeof now) != 0) {
        g.prm = now;
        check(des_set_params(g.ctx, &g.prm));
    }
    return g.ctx;
}

// sync-mode transfers around one call
void up(unsigned mask)
{
    if (g.resident) return;
    des_host_state s = view();
    check(des_upload_fields(ctx(), &s, mask | DES_F_CLOCK));
}

void down(unsigned mask)
{
    if (g.resident) return;
    des_host_state s = view();
    check(des_download_fields(ctx(), &s, mask));
}

const unsigned F_SHP = DES_F_SHP;

}  // namespace

extern "C" {

// download every Variables field the hot path keeps on the device
void desgpu_shim_sync_to_host(void)
{
    if (!g.ctx) return;
    des_host_state s = view();
    check(des_download_fields(g.ctx, &s, DES_F_ALL & ~DES_F_CLOCK));
}

// upload every Variables field (after init, restart, remeshing or any host change)
void desgpu_shim_sync_to_device(void)
{
    if (!g.var) return;
    des_host_state s = view();
    check(des_upload_fields(ctx(), &s, DES_F_ALL));
    g.vol_seen = g.var->volume->data();
    g.vol_old_seen = g.var->volume_old->data();
}

}  // extern "C"

// ---------------------------------------------------------------------
// fields.hpp
// ---------------------------------------------------------------------
void allocate_variables(const Param &param, Variables &var)   // fields.cxx:10-48
{
    const int n = var.nnode;
    const int e = var.nelem;
    var.volume = new double_vec(e);
    var.volume_old = new double_vec(e);
    var.volume_n = new double_vec(n);
    var.mass = new double_vec(n);
    var.tmass = new double_vec(n);
    var.edvoldt = new double_vec(e);
    var.temperature = new double_vec(n);
    var.coord0 = new array_t(n);
    var.plstrain = new double_vec(e);
    var.delta_plstrain = new double_vec(e);
    var.vel = new array_t(n, 0);
    var.strain = new tensor_t(e, 0);
    var.stress = new tensor_t(e, 0);
    var.stressyy = new double_vec(e, 0);
    var.ntmp = new double_vec(n);
    var.dpressure = new double_vec(e);
    var.force = new array_t(n, 0);
    var.strain_rate = new tensor_t(e, 0);
    var.shpdx = new shapefn(e);
    if (NDIMS == 3) var.shpdy = new shapefn(e);
    var.shpdz = new shapefn(e);
    var.mat = new MatProps(param, var);
    g.param = &param;
    g.var = &var;
    g.resident = std::getenv("DESGPU_SHIM_RESIDENT") && std::atoi(std::getenv("DESGPU_SHIM_RESIDENT")) != 0;
    destroy_ctx();   // created on the first hot-path call, once normals exist
}

void reallocate_variables(const Param &param, Variables &var)   // fields.cxx:51-93
{
    const int n = var.nnode;
    const int e = var.nelem;
    delete var.volume;
    delete var.volume_old;
    delete var.volume_n;
    var.volume = new double_vec(e);
    var.volume_old = new double_vec(e);
    var.volume_n = new double_vec(n);
    delete var.mass;
    delete var.tmass;
    var.mass = new double_vec(n);
    var.tmass = new double_vec(n);
    delete var.edvoldt;
    var.edvoldt = new double_vec(e);
    delete var.ntmp;
    var.ntmp = new double_vec(n);
    delete var.dpressure;
    var.dpressure = new double_vec(e);
    delete var.force;
    var.force = new array_t(n, 0);
    delete var.strain_rate;
    var.strain_rate = new tensor_t(e, 0);
    delete var.shpdx;
    delete var.shpdz;
    var.shpdx = new shapefn(e);
    if (NDIMS == 3) {
        delete var.shpdy;
        var.shpdy = new shapefn(e);
    }
    var.shpdz = new shapefn(e);
    delete var.mat;
    var.mat = new MatProps(param, var);
    g.param = &param;
    g.var = &var;
    destroy_ctx();   // the topology changed: new context on the next call
}

void update_temperature(const Param &, const Variables &, double_vec &, double_vec &)
{
    up(DES_F_TEMPERATURE | F_SHP | DES_F_VOLUME | DES_F_TMASS);
    check(des_update_temperature(ctx()));
    down(DES_F_TEMPERATURE | DES_F_NTMP);
}

void update_strain_rate(const Variables &, tensor_t &)
{
    up(DES_F_VEL | F_SHP);
    check(des_update_strain_rate(ctx()));
    down(DES_F_STRAIN_RATE);
}

void update_force(const Param &, const Variables &, array_t &)
{
    up(DES_F_STRESS | F_SHP | DES_F_VOLUME | DES_F_TEMPERATURE | DES_F_COORD | DES_F_COORD0 | DES_F_VEL);
    check(des_update_force(ctx()));
    down(DES_F_FORCE);
}

void update_velocity(const Variables &, array_t &)
{
    up(DES_F_VEL | DES_F_FORCE | DES_F_MASS);
    check(des_update_velocity(ctx()));
    if (g.resident) check(des_apply_vbcs(ctx()));
    down(DES_F_VEL);
}

void update_coordinate(const Variables &, array_t &)
{
    up(DES_F_COORD | DES_F_VEL);
    check(des_update_coordinate(ctx()));
    down(DES_F_COORD);
}

void rotate_stress(const Variables &, tensor_t &, tensor_t &)
{
    up(DES_F_VEL | F_SHP | DES_F_STRESS | DES_F_STRAIN);
    check(des_rotate_stress(ctx()));
    down(DES_F_STRESS | DES_F_STRAIN);
}

// ---------------------------------------------------------------------
// geometry.hpp
// ---------------------------------------------------------------------
double dist2(const double *a, const double *b)   // geometry.cxx:16-24
{
    double sum = 0;
    for (int i = 0; i < NDIMS; ++i) {
        double d = b[i] - a[i];
        sum += d * d;
    }
    return sum;
}

void compute_volume(const array_t &, const conn_t &, double_vec &)
{
    up(DES_F_COORD);
    des_ctx *c = ctx();
    const double *vol = g.var->volume->data(), *vol_old = g.var->volume_old->data();
    if (g.resident && vol == g.vol_old_seen && vol_old == g.vol_seen)
        check(des_swap_volume(c));   // the host swapped volume and volume_old: keep the old volume
    g.vol_seen = vol;
    g.vol_old_seen = vol_old;
    check(des_compute_volume(c));
    down(DES_F_VOLUME);
}

void compute_dvoldt(const Variables &, double_vec &)
{
    up(DES_F_STRAIN_RATE | DES_F_VOLUME | DES_F_VOLUME_N);
    check(des_compute_dvoldt(ctx()));
    down(DES_F_NTMP);
}

void compute_edvoldt(const Variables &, double_vec &, double_vec &)
{
    up(DES_F_NTMP);
    check(des_compute_edvoldt(ctx()));
    down(DES_F_EDVOLDT);
}

void NMD_stress(const Variables &, double_vec &, tensor_t &)
{
    up(DES_F_DPRESSURE | DES_F_VOLUME | DES_F_VOLUME_N | DES_F_STRESS);
    check(des_NMD_stress(ctx()));
    down(DES_F_NTMP | DES_F_STRESS);
}

double compute_dt(const Param &, const Variables &var)
{
    up(DES_F_COORD | DES_F_VOLUME | DES_F_TEMPERATURE);
    if (g.param->mat.nmat > 1 && var.elemmarkers) {   // markers may have moved (phase changes)
        const int nm = g.param->mat.nmat;
        for (int e = 0; e < var.nelem; ++e)
            for (int i = 0; i < nm; ++i) g.emark[(size_t)e * nm + i] = (*var.elemmarkers)[e][i];
        check(des_set_elemmarkers(ctx(), g.emark.data()));
    }
    double dt = 0;
    int rc = des_compute_dt(ctx(), &dt);
    if (rc == DES_ERUNTIME) {
        std::cerr << "Error: dt <= 0!\n";   // geometry.cxx:304-308
        std::exit(11);
    }
    check(rc);
    return dt;
}

void compute_mass(const Param &, const int_vec &, const conn_t &, const double_vec &, const MatProps &,
                  double, double_vec &, double_vec &, double_vec &)
{
    up(DES_F_VOLUME | DES_F_TEMPERATURE);
    check(des_compute_mass(ctx()));
    down(DES_F_VOLUME_N | DES_F_MASS | DES_F_TMASS);
}

void compute_shape_fn(const array_t &, const conn_t &, const double_vec &, const int_vec &, shapefn &,
                      shapefn &, shapefn &)
{
    up(DES_F_COORD | DES_F_VOLUME);
    check(des_compute_shape_fn(ctx()));
    down(F_SHP);
}

double elem_quality(const array_t &coord, const conn_t &connectivity, const double_vec &volume, int e)
{
    // geometry.cxx:458-496, one element on the host (bad_mesh_quality's callers)
    double vol = volume[e];
    const double *a = coord[connectivity[e][0]];
    const double *b = coord[connectivity[e][1]];
    const double *c = coord[connectivity[e][2]];
    auto area = [](const double *p, const double *q, const double *r) {
        double ab[3] = {0, 0, 0}, ac[3] = {0, 0, 0};
        for (int i = 0; i < NDIMS; ++i) {
            ab[i] = q[i] - p[i];
            ac[i] = r[i] - p[i];
        }
        if (NDIMS == 2) return std::fabs(ab[0] * ac[1] - ab[1] * ac[0]) / 2;
        double d0 = ab[1] * ac[2] - ab[2] * ac[1];
        double d1 = ab[2] * ac[0] - ab[0] * ac[2];
        double d2 = ab[0] * ac[1] - ab[1] * ac[0];
        return std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) / 2;
    };
    if (NDIMS == 3) {
        const double *d = coord[connectivity[e][NODES_PER_ELEM - 1]];
        double normalization_factor = 216 * std::sqrt(3);
        double area_sum = area(a, b, c) + area(a, b, d) + area(c, d, a) + area(c, d, b);
        return normalization_factor * vol * vol / (area_sum * area_sum * area_sum);
    }
    double normalization_factor = 4 * std::sqrt(3);
    double dist2_sum = dist2(a, b) + dist2(b, c) + dist2(a, c);
    return normalization_factor * vol / dist2_sum;
}

double worst_elem_quality(const array_t &, const conn_t &, const double_vec &, int &worst_elem)
{
    up(DES_F_COORD | DES_F_VOLUME);
    double q = 1;
    check(des_worst_elem_quality(ctx(), &q, &worst_elem));
    return q;
}

// ---------------------------------------------------------------------
// rheology.hpp
// ---------------------------------------------------------------------
void update_stress(const Variables &, tensor_t &, double_vec &, double_vec &, tensor_t &, double_vec &,
                   double_vec &, tensor_t &)
{
    up(DES_F_STRESS | DES_F_STRAIN | DES_F_STRAIN_RATE | DES_F_PLSTRAIN | DES_F_DELTA_PLSTRAIN |
       DES_F_STRESSYY | DES_F_EDVOLDT | DES_F_VOLUME | DES_F_VOLUME_OLD | DES_F_TEMPERATURE);
    check(des_update_stress(ctx()));
    down(DES_F_STRESS | DES_F_STRAIN | DES_F_STRAIN_RATE | DES_F_PLSTRAIN | DES_F_DELTA_PLSTRAIN |
         DES_F_STRESSYY | DES_F_DPRESSURE);
}

// ---------------------------------------------------------------------
// remeshing.hpp: the quality check (remeshing.cxx:1882-1935) on the device.
// remeshing.o defines this function too; the build weakens remeshing.o's
// copy (objcopy --weaken-symbol) so that this one is linked.
// ---------------------------------------------------------------------
int bad_mesh_quality(const Param &param, const Variables &, int &index)
{
    up(DES_F_COORD | DES_F_VOLUME);
    des_quality_params qp;
    qp.smallest_size = param.mesh.smallest_size;
    qp.resolution = param.mesh.resolution;
    qp.min_quality = param.mesh.min_quality;
    qp.max_boundary_distortion = param.mesh.max_boundary_distortion;
    qp.remeshing_option = param.mesh.remeshing_option;
    int code = 0, idx = index;
    double value = 0;
    check(des_bad_mesh_quality(ctx(), &qp, &code, &idx, &value));
    if (code == 3) std::cout << "    The size of element #" << idx << " is too small.\n";
    else if (code == 2) std::cout << "    Node #" << idx << " is too far from the bottm: z = " << value << "\n";
    else if (code == 1) std::cout << "    Element #" << idx << " has mesh quality = " << value << ".\n";
    if (code) index = idx;
    return code;
}
