/*
 * des_oracle.h -- CPU restatement (oracle) of the reference's explicit
 * time-step hot path.  TEST INFRASTRUCTURE ONLY: the parity tests, the
 * smoke check and the CPU-baseline leg of bench.py call it as the checker;
 * the product library never links or calls it.
 *
 * The oracle works on the reference's host layout (des_host_state, AoS rows)
 * and follows the reference's serial summation order when run with one
 * thread.  With nthreads > 1 it uses the reference's OpenMP strategy
 * (element-parallel loops and the two-colour element-band scatter of
 * utils.hpp:18-44 / mesh.cxx:1724-1817), which is what the CPU baseline
 * times.
 */
#ifndef DES_ORACLE_H
#define DES_ORACLE_H

#include "../include/desgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

/* The mesh, params and material structs (and the arrays they point to)
 * must outlive the context; state is bound with oracle_bind_state. */
oracle_ctx *oracle_create(const des_mesh *mesh, const des_params *param,
                          const des_material *mat, int nthreads);
void oracle_destroy(oracle_ctx *c);
int oracle_bind_state(oracle_ctx *c, des_host_state *st);
int oracle_set_elem_field(oracle_ctx *c, int field, const double *values);
int oracle_threads(const oracle_ctx *c);

/* per-function restatements (same names as the reference functions) */
void oracle_update_temperature(oracle_ctx *c);
void oracle_update_strain_rate(oracle_ctx *c);
void oracle_compute_dvoldt(oracle_ctx *c);
void oracle_compute_edvoldt(oracle_ctx *c);
int  oracle_update_stress(oracle_ctx *c);
void oracle_NMD_stress(oracle_ctx *c);
void oracle_update_force(oracle_ctx *c);
void oracle_update_velocity(oracle_ctx *c);
void oracle_apply_vbcs(oracle_ctx *c);
void oracle_update_coordinate(oracle_ctx *c);
void oracle_swap_volume(oracle_ctx *c);
void oracle_compute_volume(oracle_ctx *c);
void oracle_compute_mass(oracle_ctx *c);
void oracle_compute_shape_fn(oracle_ctx *c);
void oracle_rotate_stress(oracle_ctx *c);
int  oracle_compute_dt(oracle_ctx *c, double *dt);
double oracle_worst_elem_quality(oracle_ctx *c, int *worst);

/* init sequence of dynearthsol.cxx:86-94 on the bound state (masses with a
 * zero temperature field, as init() computes them before the geotherm):
 * coord0 = coord, volume, volume_old = volume, mass, shape functions,
 * apply_vbcs; then dt = compute_dt (dynearthsol.cxx:316). */
int oracle_init_fields(oracle_ctx *c);

/* nsteps of the loop body dynearthsol.cxx:325-361 (no phase changes,
 * output or remeshing).  Returns 0, or 11 when compute_dt fails. */
int oracle_run(oracle_ctx *c, int nsteps);

/* restatement of create_boundary_normals (bc.cxx:87-176); fills
 * bnormals[10][3] and edge_vectors[10][10][3].  Returns 0, or 1 when a
 * slant boundary is not planar (the reference exits with code 1). */
int oracle_boundary_normals(const des_mesh *mesh, const double *coord,
                            double bnormals[DES_NBDRYTYPES][3],
                            double edge_vectors[DES_NBDRYTYPES][DES_NBDRYTYPES][3]);

/* 3x3 symmetric eigen-solver restatement, exposed for unit tests:
 * a = {xx, yy, zz, xy, xz, yz}; returns 0 or -1 (QL non-convergence). */
int oracle_eigen3(const double a[6], double w[3], double q[9], int *used_ql);

/* principal_stresses3 (rheology.cxx:13-68): sorted p, eigenvectors v (row-major v[i][k]) */
void oracle_principal_stresses3(const double s[6], double p[3], double v[9]);

#ifdef __cplusplus
}
#endif

#endif
