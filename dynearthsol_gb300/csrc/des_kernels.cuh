// des_kernels.cuh -- host-side launchers of the explicit-step kernels.
#pragma once

#include <cuda_runtime.h>

#include "des_common.cuh"

namespace des {

// flags of the element geometry pass
enum GeoFlags : int {
    GEO_COPY_OLD = 1,    // volume_old <- volume        (dynearthsol.cxx:226)
    GEO_VOLUME = 2,      // compute_volume              (geometry.cxx:86-108)
    GEO_SHAPE = 4,       // compute_shape_fn            (geometry.cxx:368-455)
    GEO_ROTATE = 8,      // rotate_stress               (fields.cxx:411-483)
    GEO_DT = 16,         // compute_dt element terms    (geometry.cxx:254-292)
    GEO_DT_IF_STEP = 32, // ... only when steps % 10 == 0 (dynearthsol.cxx:349-361)
    GEO_MASS_TERMS = 64  // the element's mass and tmass terms -> me, tme (for launch_mass_sum)
};

// Each launcher returns the number of kernels it launched.
int launch_strain_rate(const KP &p, cudaStream_t s, bool begin_step);
int launch_heat_gather(const KP &p, cudaStream_t s);              // tdot -> p.tdot
int launch_temperature_update(const KP &p, cudaStream_t s);       // T from p.tdot
int launch_dvoldt(const KP &p, cudaStream_t s);                   // -> ntmp
int launch_heat_and_dvoldt(const KP &p, cudaStream_t s);          // fused: tdot -> p.tdot, dvoldt -> ntmp
// the FP64 step's element-centric form of strain rate + heat gather + dvoldt
// (+ clock advance) and of the node sums + temperature update: the same bits
// (needs p.qv and, with heat, p.hc64)
int launch_elem_pass(const KP &p, cudaStream_t s, bool heat);
int launch_node_pass(const KP &p, cudaStream_t s, bool heat);
int launch_edvoldt(const KP &p, cudaStream_t s);
int launch_update_stress(const KP &p, cudaStream_t s, bool fused);
// dp_nd -> ntmp; stored: the dp vol products of the fused mixed stress pass (KP::pv)
int launch_nmd_gather(const KP &p, cudaStream_t s, bool stored = false);
// in a mixed 3D context (uses_force_terms) it also forms the element force
// terms p.ft from the corrected stress, which launch_force's gather sums
int launch_nmd_correct(const KP &p, cudaStream_t s, bool with_facets);
// the force terms alone, from the current stress (mixed 3D contexts; else 0 launches)
int launch_force_terms(const KP &p, cudaStream_t s);
// a mixed 3D context's force: element terms in double-word arithmetic
inline bool uses_force_terms(const KP &p) { return p.ft != nullptr && p.nd == 3 && !p.mat.is_plane_strain; }
int launch_facet_forces(const KP &p, cudaStream_t s);
// contract: the mixed step's form: with uses_force_terms, the double-word
// gather of the force terms (k_force_dw3), else k_force's fused multiply-adds
int launch_force(const KP &p, cudaStream_t s, bool fused_motion, bool contract = false);
int launch_velocity(const KP &p, cudaStream_t s, bool contract = false);
int launch_vbcs(const KP &p, cudaStream_t s);
int launch_coordinate(const KP &p, cudaStream_t s, bool contract = false);
int launch_geometry(const KP &p, cudaStream_t s, int flags);
// the chained mixed step's geometry pass (3D mixed contexts), which also
// does the next step's element pass (k_elem_pass_mixed3's work)
int launch_geometry_ahead(const KP &p, cudaStream_t s, int flags);
int launch_mass(const KP &p, cudaStream_t s);
// compute_mass from the element terms of a GEO_MASS_TERMS geometry pass (same sums, same order)
int launch_mass_sum(const KP &p, cudaStream_t s);
int launch_dt_finalize(const KP &p, cudaStream_t s, bool only_on_step);
int launch_quality(const KP &p, cudaStream_t s, unsigned long long *red);
// red[2], red[3]: bad_mesh_quality's first tiny element and first drifted bottom node
int launch_quality_scans(const KP &p, cudaStream_t s, double smallest_vol, double bottom, double dist,
                         int check_bottom, unsigned long long *red);
// out[4][ne]: density, mesh quality, viscosity, material of an output frame
int launch_output_elem(const KP &p, double *out, cudaStream_t s);
int launch_dt_reset(const KP &p, cudaStream_t s);
// material constants: visc_coef[nmat], then 4 values per plastic table entry
int launch_material_table(const KP &p, cudaStream_t s, double *out);
// the per-element blended material properties (KP::eprop) from the marker
// counts; run whenever the counts change
int launch_elem_props(const KP &p, cudaStream_t s, double *out);

// FP32 copy of an FP64 array
int launch_f64_to_f32(const double *a, float *b, long long n, cudaStream_t s);
// a mixed 3D context's shape functions (p.shpdw non-null; else no launch):
// the double-word pairs -> FP64 p.shp, for a download
int launch_shp_join(const KP &p, cudaStream_t s);

// layout conversion between the reference's AoS rows and device SoA
int launch_aos_to_soa(const double *aos, double *soa, int n, int ncomp, cudaStream_t s);
int launch_soa_to_aos(const double *soa, double *aos, int n, int ncomp, cudaStream_t s);

// The same conversion for the rows [lo, hi) of several fields in one launch
// (one slab of the pipelined host step).
constexpr int ROWS_MAX = 12;
struct RowField {
    double *stage;   // AoS rows [n][nc]; rows lo..hi-1 are read (up) or written
    double *dev;     // SoA [nc][n]
    long long first; // index of the field's first value in the launch
    int n, nc, lo, hi;
    const float2 *dw; // download: read the double-word pairs here instead of dev, or null
};
struct RowTable {
    RowField f[ROWS_MAX];
    long long total;
    int count;
};
int launch_rows(const RowTable &t, bool up, cudaStream_t s);

}  // namespace des
