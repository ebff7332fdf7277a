/*
 * desgpu.h -- C ABI of the GB300-native explicit time-step library for
 * DynEarthSol3D-style Lagrangian finite elements (linear triangles in 2D,
 * linear tetrahedra in 3D).
 *
 * Every entry point returns an int status: DES_OK (0) on success, otherwise
 * one of the DES_E* codes below.  DES_ERUNTIME (11) and DES_EASSERT (12)
 * mirror the reference's std::exit codes ("11 runtime error", "12 assertion
 * error", DEVELOPING:32-37), so a host shim can exit with the same code.
 * The message of the last failure of a context is available through
 * des_last_error().
 *
 * Data layout at the boundary follows the reference's host arrays
 * (Array2D<T,N> rows, array2d.hpp:86-87: element i of a row-major [n][N]
 * array starts at a + N*i).  Inside the library every field is kept on the
 * device as structure-of-arrays.
 *
 * Threading: a context is used by one host thread at a time; all device work
 * of a context runs in order on one CUDA stream, which the caller may supply.
 */
#ifndef DESGPU_H
#define DESGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define DES_OK          0
#define DES_EINPUT      1    /* invalid argument (reference code 1: user input error) */
#define DES_ECUDA       3    /* a CUDA runtime call failed */
#define DES_ENOMEM      4    /* device allocation failed */
#define DES_ERUNTIME   11    /* numerical failure, e.g. dt <= 0 (geometry.cxx:304-308) */
#define DES_EASSERT    12    /* internal consistency check failed */

/* ---- sticky device error bits (des_device_status) --------------------- */
#define DES_DEV_NONFINITE    1u  /* NaN/Inf met in a node coordinate or velocity */
#define DES_DEV_NEG_VOLUME   2u  /* an element volume became <= 0 */
#define DES_DEV_QL_NOCONV    4u  /* 3x3 QL eigen iteration hit its 30-sweep cap */
#define DES_DEV_BAD_INDEX    8u  /* a connectivity or support index out of range */

/* ---- constants shared with the reference ------------------------------ */
#define DES_NBDRYTYPES 10           /* nbdrytypes, constants.hpp:38 */

/* rheology bit set, MatProps::rh_* (matprops.hpp:47-53) */
#define DES_RH_ELASTIC  1
#define DES_RH_VISCOUS  2
#define DES_RH_PLASTIC  4
#define DES_RH_MAXWELL  (DES_RH_ELASTIC | DES_RH_VISCOUS)
#define DES_RH_EP       (DES_RH_ELASTIC | DES_RH_PLASTIC)
#define DES_RH_EVP      (DES_RH_ELASTIC | DES_RH_VISCOUS | DES_RH_PLASTIC)

/* precision of a context */
#define DES_PREC_FP64   0   /* every operation in FP64 */
#define DES_PREC_MIXED  1   /* FP32 element kinematics/rheology increments, FP64 state and accumulation */

/* ---- mesh ------------------------------------------------------------- */
/* Topology of one mesh.  Mirrors Variables::{connectivity, bcflag, bfacets,
 * bnormals, edge_vectors} (parameters.hpp:229-279).  The node-to-element
 * support lists (Variables::support, mesh.cxx:1707-1721) are derived inside
 * the library from the connectivity, in ascending element order. */
typedef struct des_mesh {
    int ndims;                    /* 2 or 3 */
    int nnode;
    int nelem;
    const int *connectivity;      /* [nelem][ndims+1] node ids */
    const unsigned *bcflag;       /* [nnode] BOUNDX0.. bit flags (constants.hpp:29-38) */
    /* boundary facets: boundary i owns pairs [bfacet_offsets[i], bfacet_offsets[i+1]) */
    const int *bfacet_offsets;    /* [DES_NBDRYTYPES+1] */
    const int *bfacets;           /* [nbfacet][2] = (element, local facet 0..ndims) */
    double bnormals[DES_NBDRYTYPES][3];                 /* unit outward normals */
    double edge_vectors[DES_NBDRYTYPES][DES_NBDRYTYPES][3]; /* [i][j], i<j: boundary intersection edge */
} des_mesh;

/* ---- run-time parameters (the subset of Param the step reads) --------- */
typedef struct des_params {
    /* Control (parameters.hpp:81-101) */
    double gravity;
    double inertial_scaling;
    double dt_fraction;
    double fixed_dt;
    double damping_factor;
    double surface_diffusivity;
    double max_vbc_val;           /* Variables::max_vbc_val (dynearthsol.cxx:36-39) */
    int damping_option;
    int ref_pressure_option;
    int surface_process_option;   /* 0 only; other options stay on the host */
    int is_quasi_static;
    int has_thermal_diffusion;
    /* BC (parameters.hpp:103-135) */
    double surface_temperature;
    double mantle_temperature;
    double winkler_delta_rho;
    double elastic_foundation_constant;
    int has_fixed_bottom_temperature;
    int has_winkler_foundation;
    int has_elastic_foundation;
    int has_water_loading;
    int vbc_types[DES_NBDRYTYPES];     /* Variables::vbc_types, dynearthsol.cxx:43-52 */
    double vbc_values[DES_NBDRYTYPES]; /* Variables::vbc_values, dynearthsol.cxx:54-63 */
    /* Mesh */
    double zlength;
    /* compensation pressure of the Winkler foundation (Variables::compensation_pressure) */
    double compensation_pressure;
} des_params;

/* ---- material table (Mat, parameters.hpp:166-194; MatProps) ---------- */
/* Each array holds nmat entries.  scalar_mask bit k set means parameter k
 * was given as a single value (VectorBase::create's Vector1, matprops.cxx:
 * 176-187), for which the harmonic/arithmetic means return entry 0 unchanged
 * (matprops.cxx:105,119).  Bits: 0 bulk_modulus, 1 shear_modulus,
 * 2 heat_capacity, 3 radiogenic_heating, 4 therm_cond. */
typedef struct des_material {
    int rheol_type;          /* DES_RH_* */
    int nmat;
    int is_plane_strain;
    unsigned scalar_mask;
    double visc_min, visc_max, tension_max, therm_diff_max;
    const double *rho0, *alpha;
    const double *bulk_modulus, *shear_modulus;
    const double *visc_exponent, *visc_coefficient, *visc_activation_energy;
    const double *heat_capacity, *therm_cond, *radiogenic_heating;
    const double *pls0, *pls1;
    const double *cohesion0, *cohesion1;
    const double *friction_angle0, *friction_angle1;
    const double *dilation_angle0, *dilation_angle1;
    const int *elemmarkers;  /* [nelem][nmat] marker counts, or NULL: one marker of material 0 */
} des_material;

/* ---- host state in the reference's layout (Variables fields) ---------- */
/* Any pointer may be NULL in des_download_state (that field is skipped).
 * In des_upload_state the fields marked (in) are required. */
typedef struct des_host_state {
    double *coord;          /* (in) [nnode][ndims] */
    double *coord0;         /* [nnode][ndims]; NULL on upload = copy of coord */
    double *vel;            /* (in) [nnode][ndims] */
    double *force;          /* [nnode][ndims] */
    double *temperature;    /* (in) [nnode] */
    double *mass, *tmass, *volume_n, *ntmp;   /* [nnode] */
    double *volume;         /* [nelem]; recomputed from coord on upload when NULL */
    double *volume_old;     /* (in) [nelem] */
    double *stress;         /* (in) [nelem][nstr] */
    double *strain;         /* (in) [nelem][nstr] */
    double *strain_rate;    /* [nelem][nstr] */
    double *plstrain;       /* (in) [nelem] */
    double *delta_plstrain; /* [nelem] */
    double *stressyy;       /* [nelem] (plane strain) */
    double *dpressure;      /* [nelem] */
    double *edvoldt;        /* [nelem] */
    double *shpdx, *shpdy, *shpdz;  /* [nelem][ndims+1]; shpdy unused in 2D */
    double time;
    double dt;
    int steps;
} des_host_state;

typedef struct des_ctx des_ctx;

/* Library version string. */
const char *des_version(void);

/* Create a context on the current CUDA device.  stream may be NULL (the
 * library creates its own non-blocking stream).  precision is DES_PREC_*.
 * Replaces the device half of allocate_variables (fields.cxx:10-48). */
int des_create(const des_mesh *mesh, const des_params *param,
               const des_material *mat, int precision, void *stream,
               des_ctx **out);
int des_destroy(des_ctx *ctx);

/* Message of the last failure of ctx (or of the last failed des_create when
 * ctx is NULL), copied into buf (always NUL-terminated). */
int des_last_error(const des_ctx *ctx, char *buf, size_t len);

/* Sticky device error bits (DES_DEV_*), read and cleared. */
int des_device_status(des_ctx *ctx, unsigned *bits);

/* Host <-> device state transfer (reference AoS layout <-> device SoA).
 * des_upload_state replaces the host->device re-upload after init, restart
 * and remesh (dynearthsol.cxx:80-99,179-215; remeshing.cxx:2009-2015);
 * des_download_state is called before host readers (output.cxx:79-208).
 * A DES_PREC_MIXED 3D context keeps its shape functions as double-word FP32
 * pairs, formed from its coordinates and volumes: uploaded shape functions
 * (here or by des_upload_fields) are not used, and downloads round the pairs
 * to FP64. */
int des_upload_state(des_ctx *ctx, const des_host_state *st);
int des_download_state(des_ctx *ctx, des_host_state *st);

/* Field-wise transfer: one bit per des_host_state array (DES_F_*), plus
 * DES_F_CLOCK for time/dt/steps.  Only the selected fields move; a selected
 * field whose pointer is NULL is an input error.  Used by a host shim that
 * keeps the reference's Variables authoritative around each call. */
#define DES_F_COORD          (1u << 0)
#define DES_F_COORD0         (1u << 1)
#define DES_F_VEL            (1u << 2)
#define DES_F_FORCE          (1u << 3)
#define DES_F_TEMPERATURE    (1u << 4)
#define DES_F_MASS           (1u << 5)
#define DES_F_TMASS          (1u << 6)
#define DES_F_VOLUME_N       (1u << 7)
#define DES_F_NTMP           (1u << 8)
#define DES_F_VOLUME         (1u << 9)
#define DES_F_VOLUME_OLD     (1u << 10)
#define DES_F_STRESS         (1u << 11)
#define DES_F_STRAIN         (1u << 12)
#define DES_F_STRAIN_RATE    (1u << 13)
#define DES_F_PLSTRAIN       (1u << 14)
#define DES_F_DELTA_PLSTRAIN (1u << 15)
#define DES_F_STRESSYY       (1u << 16)
#define DES_F_DPRESSURE      (1u << 17)
#define DES_F_EDVOLDT        (1u << 18)
#define DES_F_SHP            (1u << 19)   /* shpdx, shpdy (3D), shpdz */
#define DES_F_CLOCK          (1u << 20)
#define DES_F_ALL            ((1u << 21) - 1)
int des_upload_fields(des_ctx *ctx, const des_host_state *st, unsigned mask);
int des_download_fields(des_ctx *ctx, des_host_state *st, unsigned mask);

/* Replace the per-element marker counts of a multi-material context
 * ([nelem][nmat], Variables::elemmarkers), e.g. after phase changes
 * (phasechanges.cxx:232-258) or marker remapping. */
int des_set_elemmarkers(des_ctx *ctx, const int *elemmarkers);

/* ---- markers and phase changes -----------------------------------------
 * The markers of a multi-material context on the device (MarkerSet,
 * markerset.hpp:11-84): for each marker its element, its barycentric
 * coordinates eta[ndims+1] ([nmarkers][ndims+1], the reference's layout) and
 * its material type.  Copied once after the host creates or remaps them
 * (markerset.cxx:35-64; remap_markers after remeshing); replaces the
 * previous set.  The context's per-element marker counts are not changed:
 * they are set at des_create or by des_set_elemmarkers. */
int des_set_markers(des_ctx *ctx, int nmarkers, const int *elem, const double *eta, const int *mattype);

/* phase_changes (phasechanges.cxx:232-258) on the device, on the markers of
 * des_set_markers: each marker's depth and temperature are interpolated from
 * the device's coordinates and temperatures (PhaseChange::get_ZPT,
 * phasechanges.cxx:24-39), its reference pressure follows, and the rule of
 * phase_change_option decides its new material type: 1 = SimpleSubduction
 * (phasechanges.cxx:44-160), 101 = the custom template (no change), 0 or a
 * one-material context = nothing (phase_changes_init, phasechanges.cxx:
 * 208-229).  A marker that changes moves from one material's count to the
 * other's in the element's marker counts, so the next step blends the
 * element's properties from the new counts.  hydrous_elemmarkers ([nelem],
 * Variables::hydrous_elemmarkers; NULL = none) is read by the mantle ->
 * serpentinite rule; hydration processes (the markers that dehydration
 * releases) stay on the host.  *nchanged (may be NULL) = markers changed. */
int des_phase_changes(des_ctx *ctx, int option, const int *hydrous_elemmarkers, int *nchanged);

/* Download the device's marker material types ([nmarkers], may be NULL) and
 * per-element marker counts ([nelem][nmat], may be NULL), for host-side
 * marker bookkeeping before output, checkpoints or remeshing. */
int des_get_markers(des_ctx *ctx, int *mattype, int *elemmarkers);

/* Replace the parameters (e.g. after a change of max_vbc_val). */
int des_set_params(des_ctx *ctx, const des_params *param);

/* Per-element parameter overrides (extension used by the perturbed-cohesion
 * and inverse-problem workloads; no counterpart in the reference, whose
 * properties are per material).  field is DES_EF_*; values [nelem] on the
 * host; NULL removes the override. */
#define DES_EF_COHESION0      0   /* Pa, replaces the blended cohesion0 */
#define DES_EF_COHESION1      1   /* Pa, replaces the blended cohesion1 */
#define DES_EF_LOG10_VISC     2   /* log10(Pa s), replaces MatProps::visc before clamping */
#define DES_EF_SHEAR_MODULUS  3   /* Pa, replaces MatProps::shearm */
#define DES_EF_FRICTION0      4   /* degree, replaces friction_angle0 */
#define DES_EF_FRICTION1      5   /* degree, replaces friction_angle1 */
#define DES_EF_THERM_COND     6   /* W/m/K, replaces MatProps::k */
#define DES_EF_COUNT          7
int des_set_elem_field(des_ctx *ctx, int field, const double *values);

/* ---- per-function entry points (device-resident state) --------------- */
/* Each one replaces the reference function cited beside it, reading and
 * writing the context's device copy of the corresponding Variables fields. */
int des_update_temperature(des_ctx *ctx);  /* fields.cxx:96-163 (tdot -> ntmp) */
int des_update_strain_rate(des_ctx *ctx);  /* fields.cxx:166-232 */
int des_compute_dvoldt(des_ctx *ctx);      /* geometry.cxx:111-155 (-> ntmp) */
int des_compute_edvoldt(des_ctx *ctx);     /* geometry.cxx:158-179 (ntmp -> edvoldt) */
int des_update_stress(des_ctx *ctx);       /* rheology.cxx:510-646 */
int des_NMD_stress(des_ctx *ctx);          /* geometry.cxx:182-236 (-> ntmp, stress) */
int des_update_force(des_ctx *ctx);        /* fields.cxx:291-340 + bc.cxx:493-566 */
int des_update_velocity(des_ctx *ctx);     /* fields.cxx:343-355 */
int des_apply_vbcs(des_ctx *ctx);          /* bc.cxx:179-490 */
int des_update_coordinate(des_ctx *ctx);   /* fields.cxx:358-368 */
int des_swap_volume(des_ctx *ctx);         /* dynearthsol.cxx:226 volume <-> volume_old */
int des_compute_volume(des_ctx *ctx);      /* geometry.cxx:86-108 */
int des_compute_mass(des_ctx *ctx);        /* geometry.cxx:313-365 */
int des_compute_shape_fn(des_ctx *ctx);    /* geometry.cxx:368-455 */
int des_rotate_stress(des_ctx *ctx);       /* fields.cxx:411-483 */
int des_compute_dt(des_ctx *ctx, double *dt_out); /* geometry.cxx:239-310; also sets the context dt */
int des_update_mesh(des_ctx *ctx);         /* dynearthsol.cxx:221-232 (surface_process_option 0) */

/* Worst element quality and its index (geometry.cxx:458-512, used by
 * bad_mesh_quality, remeshing.cxx:1882-1935). */
int des_worst_elem_quality(des_ctx *ctx, double *quality, int *elem);

/* The mesh-quality check that triggers remeshing, bad_mesh_quality
 * (remeshing.cxx:1882-1935), on the device-resident mesh: no coordinate or
 * volume download.  It returns, in *code, the reference's value:
 *   3  an element is smaller than smallest_size x the volume of the
 *      equilateral tetrahedron (triangle) of side resolution; *index = the
 *      first such element, *value = its volume;
 *   2  (remeshing_option 1, 2 or 11) a bottom node (BOUNDZ0) lies farther
 *      than max_boundary_distortion x resolution from z = -zlength;
 *      *index = the first such node, *value = its z;
 *   1  the worst element quality (elem_quality, geometry.cxx:458-496; its
 *      cube root in 3D) is below min_quality; *index = the first worst
 *      element, *value = that quality;
 *   0  none of these; *index and *value are left unchanged.
 * The checks run in that order, as the reference's do.  zlength is the
 * context's des_params.zlength. */
typedef struct des_quality_params {
    double smallest_size;            /* Param::mesh.smallest_size */
    double resolution;               /* Param::mesh.resolution */
    double min_quality;              /* Param::mesh.min_quality */
    double max_boundary_distortion;  /* Param::mesh.max_boundary_distortion */
    int remeshing_option;            /* Param::mesh.remeshing_option */
} des_quality_params;
int des_bad_mesh_quality(des_ctx *ctx, const des_quality_params *qp, int *code, int *index, double *value);

/* ---- the remesh hand-off ---------------------------------------------
 * A mesh as remeshing leaves it (remeshing.cxx:1937-2035): connectivity,
 * boundary flags and the boundary segments with their flags
 * (Variables::segment, segflag), in the mesher's order. */
typedef struct des_topology {
    int ndims, nnode, nelem;
    const int *connectivity;   /* [nelem][ndims+1] */
    const unsigned *bcflag;    /* [nnode] */
    int nseg;
    const int *segment;        /* [nseg][ndims] node ids of each boundary segment */
    const int *segflag;        /* [nseg] its boundary flag (0: not on a boundary) */
} des_topology;

/* create_support (mesh.cxx:1707-1721) and create_boundary_facets
 * (mesh.cxx:1637-1704) built on the device (the reference's facet search is
 * O(nseg x nelem); here one thread per segment searches the support list of
 * one of its nodes), with the reference's results bit for bit: sup_off
 * [nnode+1] and sup_elem [nelem*(ndims+1)], each node's elements in
 * ascending order; bfacet_offsets [DES_NBDRYTYPES+1] and bfacets
 * [nfacets][2] = (element, local facet), each boundary's facets in segment
 * order.  Any output may be NULL.  Needs no context; work is queued on
 * stream (NULL: the legacy default stream) and allocates temporary device
 * memory.  A segment that matches no element facet is DES_EASSERT, as the
 * reference exits with code 12. */
int des_build_topology(const des_topology *topo, int *sup_off, int *sup_elem, int *bfacet_offsets,
                       int *bfacets, void *stream);

/* The device half of reallocate_variables (fields.cxx:51-93) and the
 * topology rebuild after remeshing: the context's mesh becomes topo, its
 * support lists and boundary facets built on the device, its device arrays
 * sized for the new mesh.  Parameters, material table, boundary normals,
 * precision and stream are kept; per-element overrides (des_set_elem_field)
 * and device markers are dropped.  elemmarkers [nelem][nmat] are the new
 * mesh's marker counts (required with nmat > 1).  The state is then
 * uploaded with des_upload_state (the interpolated fields). */
int des_remesh(des_ctx *ctx, const des_topology *topo, const int *elemmarkers);

/* Read or set the context's dt / time / steps (Variables::dt, time, steps). */
int des_get_clock(des_ctx *ctx, double *time, double *dt, int *steps);
int des_set_clock(des_ctx *ctx, double time, double dt, int steps);

/* ---- whole steps ------------------------------------------------------ */
/* Run nsteps explicit steps: the body of the reference's time loop
 * (dynearthsol.cxx:325-361) without phase changes, output and remeshing,
 * with compute_dt every 10th step on the device.  Uses the fused kernel
 * schedule; results equal the per-function sequence.  In a DES_PREC_MIXED
 * context, nsteps >= 2 chains the steps (each geometry pass but the last
 * also does the next step's element pass); the results are those of
 * nsteps calls of one step, bit for bit. */
int des_step(des_ctx *ctx, int nsteps);

/* Same as des_step, but with the state in HOST memory in the reference's
 * layout: uploads st, runs nsteps, downloads into st (all inside the call).
 * This is the drop-in form for a caller whose Variables stay authoritative.
 * With nsteps >= 1, the fields that the first step writes before reading
 * them (strain_rate, force, dpressure, edvoldt, ntmp) are not uploaded, and
 * the fields that no step writes (coord0; stressyy outside plane strain) are
 * not downloaded: st ends as after upload + step + download, bit for bit,
 * with ~80 MB less host-link traffic at 1M tets.  Page-locked host arrays
 * let the copies run asynchronously at the link's rate.  With nsteps == 1,
 * a complete page-locked state and a mesh numbered slab by slab (as the
 * structured box meshes are), the upload, the step and the download overlap
 * slab by slab (one CUDA graph, built on the first such call for these host
 * arrays and reused while they stay the same).  That call also forms volume,
 * the shape functions, volume_n and, quasi-static, mass from the uploaded
 * coordinates with the kernels of the step's own update_mesh, instead of
 * uploading them (as the reference's loop keeps them: functions of the
 * coordinates); it still downloads them.  tmass is uploaded. */
int des_step_host(des_ctx *ctx, des_host_state *st, int nsteps);

/* ---- output frames in the reference's .save format ---------------------
 * Output::write (output.cxx:79-195, not averaged, no marker output) with
 * BinaryOutput's layout (binaryio.cxx:16-37): a 4096-byte ASCII header --
 * "# DynEarthSol ndims=N revision=3\n" then one "name\tbyte offset\n" line
 * per array -- followed by the arrays in the reference's row-major layout.
 * Arrays, in order: coordinate, connectivity (int32), velocity,
 * temperature, plastic strain, plastic strain-rate (delta_plstrain),
 * strain-rate, strain, stress, density, mesh quality, viscosity, material
 * (as doubles), force, coord0, bcflag (uint32). */
typedef struct des_save_frame {
    int ndims, nnode, nelem;
    const double *coord;            /* [nnode][ndims] */
    const int *connectivity;        /* [nelem][ndims+1] */
    const double *vel;              /* [nnode][ndims] */
    const double *temperature;      /* [nnode] */
    const double *plstrain;         /* [nelem] */
    const double *delta_plstrain;   /* [nelem] */
    const double *strain_rate;      /* [nelem][nstr] */
    const double *strain;           /* [nelem][nstr] */
    const double *stress;           /* [nelem][nstr] */
    const double *density;          /* [nelem] MatProps::rho */
    const double *mesh_quality;     /* [nelem] elem_quality */
    const double *viscosity;        /* [nelem] MatProps::visc */
    const double *material;         /* [nelem] index of the most abundant marker's material */
    const double *force;            /* [nnode][ndims] */
    const double *coord0;           /* [nnode][ndims] */
    const unsigned *bcflag;         /* [nnode] */
} des_save_frame;

/* Write one frame from host arrays (no device work). */
int des_write_save_host(const char *filename, const des_save_frame *frame);
/* Write the context's current state as one frame: density, mesh quality,
 * viscosity and material are evaluated on the device, and only the frame's
 * arrays come to the host.  Replaces Output::write (output.cxx:79-195) for
 * a device-resident run; the caller names the file ("%s.save.%06d"). */
int des_write_save(des_ctx *ctx, const char *filename);

/* ---- reverse mode: the adjoint of a window of steps --------------------
 * No counterpart in the reference.  Gradients of a scalar loss of the
 * state after a window of nsteps steps of the 3D FP64 step, taken with dt
 * held at the context's dt over the window (compute_dt is not called
 * inside it; des_step with fixed_dt = that dt takes the same steps).
 * Supported: 3D, DES_PREC_FP64, one material without element markers,
 * rheology elastic, Maxwell, elasto-plastic or elasto-visco-plastic.  Kinks
 * (yield, the EVP branch choice, viscosity clamps, damping signs, BC
 * overwrites) take the derivative of the branch the forward took.
 *
 * des_adjoint_forward runs the window from the current state, keeping the
 * state every checkpoint_every steps, and leaves the context at the
 * window's end.  It also records the tape of the window's last segment
 * (checkpoint_every + 1 step records of ~319 bytes per tet, the tape the
 * backward needs anyway).  des_adjoint_backward takes the adjoint of that
 * final state in seed (its fields coord, vel, temperature, stress,
 * plstrain and volume_old, in des_host_state's layout; NULL fields are
 * zero), recomputes
 * each other segment from its checkpoint onto the tape, and runs the
 * reverse steps.  With checkpoint_every >= nsteps the window is one
 * segment and the backward recomputes nothing.  Both return DES_ENOMEM
 * when the tape does not fit in device memory.  It writes the adjoint
 * of the window's start state to the same six fields of start_adjoint
 * (NULL fields, or start_adjoint NULL, are skipped) and the gradients to
 * grad, and leaves the context at the window's end.  It may be called
 * again with another seed until the next des_adjoint_forward. */
typedef struct des_adjoint_grad {
    /* [nelem] d loss / d (the element's value of DES_EF_k), or NULL.
     * DES_EF_LOG10_VISC only when that field is set (it replaces the
     * viscosity law); the others whether or not the field is set. */
    double *elem[DES_EF_COUNT];
    double vbc_values[DES_NBDRYTYPES];   /* d loss / d des_params.vbc_values[i] */
} des_adjoint_grad;

int des_adjoint_forward(des_ctx *ctx, int nsteps, int checkpoint_every);
int des_adjoint_backward(des_ctx *ctx, const des_host_state *seed, des_host_state *start_adjoint,
                         des_adjoint_grad *grad);

/* ---- nodal-mixed pressure smoothing without any device allocation ---- */
/* No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory -- a host application that owns every
 * device byte and hands out memory only from its own pools, a process under
 * a strict device-memory quota, or code running where cudaMalloc is not
 * permitted (for example while another component holds the allocator).
 * Such callers cannot use des_create, which allocates.
 *
 * It computes what des_NMD_stress computes (NMD_stress, geometry.cxx:
 * 182-236) on arrays the caller already owns, all DEVICE pointers in the
 * library's device layout: conn [ndims+1][nelem] (structure of arrays),
 * support lists sup_off [nnode+1] and sup_ent (entries e*4 + local node,
 * ascending element id per node), dpressure, volume [nelem], volume_n
 * [nnode], and stress [nstr][nelem], whose first ndims components are
 * updated in place.  Work is queued on stream (NULL: the legacy default
 * stream).
 *
 * The per-node pressure sum it needs lives in a fixed device array of
 * DES_NOALLOC_MAX_NODES doubles (16 MiB) that every GPU loading this library
 * holds until the process exits; larger meshes are rejected with DES_EINPUT
 * and a message on stderr.  The call makes no cudaMalloc, cudaFree or other
 * allocating call.  All calls share that array and it keeps the last call's
 * contents (each call overwrites every entry it reads, so nothing needs
 * clearing); calls that overlap on the GPU (different streams, or different
 * host threads) race on it and must be serialised by the caller.  Each call
 * made outside stream capture looks up the array's device address
 * (cudaGetSymbolAddress) on the current device, so a device reset between
 * calls is harmless; a call inside a capture reuses the address of the last
 * lookup on that device, so make the first call on each device before any
 * stream capture, and none inside a capture after a device reset.  A CUDA
 * error already pending on the calling thread is reported as DES_ECUDA
 * without being cleared, and nothing is launched. */
#define DES_NOALLOC_MAX_NODES 2097152
int des_nmd_stress_noalloc(int ndims, int nnode, int nelem, const int *conn, const int *sup_off,
                           const int *sup_ent, const double *dpressure, const double *volume,
                           const double *volume_n, double *stress, void *stream);

/* Synchronise the context's stream. */
int des_synchronize(des_ctx *ctx);

/* Number of CUDA kernel launches made by the context so far. */
int des_launch_count(des_ctx *ctx, long long *count);

#ifdef __cplusplus
}
#endif

#endif /* DESGPU_H */
