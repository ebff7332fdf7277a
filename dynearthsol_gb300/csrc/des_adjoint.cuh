// des_adjoint.cuh -- reverse mode of the 3D FP64 step: buffers and kernels.
//
// The differentiated map is one explicit step of the FP64 path with dt held
// fixed, as a function of the state S = (coord, vel, T, stress, plstrain,
// volume_old) and of the fields derived from it, D = (volume, shape
// functions, mass, tmass, volume_n), which the step of the reference
// recomputes from the new coordinates at its end (update_mesh,
// dynearthsol.cxx:221-232).  The adjoint of one step maps the adjoints of
// (S_{k+1}, D_{k+1}) to those of (S_k, D_k) and adds the step's share of the
// parameter gradients.  Element-to-node transfers go through per-(element,
// slot) arrays summed per node over the support lists in ascending element
// order, as the forward gathers do: no atomics, reproducible results.
#pragma once
#include "des_common.cuh"

namespace des {

// device arrays of one recorded step (all owned by the adjoint workspace)
struct TapeStep {
    // state at the start of the step
    double *x, *v, *T, *s, *pls, *volo;
    // fields derived from it
    double *vol, *shp, *mass, *tmass, *voln;
    // forward intermediates of the step
    double *edot;    // [6][ne] strain rate before the anti-locking correction
    double *tdot;    // [nn]
    double *ntmp;    // [nn] nodal dvoldt
    double *edv;     // [ne] edvoldt
    double *sstar;   // [6][ne] stress after update_stress
    double *dp;      // [ne] dpressure
    double *rho;     // [ne] element density of the step
    double *dpn;     // [nn] NMD nodal pressure change
    double *f;       // [3][nn] force after damping
    double *visc;    // [ne] viscosity the rheology used (Maxwell, EVP)
    unsigned char *evp;   // [ne] EVP branch taken: 1 elasto-plastic, 0 Maxwell
};

// adjoint buffers; "_k" fields hold the adjoint of the state at the start
// of the step being reversed once its kernels have run
struct AdjBufs {
    double *ax, *av, *aT;            // [3][nn], [3][nn], [nn]
    double *as, *apls, *avolo;       // [6][ne], [ne], [ne]
    double *avol, *ashp;             // [ne], [12][ne]
    double *am, *atm, *avn;          // [nn] x3
    double *af;                      // [3][nn] adjoint of the force before damping
    double *antmp;                   // [nn] adjoint of nodal dvoldt / volume_n
    double *adpn;                    // [nn] adjoint of NMD nodal dp / volume_n
    double *atdot;                   // [nn]
    double *aedot;                   // [6][ne]
    double *aedv, *adp, *arho;       // [ne] x3
    double *slot3;                   // [3][4][ne] nodal vector contributions
    double *slotx;                   // [3][4][ne] nodal coordinate contributions
    double *slot1;                   // [4][ne] nodal scalar contributions
    double *fslot;                   // [3][3][nbf] facet -> node coordinate contributions
    double *frho;                    // [nbf] facet -> element density adjoint
    const int *e2f_off, *e2f_ent;    // element -> boundary facets (ascending facet id)
    double *g;                       // [7][ne] parameter gradients (DES_EF_* order)
    double *gvbc;                    // [nblk][DES_NBDRYTYPES] per-block partial sums
};

// adjoint-state kernels of one step, launched in this order by the host
int launch_adj_end_geometry(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                            cudaStream_t s);
int launch_adj_motion(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                      cudaStream_t s);
int launch_adj_force(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s);
int launch_adj_nmd_nodes(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s);
int launch_adj_stress(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                      cudaStream_t s);
int launch_adj_nodes_heat(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                          cudaStream_t s);
int launch_adj_kinematics(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s);
int launch_adj_gather_vT(const KP &p, const AdjBufs &a, cudaStream_t s);
// adjoint of the derived fields at the window start -> coordinates and temperature
int launch_adj_start_geometry(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s);
int launch_adj_gather_xT(const KP &p, const AdjBufs &a, cudaStream_t s);
int adj_vbc_blocks(const KP &p);

}  // namespace des
