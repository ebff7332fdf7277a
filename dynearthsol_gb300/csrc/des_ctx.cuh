// des_ctx.cuh -- the device context behind the C ABI (internal to the
// library: des_capi.cu and the adjoint's host side share it).
#pragma once
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/desgpu.h"
#include "des_common.cuh"

namespace des {
struct AdjWork;
}

// events of one pipelined transfer: start, done, one per multi-component field
constexpr int DES_XFER_EVENTS = 32;

struct des_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int precision = DES_PREC_FP64;
    int nd = 0, npe = 0, nstr = 0, nn = 0, ne = 0, nbf = 0;
    des::KP kp{};                 // per-function parameter block (no step scratch)
    char *pool = nullptr;         // one device allocation for every array
    size_t pool_bytes = 0;
    double *d_tdot = nullptr;     // node scratch of the fused step
    double *d_rho = nullptr;      // element scratch of the fused step
    double *d_buoy = nullptr;     // element scratch of the fused step: rho g / NPE
    double *d_stage = nullptr;    // AoS staging buffer
    size_t stage_doubles = 0;
    unsigned long long *d_red = nullptr;
    double *d_ef[DES_EF_COUNT] = {};
    cudaGraphExec_t step_exec = nullptr;
    // the chained mixed step of des_step(n >= 2): its first, middle and last
    // steps (a look-ahead geometry pass does the next step's element pass,
    // and the next node pass the mass sums; the last step ends as one step)
    cudaGraphExec_t chain_exec[3] = {};
    int chain_kernels[3] = {};
    // pipelined host transfers, created by the first state transfer
    cudaStream_t xstream = nullptr;   // DMA between host rows and the device
    cudaEvent_t xev[DES_XFER_EVENTS] = {};
    double *d_xstage = nullptr;       // one AoS region per multi-component field
    size_t xstage_doubles = 0;
    cudaEvent_t ev_mid = nullptr;     // recorded by step_exec_mid once nmd_correct is done
    cudaGraphExec_t step_exec_mid = nullptr;
    // slabs of the pipelined host step (des_step_host): nfine fine slabs of
    // element rows [slab_e[j], slab_e[j+1]), node rows [slab_n[j],
    // slab_n[j+1]) and boundary facets d_fac_order[slab_f[j] .. slab_f[j+1]);
    // nslab coarse slabs of whole fine slabs; nslab 1: not pipelined
    int nfine = 0, nslab = 1;
    std::vector<int> slab_e, slab_n, slab_f;
    int *d_fac_order = nullptr;
    cudaStream_t ystream = nullptr;        // device -> host copies of the pipelined step
    cudaGraphExec_t pipe_exec = nullptr;   // the pipelined host step, for the host arrays below
    std::vector<const void *> pipe_key;
    std::vector<cudaEvent_t> pipe_ev;
    double *d_pipe_sink = nullptr;         // [2][nn]: node sums the pipelined step forms but keeps uploaded
    int pipe_kernels = 0;
    int step_kernels = 0;
    long long launches = 0;
    std::string err;
    bool has_state = false;
    des::AdjWork *adj = nullptr;  // reverse-mode workspace, created on first use
    // markers on the device (des_set_markers): one block of element ids,
    // material types, hydrous counts and barycentric coordinates
    int nmarkers = 0;
    void *d_markers = nullptr;
};

namespace des {

// helpers of des_capi.cu for the other translation units of the context
int ctx_fail(des_ctx *c, int code, const char *fmt, ...);
int ctx_cuda_fail(des_ctx *c, cudaError_t e, const char *what);
int ctx_check_launch(des_ctx *c, int n);
KP ctx_step_kp(const des_ctx *c);
// state transfer between host AoS rows and device SoA arrays (staging buffer)
int ctx_put_field(des_ctx *c, const double *host, double *dev, int n, int ncomp);
int ctx_get_field(des_ctx *c, const double *dev, double *host, int n, int ncomp);
// frees the reverse-mode workspace (des_adjoint_host.cu)
void adj_free(des_ctx *c);
// frees the device markers (des_phase.cu)
void markers_free(des_ctx *c);
// des_create with optionally pre-built support lists (des_capi.cu)
int create_context(const des_mesh *mesh, const des_params *param, const des_material *mat, int precision,
                   cudaStream_t stream, const std::vector<int> *pre_off, const std::vector<int> *pre_ent,
                   des_ctx **out);
// every device resource of a context except its stream (des_capi.cu)
void release_context(des_ctx *c);
// support and boundary facet lists of a topology built on the device (des_topology.cu)
int build_topology_device(const des_topology *t, cudaStream_t s, std::vector<int> &sup_off,
                          std::vector<int> &sup_ent, std::vector<int> &bf_off, std::vector<int> &bf,
                          std::string &err);

}  // namespace des
