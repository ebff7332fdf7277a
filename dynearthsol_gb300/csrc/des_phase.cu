// des_phase.cu -- markers on the device and the phase changes that move
// them between materials (phase_changes, phasechanges.cxx:232-258).
//
// The reference keeps its markers (MarkerSet: element, barycentric
// coordinates and material type of each marker) on the host and, every 10
// steps (dynearthsol.cxx:349-353), evaluates each marker's depth,
// temperature and reference pressure, applies the phase-change rule of its
// material, and moves the marker between the element's marker counts
// (Variables::elemmarkers), from which MatProps blends the element's
// properties.  Here the markers are copied to the device once (after they
// are created or remapped), one thread evaluates each marker against the
// device's own coordinates and temperatures, and the marker counts the
// device step blends from are updated in place with integer atomics, whose
// result does not depend on their order.  No coordinate, temperature or
// marker array crosses to the host.
#include <cstdio>
#include <vector>

#include "des_ctx.cuh"
#include "des_kernels.cuh"

namespace des {

constexpr int TPB_P = 256;

// SimpleSubduction (phasechanges.cxx:44-160): the material types and the
// transitions of a marker at depth Z, pressure P and temperature T; hydrous
// is the element's hydrous-marker count.  Hydration processes (the marker
// a dehydration releases) stay on the host and are not modelled here.
__device__ __forceinline__ int simple_subduction(int mt, double Z, double P, double T, int hydrous)
{
    enum { mantle = 0, serpentinized_mantle = 1, oceanic_crust = 2, eclogite = 3, sediment = 4, schist = 5 };
    switch (mt) {
    case oceanic_crust: {   // basalt -> eclogite
        const double min_eclogite_T = 500 + 273;
        const double transition_pressure = -0.3e9 + 2.2e6 * T;
        if (T > min_eclogite_T && P > transition_pressure) return eclogite;
        break;
    }
    case sediment: {   // sediment -> schist/gneiss
        const double min_schist_T = 650 + 273;
        const double min_schist_Z = -20e3;
        if (T > min_schist_T && Z < min_schist_Z) return schist;
        break;
    }
    case serpentinized_mantle: {   // serpentinite -> mantle
        const double transition_pressure = 2.1e9 + (7.5e9 - 2.1e9) * (T - (730 + 273)) / (500 - 730);
        const double min_serpentine_T = 550 + 273;
        if (T > min_serpentine_T && P > transition_pressure) return mantle;
        break;
    }
    case mantle: {   // mantle -> serpentinite where hydrous markers are
        const double min_serpentine_T = 550 + 273;
        if (T <= min_serpentine_T && hydrous) return serpentinized_mantle;
        break;
    }
    }
    return mt;
}

// one thread per marker: PhaseChange::get_ZPT (phasechanges.cxx:24-39) and
// the rule of option; emark [nmat][ne] counts, changed = markers moved
template <int ND>
__global__ void __launch_bounds__(TPB_P) k_phase_changes(KP p, int nm, const int *__restrict__ melem,
                                                         const double *__restrict__ meta, int *__restrict__ mtype,
                                                         const int *__restrict__ hydem, int option, int *emark,
                                                         unsigned *changed)
{
    constexpr int NPE = ND + 1;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nm) return;
    const int e = melem[m];
    if (e < 0 || e >= p.ne) {
        set_err(p, DES_DEV_BAD_INDEX);
        return;
    }
    double Z = 0, T = 0;
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        const int n = conn_at(p, i, e);
        const double eta = meta[(size_t)i * nm + m];
        Z += p.x[(size_t)(ND - 1) * p.nn + n] * eta;
        T += p.T[n] * eta;
    }
    const double P = ref_pressure_(p, Z);
    const int cur = mtype[m];
    const int nw = option == 1 ? simple_subduction(cur, Z, P, T, hydem ? hydem[e] : 0) : cur;
    if (nw == cur) return;
    if (cur < 0 || cur >= p.mat.nmat || nw < 0 || nw >= p.mat.nmat) {
        set_err(p, DES_DEV_BAD_INDEX);   // a material type beyond the table
        return;
    }
    mtype[m] = nw;
    atomicSub(&emark[(size_t)cur * p.ne + e], 1);
    atomicAdd(&emark[(size_t)nw * p.ne + e], 1);
    atomicAdd(changed, 1u);
}

void markers_free(des_ctx *c)
{
    cudaFree(c->d_markers);
    c->d_markers = nullptr;
    c->nmarkers = 0;
}

}  // namespace des

using namespace des;

extern "C" int des_set_markers(des_ctx *c, int nmarkers, const int *elem, const double *eta, const int *mattype)
{
    if (!c || nmarkers < 0 || (nmarkers > 0 && (!elem || !eta || !mattype))) return DES_EINPUT;
    const int npe = c->npe, ne = c->ne;
    for (int m = 0; m < nmarkers; ++m)
        if (elem[m] < 0 || elem[m] >= ne || mattype[m] < 0 || mattype[m] >= c->kp.mat.nmat)
            return ctx_fail(c, DES_EINPUT, "marker %d: element %d or material type %d out of range", m, elem[m],
                            mattype[m]);
    markers_free(c);
    if (nmarkers == 0) return DES_OK;
    // one block: elem, mattype [nm] ints, eta [npe][nm] doubles, hydrous counts [ne], changed
    const size_t n_int = 2 * (size_t)nmarkers + ne + 2;
    const size_t bytes = ((n_int * sizeof(int) + 15) / 16) * 16 + (size_t)npe * nmarkers * sizeof(double);
    cudaError_t ce = cudaMalloc(&c->d_markers, bytes);
    if (ce != cudaSuccess) {
        (void)cudaGetLastError();
        c->d_markers = nullptr;
        return ctx_fail(c, DES_ENOMEM, "cudaMalloc(%zu bytes) for %d markers: %s", bytes, nmarkers,
                        cudaGetErrorString(ce));
    }
    c->nmarkers = nmarkers;
    int *ip = static_cast<int *>(c->d_markers);
    double *eta_d = reinterpret_cast<double *>(static_cast<char *>(c->d_markers) +
                                               ((n_int * sizeof(int) + 15) / 16) * 16);
    std::vector<double> soa((size_t)npe * nmarkers);
    for (int m = 0; m < nmarkers; ++m)
        for (int i = 0; i < npe; ++i) soa[(size_t)i * nmarkers + m] = eta[(size_t)m * npe + i];
    cudaError_t e1 = cudaMemcpyAsync(ip, elem, nmarkers * sizeof(int), cudaMemcpyHostToDevice, c->stream);
    cudaError_t e2 = cudaMemcpyAsync(ip + nmarkers, mattype, nmarkers * sizeof(int), cudaMemcpyHostToDevice,
                                     c->stream);
    cudaError_t e3 = cudaMemcpyAsync(eta_d, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice,
                                     c->stream);
    cudaError_t e4 = cudaStreamSynchronize(c->stream);
    for (cudaError_t x : {e1, e2, e3, e4})
        if (x != cudaSuccess) return ctx_cuda_fail(c, x, "des_set_markers");
    return DES_OK;
}

extern "C" int des_phase_changes(des_ctx *c, int option, const int *hydrous_elemmarkers, int *nchanged)
{
    if (!c) return DES_EINPUT;
    if (nchanged) *nchanged = 0;
    // phase_changes_init (phasechanges.cxx:208-229): one material or option 0 -> no phase change
    if (c->kp.mat.nmat == 1 || option == 0) return DES_OK;
    if (option != 1 && option != 101) return ctx_fail(c, DES_EINPUT, "unknown phase_change_option: %d", option);
    if (!c->kp.emark) return ctx_fail(c, DES_EINPUT, "context was created without per-element markers");
    if (c->nmarkers == 0) return DES_OK;
    const int nm = c->nmarkers, ne = c->ne;
    int *ip = static_cast<int *>(c->d_markers);
    int *melem = ip, *mtype = ip + nm, *hyd = ip + 2 * nm;
    unsigned *changed = reinterpret_cast<unsigned *>(ip + 2 * nm + ne);
    const double *eta_d = reinterpret_cast<const double *>(
        static_cast<char *>(c->d_markers) + (((2 * (size_t)nm + ne + 2) * sizeof(int) + 15) / 16) * 16);
    cudaError_t e = cudaMemsetAsync(changed, 0, sizeof(unsigned), c->stream);
    if (e == cudaSuccess && hydrous_elemmarkers)
        e = cudaMemcpyAsync(hyd, hydrous_elemmarkers, ne * sizeof(int), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "des_phase_changes");
    const int grid = (nm + TPB_P - 1) / TPB_P;
    int *emark = const_cast<int *>(c->kp.emark);
    if (c->nd == 3)
        k_phase_changes<3><<<grid, TPB_P, 0, c->stream>>>(c->kp, nm, melem, eta_d, mtype,
                                                         hydrous_elemmarkers ? hyd : nullptr, option, emark, changed);
    else
        k_phase_changes<2><<<grid, TPB_P, 0, c->stream>>>(c->kp, nm, melem, eta_d, mtype,
                                                         hydrous_elemmarkers ? hyd : nullptr, option, emark, changed);
    int rc = ctx_check_launch(c, 1);
    if (rc) return rc;
    // the blended material properties follow the new counts
    if (c->kp.eprop && (rc = ctx_check_launch(c, launch_elem_props(c->kp, c->stream,
                                                                   const_cast<double *>(c->kp.eprop)))))
        return rc;
    unsigned n = 0;
    e = cudaMemcpyAsync(&n, changed, sizeof n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "des_phase_changes");
    if (nchanged) *nchanged = (int)n;
    unsigned bits = 0;
    return des_device_status(c, &bits);
}

extern "C" int des_get_markers(des_ctx *c, int *mattype, int *elemmarkers)
{
    if (!c) return DES_EINPUT;
    const int nm = c->nmarkers, ne = c->ne, nmat = c->kp.mat.nmat;
    if (mattype && nm > 0) {
        cudaError_t e = cudaMemcpyAsync(mattype, static_cast<int *>(c->d_markers) + nm, nm * sizeof(int),
                                        cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return ctx_cuda_fail(c, e, "des_get_markers");
    }
    if (elemmarkers) {
        if (!c->kp.emark) return ctx_fail(c, DES_EINPUT, "context was created without per-element markers");
        std::vector<int> soa((size_t)ne * nmat);
        cudaError_t e = cudaMemcpyAsync(soa.data(), c->kp.emark, soa.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                        c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return ctx_cuda_fail(c, e, "des_get_markers");
        for (int el = 0; el < ne; ++el)
            for (int k = 0; k < nmat; ++k) elemmarkers[(size_t)el * nmat + k] = soa[(size_t)k * ne + el];
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? DES_OK : ctx_cuda_fail(c, e, "des_get_markers");
}
