// des_noalloc.cu -- NMD_stress for callers that cannot allocate device
// memory.
//
// Some hosts of this library own every device byte themselves: a solver
// embedded in a larger GPU application that hands out memory only from its
// own pools, a process running under a strict device-memory quota, or code
// that runs while another component holds the allocator (for example inside
// a region where cudaMalloc is not permitted).  Such callers cannot create a
// context with des_create, which allocates.  des_nmd_stress_noalloc lets
// them run the nodal-mixed-discretisation pressure smoothing (the reference's
// NMD_stress, geometry.cxx:182-236) on arrays they already own: the caller
// passes every input and output as a device pointer, and the one piece of
// scratch the smoothing needs -- the per-node pressure sum -- lives in the
// fixed array below, which every GPU that loads this library holds until the
// process exits.
#include <atomic>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/desgpu.h"

namespace {

// per-node scratch: DES_NOALLOC_MAX_NODES doubles (16 MiB per device)
__device__ __align__(256) double g_nmd_scratch[DES_NOALLOC_MAX_NODES];

// Device address of the scratch, per device.  In host code g_nmd_scratch
// names a host-side stand-in, so the kernels get this address instead.  It
// is looked up again on every call made outside stream capture (a device
// reset reloads the module and can move the array); inside a capture, where
// the lookup is not allowed, the address of the last lookup on this device
// is used.  Relaxed atomics: concurrent first calls all store the same
// value, and nothing else is ordered by it.
constexpr int kMaxDevices = 64;
std::atomic<double *> g_scratch_addr[kMaxDevices] = {};

__global__ void k_nmd_nodes(int nn, const int *__restrict__ sup_off, const int *__restrict__ sup_ent,
                            const double *__restrict__ dpressure, const double *__restrict__ volume,
                            const double *__restrict__ volume_n, double *__restrict__ dp_nd)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    double acc = 0;
    for (int q = sup_off[n]; q < sup_off[n + 1]; ++q) {
        int e = sup_ent[q] >> 2;
        acc += dpressure[e] * volume[e];     // geometry.cxx:206
    }
    dp_nd[n] = acc / volume_n[n];            // geometry.cxx:216 (every entry written: no clearing needed)
}

__global__ void k_nmd_elems(int ne, int ndims, const int *__restrict__ conn, const double *__restrict__ dpressure,
                            const double *__restrict__ dp_nd, double *__restrict__ stress)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int npe = ndims + 1;
    double dp = 0;
    for (int i = 0; i < npe; ++i) dp += dp_nd[conn[(size_t)i * ne + e]];   // geometry.cxx:225-229
    double dp_el = dp / npe;
    double dp_orig = dpressure[e];
    for (int i = 0; i < ndims; ++i) stress[(size_t)i * ne + e] += (-dp_orig + dp_el) / ndims;   // :234
}

// Device address of the scratch on device dev (nullptr on failure).
double *scratch_address(int dev, cudaStream_t s)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t qe = cudaStreamIsCapturing(s, &cap);
    if (qe != cudaSuccess) {
        // the legacy stream reports an error while another stream captures
        // in global mode; the lookup is not allowed then either
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;
    }
    if (cap != cudaStreamCaptureStatusNone) return g_scratch_addr[dev].load(std::memory_order_relaxed);
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_nmd_scratch) != cudaSuccess || !ptr) {
        cudaGetLastError();
        return nullptr;
    }
    g_scratch_addr[dev].store(static_cast<double *>(ptr), std::memory_order_relaxed);
    return static_cast<double *>(ptr);
}

}  // namespace

extern "C" int des_nmd_stress_noalloc(int ndims, int nnode, int nelem, const int *conn, const int *sup_off,
                                      const int *sup_ent, const double *dpressure, const double *volume,
                                      const double *volume_n, double *stress, void *stream)
{
    if (ndims != 2 && ndims != 3) return DES_EINPUT;
    if (nnode <= 0 || nelem <= 0) return DES_EINPUT;
    if (nnode > DES_NOALLOC_MAX_NODES) {
        fprintf(stderr, "des_nmd_stress_noalloc: %d nodes exceed the fixed scratch of %d nodes\n", nnode,
                DES_NOALLOC_MAX_NODES);
        return DES_EINPUT;
    }
    if (!conn || !sup_off || !sup_ent || !dpressure || !volume || !volume_n || !stress) return DES_EINPUT;
    // An error left pending on this thread by earlier, unrelated work is the
    // caller's: report it without consuming it, and launch nothing.
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        fprintf(stderr, "des_nmd_stress_noalloc: a CUDA error from earlier work is pending (%s); nothing launched\n",
                cudaGetErrorString(pending));
        return DES_ECUDA;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DES_ECUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *scratch = scratch_address(dev, s);
    if (!scratch) return DES_ECUDA;
    const int tpb = 256;
    k_nmd_nodes<<<(nnode + tpb - 1) / tpb, tpb, 0, s>>>(nnode, sup_off, sup_ent, dpressure, volume, volume_n,
                                                         scratch);
    if (cudaGetLastError() != cudaSuccess) return DES_ECUDA;
    k_nmd_elems<<<(nelem + tpb - 1) / tpb, tpb, 0, s>>>(nelem, ndims, conn, dpressure, scratch, stress);
    if (cudaGetLastError() != cudaSuccess) return DES_ECUDA;
    return DES_OK;
}
