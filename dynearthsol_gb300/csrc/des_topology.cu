// des_topology.cu -- the mesh topology a remeshing hands over, built on the
// device: the node-to-element support lists (create_support,
// mesh.cxx:1707-1721) and the boundary facet lists (create_boundary_facets,
// mesh.cxx:1637-1704), and des_remesh, which installs a new mesh in a live
// context.
//
// The reference rebuilds both after every remeshing (remeshing.cxx:
// 1937-2035); its facet search is a double loop over segments and elements
// (O(nseg x nelem)).  Here each list is built by kernels whose result does
// not depend on the order in which threads run:
// * support: integer atomics count each node's elements and claim slots in
//   its list, then each node sorts its own list by element id (and local
//   node), which gives the reference's ascending element order exactly;
// * facets: one thread per boundary segment searches the ascending support
//   list of the segment's smallest node for the first element facet with
//   the segment's node set and a compatible flag -- the first match of the
//   reference's element loop -- and one thread per boundary type then
//   collects its segments in segment order, as the reference appends them.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "des_ctx.cuh"

namespace des {

namespace {

constexpr int TPB_T = 256;
constexpr int SCAN_B = 1024;

__constant__ int c_facet3[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};   // NODE_OF_FACET, 3D
__constant__ int c_facet2[3][2] = {{1, 2}, {2, 0}, {0, 1}};                       // NODE_OF_FACET, 2D

int grid_of(long long n, int tpb) { return (int)std::max(1LL, (n + tpb - 1) / tpb); }

__global__ void k_count_support(long long nent, const int *__restrict__ conn, int nn, int *__restrict__ cnt,
                                int *__restrict__ bad)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nent) return;
    const int n = conn[i];
    if (n < 0 || n >= nn) {
        atomicExch(bad, 1);
        return;
    }
    atomicAdd(&cnt[n], 1);
}

// exclusive scan of n ints in blocks of SCAN_B: block prefix in place, block sums to sums
__global__ void k_scan_blocks(int n, int *__restrict__ a, int *__restrict__ sums)
{
    __shared__ int warp_tot[SCAN_B / 32];
    const int i = blockIdx.x * SCAN_B + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = i < n ? a[i] : 0;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = warp_tot[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int incl = x + (w > 0 ? warp_tot[w - 1] : 0);
    if (i < n) a[i] = incl - v;
    if (threadIdx.x == SCAN_B - 1) sums[blockIdx.x] = incl;
}

// exclusive scan of the nb block sums, by one block (each thread a run of them)
__global__ void k_scan_sums(int nb, int *__restrict__ sums)
{
    __shared__ int part[SCAN_B];
    const int per = (nb + SCAN_B - 1) / SCAN_B;
    const int lo = threadIdx.x * per, hi = min(lo + per, nb);
    int t = 0;
    for (int k = lo; k < hi; ++k) t += sums[k];
    part[threadIdx.x] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < SCAN_B; ++k) {
            const int v = part[k];
            part[k] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int k = lo; k < hi; ++k) {
        const int v = sums[k];
        sums[k] = run;
        run += v;
    }
}

__global__ void k_scan_add(int n, int *__restrict__ a, const int *__restrict__ sums)
{
    const int i = blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) a[i] += sums[blockIdx.x];
}

__global__ void k_fill_support(int ne, int npe, const int *__restrict__ conn, const int *__restrict__ off,
                               int *__restrict__ cursor, int *__restrict__ ent)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)ne * npe) return;
    const int e = (int)(q / npe), i = (int)(q % npe);
    const int n = conn[q];
    ent[off[n] + atomicAdd(&cursor[n], 1)] = e * 4 + i;
}

// each node's list in ascending element order (insertion sort: the lists are short)
__global__ void k_sort_support(int nn, const int *__restrict__ off, int *__restrict__ ent)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int lo = off[n], hi = off[n + 1];
    for (int k = lo + 1; k < hi; ++k) {
        const int v = ent[k];
        int j = k - 1;
        while (j >= lo && ent[j] > v) {
            ent[j + 1] = ent[j];
            --j;
        }
        ent[j + 1] = v;
    }
}

template <int ND>
__device__ __forceinline__ void sort_nodes(int *a)
{
    if (ND == 3) {
        if (a[0] > a[1]) { int t = a[0]; a[0] = a[1]; a[1] = t; }
        if (a[1] > a[2]) { int t = a[1]; a[1] = a[2]; a[2] = t; }
        if (a[0] > a[1]) { int t = a[0]; a[0] = a[1]; a[1] = t; }
    } else if (a[0] > a[1]) {
        int t = a[0]; a[0] = a[1]; a[1] = t;
    }
}

// one thread per segment: bdry[i] = its boundary type (-1: not a boundary
// segment, -2: no element facet matches), ef[i] = element * 4 + facet
template <int ND>
__global__ void k_find_facets(int nseg, const int *__restrict__ seg, const int *__restrict__ segflag,
                              const int *__restrict__ conn, const unsigned *__restrict__ bcflag,
                              const int *__restrict__ off, const int *__restrict__ ent, int *__restrict__ bdry,
                              int *__restrict__ ef, int *__restrict__ bad)
{
    constexpr int NPE = ND + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg) return;
    const unsigned flag = (unsigned)segflag[i];
    if ((flag & 1023u) == 0) {   // not a boundary facet (BOUND_ANY)
        bdry[i] = -1;
        return;
    }
    int s[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) s[j] = seg[(size_t)i * ND + j];
    sort_nodes<ND>(s);
    int k = -1;   // the boundary type of a one-bit flag
    for (int b = 0; b < 10; ++b)
        if (flag == (1u << b)) k = b;
    for (int q = off[s[0]]; q < off[s[0] + 1]; ++q) {
        const int e = ent[q] >> 2;
        for (int f = 0; f < NPE; ++f) {
            int fn[ND];
            unsigned fl = flag;
#pragma unroll
            for (int j = 0; j < ND; ++j) {
                fn[j] = conn[(size_t)e * NPE + (ND == 3 ? c_facet3[f][j] : c_facet2[f][j])];
                fl &= bcflag[fn[j]];
            }
            if (fl == 0u) continue;
            sort_nodes<ND>(fn);
            bool same = true;
#pragma unroll
            for (int j = 0; j < ND; ++j) same = same && fn[j] == s[j];
            if (same && k >= 0) {
                bdry[i] = k;
                ef[i] = e * 4 + f;
                return;
            }
        }
    }
    bdry[i] = -2;
    atomicExch(bad, 2);
}

// one thread per boundary type: offsets[11] and the facets in segment order
__global__ void k_collect_facets(int nseg, const int *__restrict__ bdry, const int *__restrict__ ef,
                                 int *__restrict__ offsets, int *__restrict__ facets)
{
    __shared__ int cnt[10];
    const int k = threadIdx.x;
    if (k < 10) {
        int c = 0;
        for (int i = 0; i < nseg; ++i) c += bdry[i] == k;
        cnt[k] = c;
    }
    __syncthreads();
    if (k == 0) {
        offsets[0] = 0;
        for (int b = 0; b < 10; ++b) offsets[b + 1] = offsets[b] + cnt[b];
    }
    __syncthreads();
    if (k < 10) {
        int pos = offsets[k];
        for (int i = 0; i < nseg; ++i)
            if (bdry[i] == k) {
                facets[2 * pos] = ef[i] >> 2;
                facets[2 * pos + 1] = ef[i] & 3;
                ++pos;
            }
    }
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { cudaFree(p); }
};

}  // namespace

// Support lists (CSR, entries element * 4 + local node, ascending element)
// and boundary facet lists of a topology, built on the device; sup_off and
// sup_ent, bf_off and bf are filled on the host.  Returns DES_OK or an error
// code with its message in err.
int build_topology_device(const des_topology *t, cudaStream_t s, std::vector<int> &sup_off,
                          std::vector<int> &sup_ent, std::vector<int> &bf_off, std::vector<int> &bf,
                          std::string &err)
{
    const int nd = t->ndims, npe = nd + 1, nn = t->nnode, ne = t->nelem, nseg = t->nseg;
    const long long nent = (long long)ne * npe;
    const int nb = grid_of(nn + 1, SCAN_B);
    // one device block: conn [nent], cnt/off [nn+1], cursor [nn], ent [nent], sums [nb], bad [1],
    // bcflag [nn], seg [nseg*nd], segflag [nseg], bdry [nseg], ef [nseg], offsets [11], facets [2 nseg]
    const size_t n_int = 2 * (size_t)nent + 2 * (size_t)nn + 1 + nb + 1 + nn + (size_t)nseg * (nd + 5) + 11 + 8;
    DevBuf buf;
    cudaError_t ce = cudaMalloc(&buf.p, n_int * sizeof(int));
    if (ce != cudaSuccess) {
        (void)cudaGetLastError();
        err = std::string("cudaMalloc for the topology build: ") + cudaGetErrorString(ce);
        return DES_ENOMEM;
    }
    int *p = static_cast<int *>(buf.p);
    int *d_conn = p; p += nent;
    int *d_off = p; p += nn + 1;
    int *d_cursor = p; p += nn;
    int *d_ent = p; p += nent;
    int *d_sums = p; p += nb;
    int *d_bad = p; p += 1;
    unsigned *d_bcflag = reinterpret_cast<unsigned *>(p); p += nn;
    int *d_seg = p; p += (size_t)nseg * nd;
    int *d_segflag = p; p += nseg;
    int *d_bdry = p; p += nseg;
    int *d_ef = p; p += nseg;
    int *d_foff = p; p += 11;
    int *d_fac = p;
#define TCK(call)                                                   \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) {                                    \
            err = std::string(#call ": ") + cudaGetErrorString(e_); \
            return DES_ECUDA;                                       \
        }                                                           \
    } while (0)
    TCK(cudaMemcpyAsync(d_conn, t->connectivity, nent * sizeof(int), cudaMemcpyHostToDevice, s));
    TCK(cudaMemsetAsync(d_off, 0, (2 * (size_t)nn + 1) * sizeof(int), s));
    TCK(cudaMemsetAsync(d_bad, 0, sizeof(int), s));
    k_count_support<<<grid_of(nent, TPB_T), TPB_T, 0, s>>>(nent, d_conn, nn, d_off, d_bad);
    k_scan_blocks<<<nb, SCAN_B, 0, s>>>(nn + 1, d_off, d_sums);
    k_scan_sums<<<1, SCAN_B, 0, s>>>(nb, d_sums);
    k_scan_add<<<nb, SCAN_B, 0, s>>>(nn + 1, d_off, d_sums);
    k_fill_support<<<grid_of(nent, TPB_T), TPB_T, 0, s>>>(ne, npe, d_conn, d_off, d_cursor, d_ent);
    k_sort_support<<<grid_of(nn, TPB_T), TPB_T, 0, s>>>(nn, d_off, d_ent);
    TCK(cudaGetLastError());
    int bad = 0;
    TCK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    TCK(cudaStreamSynchronize(s));
    if (bad) {
        err = "connectivity holds a node id out of range";
        return DES_EINPUT;
    }
    if (nseg > 0) {
        TCK(cudaMemcpyAsync(d_bcflag, t->bcflag, nn * sizeof(unsigned), cudaMemcpyHostToDevice, s));
        TCK(cudaMemcpyAsync(d_seg, t->segment, (size_t)nseg * nd * sizeof(int), cudaMemcpyHostToDevice, s));
        TCK(cudaMemcpyAsync(d_segflag, t->segflag, nseg * sizeof(int), cudaMemcpyHostToDevice, s));
        if (nd == 3)
            k_find_facets<3><<<grid_of(nseg, TPB_T), TPB_T, 0, s>>>(nseg, d_seg, d_segflag, d_conn, d_bcflag, d_off,
                                                                    d_ent, d_bdry, d_ef, d_bad);
        else
            k_find_facets<2><<<grid_of(nseg, TPB_T), TPB_T, 0, s>>>(nseg, d_seg, d_segflag, d_conn, d_bcflag, d_off,
                                                                    d_ent, d_bdry, d_ef, d_bad);
        k_collect_facets<<<1, 32, 0, s>>>(nseg, d_bdry, d_ef, d_foff, d_fac);
        TCK(cudaGetLastError());
    }
    sup_off.resize(nn + 1);
    sup_ent.resize(nent);
    bf_off.assign(DES_NBDRYTYPES + 1, 0);
    TCK(cudaMemcpyAsync(sup_off.data(), d_off, (nn + 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
    TCK(cudaMemcpyAsync(sup_ent.data(), d_ent, nent * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (nseg > 0) {
        TCK(cudaMemcpyAsync(bf_off.data(), d_foff, 11 * sizeof(int), cudaMemcpyDeviceToHost, s));
        TCK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    TCK(cudaStreamSynchronize(s));
    if (bad) {
        err = "a boundary segment matches no element facet (create_boundary_facets, mesh.cxx:1690-1692)";
        return DES_EASSERT;
    }
    bf.resize(2 * (size_t)std::max(bf_off[DES_NBDRYTYPES], 1));
    if (bf_off[DES_NBDRYTYPES] > 0) {
        TCK(cudaMemcpyAsync(bf.data(), d_fac, 2 * (size_t)bf_off[DES_NBDRYTYPES] * sizeof(int),
                            cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
    }
#undef TCK
    return DES_OK;
}

}  // namespace des

using namespace des;

namespace {

int check_topology(const des_topology *t, std::string &err)
{
    if (!t) {
        err = "NULL topology";
        return DES_EINPUT;
    }
    if (t->ndims != 2 && t->ndims != 3) {
        err = "ndims must be 2 or 3";
        return DES_EINPUT;
    }
    if (t->nnode <= 0 || t->nelem <= 0 || t->nseg < 0 || !t->connectivity ||
        (t->nseg > 0 && (!t->bcflag || !t->segment || !t->segflag))) {
        err = "empty mesh or NULL topology array";
        return DES_EINPUT;
    }
    if ((long long)t->nelem * 4 >= (1ll << 31)) {
        err = "nelem too large for int32 support entries";
        return DES_EINPUT;
    }
    return DES_OK;
}

std::string g_topology_error;

}  // namespace

extern "C" int des_build_topology(const des_topology *t, int *sup_off, int *sup_elem, int *bfacet_offsets,
                                  int *bfacets, void *stream)
{
    std::string err;
    int rc = check_topology(t, err);
    std::vector<int> off, ent, boff, bf;
    if (!rc) rc = build_topology_device(t, static_cast<cudaStream_t>(stream), off, ent, boff, bf, err);
    if (rc) {
        fprintf(stderr, "des_build_topology: %s\n", err.c_str());
        g_topology_error = err;
        return rc;
    }
    if (sup_off) std::memcpy(sup_off, off.data(), off.size() * sizeof(int));
    if (sup_elem)
        for (size_t q = 0; q < ent.size(); ++q) sup_elem[q] = ent[q] >> 2;
    if (bfacet_offsets) std::memcpy(bfacet_offsets, boff.data(), boff.size() * sizeof(int));
    if (bfacets && boff[DES_NBDRYTYPES] > 0)
        std::memcpy(bfacets, bf.data(), 2 * (size_t)boff[DES_NBDRYTYPES] * sizeof(int));
    return DES_OK;
}

extern "C" int des_remesh(des_ctx *c, const des_topology *t, const int *elemmarkers)
{
    if (!c) return DES_EINPUT;
    std::string err;
    int rc = check_topology(t, err);
    if (!rc && t->ndims != c->nd) {
        err = "the new mesh has another dimension";
        rc = DES_EINPUT;
    }
    if (!rc && c->kp.mat.nmat > 1 && !elemmarkers) {
        err = "a multi-material context needs the new mesh's element markers";
        rc = DES_EINPUT;
    }
    std::vector<int> off, ent, boff, bf;
    if (!rc) rc = build_topology_device(t, c->stream, off, ent, boff, bf, err);
    if (rc) return ctx_fail(c, rc, "des_remesh: %s", err.c_str());
    // the new mesh with the context's boundary normals and edge vectors
    des_mesh m;
    std::memset(&m, 0, sizeof m);
    m.ndims = t->ndims;
    m.nnode = t->nnode;
    m.nelem = t->nelem;
    m.connectivity = t->connectivity;
    m.bcflag = t->bcflag;
    m.bfacet_offsets = boff.data();
    m.bfacets = bf.data();
    std::memcpy(m.bnormals, c->kp.bnormals, sizeof m.bnormals);
    std::memcpy(m.edge_vectors, c->kp.edge_vectors, sizeof m.edge_vectors);
    // the context's material table (MatC keeps every material array)
    const MatC &mt = c->kp.mat;
    des_material mat;
    std::memset(&mat, 0, sizeof mat);
    mat.rheol_type = mt.rheol_type;
    mat.nmat = mt.nmat;
    mat.is_plane_strain = mt.is_plane_strain;
    mat.scalar_mask = mt.scalar_mask;
    mat.visc_min = mt.visc_min;
    mat.visc_max = mt.visc_max;
    mat.tension_max = mt.tension_max;
    mat.therm_diff_max = mt.therm_diff_max;
    mat.rho0 = mt.rho0;
    mat.alpha = mt.alpha;
    mat.bulk_modulus = mt.bulk_modulus;
    mat.shear_modulus = mt.shear_modulus;
    mat.visc_exponent = mt.visc_exponent;
    mat.visc_coefficient = mt.visc_coefficient;
    mat.visc_activation_energy = mt.visc_activation_energy;
    mat.heat_capacity = mt.heat_capacity;
    mat.therm_cond = mt.therm_cond;
    mat.radiogenic_heating = mt.radiogenic_heating;
    mat.pls0 = mt.pls0;
    mat.pls1 = mt.pls1;
    mat.cohesion0 = mt.cohesion0;
    mat.cohesion1 = mt.cohesion1;
    mat.friction_angle0 = mt.friction_angle0;
    mat.friction_angle1 = mt.friction_angle1;
    mat.dilation_angle0 = mt.dilation_angle0;
    mat.dilation_angle1 = mt.dilation_angle1;
    mat.elemmarkers = mt.nmat > 1 ? elemmarkers : nullptr;
    const des_params prm = c->kp.prm;
    des_ctx *n = nullptr;
    rc = create_context(&m, &prm, &mat, c->precision, c->stream, &off, &ent, &n);
    if (rc) {
        char msg[512];
        des_last_error(nullptr, msg, sizeof msg);
        return ctx_fail(c, rc, "des_remesh: %s", msg);
    }
    // move the new context into the caller's handle; the stream stays the caller's or the old context's own
    const bool own = c->own_stream;
    release_context(c);
    *c = std::move(*n);
    c->own_stream = own;
    n->own_stream = false;
    delete n;
    return DES_OK;
}
