// des_capi.cu -- C ABI of the explicit-step library (include/desgpu.h):
// context creation (topology products on the host, one device pool),
// host <-> device state transfer in the reference's layout, the
// per-function entry points and the CUDA-graph-replayed fused step.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "des_ctx.cuh"
#include "des_kernels.cuh"
#include "des_mixed.cuh"

using namespace des;

namespace {

thread_local std::string g_create_error;

int fail_msg(std::string &dst, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    dst = buf;
    return code;
}

}  // namespace

namespace {

int cuda_fail(des_ctx *c, cudaError_t e, const char *what)
{
    // a failed call (an allocation, say) leaves its error as the runtime's
    // last error, which the next launch check would report as its own;
    // sticky errors stay whatever this returns
    (void)cudaGetLastError();
    std::string &dst = c ? c->err : g_create_error;
    return fail_msg(dst, DES_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                        \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
    } while (0)

int check_launch(des_ctx *c, int n)
{
    c->launches += n;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "kernel launch");
    return DES_OK;
}

KP step_kp(const des_ctx *c)
{
    KP p = c->kp;
    p.rho_e = c->d_rho;
    p.buoy_e = c->d_buoy;
    p.tdot = c->d_tdot;
    return p;
}

void invalidate_graph(des_ctx *c)
{
    if (c->step_exec) {
        cudaGraphExecDestroy(c->step_exec);
        c->step_exec = nullptr;
    }
    if (c->step_exec_mid) {
        cudaGraphExecDestroy(c->step_exec_mid);
        c->step_exec_mid = nullptr;
    }
    for (cudaGraphExec_t &g : c->chain_exec) {
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    }
    if (c->pipe_exec) {
        cudaGraphExecDestroy(c->pipe_exec);
        c->pipe_exec = nullptr;
    }
    c->pipe_key.clear();
}

void set_rho_pseudo(des_ctx *c);

int set_params(des_ctx *c, const des_params *prm)
{
    if (prm->ref_pressure_option != 0)
        return fail_msg(c->err, DES_EINPUT, "ref_pressure_option %d is not supported on the device (only 0)",
                        prm->ref_pressure_option);
    if (prm->surface_process_option != 0)
        return fail_msg(c->err, DES_EINPUT,
                        "surface_process_option %d runs on the host; the device step supports 0",
                        prm->surface_process_option);
    if (prm->damping_option < 0 || prm->damping_option > 4)
        return fail_msg(c->err, DES_EINPUT, "unknown damping_option: %d", prm->damping_option);
    c->kp.prm = *prm;
    set_rho_pseudo(c);
    invalidate_graph(c);
    return DES_OK;
}

int set_material(des_ctx *c, const des_material *m)
{
    MatC &t = c->kp.mat;
    const int rt = m->rheol_type;
    if (rt != DES_RH_ELASTIC && rt != DES_RH_VISCOUS && rt != DES_RH_MAXWELL && rt != DES_RH_EP &&
        rt != DES_RH_EVP)
        return fail_msg(c->err, DES_EINPUT, "unknown rheology type: %d", rt);
    if (m->nmat < 1 || m->nmat > DES_MAXMAT)
        return fail_msg(c->err, DES_EINPUT, "nmat = %d outside 1..%d", m->nmat, DES_MAXMAT);
    t.rheol_type = rt;
    t.nmat = m->nmat;
    t.is_plane_strain = m->is_plane_strain;
    t.scalar_mask = m->scalar_mask;
    t.visc_min = m->visc_min;
    t.visc_max = m->visc_max;
    t.tension_max = m->tension_max;
    t.therm_diff_max = m->therm_diff_max;
    const double *src[] = {m->rho0, m->alpha, m->bulk_modulus, m->shear_modulus, m->visc_exponent,
                           m->visc_coefficient, m->visc_activation_energy, m->heat_capacity, m->therm_cond,
                           m->radiogenic_heating, m->pls0, m->pls1, m->cohesion0, m->cohesion1,
                           m->friction_angle0, m->friction_angle1, m->dilation_angle0, m->dilation_angle1};
    double *dst[] = {t.rho0, t.alpha, t.bulk_modulus, t.shear_modulus, t.visc_exponent, t.visc_coefficient,
                     t.visc_activation_energy, t.heat_capacity, t.therm_cond, t.radiogenic_heating, t.pls0,
                     t.pls1, t.cohesion0, t.cohesion1, t.friction_angle0, t.friction_angle1,
                     t.dilation_angle0, t.dilation_angle1};
    for (int k = 0; k < 18; ++k) {
        if (!src[k]) return fail_msg(c->err, DES_EINPUT, "material array %d is NULL", k);
        for (int i = 0; i < m->nmat; ++i) dst[k][i] = src[k][i];
    }
    for (int i = 0; i < m->nmat; ++i) {
        t.visc_pw[i] = 1 / t.visc_exponent[i] - 1;   // IEEE division: same bits as per element
        t.visc_pw1[i] = -1 / t.visc_exponent[i];
        t.pt_phi[2 * i] = t.friction_angle0[i];
        t.pt_psi[2 * i] = t.dilation_angle0[i];
        t.pt_phi[2 * i + 1] = t.friction_angle1[i];
        t.pt_psi[2 * i + 1] = t.dilation_angle1[i];
    }
    t.pt_n = 0;   // enabled once the device has filled the table
    t.hr_over_cp = t.radiogenic_heating[0] / t.heat_capacity[0];
    return DES_OK;
}

void set_rho_pseudo(des_ctx *c)
{
    const double ps = c->kp.prm.max_vbc_val * c->kp.prm.inertial_scaling;
    c->kp.mat.rho_pseudo = c->kp.mat.bulk_modulus[0] / (ps * ps);
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Slabs of the pipelined host step: B element blocks of equal index ranges,
// node block b starting at the smallest node of element block b.  Usable
// when every element's nodes lie in its node block or the next, and every
// node's support elements in its element block or the previous one: then a
// node pass on block b reads element blocks b-1 and b, and an element pass
// on block b reads node blocks b and b+1.  Meshes numbered slab by slab (the
// structured box meshes: x is the slowest index of both numberings) qualify.
bool slab_partition(int B, const int *cn, int ne, int npe, int nn, const std::vector<int> &sup_off,
                    const std::vector<int> &sup_ent, std::vector<int> &eb, std::vector<int> &nb)
{
    if (B < 2 || ne < B) return false;
    eb.assign(B + 1, 0);
    nb.assign(B + 1, 0);
    for (int b = 0; b <= B; ++b) eb[b] = (int)((long long)ne * b / B);
    for (int b = 1; b < B; ++b) {
        int m = nn;
        for (int e = eb[b]; e < eb[b + 1]; ++e)
            for (int i = 0; i < npe; ++i) m = std::min(m, cn[(size_t)e * npe + i]);
        nb[b] = m;
    }
    nb[0] = 0;
    nb[B] = nn;
    for (int b = 0; b < B; ++b)
        if (nb[b + 1] <= nb[b]) return false;
    for (int b = 0; b < B; ++b) {
        const int hi = nb[std::min(b + 2, B)];
        for (int e = eb[b]; e < eb[b + 1]; ++e)
            for (int i = 0; i < npe; ++i) {
                const int n = cn[(size_t)e * npe + i];
                if (n < nb[b] || n >= hi) return false;
            }
        const int elo = eb[std::max(b - 1, 0)], ehi = eb[b + 1];
        for (int n = nb[b]; n < nb[b + 1]; ++n)
            for (int q = sup_off[n]; q < sup_off[n + 1]; ++q) {
                const int e = sup_ent[q] >> 2;
                if (e < elo || e >= ehi) return false;
            }
    }
    return true;
}

}  // namespace

extern "C" {

const char *des_version(void) { return "desgpu 0.2 (sm_103a; FP64 and mixed FP32/FP64 explicit step)"; }

int des_last_error(const des_ctx *c, char *buf, size_t len)
{
    if (!buf || len == 0) return DES_EINPUT;
    const std::string &s = c ? c->err : g_create_error;
    size_t n = std::min(len - 1, s.size());
    memcpy(buf, s.data(), n);
    buf[n] = 0;
    return DES_OK;
}

}  // extern "C"

namespace des {

// des_create with, optionally, the support lists already built (CSR offsets
// and entries element * 4 + local node, ascending element: des_remesh
// builds them on the device)
int create_context(const des_mesh *mesh, const des_params *param, const des_material *mat, int precision,
                   cudaStream_t stream, const std::vector<int> *pre_off, const std::vector<int> *pre_ent,
                   des_ctx **out)
{
    des_ctx *c = nullptr;
    if (!out) return fail_msg(g_create_error, DES_EINPUT, "out is NULL");
    *out = nullptr;
    if (!mesh || !param || !mat) return fail_msg(g_create_error, DES_EINPUT, "NULL mesh/param/material");
    if (mesh->ndims != 2 && mesh->ndims != 3)
        return fail_msg(g_create_error, DES_EINPUT, "ndims must be 2 or 3 (got %d)", mesh->ndims);
    if (mesh->nnode <= 0 || mesh->nelem <= 0)
        return fail_msg(g_create_error, DES_EINPUT, "empty mesh (nnode=%d, nelem=%d)", mesh->nnode, mesh->nelem);
    if ((long long)mesh->nelem * 4 >= (1ll << 31))
        return fail_msg(g_create_error, DES_EINPUT, "nelem=%d too large for int32 support entries", mesh->nelem);
    if (!mesh->connectivity || !mesh->bcflag || !mesh->bfacet_offsets)
        return fail_msg(g_create_error, DES_EINPUT, "NULL connectivity/bcflag/bfacet_offsets");
    if (precision != DES_PREC_FP64 && precision != DES_PREC_MIXED)
        return fail_msg(g_create_error, DES_EINPUT, "unknown precision %d", precision);

    c = new des_ctx();
    c->precision = precision;
    c->nd = mesh->ndims;
    c->npe = c->nd + 1;
    c->nstr = c->nd == 3 ? 6 : 3;
    c->nn = mesh->nnode;
    c->ne = mesh->nelem;
    const int nd = c->nd, npe = c->npe, nn = c->nn, ne = c->ne;
    int rc;
    if ((rc = set_params(c, param)) || (rc = set_material(c, mat))) {
        g_create_error = c->err;
        delete c;
        return rc;
    }

    // ---- topology products on the host ----
    const int *cn = mesh->connectivity;
    for (long long i = 0; i < (long long)ne * npe; ++i) {
        if (cn[i] < 0 || cn[i] >= nn) {
            int code = fail_msg(g_create_error, DES_EINPUT, "connectivity[%lld] = %d out of range [0,%d)", i,
                                cn[i], nn);
            delete c;
            return code;
        }
    }
    // support lists in ascending element order (create_support, mesh.cxx:1707-1721)
    std::vector<int> sup_off, sup_ent;
    if (pre_off && pre_ent && pre_off->size() == (size_t)nn + 1 && pre_ent->size() == (size_t)ne * npe) {
        sup_off = *pre_off;
        sup_ent = *pre_ent;
    } else {
        sup_off.assign(nn + 1, 0);
        sup_ent.resize((size_t)ne * npe);
        for (long long i = 0; i < (long long)ne * npe; ++i) sup_off[cn[i] + 1]++;
        for (int n = 0; n < nn; ++n) sup_off[n + 1] += sup_off[n];
        std::vector<int> fill(sup_off.begin(), sup_off.end() - 1);
        for (int e = 0; e < ne; ++e)
            for (int i = 0; i < npe; ++i) sup_ent[fill[cn[(size_t)e * npe + i]]++] = e * 4 + i;
    }
    // boundary facets and the node -> facet lists (ascending global facet id)
    const int nbf = mesh->bfacet_offsets[DES_NBDRYTYPES] - mesh->bfacet_offsets[0];
    c->nbf = nbf;
    std::vector<int> fac_elem(std::max(nbf, 1)), fac_f(std::max(nbf, 1)), fac_bdry(std::max(nbf, 1));
    std::vector<int> nf_off(nn + 1, 0), nf_ent;
    {
        static const int F3[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
        static const int F2[3][2] = {{1, 2}, {2, 0}, {0, 1}};
        int q = 0;
        for (int b = 0; b < DES_NBDRYTYPES; ++b) {
            for (int k = mesh->bfacet_offsets[b]; k < mesh->bfacet_offsets[b + 1]; ++k, ++q) {
                int e = mesh->bfacets[2 * k], f = mesh->bfacets[2 * k + 1];
                if (e < 0 || e >= ne || f < 0 || f > nd) {
                    int code = fail_msg(g_create_error, DES_EINPUT, "bad boundary facet (%d,%d)", e, f);
                    delete c;
                    return code;
                }
                fac_elem[q] = e;
                fac_f[q] = f;
                fac_bdry[q] = b;
                for (int j = 0; j < nd; ++j) nf_off[cn[(size_t)e * npe + (nd == 3 ? F3[f][j] : F2[f][j])] + 1]++;
            }
        }
        for (int n = 0; n < nn; ++n) nf_off[n + 1] += nf_off[n];
        nf_ent.resize(std::max(nf_off[nn], 1));
        std::vector<int> fill(nf_off.begin(), nf_off.end() - 1);
        for (int qq = 0; qq < nbf; ++qq) {
            int e = fac_elem[qq], f = fac_f[qq];
            for (int j = 0; j < nd; ++j) nf_ent[fill[cn[(size_t)e * npe + (nd == 3 ? F3[f][j] : F2[f][j])]]++] = qq;
        }
    }

    // fine slabs of the pipelined host step (the largest valid count) and the
    // boundary facets grouped by the fine slab of their element; 4 coarse
    // slabs of at least 4 fine slabs each (measured at 998,400 tets: 4 coarse
    // slabs 2.90 ms per call, 6: 2.92, 8: 3.02, 16: 4.00 -- each slab adds a
    // DMA copy per field and direction, ~2 us each)
    std::vector<int> fac_order;
    for (int F : {256, 192, 160, 128, 96, 80, 64, 48, 40, 32, 24, 20, 16}) {
        if (F * 4 > ne) continue;
        if (slab_partition(F, cn, ne, npe, nn, sup_off, sup_ent, c->slab_e, c->slab_n)) {
            c->nfine = F;
            break;
        }
    }
    if (c->nfine >= 16) c->nslab = 4;
    if (c->nslab > 1) {
        const int F = c->nfine;
        std::vector<int> blk(std::max(nbf, 1), 0);
        for (int q = 0; q < nbf; ++q)
            blk[q] = (int)(std::upper_bound(c->slab_e.begin(), c->slab_e.end(), fac_elem[q]) - c->slab_e.begin()) - 1;
        fac_order.resize(nbf);
        for (int q = 0; q < nbf; ++q) fac_order[q] = q;
        std::stable_sort(fac_order.begin(), fac_order.end(), [&](int a, int b) { return blk[a] < blk[b]; });
        c->slab_f.assign(F + 1, 0);
        for (int q = 0; q < nbf; ++q) c->slab_f[blk[q] + 1]++;
        for (int b = 0; b < F; ++b) c->slab_f[b + 1] += c->slab_f[b];
    }

    // ---- device ----
    if (cudaGetDevice(&c->device) != cudaSuccess) {
        int code = fail_msg(g_create_error, DES_ECUDA, "no CUDA device");
        delete c;
        return code;
    }
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            int code = fail_msg(g_create_error, DES_ECUDA, "cudaStreamCreate failed");
            delete c;
            return code;
        }
        c->own_stream = true;
    }

    // sizes (in bytes) of every array carved from the pool
    const size_t D = sizeof(double), I = sizeof(int);
    struct Slot { void **dst; size_t bytes; };
    KP &p = c->kp;
    std::vector<Slot> slots;
    auto add = [&](void **dst, size_t bytes) { slots.push_back({dst, align256(std::max<size_t>(bytes, 8))}); };
    int *d_conn, *d_sup_off, *d_sup_ent, *d_nf_off, *d_nf_ent, *d_fe, *d_ff, *d_fb, *d_emark = nullptr;
    double *d_eprop = nullptr;
    unsigned *d_bc;
    add((void **)&d_conn, (size_t)ne * npe * I);
    add((void **)&d_bc, (size_t)nn * sizeof(unsigned));
    add((void **)&d_sup_off, (size_t)(nn + 1) * I);
    add((void **)&d_sup_ent, (size_t)ne * npe * I);
    add((void **)&d_nf_off, (size_t)(nn + 1) * I);
    add((void **)&d_nf_ent, nf_ent.size() * I);
    add((void **)&d_fe, fac_elem.size() * I);
    add((void **)&d_ff, fac_f.size() * I);
    add((void **)&d_fb, fac_bdry.size() * I);
    if (c->nslab > 1) add((void **)&c->d_fac_order, std::max<size_t>(fac_order.size(), 1) * I);
    if (mat->elemmarkers && mat->nmat > 1) {
        add((void **)&d_emark, (size_t)ne * mat->nmat * I);
        add((void **)&d_eprop, (size_t)ne * EP_COUNT * D);
    }
    add((void **)&p.x, (size_t)nn * nd * D);
    add((void **)&p.x0, (size_t)nn * nd * D);
    add((void **)&p.v, (size_t)nn * nd * D);
    add((void **)&p.f, (size_t)nn * nd * D);
    add((void **)&p.T, (size_t)nn * D);
    add((void **)&p.mass, (size_t)nn * D);
    add((void **)&p.tmass, (size_t)nn * D);
    add((void **)&p.vol_n, (size_t)nn * D);
    add((void **)&p.ntmp, (size_t)nn * D);
    add((void **)&c->d_tdot, (size_t)nn * D);
    add((void **)&p.stress, (size_t)ne * c->nstr * D);
    add((void **)&p.strain, (size_t)ne * c->nstr * D);
    add((void **)&p.srate, (size_t)ne * c->nstr * D);
    add((void **)&p.pls, (size_t)ne * D);
    add((void **)&p.dpls, (size_t)ne * D);
    add((void **)&p.syy, (size_t)ne * D);
    add((void **)&p.dp, (size_t)ne * D);
    add((void **)&p.edvoldt, (size_t)ne * D);
    add((void **)&p.vol, (size_t)ne * D);
    add((void **)&p.vol_old, (size_t)ne * D);
    add((void **)&p.shp, (size_t)ne * npe * nd * D);
    // the mixed step's kernels are 3D; a plane-strain material runs the FP64 ones
    const bool mixed3 = (precision == DES_PREC_MIXED) && nd == 3 && !mat->is_plane_strain;
    float *d_hc = nullptr;
    float4 *d_ft = nullptr;
    float2 *d_shpdw = nullptr, *d_vdw = nullptr, *d_pv = nullptr;
    double4 *d_ndpk = nullptr;
    int *d_sup_pos = nullptr;
    double *d_qv = nullptr, *d_hc64 = nullptr;
    add((void **)&d_qv, (size_t)ne * D);
    if (mixed3) {
        add((void **)&d_hc, (size_t)ne * npe * sizeof(float));
        add((void **)&d_ft, (size_t)ne * npe * 2 * sizeof(float4));
        add((void **)&d_shpdw, (size_t)ne * npe * nd * sizeof(float2));
        add((void **)&d_vdw, (size_t)nn * nd * sizeof(float2));
        add((void **)&d_ndpk, (size_t)ne * sizeof(double4));
        add((void **)&d_pv, (size_t)ne * sizeof(float2));
        add((void **)&d_sup_pos, (size_t)ne * npe * I);
    } else {
        add((void **)&d_hc64, (size_t)ne * npe * D);
    }
    add((void **)&c->d_rho, (size_t)ne * D);
    add((void **)&c->d_buoy, (size_t)ne * D);
    add((void **)&p.me, (size_t)ne * D);
    add((void **)&p.tme, (size_t)ne * D);
    add((void **)&p.fv, (size_t)std::max(nbf, 1) * nd * D);
    add((void **)&p.clk, sizeof(Clock));
    add((void **)&p.err, sizeof(unsigned));
    add((void **)&c->d_red, 4 * sizeof(unsigned long long));
    c->stage_doubles = std::max((size_t)ne * std::max(c->nstr, npe), (size_t)nn * nd);
    add((void **)&c->d_stage, c->stage_doubles * D);
    size_t total = 0;
    for (auto &s : slots) total += s.bytes;
    cudaError_t ce = cudaMalloc((void **)&c->pool, total);
    if (ce != cudaSuccess) {
        (void)cudaGetLastError();   // the failed allocation is reported here, not at the next launch
        int code = fail_msg(g_create_error, DES_ENOMEM, "cudaMalloc(%zu bytes): %s", total, cudaGetErrorString(ce));
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return code;
    }
    c->pool_bytes = total;
    ce = cudaMemset(c->pool, 0, total);
    if (ce != cudaSuccess) {
        int code = fail_msg(g_create_error, DES_ECUDA, "cudaMemset: %s", cudaGetErrorString(ce));
        cudaFree(c->pool);
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return code;
    }
    {
        size_t off = 0;
        for (auto &s : slots) {
            *s.dst = c->pool + off;
            off += s.bytes;
        }
    }
    p.nd = nd;
    p.npe = npe;
    p.nstr = c->nstr;
    p.nn = nn;
    p.ne = ne;
    p.nbf = nbf;
    p.conn = d_conn;
    p.bcflag = d_bc;
    p.sup_off = d_sup_off;
    p.sup_ent = d_sup_ent;
    p.nf_off = d_nf_off;
    p.nf_ent = d_nf_ent;
    p.fac_elem = d_fe;
    p.fac_f = d_ff;
    p.fac_bdry = d_fb;
    p.emark = d_emark;
    p.eprop = nullptr;   // set once k_elem_props has filled d_eprop
    p.rho_e = nullptr;
    p.buoy_e = nullptr;
    p.tdot = p.ntmp;
    p.shpdw = d_shpdw;
    p.vdw = d_vdw;
    p.ndpk = d_ndpk;
    p.pv = d_pv;
    p.hc = d_hc;
    p.qv = d_qv;
    p.hc64 = d_hc64;
    p.ft = d_ft;
    p.sup_pos = d_sup_pos;
    p.e_lo = 0, p.e_hi = ne, p.n_lo = 0, p.n_hi = nn, p.f_lo = 0, p.f_hi = nbf;
    p.fac_order = nullptr;
    p.tape_visc = nullptr;
    p.tape_evp = nullptr;
    for (int i = 0; i < DES_NBDRYTYPES; ++i)
        for (int d = 0; d < 3; ++d) {
            p.bnormals[i][d] = mesh->bnormals[i][d];
            for (int j = 0; j < DES_NBDRYTYPES; ++j) p.edge_vectors[i][j][d] = mesh->edge_vectors[i][j][d];
        }

    // uploads (synchronous: creation time only)
    std::vector<int> conn_soa((size_t)ne * npe);
    for (int e = 0; e < ne; ++e)
        for (int i = 0; i < npe; ++i) conn_soa[(size_t)i * ne + e] = cn[(size_t)e * npe + i];
    cudaError_t e1 = cudaSuccess;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        if (e1 == cudaSuccess && bytes) e1 = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up(d_conn, conn_soa.data(), conn_soa.size() * I);
    up(d_bc, mesh->bcflag, (size_t)nn * sizeof(unsigned));
    up(d_sup_off, sup_off.data(), sup_off.size() * I);
    up(d_sup_ent, sup_ent.data(), sup_ent.size() * I);
    if (d_sup_pos) {   // the support-list entry of each (element, slot), slot-major
        std::vector<int> pos((size_t)ne * npe);
        for (size_t q = 0; q < sup_ent.size(); ++q) pos[(size_t)(sup_ent[q] & 3) * ne + (sup_ent[q] >> 2)] = (int)q;
        up(d_sup_pos, pos.data(), pos.size() * I);
    }
    up(d_nf_off, nf_off.data(), nf_off.size() * I);
    up(d_nf_ent, nf_ent.data(), nf_ent.size() * I);
    up(d_fe, fac_elem.data(), fac_elem.size() * I);
    up(d_ff, fac_f.data(), fac_f.size() * I);
    up(d_fb, fac_bdry.data(), fac_bdry.size() * I);
    if (c->d_fac_order && !fac_order.empty()) up(c->d_fac_order, fac_order.data(), fac_order.size() * I);
    if (d_emark) {
        std::vector<int> em((size_t)ne * mat->nmat);
        for (int e = 0; e < ne; ++e)
            for (int m = 0; m < mat->nmat; ++m) em[(size_t)m * ne + e] = mat->elemmarkers[(size_t)e * mat->nmat + m];
        up(d_emark, em.data(), em.size() * I);
        if (e1 == cudaSuccess) {
            launch_elem_props(p, c->stream, d_eprop);
            e1 = cudaGetLastError();
            if (e1 == cudaSuccess) e1 = cudaStreamSynchronize(c->stream);
            p.eprop = d_eprop;
        }
    }
    if (e1 == cudaSuccess) {
        Clock ck{};
        ck.red_minh = ck.red_maxwell = ck.red_diffusion = ~0ull;
        e1 = cudaMemcpy(p.clk, &ck, sizeof ck, cudaMemcpyHostToDevice);
    }
    if (e1 == cudaSuccess) {
        // material constants computed by the device's own functions
        set_rho_pseudo(c);
        const int nm = p.mat.nmat;
        std::vector<double> tab(nm + 8 * nm);
        launch_material_table(p, c->stream, c->d_stage);
        e1 = cudaMemcpyAsync(tab.data(), c->d_stage, tab.size() * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream);
        if (e1 == cudaSuccess) e1 = cudaStreamSynchronize(c->stream);
        if (e1 == cudaSuccess) {
            for (int m = 0; m < nm; ++m) p.mat.visc_coef[m] = tab[m];
            p.mat.visc_skip_empty = 1;
            for (int m = 0; m < nm; ++m) {
                p.mat.visc_lnc[m] = std::log(0.25e6 * tab[m]);
                p.mat.visc_qnr[m] = p.mat.visc_activation_energy[m] / (p.mat.visc_exponent[m] * 8.3144);
                if (!(tab[m] > 0 && std::isfinite(tab[m]) && p.mat.visc_activation_energy[m] >= 0
                      && p.mat.visc_exponent[m] > 0))
                    p.mat.visc_skip_empty = 0;
            }
            p.mat.visc_lnmin = std::log(p.mat.visc_min);
            p.mat.visc_lnmax = std::log(p.mat.visc_max);
            for (int k = 0; k < 2 * nm; ++k) {
                p.mat.pt_anphi[k] = tab[nm + 4 * k + 0];
                p.mat.pt_anpsi[k] = tab[nm + 4 * k + 1];
                p.mat.pt_sqrt_anphi[k] = tab[nm + 4 * k + 2];
                p.mat.pt_tanphi[k] = tab[nm + 4 * k + 3];
            }
            for (int m = 0; m < nm; ++m) {
                // IEEE division: the same bits the per-element code computes
                p.mat.pt_coh_over_tan[2 * m] = p.mat.cohesion0[m] / p.mat.pt_tanphi[2 * m];
                p.mat.pt_coh_over_tan[2 * m + 1] = p.mat.cohesion1[m] / p.mat.pt_tanphi[2 * m + 1];
                p.mat.hardening[m] = (p.mat.cohesion1[m] - p.mat.cohesion0[m]) / (p.mat.pls1[m] - p.mat.pls0[m]);
            }
            p.mat.pt_n = 2 * nm;
        }
    }
    if (e1 != cudaSuccess) {
        int code = fail_msg(g_create_error, DES_ECUDA, "device setup: %s", cudaGetErrorString(e1));
        cudaFree(c->pool);
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return code;
    }
    *out = c;
    return DES_OK;
}

}  // namespace des

extern "C" {

int des_create(const des_mesh *mesh, const des_params *param, const des_material *mat, int precision,
               void *stream, des_ctx **out)
{
    return create_context(mesh, param, mat, precision, static_cast<cudaStream_t>(stream), nullptr, nullptr, out);
}

}  // extern "C"

namespace des {

// every device resource of c except its stream; c itself is not deleted
void release_context(des_ctx *c)
{
    cudaStreamSynchronize(c->stream);
    invalidate_graph(c);
    adj_free(c);
    markers_free(c);
    if (c->ystream) {
        cudaStreamSynchronize(c->ystream);
        cudaStreamDestroy(c->ystream);
        for (cudaEvent_t e : c->pipe_ev) cudaEventDestroy(e);
        cudaFree(c->d_pipe_sink);
    }
    if (c->xstream) {
        cudaStreamSynchronize(c->xstream);
        cudaStreamDestroy(c->xstream);
        for (cudaEvent_t e : c->xev) cudaEventDestroy(e);
        cudaEventDestroy(c->ev_mid);
        cudaFree(c->d_xstage);
    }
    for (int k = 0; k < DES_EF_COUNT; ++k)
        if (c->d_ef[k]) cudaFree(c->d_ef[k]);
    cudaFree(c->pool);
    c->pool = nullptr;
}

}  // namespace des

extern "C" {

int des_destroy(des_ctx *c)
{
    if (!c) return DES_OK;
    release_context(c);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return DES_OK;
}

int des_device_status(des_ctx *c, unsigned *bits)
{
    if (!c || !bits) return DES_EINPUT;
    unsigned h = 0;
    CK(cudaMemcpyAsync(&h, c->kp.err, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->kp.err, 0, sizeof(unsigned), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *bits = h & 0xffu;
    if (h & 0x100u) {
        fail_msg(c->err, DES_ERUNTIME, "Error: dt <= 0!");
        return DES_ERUNTIME;
    }
    return DES_OK;
}

int des_set_params(des_ctx *c, const des_params *prm)
{
    if (!c || !prm) return DES_EINPUT;
    return set_params(c, prm);
}

int des_set_elem_field(des_ctx *c, int field, const double *values)
{
    if (!c || field < 0 || field >= DES_EF_COUNT) return DES_EINPUT;
    invalidate_graph(c);
    if (!values) {
        if (c->d_ef[field]) {
            CK(cudaStreamSynchronize(c->stream));
            cudaFree(c->d_ef[field]);
        }
        c->d_ef[field] = nullptr;
        c->kp.ef[field] = nullptr;
        return DES_OK;
    }
    if (!c->d_ef[field]) CK(cudaMalloc((void **)&c->d_ef[field], (size_t)c->ne * sizeof(double)));
    CK(cudaMemcpyAsync(c->d_ef[field], values, (size_t)c->ne * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->kp.ef[field] = c->d_ef[field];
    return DES_OK;
}

// ---- state transfer ----
namespace {

int put_field(des_ctx *c, const double *host, double *dev, int n, int ncomp)
{
    size_t bytes = (size_t)n * ncomp * sizeof(double);
    if (ncomp == 1) {
        CK(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, c->stream));
        return DES_OK;
    }
    CK(cudaMemcpyAsync(c->d_stage, host, bytes, cudaMemcpyHostToDevice, c->stream));
    return check_launch(c, launch_aos_to_soa(c->d_stage, dev, n, ncomp, c->stream));
}

int get_field(des_ctx *c, double *host, const double *dev, int n, int ncomp)
{
    size_t bytes = (size_t)n * ncomp * sizeof(double);
    if (ncomp == 1) {
        CK(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
        return DES_OK;
    }
    int rc = check_launch(c, launch_soa_to_aos(dev, c->d_stage, n, ncomp, c->stream));
    if (rc) return rc;
    // stream order keeps the staging buffer's next writer behind this copy
    CK(cudaMemcpyAsync(host, c->d_stage, bytes, cudaMemcpyDeviceToHost, c->stream));
    return DES_OK;
}

// Pipelined state transfer.  The host rows of every field move by DMA on the
// copy stream, back to back; a multi-component field lands in its own region
// of the staging area and is converted between the reference's AoS rows and
// the device SoA arrays on the compute stream while the next field's copy
// runs.  Events order each conversion against its copy.  The host link is
// then busy for the whole transfer (one DMA and one conversion per field,
// serialised on one stream, left it idle during every conversion).
int ensure_xfer(des_ctx *c)
{
    if (c->xstream) return DES_OK;
    if (!c->d_xstage) {
        const size_t need = (size_t)4 * c->nn * c->nd + (size_t)3 * c->ne * c->nstr + (size_t)c->nd * c->ne * c->npe;
        CK(cudaMalloc((void **)&c->d_xstage, need * sizeof(double)));
        c->xstage_doubles = need;
    }
    for (cudaEvent_t &e : c->xev)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!c->ev_mid) CK(cudaEventCreateWithFlags(&c->ev_mid, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&c->xstream, cudaStreamNonBlocking));
    return DES_OK;
}

// One direction of a pipelined transfer: begin(), field() per field, end().
struct Pipe {
    des_ctx *c;
    bool up;
    size_t off = 0;   // staging doubles handed out
    int nev = 2;      // xev[0]: start, xev[1]: done, then one per converted field

    // The copies start after what the compute stream has queued so far
    // (or after `after`, an event of it).
    int begin(cudaEvent_t after = nullptr)
    {
        if (!after) {
            CK(cudaEventRecord(c->xev[0], c->stream));
            after = c->xev[0];
        }
        CK(cudaStreamWaitEvent(c->xstream, after, 0));
        return DES_OK;
    }
    // on_copy_stream: a download whose conversion runs on the copy stream
    // (the compute stream is still busy with kernels that do not write `dev`)
    int field(double *host, double *dev, int n, int ncomp, bool on_copy_stream = false)
    {
        const size_t cnt = (size_t)n * ncomp, bytes = cnt * sizeof(double);
        if (cnt == 0) return DES_OK;
        if (ncomp == 1) {
            if (up) CK(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, c->xstream));
            else CK(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->xstream));
            return DES_OK;
        }
        if (off + cnt > c->xstage_doubles || nev >= DES_XFER_EVENTS)
            return fail_msg(c->err, DES_EINPUT, "state transfer: a field was given twice");
        double *stg = c->d_xstage + off;
        off += cnt;
        cudaEvent_t ev = c->xev[nev++];
        int rc;
        if (up) {
            CK(cudaMemcpyAsync(stg, host, bytes, cudaMemcpyHostToDevice, c->xstream));
            CK(cudaEventRecord(ev, c->xstream));
            CK(cudaStreamWaitEvent(c->stream, ev, 0));
            return check_launch(c, launch_aos_to_soa(stg, dev, n, ncomp, c->stream));
        }
        if (on_copy_stream) {
            if ((rc = check_launch(c, launch_soa_to_aos(dev, stg, n, ncomp, c->xstream)))) return rc;
        } else {
            if ((rc = check_launch(c, launch_soa_to_aos(dev, stg, n, ncomp, c->stream)))) return rc;
            CK(cudaEventRecord(ev, c->stream));
            CK(cudaStreamWaitEvent(c->xstream, ev, 0));
        }
        CK(cudaMemcpyAsync(host, stg, bytes, cudaMemcpyDeviceToHost, c->xstream));
        return DES_OK;
    }
    // the compute stream's later work waits for every copy
    int end()
    {
        CK(cudaEventRecord(c->xev[1], c->xstream));
        CK(cudaStreamWaitEvent(c->stream, c->xev[1], 0));
        return DES_OK;
    }
};

// A state field: host rows, device array, rows, values per row, and whether
// the step is done writing it once nmd_correct is (see enqueue_step).
struct StateField {
    double *host;
    double *dev;
    int n, ncomp;
    bool early;
};

int state_fields(des_ctx *c, const des_host_state *st, StateField *out)
{
    KP &p = c->kp;
    const int nn = c->nn, ne = c->ne, nd = c->nd, npe = c->npe, nstr = c->nstr;
    const size_t shp1 = (size_t)ne * npe;
    const StateField all[] = {
        {st->coord, p.x, nn, nd, false},
        {st->coord0, p.x0, nn, nd, true},
        {st->vel, p.v, nn, nd, false},
        {st->force, p.f, nn, nd, false},
        {st->temperature, p.T, nn, 1, true},
        {st->mass, p.mass, nn, 1, false},
        {st->tmass, p.tmass, nn, 1, false},
        {st->volume_n, p.vol_n, nn, 1, false},
        {st->ntmp, p.ntmp, nn, 1, true},
        {st->volume, p.vol, ne, 1, false},
        {st->volume_old, p.vol_old, ne, 1, false},
        {st->stress, p.stress, ne, nstr, false},
        {st->strain, p.strain, ne, nstr, false},
        {st->strain_rate, p.srate, ne, nstr, true},
        {st->plstrain, p.pls, ne, 1, true},
        {st->delta_plstrain, p.dpls, ne, 1, true},
        {st->stressyy, p.syy, ne, 1, true},
        {st->dpressure, p.dp, ne, 1, true},
        {st->edvoldt, p.edvoldt, ne, 1, true},
        {st->shpdx, p.shp, ne, npe, false},
        {nd == 3 ? st->shpdy : nullptr, p.shp + shp1, ne, npe, false},
        {st->shpdz, p.shp + (size_t)(nd - 1) * shp1, ne, npe, false},
    };
    int k = 0;
    for (const StateField &f : all)
        if (f.host) out[k++] = f;
    return k;
}

constexpr int MAX_STATE_FIELDS = 22;

// download of every non-NULL field; with `early`, the fields the step's tail
// does not write are copied once the step records ev_mid (the step must have
// been launched from step_exec_mid), while the tail kernels still run.  With
// `after_step`, coord0 and (outside plane strain) stressyy are skipped: no
// step writes them, so the host arrays they were uploaded from hold them.
int download_state(des_ctx *c, des_host_state *st, bool early, bool after_step = false)
{
    int rc;
    if ((rc = ensure_xfer(c))) return rc;
    des_host_state out = *st;
    if (after_step) {
        out.coord0 = nullptr;
        if (!c->kp.mat.is_plane_strain) out.stressyy = nullptr;
    }
    StateField f[MAX_STATE_FIELDS];
    const int nf = state_fields(c, &out, f);
    Pipe pp{c, false};
    if (early) {
        if ((rc = pp.begin(c->ev_mid))) return rc;
        for (int k = 0; k < nf; ++k)
            if (f[k].early && (rc = pp.field(f[k].host, f[k].dev, f[k].n, f[k].ncomp, true))) return rc;
    }
    // a mixed context keeps its shape functions as double-word pairs
    if ((out.shpdx || out.shpdy || out.shpdz) && (rc = check_launch(c, launch_shp_join(c->kp, c->stream))))
        return rc;
    if ((rc = pp.begin())) return rc;
    for (int k = 0; k < nf; ++k)
        if (!(early && f[k].early) && (rc = pp.field(f[k].host, f[k].dev, f[k].n, f[k].ncomp))) return rc;
    if ((rc = pp.end())) return rc;
    Clock ck;
    CK(cudaMemcpyAsync(&ck, c->kp.clk, sizeof ck, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    st->time = ck.time;
    st->dt = ck.dt;
    st->steps = ck.steps;
    return DES_OK;
}

}  // namespace

int des_upload_state(des_ctx *c, const des_host_state *st)
{
    if (!c || !st) return DES_EINPUT;
    if (!st->coord || !st->vel || !st->temperature || !st->volume_old || !st->stress || !st->strain ||
        !st->plstrain)
        return fail_msg(c->err, DES_EINPUT, "upload: coord, vel, temperature, volume_old, stress, strain and "
                        "plstrain are required");
    KP &p = c->kp;
    const int nn = c->nn, ne = c->ne, nd = c->nd, nstr = c->nstr;
    int rc;
    if ((rc = ensure_xfer(c))) return rc;
    // derived fields are taken from the host only when given as a set
    des_host_state in = *st;
    const bool have_shp = st->shpdx && st->shpdz && (nd == 2 || st->shpdy);
    const bool have_mass = st->mass && st->tmass && st->volume_n;
    if (!have_shp || p.shpdw) in.shpdx = in.shpdy = in.shpdz = nullptr;
    if (!have_mass) in.mass = in.tmass = in.volume_n = nullptr;
    StateField f[MAX_STATE_FIELDS];
    const int nf = state_fields(c, &in, f);
    Pipe pp{c, true};
    if ((rc = pp.begin())) return rc;
    for (int k = 0; k < nf; ++k)
        if ((rc = pp.field(f[k].host, f[k].dev, f[k].n, f[k].ncomp))) return rc;
#define ZERO(d, bytes) CK(cudaMemsetAsync((d), 0, (bytes), c->stream))
    if (!st->force) ZERO(p.f, (size_t)nn * nd * sizeof(double));
    if (!st->strain_rate) ZERO(p.srate, (size_t)ne * nstr * sizeof(double));
    if (!st->delta_plstrain) ZERO(p.dpls, (size_t)ne * sizeof(double));
    if (!st->stressyy) ZERO(p.syy, (size_t)ne * sizeof(double));
    if (!st->dpressure) ZERO(p.dp, (size_t)ne * sizeof(double));
    if (!st->edvoldt) ZERO(p.edvoldt, (size_t)ne * sizeof(double));
    if (!st->ntmp) ZERO(p.ntmp, (size_t)nn * sizeof(double));
#undef ZERO
    if ((rc = pp.end())) return rc;
    // what follows reads the uploaded fields
    if (!st->coord0)
        CK(cudaMemcpyAsync(p.x0, p.x, (size_t)nn * nd * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    {
        Clock ck{};
        ck.time = st->time;
        ck.dt = st->dt;
        ck.steps = st->steps;
        ck.red_minh = ck.red_maxwell = ck.red_diffusion = ~0ull;
        CK(cudaMemcpyAsync(p.clk, &ck, sizeof ck, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));   // ck lives on this stack frame
    }
    KP q = p;   // per-function form
    if (!st->volume && (rc = check_launch(c, launch_geometry(q, c->stream, GEO_VOLUME)))) return rc;
    // a mixed 3D context forms its double-word shape functions from the
    // coordinates: FP64 values do not split into pairs exactly, and so do not
    // carry its own pairs through a download and an upload
    if (!have_shp || p.shpdw) {
        if ((rc = check_launch(c, launch_geometry(q, c->stream, GEO_SHAPE)))) return rc;
    }
    if (!have_mass && (rc = check_launch(c, launch_mass(q, c->stream)))) return rc;
    CK(cudaStreamSynchronize(c->stream));
    c->has_state = true;
    return DES_OK;
}

int des_download_state(des_ctx *c, des_host_state *st)
{
    if (!c || !st) return DES_EINPUT;
    return download_state(c, st, false);
}

namespace {

struct FieldDesc {
    unsigned bit;
    double *des_host_state::*member;
    int node;    // 1: node field, 0: element field
    int ncomp;   // 0: nd, -1: nstr, -2: npe (shape functions), else the count
};

const FieldDesc kFields[] = {
    {DES_F_COORD, &des_host_state::coord, 1, 0},
    {DES_F_COORD0, &des_host_state::coord0, 1, 0},
    {DES_F_VEL, &des_host_state::vel, 1, 0},
    {DES_F_FORCE, &des_host_state::force, 1, 0},
    {DES_F_TEMPERATURE, &des_host_state::temperature, 1, 1},
    {DES_F_MASS, &des_host_state::mass, 1, 1},
    {DES_F_TMASS, &des_host_state::tmass, 1, 1},
    {DES_F_VOLUME_N, &des_host_state::volume_n, 1, 1},
    {DES_F_NTMP, &des_host_state::ntmp, 1, 1},
    {DES_F_VOLUME, &des_host_state::volume, 0, 1},
    {DES_F_VOLUME_OLD, &des_host_state::volume_old, 0, 1},
    {DES_F_STRESS, &des_host_state::stress, 0, -1},
    {DES_F_STRAIN, &des_host_state::strain, 0, -1},
    {DES_F_STRAIN_RATE, &des_host_state::strain_rate, 0, -1},
    {DES_F_PLSTRAIN, &des_host_state::plstrain, 0, 1},
    {DES_F_DELTA_PLSTRAIN, &des_host_state::delta_plstrain, 0, 1},
    {DES_F_STRESSYY, &des_host_state::stressyy, 0, 1},
    {DES_F_DPRESSURE, &des_host_state::dpressure, 0, 1},
    {DES_F_EDVOLDT, &des_host_state::edvoldt, 0, 1},
};

double *device_field(des_ctx *c, unsigned bit)
{
    KP &p = c->kp;
    switch (bit) {
    case DES_F_COORD: return p.x;
    case DES_F_COORD0: return p.x0;
    case DES_F_VEL: return p.v;
    case DES_F_FORCE: return p.f;
    case DES_F_TEMPERATURE: return p.T;
    case DES_F_MASS: return p.mass;
    case DES_F_TMASS: return p.tmass;
    case DES_F_VOLUME_N: return p.vol_n;
    case DES_F_NTMP: return p.ntmp;
    case DES_F_VOLUME: return p.vol;
    case DES_F_VOLUME_OLD: return p.vol_old;
    case DES_F_STRESS: return p.stress;
    case DES_F_STRAIN: return p.strain;
    case DES_F_STRAIN_RATE: return p.srate;
    case DES_F_PLSTRAIN: return p.pls;
    case DES_F_DELTA_PLSTRAIN: return p.dpls;
    case DES_F_STRESSYY: return p.syy;
    case DES_F_DPRESSURE: return p.dp;
    case DES_F_EDVOLDT: return p.edvoldt;
    default: return nullptr;
    }
}

int transfer_fields(des_ctx *c, des_host_state *st, unsigned mask, bool up)
{
    if (!c || !st) return DES_EINPUT;
    if (mask & ~DES_F_ALL) return fail_msg(c->err, DES_EINPUT, "unknown field bits %#x", mask & ~DES_F_ALL);
    int rc;
    if ((rc = ensure_xfer(c))) return rc;
    Pipe pp{c, up};
    // a mixed context keeps its shape functions as double-word pairs
    if ((mask & DES_F_SHP) && !up && (rc = check_launch(c, launch_shp_join(c->kp, c->stream)))) return rc;
    if ((rc = pp.begin())) return rc;
    for (const FieldDesc &fd : kFields) {
        if (!(mask & fd.bit)) continue;
        double *h = st->*fd.member;
        if (!h) return fail_msg(c->err, DES_EINPUT, "field %#x selected but NULL", fd.bit);
        const int n = fd.node ? c->nn : c->ne;
        const int k = fd.ncomp == 0 ? c->nd : (fd.ncomp == -1 ? c->nstr : fd.ncomp);
        if ((rc = pp.field(h, device_field(c, fd.bit), n, k))) return rc;
    }
    if (mask & DES_F_SHP) {
        double *arr[3] = {st->shpdx, c->nd == 3 ? st->shpdy : nullptr, st->shpdz};
        int slot = 0;
        for (int a = 0; a < 3; ++a) {
            if (a == 1 && c->nd == 2) continue;
            if (!arr[a]) return fail_msg(c->err, DES_EINPUT, "shape function array NULL");
            double *d = c->kp.shp + (size_t)slot * c->ne * c->npe;
            if ((rc = pp.field(arr[a], d, c->ne, c->npe))) return rc;
            ++slot;
        }
    }
    if ((rc = pp.end())) return rc;
    if ((mask & DES_F_SHP) && up && c->kp.shpdw) {   // a mixed 3D context forms them from its coordinates
        rc = check_launch(c, launch_geometry(c->kp, c->stream, GEO_SHAPE));
        if (rc) return rc;
    }
    if (mask & DES_F_CLOCK) {
        Clock ck;
        CK(cudaMemcpyAsync(&ck, c->kp.clk, sizeof ck, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (up) {
            ck.time = st->time;
            ck.dt = st->dt;
            ck.steps = st->steps;
            CK(cudaMemcpyAsync(c->kp.clk, &ck, sizeof ck, cudaMemcpyHostToDevice, c->stream));
        } else {
            st->time = ck.time;
            st->dt = ck.dt;
            st->steps = ck.steps;
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return DES_OK;
}

}  // namespace

int des_upload_fields(des_ctx *c, const des_host_state *st, unsigned mask)
{
    int rc = transfer_fields(c, const_cast<des_host_state *>(st), mask, true);
    if (rc == DES_OK) c->has_state = true;
    return rc;
}

int des_download_fields(des_ctx *c, des_host_state *st, unsigned mask)
{
    return transfer_fields(c, st, mask, false);
}

int des_set_elemmarkers(des_ctx *c, const int *em)
{
    if (!c || !em) return DES_EINPUT;
    if (!c->kp.emark) return fail_msg(c->err, DES_EINPUT, "context was created without per-element markers");
    const int nm = c->kp.mat.nmat, ne = c->ne;
    std::vector<int> soa((size_t)ne * nm);
    for (int e = 0; e < ne; ++e)
        for (int m = 0; m < nm; ++m) soa[(size_t)m * ne + e] = em[(size_t)e * nm + m];
    CK(cudaMemcpyAsync(const_cast<int *>(c->kp.emark), soa.data(), soa.size() * sizeof(int),
                       cudaMemcpyHostToDevice, c->stream));
    if (c->kp.eprop) {
        int rc = check_launch(c, launch_elem_props(c->kp, c->stream, const_cast<double *>(c->kp.eprop)));
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    return DES_OK;
}

int des_get_clock(des_ctx *c, double *time, double *dt, int *steps)
{
    if (!c) return DES_EINPUT;
    Clock ck;
    CK(cudaMemcpyAsync(&ck, c->kp.clk, sizeof ck, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (time) *time = ck.time;
    if (dt) *dt = ck.dt;
    if (steps) *steps = ck.steps;
    return DES_OK;
}

int des_set_clock(des_ctx *c, double time, double dt, int steps)
{
    if (!c) return DES_EINPUT;
    Clock ck;
    CK(cudaMemcpyAsync(&ck, c->kp.clk, sizeof ck, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    ck.time = time;
    ck.dt = dt;
    ck.steps = steps;
    CK(cudaMemcpyAsync(c->kp.clk, &ck, sizeof ck, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DES_OK;
}

// ---- per-function entry points ----
#define PERFN(name, body)                     \
    int name(des_ctx *c)                      \
    {                                         \
        if (!c) return DES_EINPUT;            \
        const KP &p = c->kp;                  \
        cudaStream_t s = c->stream;           \
        int n = 0;                            \
        body;                                 \
        return check_launch(c, n);            \
    }

PERFN(des_update_temperature,
      n += (p.shpdw ? launch_heat_and_dvoldt_mixed(p, s, true, false) : launch_heat_gather(p, s));
      n += launch_temperature_update(p, s))
PERFN(des_update_strain_rate,
      n += (p.shpdw ? launch_strain_rate_mixed(p, s, false) : launch_strain_rate(p, s, false)))
PERFN(des_compute_dvoldt, n += launch_dvoldt(p, s))
PERFN(des_compute_edvoldt, n += launch_edvoldt(p, s))
PERFN(des_update_stress,
      n += (p.shpdw ? launch_update_stress_mixed(p, s, false)
                                                 : launch_update_stress(p, s, false)))
PERFN(des_NMD_stress, n += launch_nmd_gather(p, s); n += launch_nmd_correct(p, s, false))
// in a mixed context, the fused-multiply-add forms of the mixed step
PERFN(des_update_force,
      n += launch_facet_forces(p, s); n += launch_force_terms(p, s);
      n += launch_force(p, s, false, p.shpdw != nullptr))
PERFN(des_update_velocity, n += launch_velocity(p, s, p.shpdw != nullptr))
PERFN(des_apply_vbcs, n += launch_vbcs(p, s))
PERFN(des_update_coordinate, n += launch_coordinate(p, s, p.shpdw != nullptr))
PERFN(des_swap_volume, n += launch_geometry(p, s, GEO_COPY_OLD))
PERFN(des_compute_volume, n += launch_geometry(p, s, GEO_VOLUME))
PERFN(des_compute_mass, n += launch_mass(p, s))
PERFN(des_compute_shape_fn, n += launch_geometry(p, s, GEO_SHAPE))
PERFN(des_rotate_stress, n += launch_geometry(p, s, GEO_ROTATE))
PERFN(des_update_mesh, n += launch_coordinate(p, s, p.shpdw != nullptr);
      n += launch_geometry(p, s, GEO_COPY_OLD | GEO_VOLUME); n += launch_mass(p, s);
      n += launch_geometry(p, s, GEO_SHAPE))

int des_compute_dt(des_ctx *c, double *dt_out)
{
    if (!c) return DES_EINPUT;
    int rc = check_launch(c, launch_geometry(c->kp, c->stream, GEO_DT) + launch_dt_finalize(c->kp, c->stream, false));
    if (rc) return rc;
    double dt;
    rc = des_get_clock(c, nullptr, &dt, nullptr);
    if (rc) return rc;
    if (dt_out) *dt_out = dt;
    unsigned bits;
    return des_device_status(c, &bits);
}

int des_worst_elem_quality(des_ctx *c, double *quality, int *elem)
{
    if (!c) return DES_EINPUT;
    unsigned long long init[2] = {~0ull, ~0ull}, res[2];
    CK(cudaMemcpyAsync(c->d_red, init, sizeof init, cudaMemcpyHostToDevice, c->stream));
    int rc = check_launch(c, launch_quality(c->kp, c->stream, c->d_red));
    if (rc) return rc;
    CK(cudaMemcpyAsync(res, c->d_red, sizeof res, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double q;
    memcpy(&q, &res[0], sizeof q);
    int w = (int)res[1];
    if (!(q < 1)) {   // worst_elem_quality starts from q = 1, worst = 0
        q = 1;
        w = 0;
    }
    if (quality) *quality = q;
    if (elem) *elem = w;
    return DES_OK;
}

int des_bad_mesh_quality(des_ctx *c, const des_quality_params *qp, int *code, int *index, double *value)
{
    if (!c || !qp || !code || !index) return DES_EINPUT;
    const int nd = c->kp.nd;
    // the volume of the equilateral triangle / tetrahedron of unit side
    // (remeshing.cxx:76-82), and the thresholds as the reference forms them
    const double sizefactor = nd == 3 ? 0.118 : 0.433;
    const double smallest_vol = qp->smallest_size * sizefactor * std::pow(qp->resolution, nd);
    const double bottom = -c->kp.prm.zlength;
    const double dist = qp->max_boundary_distortion * qp->resolution;
    const int opt = qp->remeshing_option;
    const int check_bottom = (opt == 1 || opt == 2 || opt == 11);
    unsigned long long init[4] = {~0ull, ~0ull, ~0ull, ~0ull}, res[4];
    CK(cudaMemcpyAsync(c->d_red, init, sizeof init, cudaMemcpyHostToDevice, c->stream));
    int rc = check_launch(c, launch_quality_scans(c->kp, c->stream, smallest_vol, bottom, dist, check_bottom,
                                                  c->d_red) +
                                 launch_quality(c->kp, c->stream, c->d_red));
    if (rc) return rc;
    CK(cudaMemcpyAsync(res, c->d_red, sizeof res, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (res[2] != ~0ull) {
        *code = 3;
        *index = (int)res[2];
        if (value) CK(cudaMemcpy(value, c->kp.vol + res[2], sizeof(double), cudaMemcpyDeviceToHost));
        return DES_OK;
    }
    if (check_bottom && res[3] != ~0ull) {
        *code = 2;
        *index = (int)res[3];
        if (value)
            CK(cudaMemcpy(value, c->kp.x + (size_t)(nd - 1) * c->kp.nn + res[3], sizeof(double),
                          cudaMemcpyDeviceToHost));
        return DES_OK;
    }
    double q;
    memcpy(&q, &res[0], sizeof q);
    int w = (int)res[1];
    if (!(q < 1)) {   // worst_elem_quality starts from q = 1, worst = 0
        q = 1;
        w = 0;
    }
    if (nd == 3) q = std::pow(q, 1.0 / 3);   // remeshing.cxx:1924-1927
    if (q < qp->min_quality) {
        *code = 1;
        *index = w;
        if (value) *value = q;
        return DES_OK;
    }
    *code = 0;
    return DES_OK;
}

// ---- the fused step ----
namespace {

bool use_mixed(const des_ctx *c) { return c->kp.shpdw != nullptr; }

// `mid` (optional) is recorded once nmd_correct is done: the kernels after it
// (force and motion, geometry and rotation, mass sums, dt) write only x, v, f,
// vol_old, vol, the shape functions, stress, strain, mass, tmass, volume_n
// and the clock, so every other state field is final at that point.
int record_mid(cudaEvent_t mid, cudaStream_t s)
{
    return mid ? (cudaEventRecordWithFlags(mid, s, cudaEventRecordExternal) == cudaSuccess ? 0 : -1) : 0;
}

int enqueue_step_mixed(des_ctx *c, cudaEvent_t mid)
{
    const KP p = step_kp(c);
    cudaStream_t s = c->stream;
    int n = 0;
    const bool thermal = p.prm.has_thermal_diffusion != 0;
    n += launch_elem_pass_mixed(p, s, thermal);
    n += launch_node_pass_mixed(p, s, thermal);
    n += launch_update_stress_mixed(p, s, true);
    n += launch_nmd_gather(p, s, true);
    n += launch_nmd_correct(p, s, true);
    if (record_mid(mid, s)) return -1;
    n += launch_force(p, s, true, true);
    int geo = GEO_COPY_OLD | GEO_VOLUME | GEO_SHAPE | GEO_DT | GEO_DT_IF_STEP | GEO_MASS_TERMS;
    if (p.mat.rheol_type & DES_RH_ELASTIC) geo |= GEO_ROTATE;   // FP32 increments in a mixed context
    n += launch_geometry(p, s, geo);
    n += launch_mass_sum(p, s);
    n += launch_dt_finalize(p, s, true);
    return n;
}

// The chained mixed step (part 0 first, 1 middle, 2 last of des_step(n),
// n >= 2).  update_mesh's passes end each step but the last as one
// look-ahead pass that also does the next step's element pass (strain rate,
// dvoldt and heat terms: the next step reads the same velocities, shape
// functions, volumes and temperatures), and the next step's node pass forms
// the mass sums before its own (nothing in between reads mass, tmass or
// volume_n).  Every kernel does the arithmetic of enqueue_step_mixed's, so
// n chained steps give the bits of n single steps; the last step ends as a
// single step does, leaving the same state.
int enqueue_step_mixed_chain(des_ctx *c, int part)
{
    const KP p = step_kp(c);
    cudaStream_t s = c->stream;
    int n = 0;
    const bool thermal = p.prm.has_thermal_diffusion != 0;
    if (part == 0) n += launch_elem_pass_mixed(p, s, thermal);
    n += launch_node_pass_mixed(p, s, thermal, part != 0, part != 0);
    n += launch_update_stress_mixed(p, s, true);
    n += launch_nmd_gather(p, s, true);
    n += launch_nmd_correct(p, s, true);
    n += launch_force(p, s, true, true);
    int geo = GEO_COPY_OLD | GEO_VOLUME | GEO_SHAPE | GEO_DT | GEO_DT_IF_STEP | GEO_MASS_TERMS;
    if (p.mat.rheol_type & DES_RH_ELASTIC) geo |= GEO_ROTATE;
    if (part == 2) {
        n += launch_geometry(p, s, geo);
        n += launch_mass_sum(p, s);
    } else {
        n += launch_geometry_ahead(p, s, geo);
    }
    n += launch_dt_finalize(p, s, true);
    return n;
}

int enqueue_step(des_ctx *c, cudaEvent_t mid)
{
    if (use_mixed(c)) return enqueue_step_mixed(c, mid);
    const KP p = step_kp(c);
    cudaStream_t s = c->stream;
    int n = 0;
    const bool thermal = p.prm.has_thermal_diffusion != 0;
    n += launch_elem_pass(p, s, thermal);   // strain rate, element dvoldt and heat terms
    n += launch_node_pass(p, s, thermal);   // nodal sums, temperature update
    n += launch_update_stress(p, s, true);
    n += launch_nmd_gather(p, s);
    n += launch_nmd_correct(p, s, true);
    if (record_mid(mid, s)) return -1;
    n += launch_force(p, s, true);
    int geo = GEO_COPY_OLD | GEO_VOLUME | GEO_SHAPE | GEO_DT | GEO_DT_IF_STEP | GEO_MASS_TERMS;
    if (p.mat.rheol_type & DES_RH_ELASTIC) geo |= GEO_ROTATE;
    n += launch_geometry(p, s, geo);
    n += launch_mass_sum(p, s);
    n += launch_dt_finalize(p, s, true);
    return n;
}

// One step as a CUDA graph; with `mid`, the graph also records it once
// nmd_correct is done (step_exec_mid).
int build_step_graph(des_ctx *c, cudaEvent_t mid = nullptr)
{
    cudaGraph_t g;
    cudaGraphExec_t &exec = mid ? c->step_exec_mid : c->step_exec;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int n = enqueue_step(c, mid);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    if (n < 0) {
        cudaGraphDestroy(g);
        return fail_msg(c->err, DES_ECUDA, "step capture: recording the mid-step event failed");
    }
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        exec = nullptr;
        return cuda_fail(c, e, "cudaGraphInstantiate");
    }
    c->step_kernels = n;
    return DES_OK;
}

int build_chain_graph(des_ctx *c, int part)
{
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int n = enqueue_step_mixed_chain(c, part);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->chain_exec[part], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->chain_exec[part] = nullptr;
        return cuda_fail(c, e, "cudaGraphInstantiate");
    }
    c->chain_kernels[part] = n;
    return DES_OK;
}

}  // namespace

// ---- the slab-pipelined host step ----
namespace {

// A field of the pipelined host step: host rows, device SoA array (and its
// FP32 copy for the mixed shape functions), values per row, node or element
// rows, whether it is uploaded / downloaded, and its staging region.
struct SlabField {
    double *host;
    double *dev;
    int ncomp;
    bool node, up, down;
    double *stage;
    const float2 *dw;   // download from these double-word pairs instead of dev (mixed shape functions)
};

// The fields of one call, or false when the call does not qualify: the
// state must be complete (coord0 and the derived fields given, as the
// reference's Variables hold them) and page-locked (graph copy nodes).
// Volume, shape functions and volume_n are functions of the coordinates,
// and in the quasi-static mode so is the mass (pseudo-density x volume /
// NPE): the step forms them on the device from the uploaded coordinates,
// with the kernels and bits of its own update_mesh, instead of uploading
// them (~108 MB of the 998,400-tet state).  tmass is uploaded: the
// reference's init forms it before it sets the temperature.
bool slab_fields(des_ctx *c, const des_host_state *st, std::vector<SlabField> &out)
{
    KP &p = c->kp;
    const int nd = c->nd, npe = c->npe, nstr = c->nstr, ne = c->ne;
    const size_t shp1 = (size_t)ne * npe;
    const float2 *dw = p.shpdw;
    const bool ps = p.mat.is_plane_strain != 0;
    const bool qs = p.prm.is_quasi_static != 0;
    // up: needed by the step; down: written by it (strain_rate, force,
    // dpressure, edvoldt and ntmp are written before they are read; coord0
    // and, outside plane strain, stressyy are never written)
    const SlabField all[] = {
        {st->coord, p.x, nd, true, true, true, nullptr},
        {st->coord0, p.x0, nd, true, true, false, nullptr},
        {st->vel, p.v, nd, true, true, true, nullptr},
        {st->force, p.f, nd, true, false, true, nullptr},
        {st->temperature, p.T, 1, true, true, true, nullptr},
        {st->mass, p.mass, 1, true, !qs, true, nullptr},
        {st->tmass, p.tmass, 1, true, true, true, nullptr},
        {st->volume_n, p.vol_n, 1, true, false, true, nullptr},
        {st->ntmp, p.ntmp, 1, true, false, true, nullptr},
        {st->volume, p.vol, 1, false, false, true, nullptr},
        {st->volume_old, p.vol_old, 1, false, true, true, nullptr},
        {st->stress, p.stress, nstr, false, true, true, nullptr},
        {st->strain, p.strain, nstr, false, true, true, nullptr},
        {st->strain_rate, p.srate, nstr, false, false, true, nullptr},
        {st->plstrain, p.pls, 1, false, true, true, nullptr},
        {st->delta_plstrain, p.dpls, 1, false, true, true, nullptr},
        {st->stressyy, p.syy, 1, false, true, ps, nullptr},
        {st->dpressure, p.dp, 1, false, false, true, nullptr},
        {st->edvoldt, p.edvoldt, 1, false, false, true, nullptr},
        {st->shpdx, p.shp, npe, false, false, true, nullptr, dw},
        {nd == 3 ? st->shpdy : nullptr, p.shp + shp1, npe, false, false, nd == 3, nullptr,
         dw ? dw + shp1 : nullptr},
        {st->shpdz, p.shp + (size_t)(nd - 1) * shp1, npe, false, false, true, nullptr,
         dw ? dw + (size_t)(nd - 1) * shp1 : nullptr},
    };
    out.clear();
    size_t off = 0;
    for (SlabField f : all) {
        if (!f.up && !f.down) continue;
        if (!f.host) {
            if (f.up) return false;   // an input is missing: the general path
            continue;
        }
        const size_t cnt = (size_t)(f.node ? c->nn : c->ne) * f.ncomp;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, f.host) != cudaSuccess || a.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            return false;
        }
        if (f.ncomp > 1) {
            if (off + cnt > c->xstage_doubles) return false;
            f.stage = c->d_xstage + off;
            off += cnt;
        }
        out.push_back(f);
    }
    return true;
}

// One step with the host transfers pipelined over the slabs (captured into
// c->pipe_exec).  The mesh is cut into F fine slabs (element and node index
// ranges such that an element's nodes lie in its fine slab or the next and a
// node's support elements in its fine slab or the previous one) and B coarse
// slabs of fine slabs [C_b, C_b+1).  The step's eight stages alternate
// between element passes (reading the node slabs j, j+1 for element slab j)
// and node passes (reading the element slabs j-1, j for node slab j).  Stage
// s of coarse slab b covers the fine slabs [C_b - g_s, C_b+1 - g_s), with the
// skew g = 0,0,1,1,2,2,3,3: every stage then reads only what the stages of
// coarse slabs <= b have written, and writes nothing that a stage of a later
// slab, run afterwards, still has to read in its old state (each element pass
// lies one fine slab behind the node pass before it).  So the slabs run one
// after the other on the compute stream, while three streams overlap:
// uploads (xstream), coarse slab b uploads the element fine slabs [C_b,
// C_b+1) and the node fine slabs [C_b + 1, C_b+1 + 1), all that slab b's first
// stage reads; downloads (ystream), once slab b has run, the fine slabs
// [C_b - 4, C_b+1 - 4), which no later stage writes.  Two stages lead the
// step's eight: an element pass that forms the volume, shape functions and
// mass terms from the uploaded coordinates (those fields are not uploaded)
// and a node pass that sums mass and volume_n, so the skew is
// 0,0,1,1,2,2,3,3,4,4.  The uploaded tmass (and, outside the quasi-static
// mode, mass) is kept: the node pass writes those sums to a scratch sink.
int capture_pipelined(des_ctx *c, const std::vector<SlabField> &F, cudaGraphExec_t *exec, int *nkern)
{
    const int B = c->nslab, NF = c->nfine;
    const bool mixed = use_mixed(c);
    const KP p0 = step_kp(c);
    const bool thermal = p0.prm.has_thermal_diffusion != 0;
    cudaStream_t cs = c->stream, xs = c->xstream, ys = c->ystream;
    std::vector<cudaEvent_t> &ev = c->pipe_ev;   // [0,B) uploaded, [B,2B) slab done, 2B fork, 2B+1/2 joins
    constexpr int NSTAGE = 10, LAG = 4;
    static const int SKEW[NSTAGE] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4};
    auto cb = [&](int b) { return (int)((long long)NF * b / B); };   // C_b
    // a fine-slab range, clipped to [0, NF); the last coarse slab runs to NF
    auto fine = [&](int b, int shift, int &lo, int &hi) {
        lo = b == 0 ? 0 : std::max(0, cb(b) - shift);
        hi = b == B - 1 ? NF : std::min(NF, cb(b + 1) - shift);
    };
    int n = 0;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
#define CKC(call)                                \
    do {                                         \
        if ((e = (call)) != cudaSuccess) goto end; \
    } while (0)
    CKC(cudaEventRecord(ev[2 * B], cs));
    CKC(cudaStreamWaitEvent(xs, ev[2 * B], 0));
    CKC(cudaStreamWaitEvent(ys, ev[2 * B], 0));
    // uploads
    for (int b = 0; b < B; ++b) {
        int elo, ehi, nlo, nhi;
        fine(b, 0, elo, ehi);
        fine(b, -1, nlo, nhi);
        RowTable t{};
        for (const SlabField &f : F) {
            if (!f.up) continue;
            const int lo = f.node ? c->slab_n[nlo] : c->slab_e[elo], hi = f.node ? c->slab_n[nhi] : c->slab_e[ehi];
            if (hi <= lo) continue;
            const size_t o = (size_t)lo * f.ncomp, bytes = (size_t)(hi - lo) * f.ncomp * sizeof(double);
            CKC(cudaMemcpyAsync((f.ncomp == 1 ? f.dev : f.stage) + o, f.host + o, bytes, cudaMemcpyHostToDevice, xs));
            if (f.ncomp > 1) {
                RowField &r = t.f[t.count++];
                r = {f.stage, f.dev, t.total, f.node ? c->nn : c->ne, f.ncomp, lo, hi, nullptr};
                t.total += (long long)(hi - lo) * f.ncomp;
            }
        }
        n += launch_rows(t, true, xs);
        CKC(cudaGetLastError());
        CKC(cudaEventRecord(ev[b], xs));
    }
    // the step, coarse slab by coarse slab
    for (int b = 0; b < B; ++b) {
        CKC(cudaStreamWaitEvent(cs, ev[b], 0));
        for (int st = 0; st < NSTAGE; ++st) {
            int lo, hi;
            fine(b, SKEW[st], lo, hi);
            if (hi <= lo) continue;
            KP q = p0;
            q.e_lo = c->slab_e[lo], q.e_hi = c->slab_e[hi];
            q.n_lo = c->slab_n[lo], q.n_hi = c->slab_n[hi];
            q.f_lo = c->slab_f[lo], q.f_hi = c->slab_f[hi];
            q.fac_order = c->d_fac_order;
            switch (st) {
            case 0: {   // the derived fields of the start state: the element density from T, as compute_mass forms it
                KP g = q;
                g.rho_e = nullptr;
                n += launch_geometry(g, cs, GEO_VOLUME | GEO_SHAPE | GEO_MASS_TERMS);
                break;
            }
            case 1: {   // mass (quasi-static) and volume_n; the uploaded tmass (and mass) stay
                KP g = q;
                g.tmass = c->d_pipe_sink;
                if (!g.prm.is_quasi_static) g.mass = c->d_pipe_sink + c->nn;
                n += launch_mass_sum(g, cs);
                break;
            }
            case 2: n += mixed ? launch_elem_pass_mixed(q, cs, thermal) : launch_elem_pass(q, cs, thermal); break;
            case 3: n += mixed ? launch_node_pass_mixed(q, cs, thermal) : launch_node_pass(q, cs, thermal); break;
            case 4: n += mixed ? launch_update_stress_mixed(q, cs, true) : launch_update_stress(q, cs, true); break;
            case 5: n += launch_nmd_gather(q, cs, mixed); break;
            case 6: n += launch_nmd_correct(q, cs, true); break;
            case 7: n += launch_force(q, cs, true, mixed); break;
            case 8: {
                int geo = GEO_COPY_OLD | GEO_VOLUME | GEO_SHAPE | GEO_DT | GEO_DT_IF_STEP | GEO_MASS_TERMS;
                if (q.mat.rheol_type & DES_RH_ELASTIC) geo |= GEO_ROTATE;
                n += launch_geometry(q, cs, geo);
                break;
            }
            case 9: n += launch_mass_sum(q, cs); break;
            }
            CKC(cudaGetLastError());
        }
        CKC(cudaEventRecord(ev[B + b], cs));
    }
    n += launch_dt_finalize(p0, cs, true);
    CKC(cudaGetLastError());
    // downloads
    for (int b = 0; b < B; ++b) {
        CKC(cudaStreamWaitEvent(ys, ev[B + b], 0));
        int flo, fhi;
        fine(b, LAG, flo, fhi);
        RowTable t{};
        for (const SlabField &f : F) {
            if (!f.down || f.ncomp == 1) continue;
            const int lo = f.node ? c->slab_n[flo] : c->slab_e[flo], hi = f.node ? c->slab_n[fhi] : c->slab_e[fhi];
            if (hi <= lo) continue;
            RowField &r = t.f[t.count++];
            r = {f.stage, f.dev, t.total, f.node ? c->nn : c->ne, f.ncomp, lo, hi, f.dw};
            t.total += (long long)(hi - lo) * f.ncomp;
        }
        n += launch_rows(t, false, ys);
        CKC(cudaGetLastError());
        for (const SlabField &f : F) {
            if (!f.down) continue;
            const int lo = f.node ? c->slab_n[flo] : c->slab_e[flo], hi = f.node ? c->slab_n[fhi] : c->slab_e[fhi];
            if (hi <= lo) continue;
            const size_t o = (size_t)lo * f.ncomp, bytes = (size_t)(hi - lo) * f.ncomp * sizeof(double);
            CKC(cudaMemcpyAsync(f.host + o, (f.ncomp == 1 ? f.dev : f.stage) + o, bytes, cudaMemcpyDeviceToHost, ys));
        }
    }
    CKC(cudaEventRecord(ev[2 * B + 1], xs));
    CKC(cudaEventRecord(ev[2 * B + 2], ys));
    CKC(cudaStreamWaitEvent(cs, ev[2 * B + 1], 0));
    CKC(cudaStreamWaitEvent(cs, ev[2 * B + 2], 0));
end:
#undef CKC
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *exec = nullptr;
        return cuda_fail(c, e, "pipelined host step capture");
    }
    *nkern = n;
    return DES_OK;
}

int ensure_pipe(des_ctx *c)
{
    if (c->ystream) return DES_OK;
    c->pipe_ev.assign(2 * c->nslab + 3, nullptr);
    for (cudaEvent_t &e : c->pipe_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(cudaMalloc((void **)&c->d_pipe_sink, 2 * (size_t)c->nn * sizeof(double)));
    CK(cudaStreamCreateWithFlags(&c->ystream, cudaStreamNonBlocking));
    return DES_OK;
}

// des_step_host for one step over the slabs; *done false: not applicable
int step_host_pipelined(des_ctx *c, des_host_state *st, bool *done)
{
    *done = false;
    if (c->nslab < 2) return DES_OK;
    int rc;
    if ((rc = ensure_xfer(c)) || (rc = ensure_pipe(c))) return rc;
    std::vector<SlabField> F;
    if (!slab_fields(c, st, F)) return DES_OK;
    std::vector<const void *> key;
    for (const SlabField &f : F) key.push_back(f.host);
    if (!c->pipe_exec || key != c->pipe_key) {
        if (c->pipe_exec) {
            cudaGraphExecDestroy(c->pipe_exec);
            c->pipe_exec = nullptr;
        }
        if ((rc = capture_pipelined(c, F, &c->pipe_exec, &c->pipe_kernels))) return rc;
        c->pipe_key = key;
    }
    // the clock, as des_upload_state sets it
    Clock ck{};
    ck.time = st->time;
    ck.dt = st->dt;
    ck.steps = st->steps;
    ck.red_minh = ck.red_maxwell = ck.red_diffusion = ~0ull;
    CK(cudaMemcpyAsync(c->kp.clk, &ck, sizeof ck, cudaMemcpyHostToDevice, c->stream));
    CK(cudaGraphLaunch(c->pipe_exec, c->stream));
    c->launches += c->pipe_kernels;
    CK(cudaMemcpyAsync(&ck, c->kp.clk, sizeof ck, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    st->time = ck.time;
    st->dt = ck.dt;
    st->steps = ck.steps;
    c->has_state = true;
    *done = true;
    return DES_OK;
}

}  // namespace

int des_step(des_ctx *c, int nsteps)
{
    if (!c || nsteps < 0) return DES_EINPUT;
    if (!c->has_state) return fail_msg(c->err, DES_EINPUT, "des_step before des_upload_state");
    if (nsteps >= 2 && use_mixed(c)) {   // the chained step
        for (int part = 0; part < 3; ++part) {
            int rc;
            if (!c->chain_exec[part] && (rc = build_chain_graph(c, part))) return rc;
        }
        for (int i = 0; i < nsteps; ++i) {
            const int part = i == 0 ? 0 : (i == nsteps - 1 ? 2 : 1);
            CK(cudaGraphLaunch(c->chain_exec[part], c->stream));
            c->launches += c->chain_kernels[part];
        }
        return DES_OK;
    }
    if (!c->step_exec) {
        int rc = build_step_graph(c);
        if (rc) return rc;
    }
    for (int i = 0; i < nsteps; ++i) CK(cudaGraphLaunch(c->step_exec, c->stream));
    c->launches += (long long)nsteps * c->step_kernels;
    return DES_OK;
}

int des_step_host(des_ctx *c, des_host_state *st, int nsteps)
{
    if (!c || !st || nsteps < 0) return DES_EINPUT;
    int rc;
    if (nsteps == 1) {   // transfers overlapped with the step, slab by slab
        bool done = false;
        if ((rc = step_host_pipelined(c, st, &done))) return rc;
        if (done) return DES_OK;
    }
    if (nsteps == 0) {
        if ((rc = des_upload_state(c, st))) return rc;
        return download_state(c, st, false);
    }
    // The first step writes strain_rate, force, dpressure, edvoldt and ntmp
    // before it reads them (element pass, force, stress, stress, node pass),
    // so their host values cannot change the result: they are not uploaded,
    // and the download brings back their new values.
    des_host_state in = *st;
    in.strain_rate = in.force = in.dpressure = in.edvoldt = in.ntmp = nullptr;
    if ((rc = des_upload_state(c, &in))) return rc;
    // the last step comes from the graph that records ev_mid, so that the
    // fields it no longer writes go back to the host while its tail runs
    if ((rc = des_step(c, nsteps - 1))) return rc;
    if (!c->step_exec_mid && (rc = build_step_graph(c, c->ev_mid))) return rc;
    CK(cudaGraphLaunch(c->step_exec_mid, c->stream));
    c->launches += c->step_kernels;
    return download_state(c, st, true, true);
}

int des_synchronize(des_ctx *c)
{
    if (!c) return DES_EINPUT;
    CK(cudaStreamSynchronize(c->stream));
    return DES_OK;
}

int des_launch_count(des_ctx *c, long long *count)
{
    if (!c || !count) return DES_EINPUT;
    *count = c->launches;
    return DES_OK;
}

}  // extern "C"

// ------------------------------------------------------------------
// helpers shared with the other translation units of the context
// ------------------------------------------------------------------
namespace des {

int ctx_fail(des_ctx *c, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
    return code;
}

int ctx_cuda_fail(des_ctx *c, cudaError_t e, const char *what) { return cuda_fail(c, e, what); }
int ctx_check_launch(des_ctx *c, int n) { return check_launch(c, n); }
KP ctx_step_kp(const des_ctx *c) { return step_kp(c); }
int ctx_put_field(des_ctx *c, const double *host, double *dev, int n, int ncomp)
{
    return put_field(c, host, dev, n, ncomp);
}
int ctx_get_field(des_ctx *c, const double *dev, double *host, int n, int ncomp)
{
    return get_field(c, host, dev, n, ncomp);
}

}  // namespace des
