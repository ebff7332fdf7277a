// des_kernels.cu -- sm_103a kernels of the explicit time step.
//
// Element kernels run one thread per element (SoA loads coalesce across a
// warp); node kernels run one thread per node and gather the contributions
// of the node's support elements in ascending element order -- the order in
// which the reference's serial element loops scatter them -- so every nodal
// sum is reproducible and matches the reference's serial order.
//
// All arithmetic is FP64 and written in the reference's expression order
// (the library is compiled without FMA contraction), so FP64 results track
// the reference's CPU run to the last few ulps of the transcendental
// functions.
#include "des_kernels.cuh"
#include "des_rheology.cuh"
#include "des_bc.cuh"
#include "des_dw.cuh"
#include "des_mixed_elem.cuh"

namespace des {

constexpr int TPB = 256;

static inline int nblocks(long long n, int tpb = TPB)
{
    long long b = (n + tpb - 1) / tpb;
    return (int)(b < 1 ? 1 : b);
}

// ==================================================================
// strain rate (fields.cxx:166-232)
// ==================================================================
template <int ND>
__device__ __forceinline__ void strain_rate_elem(const KP &p, int e, double *s)
{
    constexpr int NPE = ND + 1;
    double v[NPE][ND];
    double sx[NPE], sy[NPE], sz[NPE];
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        int n = conn_at(p, i, e);
        load_node_v<ND>(p, n, v[i]);
        sx[i] = shp_at(p, 0, i, e);
        if (ND == 3) sy[i] = shp_at(p, 1, i, e);
        sz[i] = shp_at(p, ND - 1, i, e);
    }
    if (ND == 3) {
        s[0] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[0] += v[i][0] * sx[i];
        s[1] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[1] += v[i][1] * sy[i];
        s[2] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[2] += v[i][ND - 1] * sz[i];
        s[3] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[3] += 0.5 * (v[i][0] * sy[i] + v[i][1] * sx[i]);
        s[4] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[4] += 0.5 * (v[i][0] * sz[i] + v[i][ND - 1] * sx[i]);
        s[5] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[5] += 0.5 * (v[i][1] * sz[i] + v[i][ND - 1] * sy[i]);
    } else {
        s[0] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[0] += v[i][0] * sx[i];
        s[1] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[1] += v[i][ND - 1] * sz[i];
        s[2] = 0;
#pragma unroll
        for (int i = 0; i < NPE; ++i) s[2] += 0.5 * (v[i][0] * sz[i] + v[i][ND - 1] * sx[i]);
    }
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_strain_rate(KP p, int begin_step)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (begin_step && e == 0) {
        // var.steps++; var.time += var.dt (dynearthsol.cxx:325-326)
        p.clk->steps += 1;
        p.clk->time += p.clk->dt;
    }
    if (e >= p.ne) return;
    double s[NSTR];
    strain_rate_elem<ND>(p, e, s);
#pragma unroll
    for (int c = 0; c < NSTR; ++c) p.srate[(size_t)c * p.ne + e] = s[c];
}

// ==================================================================
// nodal gathers: heat (fields.cxx:99-146) and dvoldt (geometry.cxx:111-155)
// ==================================================================
// contribution of element e to tdot of its local node i
template <int ND>
__device__ __forceinline__ double heat_term(const KP &p, int e, int i)
{
    constexpr int NPE = ND + 1;
    double vol = p.vol[e];
    double kv = m_k(p, e) * vol;
    double rh = m_hr_over_cp(p, e) * vol;
    double sxi = shp_at(p, 0, i, e), szi = shp_at(p, ND - 1, i, e);
    double syi = (ND == 3) ? shp_at(p, 1, i, e) : 0.0;
    double diffusion = 0;
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        double sxj = shp_at(p, 0, j, e), szj = shp_at(p, ND - 1, j, e);
        double D;
        if (ND == 3) {
            double syj = shp_at(p, 1, j, e);
            D = (sxi * sxj + syi * syj + szi * szj);
        } else {
            D = (sxi * sxj + szi * szj);
        }
        diffusion += D * p.T[conn_at(p, j, e)];
    }
    return diffusion * kv - rh;
}

template <int ND, bool HEAT, bool DVOLDT>
__global__ void __launch_bounds__(TPB) k_node_gather1(KP p)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    int b = p.sup_off[n], end = p.sup_off[n + 1];
    double tdot = 0, dvoldt = 0;
    for (int q = b; q < end; ++q) {
        int ent = p.sup_ent[q];
        int e = ent >> 2, i = ent & 3;
        if (HEAT) tdot += heat_term<ND>(p, e, i);
        if (DVOLDT) {
            double dj;
            if (ND == 3) dj = p.srate[e] + p.srate[(size_t)p.ne + e] + p.srate[2 * (size_t)p.ne + e];
            else dj = p.srate[e] + p.srate[(size_t)p.ne + e];
            dvoldt += dj * p.vol[e];
        }
    }
    if (HEAT) p.tdot[n] = tdot;
    if (DVOLDT) p.ntmp[n] = dvoldt / p.vol_n[n];
}

// The fused step's form of the same three functions (update_strain_rate,
// the heat gather of update_temperature, compute_dvoldt), element-centric.
// k_elem_pass writes the strain rate, the element's dvoldt term qv = tr(edot)
// vol and, with heat, its contribution to each of its nodes' tdot (slot i of
// hc64).  The stencil D_ij = dN_i . dN_j is formed once per element: D_ji is
// the same products in the same order, so every slot holds the very value
// heat_term gives for (e, i), at 10 instead of 16 dot products.
// k_node_pass sums the slots and the qv over each node's support in
// ascending element order -- the node-centric kernels' order -- and applies
// the temperature update.  The bits are those of k_strain_rate,
// k_node_gather1 and k_temperature_update.
template <int ND>
__global__ void __launch_bounds__(TPB) k_elem_pass(KP p, int heat)
{
    constexpr int NPE = ND + 1, NSTR = ND * (ND + 1) / 2;
    const int e = p.e_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 0) {   // var.steps++; var.time += var.dt (dynearthsol.cxx:325-326)
        p.clk->steps += 1;
        p.clk->time += p.clk->dt;
    }
    if (e >= p.e_hi) return;
    const size_t ne = p.ne;
    double sr[NSTR];
    strain_rate_elem<ND>(p, e, sr);
#pragma unroll
    for (int c = 0; c < NSTR; ++c) p.srate[(size_t)c * ne + e] = sr[c];
    const double vol = p.vol[e];
    double dj;
    if (ND == 3) dj = sr[0] + sr[1] + sr[2];
    else dj = sr[0] + sr[1];
    p.qv[e] = dj * vol;
    if (!heat) return;
    const double kv = m_k(p, e) * vol;
    const double rh = m_hr_over_cp(p, e) * vol;
    double sx[NPE], sy[NPE], sz[NPE], T[NPE];
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        sx[i] = shp_at(p, 0, i, e);
        sy[i] = (ND == 3) ? shp_at(p, 1, i, e) : 0.0;
        sz[i] = shp_at(p, ND - 1, i, e);
        T[i] = p.T[conn_at(p, i, e)];
    }
    double D[NPE][NPE];
#pragma unroll
    for (int i = 0; i < NPE; ++i)
#pragma unroll
        for (int j = i; j < NPE; ++j) {
            D[i][j] = (ND == 3) ? (sx[i] * sx[j] + sy[i] * sy[j] + sz[i] * sz[j]) : (sx[i] * sx[j] + sz[i] * sz[j]);
            D[j][i] = D[i][j];
        }
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        double diffusion = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) diffusion += D[i][j] * T[j];
        p.hc64[(size_t)i * ne + e] = diffusion * kv - rh;
    }
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_node_pass(KP p, int heat)
{
    const int n = p.n_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.n_hi) return;
    const size_t ne = p.ne;
    double tdot = 0, dvoldt = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        const int ent = p.sup_ent[q];
        const int e = ent >> 2, i = ent & 3;
        if (heat) tdot += p.hc64[(size_t)i * ne + e];
        dvoldt += p.qv[e];
    }
    p.ntmp[n] = dvoldt / p.vol_n[n];
    if (heat) {   // temperature update + Dirichlet BC (fields.cxx:151-162)
        p.tdot[n] = tdot;
        const unsigned flag = p.bcflag[n];
        if (flag & BOUNDZ1) p.T[n] = p.prm.surface_temperature;
        else if ((flag & BOUNDZ0) && !p.prm.has_fixed_bottom_temperature) p.T[n] = p.prm.mantle_temperature;
        else p.T[n] -= tdot * p.clk->dt / p.tmass[n];
    }
}

// temperature update + Dirichlet BC (fields.cxx:151-162)
__global__ void __launch_bounds__(TPB) k_temperature_update(KP p)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    unsigned flag = p.bcflag[n];
    if (flag & BOUNDZ1) p.T[n] = p.prm.surface_temperature;
    else if ((flag & BOUNDZ0) && !p.prm.has_fixed_bottom_temperature) p.T[n] = p.prm.mantle_temperature;
    else p.T[n] -= p.tdot[n] * p.clk->dt / p.tmass[n];
}

// compute_edvoldt (geometry.cxx:158-179)
template <int ND>
__global__ void __launch_bounds__(TPB) k_edvoldt(KP p)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    double dj = 0;
#pragma unroll
    for (int i = 0; i < ND + 1; ++i) dj += p.ntmp[conn_at(p, i, e)];
    p.edvoldt[e] = dj / (ND + 1);
}

// ==================================================================
// update_stress (rheology.cxx:510-646)
// ==================================================================
template <int ND>
__global__ void __launch_bounds__(TPB) k_update_stress(KP p, int fused)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    int e = p.e_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.e_hi) return;
    const size_t ne = p.ne;
    double edv;
    if (fused) {
        // compute_edvoldt fused in: dvoldt of the step is in ntmp
        double dj = 0;
#pragma unroll
        for (int i = 0; i < ND + 1; ++i) dj += p.ntmp[conn_at(p, i, e)];
        edv = dj / (ND + 1);
        p.edvoldt[e] = edv;
    } else {
        edv = p.edvoldt[e];
    }
    double s[NSTR], es[NSTR], edot[NSTR];
#pragma unroll
    for (int c = 0; c < NSTR; ++c) {
        s[c] = p.stress[c * ne + e];
        es[c] = p.strain[c * ne + e];
        edot[c] = p.srate[c * ne + e];
    }
    double syy = p.syy[e], pls = p.pls[e], dpls = p.dpls[e], dpr;
    unsigned bits = update_stress_elem<ND>(p, e, p.clk->dt, s, syy, es, edot, pls, dpls, edv, p.vol[e],
                                           p.vol_old[e], dpr);
#pragma unroll
    for (int c = 0; c < NSTR; ++c) {
        p.stress[c * ne + e] = s[c];
        p.strain[c * ne + e] = es[c];
        p.srate[c * ne + e] = edot[c];
    }
    p.syy[e] = syy;
    p.pls[e] = pls;
    p.dpls[e] = dpls;
    p.dp[e] = dpr;
    if (fused && p.rho_e) {   // temperature is final for this step
        const double rho = m_rho<ND>(p, e);
        p.rho_e[e] = rho;
        // the force gather's buoyancy term, once per element instead of per node
        if (p.buoy_e) p.buoy_e[e] = p.prm.gravity != 0 ? rho * p.prm.gravity / (ND + 1) : 0.0;
    }
    if (bits) set_err(p, bits);
}

// ==================================================================
// NMD_stress (geometry.cxx:182-236)
// ==================================================================
// stored: read the products the fused stress pass formed (KP::pv), the same
// dw_mul of the same pairs, instead of forming them for each support entry
template <int ND>
__global__ void __launch_bounds__(TPB) k_nmd_gather(KP p, int stored)
{
    int n = p.n_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.n_hi) return;
    if (ND == 3 && p.shpdw) {   // a mixed context: double-word products, compensated FP32 sum (des_dw.cuh)
        dw_sum acc;
        for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
            const int e = p.sup_ent[q] >> 2;
            acc.add(stored ? dw_of2(p.pv[e]) : dw_mul(dw_split(p.dp[e]), dw_split(p.vol[e])));
        }
        p.ntmp[n] = acc.value() / p.vol_n[n];
        return;
    }
    double acc = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        int e = p.sup_ent[q] >> 2;
        acc += p.dp[e] * p.vol[e];
    }
    p.ntmp[n] = acc / p.vol_n[n];
}

// per-facet force of the gravity-induced stress BCs (bc.cxx:493-557);
// inactive facets get exactly +0 so that subtracting them is exact
template <int ND>
__device__ void facet_force(const KP &p, int q)
{
    const int i = p.fac_bdry[q];
    const int t = p.prm.vbc_types[i];
    double out[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) out[d] = 0.0;
    bool active = p.prm.gravity != 0 && (t == 0 || t == 2 || t == 4) &&
                  !(i == 4 && !p.prm.has_winkler_foundation) && !(i == 5 && !p.prm.has_water_loading);
    if (active) {
        const int e = p.fac_elem[q], f = p.fac_f[q];
        double normal[ND], zcenter;
        if (ND == 3) {
            const int F[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
            double c0[3], c1[3], c2[3];
            load_node_x<3>(p, conn_at(p, F[f][0], e), c0);
            load_node_x<3>(p, conn_at(p, F[f][1], e), c1);
            load_node_x<3>(p, conn_at(p, F[f][2], e), c2);
            double v01[3], v02[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                v01[d] = c1[d] - c0[d];
                v02[d] = c2[d] - c0[d];
            }
            normal[0] = (v01[1] * v02[2] - v01[2] * v02[1]) / 2;
            normal[1] = (v01[2] * v02[0] - v01[0] * v02[2]) / 2;
            normal[ND - 1] = (v01[0] * v02[1] - v01[1] * v02[0]) / 2;
            zcenter = div3(c0[2] + c1[2] + c2[2]);   // x / 3, bit for bit
        } else {
            const int F[3][2] = {{1, 2}, {2, 0}, {0, 1}};
            double c0[2], c1[2];
            load_node_x<2>(p, conn_at(p, F[f][0], e), c0);
            load_node_x<2>(p, conn_at(p, F[f][1], e), c1);
            double v01[2] = {c1[0] - c0[0], c1[1] - c0[1]};
            normal[0] = v01[1];
            normal[ND - 1] = -v01[0];
            zcenter = (c0[1] + c1[1]) / 2;
        }
        double pr;
        if (i == 4 && p.prm.has_winkler_foundation) {
            double rho = p.rho_e ? p.rho_e[e] : m_rho<ND>(p, e);
            pr = p.prm.compensation_pressure
                - (rho + p.prm.winkler_delta_rho) * p.prm.gravity * (zcenter + p.prm.zlength);
        } else if (i == 5 && p.prm.has_water_loading) {
            const double sea_level = 0;
            pr = 0;
            if (zcenter < sea_level) {
                const double sea_water_density = 1030;
                pr = sea_water_density * p.prm.gravity * (sea_level - zcenter);
            }
        } else {
            pr = ref_pressure_(p, zcenter);
        }
#pragma unroll
        for (int d = 0; d < ND; ++d) out[d] = divnd<ND>(pr * normal[d]);
    }
#pragma unroll
    for (int d = 0; d < ND; ++d) p.fv[(size_t)d * p.nbf + q] = out[d];
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_nmd_correct(KP p, int with_facets)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nel = p.e_hi - p.e_lo;
    if (t < nel) {
        const int e = p.e_lo + t;
        double dpn = 0;
#pragma unroll
        for (int i = 0; i < ND + 1; ++i) dpn += p.ntmp[conn_at(p, i, e)];
        double dp_el = dpn / (ND + 1);
        double dp_orig = p.dp[e];
#pragma unroll
        for (int i = 0; i < ND; ++i) p.stress[(size_t)i * p.ne + e] += divnd<ND>(-dp_orig + dp_el);
    } else if (with_facets && t < nel + (p.f_hi - p.f_lo)) {
        const int i = p.f_lo + (t - nel);
        facet_force<ND>(p, p.fac_order ? p.fac_order[i] : i);
    }
}

// The mixed 3D step's force terms of one element (fields.cxx:291-340, the
// element's part): for each node slot i the vector
//   T_i = (sigma . dN_i/dx + rho g / 4 z) vol,
// which the node gather k_force_dw3 subtracts.  Formed in double-word
// arithmetic (des_dw.cuh) from the FP64 stress, volume and buoyancy and the
// double-word shape functions: sigma vol first (6 products), then T_1..T_3 as compensated dot
// products with dN_1..3/dx, T_0 = -(T_1 + T_2 + T_3) (the four shape-function
// gradients of a tetrahedron sum to zero: the element's stress forces
// balance exactly), and the buoyancy term rho g / 4 vol added to every z
// component.  Each T is within ~2^-44 of its FP64 value, relative to the
// terms it sums.  T_i goes to the support-list entry of (e, i), so that
// each node's gather reads its terms from consecutive memory.
__device__ __forceinline__ void force_terms_dw3(const KP &p, int e, const double *s)
{
    const size_t ne = p.ne;
    double buoy = 0;
    if (p.buoy_e) {
        buoy = p.buoy_e[e];
    } else if (p.prm.gravity != 0) {
        const double rho = p.rho_e ? p.rho_e[e] : m_rho<3>(p, e);
        buoy = rho * p.prm.gravity / 4;
    }
    const dw v = dw_split(p.vol[e]);
    dw sv[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) sv[c] = dw_mul(dw_split(s[c]), v);
    dw t[4][3];
#pragma unroll
    for (int i = 1; i < 4; ++i) {
        const dw sx = dw_of2(p.shpdw[(size_t)i * ne + e]), sy = dw_of2(p.shpdw[(size_t)(4 + i) * ne + e]),
                 sz = dw_of2(p.shpdw[(size_t)(8 + i) * ne + e]);
        t[i][0] = dw_dot3c(sv[0], sx, sv[3], sy, sv[4], sz);
        t[i][1] = dw_dot3c(sv[3], sx, sv[1], sy, sv[5], sz);
        t[i][2] = dw_dot3c(sv[4], sx, sv[5], sy, sv[2], sz);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) t[0][k] = dw_neg(dw_sum3(t[1][k], t[2][k], t[3][k]));
    const dw bv = dw_mul(dw_split(buoy), v);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        t[i][2] = dw_add(t[i][2], bv);
        float4 *o = p.ft + 2 * (size_t)p.sup_pos[(size_t)i * ne + e];
        o[0] = make_float4(t[i][0].hi, t[i][1].hi, t[i][2].hi, 0.0f);
        o[1] = make_float4(t[i][0].lo, t[i][1].lo, t[i][2].lo, 0.0f);
    }
}

// k_nmd_correct<3> for the mixed step, which also forms the element's force
// terms from the corrected stress (the same bits of stress as k_nmd_correct)
__global__ void __launch_bounds__(TPB) k_nmd_correct_ft3(KP p, int with_facets)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nel = p.e_hi - p.e_lo;
    if (t < nel) {
        const int e = p.e_lo + t;
        const size_t ne = p.ne;
        double dpn = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) dpn += p.ntmp[conn_at(p, i, e)];
        const double dp_el = dpn / 4;
        const double dp_orig = p.dp[e];
        double s[6];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s[i] = p.stress[(size_t)i * ne + e] + divnd<3>(-dp_orig + dp_el);
            p.stress[(size_t)i * ne + e] = s[i];
        }
#pragma unroll
        for (int i = 3; i < 6; ++i) s[i] = p.stress[(size_t)i * ne + e];
        force_terms_dw3(p, e, s);
    } else if (with_facets && t < nel + (p.f_hi - p.f_lo)) {
        const int i = p.f_lo + (t - nel);
        facet_force<3>(p, p.fac_order ? p.fac_order[i] : i);
    }
}

// the force terms alone (des_update_force in a mixed context)
__global__ void __launch_bounds__(TPB) k_force_terms3(KP p)
{
    const int e = p.e_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.e_hi) return;
    double s[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) s[c] = p.stress[(size_t)c * p.ne + e];
    force_terms_dw3(p, e, s);
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_facet_forces(KP p)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < p.nbf) facet_force<ND>(p, q);
}

// ==================================================================
// update_force (fields.cxx:291-340) with stress BCs (bc.cxx:493-566) and
// damping (fields.cxx:235-288); optionally fused with update_velocity,
// apply_vbcs and update_coordinate (dynearthsol.cxx:340-343, fields.cxx:343-368)
// ==================================================================
template <int ND>
__device__ __forceinline__ void damp(const KP &p, double &ff, double v)
{
    const double df = p.prm.damping_factor;
    switch (p.prm.damping_option) {
    case 1:
        if (fabs(v) > 1e-13) ff -= df * copysign(ff, v);
        break;
    case 2:
        ff -= df * ff;
        break;
    case 3:
        if ((ff < 0) == (v < 0)) ff -= df * ff;
        else ff += (1 - df) * ff;
        break;
    default:
        break;
    }
}

// a * b + c; with C, one fused multiply-add (the mixed step's kernels).
// Without C it is the separately rounded product and sum of the FP64 step.
template <bool C>
__device__ __forceinline__ double madd(double a, double b, double c)
{
    return C ? fma(a, b, c) : a * b + c;
}

// CONTRACT: the mixed step's form, with the sums of products fused
// (1 + 2 instead of 3 + 2 FP64 operations per component, and the update
// f -= t * vol one fma), and dt f / m as dt f (1/m) with one recip_newton.
// Rounding moves by an ulp of each force term, far below the FP32 strain
// rate terms of the same step.
template <int ND, bool CONTRACT>
__device__ __forceinline__ void force_tail(const KP &p, int n, double *f, int fused_motion);

template <int ND, bool CONTRACT = false>
__global__ void __launch_bounds__(TPB) k_force(KP p, int fused_motion)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    constexpr int NPE = ND + 1;
    int n = p.n_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.n_hi) return;
    const size_t ne = p.ne;
    const double gravity = p.prm.gravity;
    double f[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) f[d] = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        int ent = p.sup_ent[q];
        int e = ent >> 2, i = ent & 3;
        double s[NSTR];
#pragma unroll
        for (int c = 0; c < NSTR; ++c) s[c] = p.stress[c * ne + e];
        double vol = p.vol[e];
        double buoy = 0;
        if (p.buoy_e) {
            buoy = p.buoy_e[e];
        } else if (gravity != 0) {
            double rho = p.rho_e ? p.rho_e[e] : m_rho<ND>(p, e);
            buoy = rho * gravity / NPE;
        }
        double sx = shp_at(p, 0, i, e), sz = shp_at(p, ND - 1, i, e);
        // f -= (sum of products) * vol, written as madd(-t, vol, f): the same
        // bits as the reference's expression when not contracted
        if (ND == 3) {
            double sy = shp_at(p, 1, i, e);
            f[0] = madd<CONTRACT>(-madd<CONTRACT>(s[4], sz, madd<CONTRACT>(s[3], sy, s[0] * sx)), vol, f[0]);
            f[1] = madd<CONTRACT>(-madd<CONTRACT>(s[5], sz, madd<CONTRACT>(s[1], sy, s[3] * sx)), vol, f[1]);
            const double tz = CONTRACT ? fma(s[2], sz, fma(s[5], sy, fma(s[4], sx, buoy)))
                                       : madd<false>(s[2], sz, madd<false>(s[5], sy, s[4] * sx)) + buoy;
            f[ND - 1] = madd<CONTRACT>(-tz, vol, f[ND - 1]);
        } else {
            f[0] = madd<CONTRACT>(-madd<CONTRACT>(s[2], sz, s[0] * sx), vol, f[0]);
            const double tz = CONTRACT ? fma(s[1], sz, fma(s[2], sx, buoy)) : madd<false>(s[1], sz, s[2] * sx) + buoy;
            f[ND - 1] = madd<CONTRACT>(-tz, vol, f[ND - 1]);
        }
    }
    force_tail<ND, CONTRACT>(p, n, f, fused_motion);
}

// k_force after its element gather: the gravity-induced stress BCs, the
// elastic foundation, damping and the force store, then (fused_motion) the
// velocity update, velocity BCs and coordinate update
template <int ND, bool CONTRACT>
__device__ __forceinline__ void force_tail(const KP &p, int n, double *f, int fused_motion)
{
    // gravity-induced stress BCs, in the reference's facet order
    for (int q = p.nf_off[n]; q < p.nf_off[n + 1]; ++q) {
        int fq = p.nf_ent[q];
#pragma unroll
        for (int d = 0; d < ND; ++d) f[d] -= p.fv[(size_t)d * p.nbf + fq];
    }
    const unsigned flag = p.bcflag[n];
    if (p.prm.has_elastic_foundation && (flag & BOUNDZ0)) {
        const size_t o = (size_t)(ND - 1) * p.nn + n;
        f[ND - 1] -= p.prm.elastic_foundation_constant * (p.x[o] - p.x0[o]);
    }
    double v[ND];
    load_node_v<ND>(p, n, v);
    if (p.prm.is_quasi_static) {
#pragma unroll
        for (int d = 0; d < ND; ++d) damp<ND>(p, f[d], v[d]);
    }
#pragma unroll
    for (int d = 0; d < ND; ++d) p.f[(size_t)d * p.nn + n] = f[d];
    if (!fused_motion) return;
    const double dt = p.clk->dt;
    const double m = p.mass[n];
    if (CONTRACT) {
        const double im = recip_newton(m);
#pragma unroll
        for (int d = 0; d < ND; ++d) v[d] = fma(dt * f[d], im, v[d]);
    } else {
#pragma unroll
        for (int d = 0; d < ND; ++d) v[d] += dt * f[d] / m;
    }
    apply_vbcs_node<ND>(p, flag, v);
    bool bad = false;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const size_t o = (size_t)d * p.nn + n;
        p.v[o] = v[d];
        if (ND == 3 && p.vdw) {   // a mixed context: the pairs the look-ahead geometry pass reads
            const dw w = dw_split(v[d]);
            p.vdw[o] = make_float2(w.hi, w.lo);
        }
        double xn = madd<CONTRACT>(v[d], dt, p.x[o]);
        p.x[o] = xn;
        bad |= !isfinite(xn) || !isfinite(v[d]);
    }
    if (bad) set_err(p, DES_DEV_NONFINITE);
}

// update_force of the mixed 3D step: each node sums the force terms T of its
// support (k_nmd_correct_ft3 / k_force_terms3, stored in the support list's
// order: one contiguous run per node) in ascending element order in
// double-word arithmetic -- whose sums are accurate relative to the exact
// sum (Algorithm 6 of des_dw.cuh), however much the elements' terms cancel
// -- and rounds the sum to FP64 once; the rest is k_force's FP64 tail.
__global__ void __launch_bounds__(TPB) k_force_dw3(KP p, int fused_motion)
{
    const int n = p.n_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.n_hi) return;
    dw a0{0.0f, 0.0f}, a1{0.0f, 0.0f}, a2{0.0f, 0.0f};
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        const float4 h = __ldg(p.ft + 2 * (size_t)q), l = __ldg(p.ft + 2 * (size_t)q + 1);
        a0 = dw_add(a0, {h.x, l.x});
        a1 = dw_add(a1, {h.y, l.y});
        a2 = dw_add(a2, {h.z, l.z});
    }
    double f[3] = {-f64_of(a0), -f64_of(a1), -f64_of(a2)};
    force_tail<3, true>(p, n, f, fused_motion);
}

// CONTRACT: the form of k_force<ND, true>'s fused velocity update
template <int ND, bool CONTRACT = false>
__global__ void __launch_bounds__(TPB) k_velocity(KP p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nn * ND) return;
    int d = i / p.nn, n = i - d * p.nn;
    if (CONTRACT) p.v[i] = fma(p.clk->dt * p.f[i], recip_newton(p.mass[n]), p.v[i]);
    else p.v[i] += p.clk->dt * p.f[i] / p.mass[n];
    (void)d;
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_vbcs(KP p)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    unsigned flag = p.bcflag[n];
    if (!(flag & BOUND_ANY)) return;
    double v[ND];
    load_node_v<ND>(p, n, v);
    apply_vbcs_node<ND>(p, flag, v);
#pragma unroll
    for (int d = 0; d < ND; ++d) p.v[(size_t)d * p.nn + n] = v[d];
}

template <int ND, bool CONTRACT = false>
__global__ void __launch_bounds__(TPB) k_coordinate(KP p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nn * ND) return;
    p.x[i] = madd<CONTRACT>(p.v[i], p.clk->dt, p.x[i]);
}

// ==================================================================
// element geometry: volume_old swap, compute_volume, compute_shape_fn,
// rotate_stress, compute_dt element terms
// ==================================================================
// compute_shape_fn (geometry.cxx:368-455) of the FP64 step
template <int ND>
__device__ __forceinline__ void shape_fn_elem(const double (*d)[ND], const TetEdges &te, double vol,
                                              double (*shp)[ND + 1])
{
    if (ND == 3) {
        double iv = 1 / (6 * vol);
        const double x01 = te.x01, x02 = te.x02, x03 = te.x03, x12 = te.x12, x13 = te.x13, x23 = te.x23;
        const double y01 = te.y01, y02 = te.y02, y03 = te.y03, y12 = te.y12, y13 = te.y13, y23 = te.y23;
        const double z01 = te.z01, z02 = te.z02, z03 = te.z03, z12 = te.z12, z13 = te.z13, z23 = te.z23;
        shp[0][0] = iv * (y13 * z12 - y12 * z13);
        shp[1][0] = iv * (z13 * x12 - z12 * x13);
        shp[ND - 1][0] = iv * (x13 * y12 - x12 * y13);
        shp[0][1] = iv * (y02 * z23 - y23 * z02);
        shp[0][2] = iv * (y13 * z03 - y03 * z13);
        shp[0][3] = iv * (y01 * z02 - y02 * z01);
        shp[1][1] = iv * (z02 * x23 - z23 * x02);
        shp[1][2] = iv * (z13 * x03 - z03 * x13);
        shp[1][3] = iv * (z01 * x02 - z02 * x01);
        shp[ND - 1][1] = iv * (x02 * y23 - x23 * y02);
        shp[ND - 1][2] = iv * (x13 * y03 - x03 * y13);
        shp[ND - 1][3] = iv * (x01 * y02 - x02 * y01);
    } else {
        const double *d0 = d[0], *d1 = d[1], *d2 = d[2];
        double iv = 1 / (2 * vol);
        shp[0][0] = iv * (d1[1] - d2[1]);
        shp[0][1] = iv * (d2[1] - d0[1]);
        shp[0][2] = iv * (d0[1] - d1[1]);
        shp[ND - 1][0] = iv * (d2[0] - d1[0]);
        shp[ND - 1][1] = iv * (d0[0] - d2[0]);
        shp[ND - 1][2] = iv * (d1[0] - d0[0]);
    }
}

// The mixed context's tet geometry from the edges at node 0, d_i = x_i - x_0
// (9 FP64 differences instead of the reference formulas' 18): with the cross
// products c1 = d2 x d3, c2 = d3 x d1, c3 = d1 x d2, the signed volume is
// d1 . c1 / 6 in FP64 (geometry.cxx:29-49 evaluates the same determinant from
// other edges), dN_i/dx = c_i / (6 vol) for i = 1..3 and dN_0/dx = -(sum of
// the other three) (geometry.cxx:368-455), the latter in double-word
// arithmetic (rel_shape_fn_dw).
struct RelEdges {
    double d[3][3];   // d[i - 1][k]: component k of x_i - x_0
};

__device__ __forceinline__ RelEdges rel_edges(const double *x0, const double *x1, const double *x2, const double *x3)
{
    RelEdges r;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r.d[0][k] = x1[k] - x0[k];
        r.d[1][k] = x2[k] - x0[k];
        r.d[2][k] = x3[k] - x0[k];
    }
    return r;
}

// a x b, each component one fused multiply-add and one product
__device__ __forceinline__ void cross3(const double *a, const double *b, double *out)
{
    out[0] = fma(a[1], b[2], -(a[2] * b[1]));
    out[1] = fma(a[2], b[0], -(a[0] * b[2]));
    out[2] = fma(a[0], b[1], -(a[1] * b[0]));
}

// The mixed context's shape functions as double-word pairs: with the FP64
// edges d_i and the volume's FP64 cross product c1 = d2 x d3, the cross
// products c2 = d3 x d1 and c3 = d1 x d2 (compensated, dw_diff2), 1/(6 vol)
// (dw_recip) and dN_i/dx = c_i / (6 vol), dN_0/dx = -(the other three),
// all on the FP32 pipe; within ~2^-45 of the exact values where the FP64
// forms carry one rounding per product.
__device__ __forceinline__ void rel_shape_fn_dw(const RelEdges &r, const double *c1, double vol, dw (*shp)[4])
{
    dw d[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) d[i][k] = dw_split(r.d[i][k]);
    dw cc[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) cc[0][k] = dw_split(c1[k]);
    cc[1][0] = dw_diff2(d[2][1], d[0][2], d[2][2], d[0][1]);
    cc[1][1] = dw_diff2(d[2][2], d[0][0], d[2][0], d[0][2]);
    cc[1][2] = dw_diff2(d[2][0], d[0][1], d[2][1], d[0][0]);
    cc[2][0] = dw_diff2(d[0][1], d[1][2], d[0][2], d[1][1]);
    cc[2][1] = dw_diff2(d[0][2], d[1][0], d[0][0], d[1][2]);
    cc[2][2] = dw_diff2(d[0][0], d[1][1], d[0][1], d[1][0]);
    const dw iv = dw_recip(dw_mul(dw_split(vol), dw{6.0f, 0.0f}));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int i = 1; i < 4; ++i) shp[k][i] = dw_mul(cc[i - 1][k], iv);
        shp[k][0] = dw_neg(dw_sum3(shp[k][1], shp[k][2], shp[k][3]));
    }
}

// jaumann_rate_3d / _2d (fields.cxx:375-404)
__device__ __forceinline__ void jaumann3(double *s, double dt, double w3, double w4, double w5)
{
    double si[6];
    si[0] = -2.0 * s[3] * w3 - 2.0 * s[4] * w4;
    si[1] = 2.0 * s[3] * w3 - 2.0 * s[5] * w5;
    si[2] = 2.0 * s[4] * w4 + 2.0 * s[5] * w5;
    si[3] = s[0] * w3 - s[1] * w3 - s[4] * w5 - s[5] * w4;
    si[4] = s[0] * w4 - s[2] * w4 + s[3] * w5 - s[5] * w3;
    si[5] = s[1] * w5 - s[2] * w5 + s[3] * w4 + s[4] * w3;
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] += dt * si[i];
}

__device__ __forceinline__ void jaumann2(double *s, double dt, double w2)
{
    double si[3];
    si[0] = -2.0 * s[2] * w2;
    si[1] = 2.0 * s[2] * w2;
    si[2] = s[0] * w2 - s[1] * w2;
#pragma unroll
    for (int i = 0; i < 3; ++i) s[i] += dt * si[i];
}

template <int ND>
__device__ __forceinline__ void warp_block_min(unsigned long long val, unsigned long long *target)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, val, o);
        val = other < val ? other : val;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(target, val);
}

// The element geometry pass.  AHEAD (3D mixed contexts, the chained step's
// look-ahead): with the shape-function pairs still in registers and the
// velocities as the pairs the force pass stored (KP::vdw), it also does the
// next step's element pass (strain rate, dvoldt and heat terms) -- the next
// step reads the same velocities, shape functions, volume and temperature,
// none of which changes in between -- so the pairs are not read back and one
// pass over the elements is saved.  What the next node pass gathers per
// support entry (dvoldt term, volume, mass and tmass terms) goes into one
// record per element (KP::ndpk) instead of four arrays.
template <int ND, bool AHEAD>
__device__ __forceinline__ void geometry_body(const KP &p, int flags)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    constexpr int NPE = ND + 1;
    int e = p.e_lo + blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = e < p.e_hi;
    const size_t ne = p.ne;
    bool do_dt = (flags & GEO_DT) != 0;
    if (flags & GEO_DT_IF_STEP) do_dt = do_dt && (p.clk->steps % 10 == 0);
    do_dt = do_dt && p.prm.fixed_dt == 0;
    unsigned long long b_minh = ~0ull, b_maxwell = ~0ull;
    if (in) {
        double c[NPE][ND];
        int nodes[NPE];
#pragma unroll
        for (int i = 0; i < NPE; ++i) {
            nodes[i] = conn_at(p, i, e);
            load_node_x<ND>(p, nodes[i], c[i]);
        }
        double vol;
        TetEdges te{};
        // a mixed context's 3D geometry works from the edges at node 0
        const bool rel0 = ND == 3 && p.shpdw != nullptr;
        RelEdges re{};
        if (rel0 && (flags & (GEO_VOLUME | GEO_SHAPE))) re = rel_edges(c[0], c[1], c[2], c[NPE - 1]);
        else if (ND == 3 && (flags & (GEO_VOLUME | GEO_SHAPE))) te = tet_edges(c[0], c[1], c[2], c[NPE - 1]);
        // the FP64 cross product d2 x d3 that the volume and the shape functions share
        double c1[3] = {0, 0, 0};
        if (rel0 && (flags & (GEO_VOLUME | GEO_SHAPE))) cross3(re.d[1], re.d[2], c1);
        if (flags & GEO_COPY_OLD) p.vol_old[e] = p.vol[e];
        if (flags & GEO_VOLUME) {
            if (rel0) vol = div6(fma(re.d[0][2], c1[2], fma(re.d[0][1], c1[1], re.d[0][0] * c1[0])));
            else if (ND == 3) vol = tet_volume(te);
            else vol = tri_area<2>(c[0], c[1], c[2]);
            p.vol[e] = vol;
            if (!(vol > 0)) set_err(p, DES_DEV_NEG_VOLUME);
        } else {
            vol = p.vol[e];
        }
        if (do_dt) {
            // compute_dt element terms (geometry.cxx:254-292), while the coordinates are at hand
            double minh;
            if (ND == 3) {
                // the largest face area: sqrt is correctly rounded and
                // monotonic and /2 exact, so max_i sqrt(s_i) / 2 equals
                // sqrt(max_i s_i) / 2 -- one square root instead of four
                const double s2 = dmax_(dmax_(tri_area2_3d(c[0], c[1], c[2]), tri_area2_3d(c[0], c[1], c[NPE - 1])),
                                        dmax_(tri_area2_3d(c[2], c[NPE - 1], c[0]),
                                              tri_area2_3d(c[2], c[NPE - 1], c[1])));
                double maxa = sqrt(s2) / 2;
                minh = 3 * vol / maxa;
            } else {
                double d01 = 0, d12 = 0, d02 = 0;
#pragma unroll
                for (int k = 0; k < ND; ++k) {
                    double a = c[1][k] - c[0][k], b = c[2][k] - c[1][k], cc = c[2][k] - c[0][k];
                    d01 += a * a;
                    d12 += b * b;
                    d02 += cc * cc;
                }
                double maxl = sqrt(dmax_(dmax_(d01, d12), d02));
                minh = 2 * vol / maxl;
            }
            b_minh = dbits(minh);
            // uniform, the Maxwell time is formed once by k_dt_finalize
            if (!uniform_maxwell_time(p)) b_maxwell = dbits(0.5 * p.mat.visc_min / (1e-40 + m_shearm(p, e)));
            // the diffusion time 0.5 minh^2 / kappa is non-decreasing in minh,
            // so its minimum over the elements is k_dt_finalize's 0.5 min(minh)^2 / kappa
        }
        double shp[ND][NPE];
        float s32[ND][NPE];   // a mixed context's FP32 shape functions (its rotation's)
        dw sdw[3][4];         // a mixed context's shape-function pairs
        if (flags & GEO_SHAPE) {
            if constexpr (ND == 3) {
                if (rel0) {   // the mixed context: double-word pairs (their high parts are the FP32 values)
                    rel_shape_fn_dw(re, c1, vol, sdw);
#pragma unroll
                    for (int k = 0; k < 3; ++k)
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const size_t o = ((size_t)k * 4 + i) * ne + e;
                            p.shpdw[o] = make_float2(sdw[k][i].hi, sdw[k][i].lo);
                            s32[k][i] = sdw[k][i].hi;
                        }
                } else {
                    shape_fn_elem<ND>(c, te, vol, shp);
                }
            } else {
                shape_fn_elem<ND>(c, te, vol, shp);
            }
            if (!rel0) {
#pragma unroll
                for (int k = 0; k < ND; ++k)
#pragma unroll
                    for (int i = 0; i < NPE; ++i) p.shp[((size_t)k * NPE + i) * ne + e] = shp[k][i];
            }
        } else if (flags & GEO_ROTATE) {
#pragma unroll
            for (int k = 0; k < ND; ++k)
#pragma unroll
                for (int i = 0; i < NPE; ++i) {
                    const size_t o = ((size_t)k * NPE + i) * ne + e;
                    if (rel0) s32[k][i] = p.shpdw[o].x;
                    else shp[k][i] = p.shp[o];
                }
        }
        // a mixed context's node velocities as double-word pairs (dw_split of
        // the FP64 values): the look-ahead reads the pairs the force pass
        // stored (KP::vdw), the other passes split the velocities
        dw vd[NPE][3];
        float w3 = 0, w4 = 0, w5 = 0;   // a mixed context's spin
        if (rel0 && ((flags & GEO_ROTATE) || AHEAD)) {
#pragma unroll
            for (int i = 0; i < NPE; ++i) {
                if constexpr (AHEAD) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) vd[i][d] = dw_of2(p.vdw[(size_t)d * p.nn + nodes[i]]);
                } else {
                    double vi[ND];
                    load_node_v<ND>(p, nodes[i], vi);
#pragma unroll
                    for (int d = 0; d < ND; ++d) vd[i][d] = dw_split(vi[d]);
                }
            }
        }
        if ((flags & GEO_ROTATE) && rel0) {
            // mixed step: spin from FP32 velocity differences (the pairs'
            // high parts, the nearest floats), FP32 Jaumann increments added
            // to the FP64 stress and strain.  Rounding the velocities to FP32
            // moves a difference by ~2^-23 |v|: against differences ~|v| h / L
            // across an element of size h in a field varying over L, a
            // relative error ~2^-23 L / h in the spin, whose increment dt W s
            // is itself ~1e-8 of the stress per step.
#pragma unroll
            for (int i = 1; i < NPE; ++i) {
                const float d0 = vd[i][0].hi - vd[0][0].hi, d1 = vd[i][1].hi - vd[0][1].hi,
                            d2 = vd[i][ND - 1].hi - vd[0][ND - 1].hi;
                const float sx = s32[0][i], sy = s32[1][i], sz = s32[ND - 1][i];
                w3 += 0.5f * (d0 * sy - d1 * sx);
                w4 += 0.5f * (d0 * sz - d2 * sx);
                w5 += 0.5f * (d1 * sz - d2 * sy);
            }
        }
        double qv_next = 0;   // the look-ahead: the next step's dvoldt term
        if constexpr (AHEAD && ND == 3) {   // the next step's element pass (k_elem_pass_mixed3's arithmetic)
            float2 h[3][3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int i = 1; i < 4; ++i) h[k][i - 1] = make_float2(sdw[k][i].hi, sdw[k][i].lo);
            double sr[6];
            strain_rate_mixed_vals(vd, h, sr);
#pragma unroll
            for (int cc = 0; cc < 6; ++cc) p.srate[cc * ne + e] = sr[cc];
            qv_next = elem_terms_mixed(p, e, sr, vol, s32, p.prm.has_thermal_diffusion != 0, false);
        }
        if ((flags & GEO_ROTATE) && rel0) {
            const float dtf = f32_of(p.clk->dt);
            double *arr[2] = {p.stress, p.strain};
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                double S[6];
#pragma unroll
                for (int cc = 0; cc < 6; ++cc) S[cc] = arr[a][cc * ne + e];
                // the isotropic part does not rotate: only normal-stress
                // differences enter.  Taken in FP32, each is off by ~2^-23
                // |S|, which the increment scales by dt |W| (~1e-8): ~1e-15
                // of the stress per step, of random sign
                const float S0 = f32_of(S[0]), S1 = f32_of(S[1]), S2 = f32_of(S[2]);
                const float d01 = S0 - S1, d02 = S0 - S2, d12 = S1 - S2;
                const float f3 = f32_of(S[3]), f4 = f32_of(S[4]), f5 = f32_of(S[5]);
                float si[6];
                si[0] = -2.0f * f3 * w3 - 2.0f * f4 * w4;
                si[1] = 2.0f * f3 * w3 - 2.0f * f5 * w5;
                si[2] = 2.0f * f4 * w4 + 2.0f * f5 * w5;
                si[3] = d01 * w3 - f4 * w5 - f5 * w4;
                si[4] = d02 * w4 + f3 * w5 - f5 * w3;
                si[5] = d12 * w5 + f3 * w4 + f4 * w3;
#pragma unroll
                for (int cc = 0; cc < 6; ++cc) arr[a][cc * ne + e] = S[cc] + f64_of(dtf * si[cc]);
            }
        } else if (flags & GEO_ROTATE) {
            double v[NPE][ND];
#pragma unroll
            for (int i = 0; i < NPE; ++i) load_node_v<ND>(p, nodes[i], v[i]);
            const double dt = p.clk->dt;
            double s[NSTR], es[NSTR];
#pragma unroll
            for (int cc = 0; cc < NSTR; ++cc) {
                s[cc] = p.stress[cc * ne + e];
                es[cc] = p.strain[cc * ne + e];
            }
            if (ND == 3) {
                double w3 = 0, w4 = 0, w5 = 0;
#pragma unroll
                for (int i = 0; i < NPE; ++i) w3 += 0.5 * (v[i][0] * shp[1][i] - v[i][1] * shp[0][i]);
#pragma unroll
                for (int i = 0; i < NPE; ++i) w4 += 0.5 * (v[i][0] * shp[ND - 1][i] - v[i][ND - 1] * shp[0][i]);
#pragma unroll
                for (int i = 0; i < NPE; ++i) w5 += 0.5 * (v[i][1] * shp[ND - 1][i] - v[i][ND - 1] * shp[1][i]);
                jaumann3(s, dt, w3, w4, w5);
                jaumann3(es, dt, w3, w4, w5);
            } else {
                double w2 = 0;
#pragma unroll
                for (int i = 0; i < NPE; ++i) w2 += 0.5 * (v[i][ND - 1] * shp[0][i] - v[i][0] * shp[ND - 1][i]);
                jaumann2(s, dt, w2);
                jaumann2(es, dt, w2);
            }
#pragma unroll
            for (int cc = 0; cc < NSTR; ++cc) {
                p.stress[cc * ne + e] = s[cc];
                p.strain[cc * ne + e] = es[cc];
            }
        }
        if (flags & GEO_MASS_TERMS) {
            // compute_mass element terms (geometry.cxx:313-365), as k_mass forms them
            const double rho_e = p.rho_e ? p.rho_e[e] : m_rho<ND>(p, e);
            const double pseudo_speed = p.prm.max_vbc_val * p.prm.inertial_scaling;
            const double rho = p.prm.is_quasi_static
                ? ((p.mat.nmat == 1) ? p.mat.rho_pseudo : m_bulkm(p, e) / (pseudo_speed * pseudo_speed))
                : rho_e;
            const double me = rho * vol / NPE;
            const double tme = p.prm.has_thermal_diffusion ? rho_e * m_cp(p, e) * vol / NPE : 0.0;
            if constexpr (AHEAD) {
                // what the next node pass gathers per support entry, in one
                // 32-byte record (one sector instead of four)
                p.ndpk[e] = make_double4(qv_next, vol, me, tme);
            } else {
                p.me[e] = me;
                if (p.prm.has_thermal_diffusion) p.tme[e] = tme;
            }
        }
    }
    if (do_dt) {   // uniform across the grid: every thread reaches the shuffles
        warp_block_min<ND>(b_minh, &p.clk->red_minh);
        if (!uniform_maxwell_time(p)) warp_block_min<ND>(b_maxwell, &p.clk->red_maxwell);
    }
}

// three blocks of 256 per SM (80 registers, ~150 bytes of spills to L1):
// 24 warps hide the node gathers' latency better than 16 with 128 registers
// (mixed step at 998,400 tets: 23 us less per step)
template <int ND>
__global__ void __launch_bounds__(TPB, 3) k_geometry(KP p, int flags)
{
    geometry_body<ND, false>(p, flags);
}

__global__ void __launch_bounds__(TPB, 3) k_geometry_ahead3(KP p, int flags)
{
    geometry_body<3, true>(p, flags);
}

// compute_dt final combination (geometry.cxx:294-309), single thread
template <int ND>
__global__ void k_dt_finalize(KP p, int only_on_step)
{
    Clock *ck = p.clk;
    if (only_on_step && ck->steps % 10 != 0) return;
    double dt;
    if (p.prm.fixed_dt != 0) {
        dt = p.prm.fixed_dt;
    } else {
        double minl = bitsd(ck->red_minh);
        const bool any = ck->red_minh != ~0ull;
        if (!any) minl = DBL_MAX;
        double dt_maxwell;
        if (uniform_maxwell_time(p)) dt_maxwell = any ? 0.5 * p.mat.visc_min / (1e-40 + m_shearm(p, 0)) : DBL_MAX;
        else dt_maxwell = ck->red_maxwell == ~0ull ? DBL_MAX : bitsd(ck->red_maxwell);
        double dt_diffusion = (any && p.prm.has_thermal_diffusion) ? 0.5 * minl * minl / p.mat.therm_diff_max : DBL_MAX;
        double dt_advection = 0.5 * minl / p.prm.max_vbc_val;
        double dt_elastic = p.prm.is_quasi_static
            ? 0.5 * minl / (p.prm.max_vbc_val * p.prm.inertial_scaling)
            : 0.5 * minl / sqrt(m_bulkm(p, 0) / m_rho<ND>(p, 0));
        dt = dmin_(dmin_(dt_elastic, dt_maxwell), dmin_(dt_advection, dt_diffusion)) * p.prm.dt_fraction;
        ck->last_dt_terms[0] = dt_maxwell;
        ck->last_dt_terms[1] = dt_diffusion;
        ck->last_dt_terms[2] = dt_advection;
        ck->last_dt_terms[3] = dt_elastic;
        if (dt <= 0) atomicOr(p.err, 0x100u);   // reported as DES_ERUNTIME
    }
    ck->dt = dt;
    ck->red_minh = ck->red_maxwell = ck->red_diffusion = ~0ull;
}

__global__ void k_dt_reset(KP p)
{
    p.clk->red_minh = p.clk->red_maxwell = p.clk->red_diffusion = ~0ull;
}

// ==================================================================
// compute_mass (geometry.cxx:313-365)
// ==================================================================
template <int ND>
__global__ void __launch_bounds__(TPB) k_mass(KP p)
{
    constexpr int NPE = ND + 1;
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const double pseudo_speed = p.prm.max_vbc_val * p.prm.inertial_scaling;
    const bool quasi = p.prm.is_quasi_static, thermal = p.prm.has_thermal_diffusion;
    const bool cs = ND == 3 && p.shpdw;   // a mixed context: compensated FP32 sums, as k_mass_sum's
    double vn = 0, ms = 0, tm = 0;
    dw_sum vs, mss, tms;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        int e = p.sup_ent[q] >> 2;
        double vol = p.vol[e];
        double rho_e = p.rho_e ? p.rho_e[e] : m_rho<ND>(p, e);
        double rho = quasi ? ((p.mat.nmat == 1) ? p.mat.rho_pseudo : m_bulkm(p, e) / (pseudo_speed * pseudo_speed))
                           : rho_e;
        double m = rho * vol / NPE;
        double tme = thermal ? rho_e * m_cp(p, e) * vol / NPE : 0.0;
        if (cs) {
            vs.add(dw_split(vol));
            mss.add(dw_split(m));
            if (thermal) tms.add(dw_split(tme));
        } else {
            vn += vol;
            ms += m;
            if (thermal) tm += tme;
        }
    }
    if (cs) {
        vn = vs.value();
        ms = mss.value();
        tm = tms.value();
    }
    p.vol_n[n] = vn;
    p.mass[n] = ms;
    p.tmass[n] = tm;
}

// the node sums of compute_mass from the element terms that the geometry
// pass wrote (GEO_MASS_TERMS): per pair 3 additions instead of the terms
template <int ND>
__global__ void __launch_bounds__(TPB) k_mass_sum(KP p)
{
    int n = p.n_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.n_hi) return;
    const bool thermal = p.prm.has_thermal_diffusion;
    if (ND == 3 && p.shpdw) {   // a mixed context: compensated FP32 sums (des_dw.cuh), as k_mass's
        dw_sum vs, mss, tms;
        for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
            const int e = p.sup_ent[q] >> 2;
            vs.add(dw_split(p.vol[e]));
            mss.add(dw_split(p.me[e]));
            if (thermal) tms.add(dw_split(p.tme[e]));
        }
        p.vol_n[n] = vs.value();
        p.mass[n] = mss.value();
        p.tmass[n] = thermal ? tms.value() : 0.0;
        return;
    }
    double vn = 0, ms = 0, tm = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        int e = p.sup_ent[q] >> 2;
        vn += p.vol[e];
        ms += p.me[e];
        if (thermal) tm += p.tme[e];
    }
    p.vol_n[n] = vn;
    p.mass[n] = ms;
    p.tmass[n] = tm;
}

// ==================================================================
// worst element quality (geometry.cxx:458-512)
// ==================================================================
template <int ND>
__device__ __forceinline__ double elem_quality(const KP &p, int e)
{
    constexpr int NPE = ND + 1;
    double c[NPE][ND];
#pragma unroll
    for (int i = 0; i < NPE; ++i) load_node_x<ND>(p, conn_at(p, i, e), c[i]);
    double vol = p.vol[e];
    if (ND == 3) {
        double normalization_factor = 216 * sqrt(3.0);
        double area_sum = (tri_area<3>(c[0], c[1], c[2]) + tri_area<3>(c[0], c[1], c[NPE - 1])
                           + tri_area<3>(c[2], c[NPE - 1], c[0]) + tri_area<3>(c[2], c[NPE - 1], c[1]));
        return normalization_factor * vol * vol / (area_sum * area_sum * area_sum);
    }
    double normalization_factor = 4 * sqrt(3.0);
    double d01 = 0, d12 = 0, d02 = 0;
#pragma unroll
    for (int k = 0; k < ND; ++k) {
        double a = c[1][k] - c[0][k], b = c[2][k] - c[1][k], cc = c[2][k] - c[0][k];
        d01 += a * a;
        d12 += b * b;
        d02 += cc * cc;
    }
    double dist2_sum = d01 + d12 + d02;
    return normalization_factor * vol / dist2_sum;
}

// red[0] = min quality bits (quality > 0), red[1] = smallest index at that minimum

// per-element fields of an output frame (output.cxx:146-173): density
// (MatProps::rho), mesh quality (elem_quality), viscosity (MatProps::visc of
// the current strain rate) and the most abundant marker's material
template <int ND>
__global__ void __launch_bounds__(TPB) k_output_elem(KP p, double *out)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne;
    double edot[NSTR];
#pragma unroll
    for (int c = 0; c < NSTR; ++c) edot[c] = p.srate[c * ne + e];
    out[e] = m_rho<ND>(p, e);
    out[ne + e] = elem_quality<ND>(p, e);
    out[2 * ne + e] = m_visc<ND>(p, e, edot);
    int best = 0, bc = -1;
    for (int m = 0; m < p.mat.nmat; ++m) {
        const int k = mcount(p, e, m);
        if (k > bc) {   // std::max_element: the first of equal maxima
            bc = k;
            best = m;
        }
    }
    out[3 * ne + e] = best;
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_quality_min(KP p, unsigned long long *red)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long b = ~0ull;
    if (e < p.ne) {
        double q = elem_quality<ND>(p, e);
        b = q > 0 ? dbits(q) : 0ull;
    }
    warp_block_min<ND>(b, &red[0]);
}

template <int ND>
__global__ void __launch_bounds__(TPB) k_quality_arg(KP p, unsigned long long *red)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    double q = elem_quality<ND>(p, e);
    unsigned long long b = q > 0 ? dbits(q) : 0ull;
    if (b == red[0]) atomicMin(&red[1], (unsigned long long)e);
}

// bad_mesh_quality's index scans (remeshing.cxx:1892-1919), one thread per
// element and node: red[2] = the first element whose volume is below
// smallest_vol, red[3] (check_bottom) = the first bottom node whose depth is
// farther than dist from z = bottom.  Each warp takes the smallest candidate
// index before one atomicMin, so the result is the first index whatever the
// order the blocks run in.
template <int ND>
__global__ void __launch_bounds__(TPB) k_quality_scans(KP p, double smallest_vol, double bottom, double dist,
                                                       int check_bottom, unsigned long long *red)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned small = 0xffffffffu, far = 0xffffffffu;
    if (i < p.ne && p.vol[i] < smallest_vol) small = (unsigned)i;
    if (check_bottom && i < p.nn && (p.bcflag[i] & BOUNDZ0)) {
        const double z = p.x[(size_t)(ND - 1) * p.nn + i];
        if (fabs(z - bottom) > dist) far = (unsigned)i;
    }
    small = __reduce_min_sync(0xffffffffu, small);
    far = __reduce_min_sync(0xffffffffu, far);
    if ((threadIdx.x & 31) == 0) {
        if (small != 0xffffffffu) atomicMin(&red[2], (unsigned long long)small);
        if (far != 0xffffffffu) atomicMin(&red[3], (unsigned long long)far);
    }
}

// ==================================================================
// material constants (see MatC): out[0..] = visc_coef[nmat], then for each
// of the 2*nmat plastic table entries anphi, anpsi, sqrt(anphi), tan(phi)
// ==================================================================
__global__ void k_material_table(KP p, double *out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int nm = p.mat.nmat;
    for (int m = 0; m < nm; ++m) out[m] = pow(0.75 * p.mat.visc_coefficient[m], p.mat.visc_pw1[m]);
    for (int k = 0; k < 2 * nm; ++k) {
        double an, ap, sq, tn;
        plastic_angles(p.mat.pt_phi[k], p.mat.pt_psi[k], an, ap, sq, tn);
        out[nm + 4 * k + 0] = an;
        out[nm + 4 * k + 1] = ap;
        out[nm + 4 * k + 2] = sq;
        out[nm + 4 * k + 3] = tn;
    }
}

int launch_material_table(const KP &p, cudaStream_t s, double *out)
{
    k_material_table<<<1, 1, 0, s>>>(p, out);
    return 1;
}

// the elements' marker-blended material properties (matprops.cxx:103-128)
// into out [EP_COUNT][ne], by the functions a kernel would otherwise call
// per use (hmean, amean, and the division of m_hr_over_cp)
__global__ void __launch_bounds__(TPB) k_elem_props(KP p, double *out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne;
    const double cp = amean(p, p.mat.heat_capacity, 2, e), hr = amean(p, p.mat.radiogenic_heating, 3, e);
    out[EP_BULKM * ne + e] = hmean(p, p.mat.bulk_modulus, 0, e);
    out[EP_SHEARM * ne + e] = hmean(p, p.mat.shear_modulus, 1, e);
    out[EP_CP * ne + e] = cp;
    out[EP_HR * ne + e] = hr;
    out[EP_K * ne + e] = amean(p, p.mat.therm_cond, 4, e);
    out[EP_HR_OVER_CP * ne + e] = hr / cp;
}

int launch_elem_props(const KP &p, cudaStream_t s, double *out)
{
    KP q = p;
    q.eprop = nullptr;
    k_elem_props<<<nblocks(p.ne), TPB, 0, s>>>(q, out);
    return 1;
}

// ==================================================================
// AoS <-> SoA
// ==================================================================
__global__ void k_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, int n, int nc)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)n * nc) return;
    long long r = i / nc, c = i - r * nc;
    soa[c * n + r] = aos[i];
}

__global__ void k_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, int n, int nc)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)n * nc) return;
    long long r = i / nc, c = i - r * nc;
    aos[i] = soa[c * n + r];
}

// rows [lo, hi) of several fields between AoS staging and SoA arrays; a
// thread's flat index only grows, so its field index only grows
template <bool UP>
__global__ void __launch_bounds__(TPB) k_rows(const __grid_constant__ RowTable t)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    int k = 0;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < t.total; g += stride) {
        while (g >= t.f[k].first + (long long)(t.f[k].hi - t.f[k].lo) * t.f[k].nc) ++k;
        const RowField &f = t.f[k];
        const long long j = g - f.first;
        const long long r = f.lo + j / f.nc, c = j % f.nc;
        const size_t aos = (size_t)r * f.nc + c, soa = (size_t)c * f.n + r;
        if (UP) {
            f.dev[soa] = f.stage[aos];
        } else {
            f.stage[aos] = f.dw ? f64_of(dw_of2(f.dw[soa])) : f.dev[soa];
        }
    }
}

// ==================================================================
// launchers
// ==================================================================
#define DISPATCH(KERNEL, GRID, ...)                                       \
    do {                                                                  \
        if (p.nd == 3) KERNEL<3><<<(GRID), TPB, 0, s>>>(__VA_ARGS__);     \
        else KERNEL<2><<<(GRID), TPB, 0, s>>>(__VA_ARGS__);               \
    } while (0)

int launch_strain_rate(const KP &p, cudaStream_t s, bool begin_step)
{
    DISPATCH(k_strain_rate, nblocks(p.ne), p, (int)begin_step);
    return 1;
}

int launch_heat_gather(const KP &p, cudaStream_t s)
{
    if (p.nd == 3) k_node_gather1<3, true, false><<<nblocks(p.nn), TPB, 0, s>>>(p);
    else k_node_gather1<2, true, false><<<nblocks(p.nn), TPB, 0, s>>>(p);
    return 1;
}

int launch_dvoldt(const KP &p, cudaStream_t s)
{
    if (p.nd == 3) k_node_gather1<3, false, true><<<nblocks(p.nn), TPB, 0, s>>>(p);
    else k_node_gather1<2, false, true><<<nblocks(p.nn), TPB, 0, s>>>(p);
    return 1;
}

int launch_elem_pass(const KP &p, cudaStream_t s, bool heat)
{
    DISPATCH(k_elem_pass, nblocks(p.e_hi - p.e_lo), p, (int)heat);
    return 1;
}

int launch_node_pass(const KP &p, cudaStream_t s, bool heat)
{
    DISPATCH(k_node_pass, nblocks(p.n_hi - p.n_lo), p, (int)heat);
    return 1;
}

int launch_heat_and_dvoldt(const KP &p, cudaStream_t s)
{
    if (p.nd == 3) k_node_gather1<3, true, true><<<nblocks(p.nn), TPB, 0, s>>>(p);
    else k_node_gather1<2, true, true><<<nblocks(p.nn), TPB, 0, s>>>(p);
    return 1;
}

int launch_temperature_update(const KP &p, cudaStream_t s)
{
    k_temperature_update<<<nblocks(p.nn), TPB, 0, s>>>(p);
    return 1;
}

int launch_edvoldt(const KP &p, cudaStream_t s)
{
    DISPATCH(k_edvoldt, nblocks(p.ne), p);
    return 1;
}

int launch_update_stress(const KP &p, cudaStream_t s, bool fused)
{
    DISPATCH(k_update_stress, nblocks(p.e_hi - p.e_lo), p, (int)fused);
    return 1;
}

int launch_nmd_gather(const KP &p, cudaStream_t s, bool stored)
{
    DISPATCH(k_nmd_gather, nblocks(p.n_hi - p.n_lo), p, (int)(stored && p.pv));
    return 1;
}

int launch_nmd_correct(const KP &p, cudaStream_t s, bool with_facets)
{
    long long n = (long long)(p.e_hi - p.e_lo) + (with_facets ? p.f_hi - p.f_lo : 0);
    if (uses_force_terms(p)) {
        k_nmd_correct_ft3<<<nblocks(n), TPB, 0, s>>>(p, (int)with_facets);
        return 1;
    }
    DISPATCH(k_nmd_correct, nblocks(n), p, (int)with_facets);
    return 1;
}

int launch_force_terms(const KP &p, cudaStream_t s)
{
    if (!uses_force_terms(p)) return 0;
    k_force_terms3<<<nblocks(p.e_hi - p.e_lo), TPB, 0, s>>>(p);
    return 1;
}

int launch_facet_forces(const KP &p, cudaStream_t s)
{
    if (p.nbf == 0) return 0;
    DISPATCH(k_facet_forces, nblocks(p.nbf), p);
    return 1;
}

int launch_force(const KP &p, cudaStream_t s, bool fused_motion, bool contract)
{
    if (contract && uses_force_terms(p)) {
        k_force_dw3<<<nblocks(p.n_hi - p.n_lo), TPB, 0, s>>>(p, (int)fused_motion);
        return 1;
    }
    if (contract) {
        if (p.nd == 3) k_force<3, true><<<nblocks(p.n_hi - p.n_lo), TPB, 0, s>>>(p, (int)fused_motion);
        else k_force<2, true><<<nblocks(p.n_hi - p.n_lo), TPB, 0, s>>>(p, (int)fused_motion);
        return 1;
    }
    DISPATCH(k_force, nblocks(p.n_hi - p.n_lo), p, (int)fused_motion);
    return 1;
}

int launch_velocity(const KP &p, cudaStream_t s, bool contract)
{
    const int g = nblocks((long long)p.nn * p.nd);
    if (contract) {
        if (p.nd == 3) k_velocity<3, true><<<g, TPB, 0, s>>>(p);
        else k_velocity<2, true><<<g, TPB, 0, s>>>(p);
        return 1;
    }
    DISPATCH(k_velocity, g, p);
    return 1;
}

int launch_vbcs(const KP &p, cudaStream_t s)
{
    DISPATCH(k_vbcs, nblocks(p.nn), p);
    return 1;
}

int launch_coordinate(const KP &p, cudaStream_t s, bool contract)
{
    const int g = nblocks((long long)p.nn * p.nd);
    if (contract) {
        if (p.nd == 3) k_coordinate<3, true><<<g, TPB, 0, s>>>(p);
        else k_coordinate<2, true><<<g, TPB, 0, s>>>(p);
        return 1;
    }
    DISPATCH(k_coordinate, g, p);
    return 1;
}

int launch_geometry(const KP &p, cudaStream_t s, int flags)
{
    DISPATCH(k_geometry, nblocks(p.e_hi - p.e_lo), p, flags);
    return 1;
}

int launch_geometry_ahead(const KP &p, cudaStream_t s, int flags)
{
    k_geometry_ahead3<<<nblocks(p.e_hi - p.e_lo), TPB, 0, s>>>(p, flags);
    return 1;
}

int launch_mass(const KP &p, cudaStream_t s)
{
    DISPATCH(k_mass, nblocks(p.nn), p);
    return 1;
}

int launch_mass_sum(const KP &p, cudaStream_t s)
{
    DISPATCH(k_mass_sum, nblocks(p.n_hi - p.n_lo), p);
    return 1;
}

int launch_dt_finalize(const KP &p, cudaStream_t s, bool only_on_step)
{
    if (p.nd == 3) k_dt_finalize<3><<<1, 1, 0, s>>>(p, (int)only_on_step);
    else k_dt_finalize<2><<<1, 1, 0, s>>>(p, (int)only_on_step);
    return 1;
}

int launch_dt_reset(const KP &p, cudaStream_t s)
{
    k_dt_reset<<<1, 1, 0, s>>>(p);
    return 1;
}

int launch_output_elem(const KP &p, double *out, cudaStream_t s)
{
    DISPATCH(k_output_elem, nblocks(p.ne), p, out);
    return 1;
}

int launch_quality(const KP &p, cudaStream_t s, unsigned long long *red)
{
    DISPATCH(k_quality_min, nblocks(p.ne), p, red);
    DISPATCH(k_quality_arg, nblocks(p.ne), p, red);
    return 2;
}

int launch_quality_scans(const KP &p, cudaStream_t s, double smallest_vol, double bottom, double dist,
                         int check_bottom, unsigned long long *red)
{
    DISPATCH(k_quality_scans, nblocks(std::max(p.ne, p.nn)), p, smallest_vol, bottom, dist, check_bottom, red);
    return 1;
}

__global__ void k_f64_to_f32(const double *__restrict__ a, float *__restrict__ b, long long n)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = f32_of(a[i]);   // as the mixed geometry pass rounds them
}

int launch_f64_to_f32(const double *a, float *b, long long n, cudaStream_t s)
{
    k_f64_to_f32<<<nblocks(n), TPB, 0, s>>>(a, b, n);
    return 1;
}

// a mixed 3D context's shape functions: the double-word pairs -> FP64 (for downloads)
__global__ void k_shp_join(const float2 *__restrict__ w, double *__restrict__ a, long long n)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) a[i] = f64_of(dw_of2(w[i]));
}

int launch_shp_join(const KP &p, cudaStream_t s)
{
    if (!p.shpdw) return 0;
    const long long n = (long long)p.ne * p.npe * p.nd;
    k_shp_join<<<nblocks(n), TPB, 0, s>>>(p.shpdw, p.shp, n);
    return 1;
}

int launch_aos_to_soa(const double *aos, double *soa, int n, int ncomp, cudaStream_t s)
{
    k_aos_to_soa<<<nblocks((long long)n * ncomp), TPB, 0, s>>>(aos, soa, n, ncomp);
    return 1;
}

int launch_soa_to_aos(const double *soa, double *aos, int n, int ncomp, cudaStream_t s)
{
    k_soa_to_aos<<<nblocks((long long)n * ncomp), TPB, 0, s>>>(soa, aos, n, ncomp);
    return 1;
}

int launch_rows(const RowTable &t, bool up, cudaStream_t s)
{
    if (t.total <= 0) return 0;
    const int grid = (int)(t.total < 152LL * 8 * TPB ? nblocks(t.total) : 152 * 8);
    if (up) k_rows<true><<<grid, TPB, 0, s>>>(t);
    else k_rows<false><<<grid, TPB, 0, s>>>(t);
    return 1;
}

}  // namespace des
