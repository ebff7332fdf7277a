// des_mixed_elem.cuh -- the per-element work of the mixed step's element
// pass (strain rate, dvoldt term, heat terms) on values held in registers.
// The element pass (k_elem_pass_mixed3) loads them from memory; the
// look-ahead geometry pass of the chained step (k_geometry_ahead3) forms the
// shape functions itself and hands them over directly.  Both call these
// functions, so both form the very same bits.
#pragma once

#include "des_common.cuh"
#include "des_dw.cuh"

namespace des {

// strain rate (fields.cxx:166-232) from the velocity differences to node 0.
// Each product dv_i,k * dN_i/dx_l is of the size of the whole row k of the
// velocity gradient, so an FP32 sum carries an absolute error ~eps32 |L|
// into every component.  In the shear components that is harmless, but the
// normal components set the volumetric rate, which the pressure integrates
// with the bulk modulus (through the nodal-mixed dvoldt): in FP32 they alone
// moved the stress by 1e-4 (relative L2) in 150 steps of a yielding case.
// So the normal components are double-word dot products (des_dw.cuh) of the
// double-word velocity differences and shape functions, rounded to FP64
// (~2^-45 of the row's terms), the shear ones FP32 from the pairs' high parts.
//   v: the four nodes' velocities as double-word pairs (dw_split of the FP64
//   values); h[k][i - 1]: the pair of dN_i/dx_k, i = 1..3
__device__ __forceinline__ void strain_rate_mixed_vals(const dw (*v)[3], const float2 (*h)[3], double *out)
{
    dw w0[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) w0[d] = dw_neg(v[0][d]);
    dw dd[3][3];
    float dv[3][3], sx[3], sy[3], sz[3];
#pragma unroll
    for (int i = 1; i < 4; ++i) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            dd[i - 1][d] = dw_add(v[i][d], w0[d]);
            dv[i - 1][d] = dd[i - 1][d].hi;
        }
        sx[i - 1] = h[0][i - 1].x;
        sy[i - 1] = h[1][i - 1].x;
        sz[i - 1] = h[2][i - 1].x;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        out[k] = f64_of(dw_dot3c(dd[0][k], dw_of2(h[k][0]), dd[1][k], dw_of2(h[k][1]), dd[2][k], dw_of2(h[k][2])));
    float s3 = 0, s4 = 0, s5 = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        s3 += 0.5f * (dv[i][0] * sy[i] + dv[i][1] * sx[i]);
        s4 += 0.5f * (dv[i][0] * sz[i] + dv[i][2] * sx[i]);
        s5 += 0.5f * (dv[i][1] * sz[i] + dv[i][2] * sy[i]);
    }
    out[3] = f64_of(s3);
    out[4] = f64_of(s4);
    out[5] = f64_of(s5);
}

// the four nodes' velocities of element e as double-word pairs
__device__ __forceinline__ void load_elem_v_dw(const KP &p, int e, dw (*v)[3])
{
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double vi[3];
        load_node_v<3>(p, conn_at(p, i, e), vi);
#pragma unroll
        for (int d = 0; d < 3; ++d) v[i][d] = dw_split(vi[d]);
    }
}

// The element's dvoldt term (geometry.cxx:127-135), returned and (store_qv)
// stored, and, with heat, its four heat terms (fields.cxx:99-146): the
// stencil on FP64 temperature differences (sum_j D_ij = 0), FP32 products.
// sr: the element's strain rate; s32[k][i]: dN_i/dx_k in FP32 (the pairs'
// high parts).
__device__ __forceinline__ double elem_terms_mixed(const KP &p, int e, const double *sr, double vol,
                                                   const float (*s32)[4], bool heat, bool store_qv = true)
{
    const size_t ne = p.ne;
    const double qv = (sr[0] + sr[1] + sr[2]) * vol;
    if (store_qv) p.qv[e] = qv;
    if (!heat) return qv;
    double T[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) T[i] = p.T[conn_at(p, i, e)];
    // D_ij = D_ji and f32_of(T_i - T_j) = -f32_of(T_j - T_i) bit for bit,
    // so each of the six products serves both rows
    float P[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i + 1; j < 4; ++j) {
            const float D = s32[0][i] * s32[0][j] + s32[1][i] * s32[1][j] + s32[2][i] * s32[2][j];
            const float t = D * f32_of(T[j] - T[i]);
            P[i][j] = t;
            P[j][i] = -t;
        }
    const bool k_const = (p.mat.nmat == 1) && !p.ef[DES_EF_THERM_COND];
    const float volf = f32_of(vol);
    const float kv = f32_of(k_const ? p.mat.therm_cond[0] : m_k(p, e)) * volf;
    const float rh = f32_of(m_hr_over_cp(p, e)) * volf;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float diffusion = 0.0f;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j != i) diffusion += P[i][j];
        p.hc[(size_t)i * ne + e] = kv * diffusion - rh;
    }
    return qv;
}

}  // namespace des
