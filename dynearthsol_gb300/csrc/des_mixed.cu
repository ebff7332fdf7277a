// des_mixed.cu -- kernels of the mixed-precision step (DES_PREC_MIXED).
//
// On GB300 an FP64 instruction issues at 1/64 of the FP32 rate, and the FP64
// step is FP64-pipe-bound (update_stress keeps the FP64 pipe ~86% busy).
// The mixed step keeps every state variable, every stress and strain
// increment and every nodal sum in FP64, and moves to FP32 the expensive
// work whose result is a coefficient or a small correction:
//
// * the viscosity (Arrhenius power law: pow, exp), evaluated to ~2e-7 with
//   FP32 transcendentals on an exact exponent split (visc_mixed);
// * the Mohr-Coulomb return map's eigen-solve: the DEVIATORIC trial stress
//   is diagonalised in FP32 (branch-free cyclic Jacobi); the principal
//   stresses, yield functions and plastic multiplier are formed in FP64 and
//   the correction -alam * sum_k c_k v_k v_k^T (FP32 tensor, FP64 scale and
//   sum) is applied to the FP64 trial stress;
// * strain rate, spin and the heat stencil: sums of products of shape
//   function derivatives with nodal values whose sum over the element
//   vanishes, evaluated in FP32 on FP64 differences (v_i - v_0, T_j - T_i)
//   so that nothing cancels in FP32; the Jaumann rotation increments.
// The elastic and Maxwell increments stay FP64: the quasi-static explicit
// scheme integrates their rounding without dissipating it (damping option 2
// only scales the force), and in FP32 they alone moved the stress by 4e-6
// (relative L2) after 2000 steps of the 998,400-tet workload.
// Element volumes, shape functions, forces and masses stay FP64.
#include "des_kernels.cuh"
#include "des_rheology.cuh"
#include "des_mixed.cuh"

namespace des {

constexpr int TPB_M = 256;

__device__ __forceinline__ float shp32_at(const KP &p, int k, int i, int e)
{
    return p.shp32[((size_t)k * 4 + i) * p.ne + e];
}

static inline int nblocks_m(long long n)
{
    long long b = (n + TPB_M - 1) / TPB_M;
    return (int)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------------
// FP32 cyclic Jacobi for a symmetric 3x3 matrix (Jacobi 1846; the stable
// rotation formulas of Rutishauser, as in Golub & Van Loan, "Matrix
// Computations", sec. 8.5).  Fixed sweep count: no data-dependent branches
// besides skipping exact zeros.  v[r][k] is component r of eigenvector k.
// ------------------------------------------------------------------
template <int P, int Q>
__device__ __forceinline__ void jrot(float (&a)[3][3], float (&v)[3][3])
{
    constexpr int R = 3 - P - Q;
    const float apq = a[P][Q];
    if (apq == 0.0f) return;
    const float theta = __fdividef(a[Q][Q] - a[P][P], 2.0f * apq);
    // |theta| -> inf (negligible apq) gives t = 0: no rotation
    const float at = fabsf(theta);
    const float t = copysignf(__frcp_rn(at + __fsqrt_rn(fmaf(at, at, 1.0f))), theta);
    const float c = rsqrtf(fmaf(t, t, 1.0f));
    const float s = t * c;
    const float tau = __fdividef(s, 1.0f + c);
    a[P][P] -= t * apq;
    a[Q][Q] += t * apq;
    a[P][Q] = a[Q][P] = 0.0f;
    const float arp = a[R][P], arq = a[R][Q];
    a[R][P] = a[P][R] = arp - s * (arq + tau * arp);
    a[R][Q] = a[Q][R] = arq + s * (arp - tau * arq);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float vkp = v[k][P], vkq = v[k][Q];
        v[k][P] = vkp - s * (vkq + tau * vkp);
        v[k][Q] = vkq + s * (vkp - tau * vkq);
    }
}

// eigenvalues ascending in w, eigenvectors in the columns of v
__device__ __forceinline__ void jacobi3f(const float d[6], float w[3], float (&v)[3][3])
{
    float a[3][3] = {{d[0], d[3], d[4]}, {d[3], d[1], d[5]}, {d[4], d[5], d[2]}};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? 1.0f : 0.0f;
#pragma unroll
    for (int sweep = 0; sweep < 4; ++sweep) {
        jrot<0, 1>(a, v);
        jrot<0, 2>(a, v);
        jrot<1, 2>(a, v);
    }
    w[0] = a[0][0];
    w[1] = a[1][1];
    w[2] = a[2][2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = (k == 1) ? 1 : 0, j = i + 1;
        if (w[i] > w[j]) {
            float t = w[i];
            w[i] = w[j];
            w[j] = t;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                float b = v[r][i];
                v[r][i] = v[r][j];
                v[r][j] = b;
            }
        }
    }
}

// Arrhenius power-law viscosity (matprops.cxx:276-312) for nmat == 1:
//   ln visc = ln(0.25e6 coef) + pw ln(edot_II) + Q / (n R T),
// with every term kept to ~1e-8 absolute at ~10 FP64 operations:
// ln(edot_II) = logf(mantissa) + exponent ln 2 (the FP32 log only sees
// [0.5, 1)); 1/T from an FP32 seed and one FP64 Newton step; exp(ln visc) =
// 2^k expf(r) with |r| <= ln2/2; the clamps to [visc_min, visc_max] are
// exact.  The resulting viscosity is within ~2e-7 of the FP64 law.
__device__ __forceinline__ double visc_mixed(const KP &p, int e, const double *edot, double T)
{
    if (p.mat.nmat != 1 || p.ef[DES_EF_LOG10_VISC]) return m_visc<3>(p, e, edot);
    const double LN2 = 0.6931471805599453, INV_LN2 = 1.4426950408889634;
    float t[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = (float)edot[i];
    const float a = (t[0] + t[1] + t[2]) * (1.0f / 3.0f);
    const float j2 = 0.5f * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a))
        + t[3] * t[3] + t[4] * t[4] + t[5] * t[5];
    const float ed = fmaxf(sqrtf(j2), 1e-30f);
    int ex;
    const float mant = frexpf(ed, &ex);
    const double ln_ed = (double)logf(mant) + (double)ex * LN2;
    double r = (double)(1.0f / (float)T);
    r = r * (2.0 - T * r);
    const double lnv = p.mat.visc_lnc + p.mat.visc_pw[0] * ln_ed + p.mat.visc_qnr * r;
    if (lnv <= p.mat.visc_lnmin) return p.mat.visc_min;
    if (lnv >= p.mat.visc_lnmax) return p.mat.visc_max;
    const double k = rint(lnv * INV_LN2);
    const float rr = (float)(lnv - k * LN2);
    return ldexp((double)expf(rr), (int)k);
}

// Mohr-Coulomb return map (rheology.cxx:151-299) on the FP64 trial stress s
// (already holding the elastic trial), FP32 eigen-solve of its deviator.
__device__ __forceinline__ unsigned elasto_plastic_mixed(double bulkm, double shearm, double amc, double anphi,
                                                         double anpsi, double hardn, double ten_max,
                                                         double &depls, double *s)
{
    depls = 0;
    const double m = (s[0] + s[1] + s[2]) * (1.0 / 3);
    float d[6] = {(float)(s[0] - m), (float)(s[1] - m), (float)(s[2] - m), (float)s[3], (float)s[4], (float)s[5]};
    float w[3], v[3][3];
    jacobi3f(d, w, v);
    double p0 = m + (double)w[0], p2 = m + (double)w[2];
    double fs = p0 - p2 * anphi + amc;
    double ft = p2 - ten_max;
    if (fs > 0 && ft < 0) return 0;
    double pa = sqrt(1 + anphi * anphi) + anphi;
    double ps = ten_max * anphi - amc;
    double h = p2 - ten_max + pa * (p0 - ps);
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double alam;
    float c[3];
    if (h < 0) {
        alam = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2 * sqrt(anphi) * hardn);
        c[0] = (float)(a1 - a2 * anpsi);
        c[1] = (float)(a2 - a2 * anpsi);
        c[2] = (float)(a2 - a1 * anpsi);
        depls = fabs(alam) * sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18);
    } else {
        alam = ft / a1;
        c[0] = (float)a2;
        c[1] = (float)a2;
        c[2] = (float)a1;
        depls = fabs(alam) * sqrt(7. / 18);
    }
    // s -= alam * sum_k c_k v_k v_k^T
    float M[6];
    M[0] = c[0] * v[0][0] * v[0][0] + c[1] * v[0][1] * v[0][1] + c[2] * v[0][2] * v[0][2];
    M[1] = c[0] * v[1][0] * v[1][0] + c[1] * v[1][1] * v[1][1] + c[2] * v[1][2] * v[1][2];
    M[2] = c[0] * v[2][0] * v[2][0] + c[1] * v[2][1] * v[2][1] + c[2] * v[2][2] * v[2][2];
    M[3] = c[0] * v[0][0] * v[1][0] + c[1] * v[0][1] * v[1][1] + c[2] * v[0][2] * v[1][2];
    M[4] = c[0] * v[0][0] * v[2][0] + c[1] * v[0][1] * v[2][1] + c[2] * v[0][2] * v[2][2];
    M[5] = c[0] * v[1][0] * v[2][0] + c[1] * v[1][1] * v[2][1] + c[2] * v[1][2] * v[2][2];
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] -= alam * (double)M[i];
    return 0;
}

// update_stress (rheology.cxx:510-646), 3D, mixed precision
__global__ void __launch_bounds__(TPB_M) k_update_stress_mixed3(KP p, int fused)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne;
    double edv;
    if (fused) {
        double dj = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) dj += p.ntmp[conn_at(p, i, e)];
        edv = dj / 4;
        p.edvoldt[e] = edv;
    } else {
        edv = p.edvoldt[e];
    }
    double s[6], es[6], edot[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        s[c] = p.stress[c * ne + e];
        es[c] = p.strain[c * ne + e];
        edot[c] = p.srate[c * ne + e];
    }
    double pls = p.pls[e], dpls = p.dpls[e];
    const double dt = p.clk->dt;
    const double old_s = s[0] + s[1] + s[2];
    {
        const double div = edot[0] + edot[1] + edot[2];
        const double corr = (edv - div) * (1.0 / 3);
#pragma unroll
        for (int i = 0; i < 3; ++i) edot[i] += corr;
    }
    double de[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        de[i] = edot[i] * dt;
        es[i] += de[i];
    }
    const int rt = p.mat.rheol_type;
    const double bulkm = m_bulkm(p, e), shearm = m_shearm(p, e);
    const double T = elem_avg_T<4>(p, e);
    unsigned bits = 0;
    if (rt == DES_RH_ELASTIC) {
        elastic_<3>(bulkm, shearm, de, s);
    } else if (rt == DES_RH_VISCOUS) {
        viscous_<3>(bulkm, visc_mixed(p, e, edot, T), es[0] + es[1] + es[2], edot, s);
    } else if (rt == DES_RH_MAXWELL) {
        const double dv = p.vol[e] / p.vol_old[e] - 1;
        maxwell_<3>(bulkm, shearm, visc_mixed(p, e, edot, T), dt, dv, de, s);
    } else {
        double amc, anphi, anpsi, hardn, ten_max;
        m_plastic_props(p, e, pls, amc, anphi, anpsi, hardn, ten_max);
        double sp[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) sp[i] = s[i];
        elastic_<3>(bulkm, shearm, de, sp);
        double depls = 0;
        bits |= elasto_plastic_mixed(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, depls, sp);
        if (rt == DES_RH_EP) {
#pragma unroll
            for (int i = 0; i < 6; ++i) s[i] = sp[i];
            pls += depls;
            dpls = depls;
        } else {   // EVP: the smaller second invariant wins (rheology.cxx:594-634)
            const double dv = p.vol[e] / p.vol_old[e] - 1;
            double sv[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) sv[i] = s[i];
            maxwell_<3>(bulkm, shearm, visc_mixed(p, e, edot, T), dt, dv, de, sv);
            const double svII = second_invariant2_<3>(sv), spII = second_invariant2_<3>(sp);
            if (svII < spII) {
#pragma unroll
                for (int i = 0; i < 6; ++i) s[i] = sv[i];
            } else {
#pragma unroll
                for (int i = 0; i < 6; ++i) s[i] = sp[i];
                pls += depls;
                dpls = depls;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        p.stress[c * ne + e] = s[c];
        p.strain[c * ne + e] = es[c];
        p.srate[c * ne + e] = edot[c];
    }
    p.pls[e] = pls;
    p.dpls[e] = dpls;
    p.dp[e] = (s[0] + s[1] + s[2]) - old_s;
    if (fused && p.rho_e) p.rho_e[e] = m_rho_T(p, e, T);
    if (bits) set_err(p, bits);
}

// strain rate (fields.cxx:166-232) from FP64 velocity differences, FP32 sums
__global__ void __launch_bounds__(TPB_M) k_strain_rate_mixed3(KP p, int begin_step)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (begin_step && e == 0) {
        p.clk->steps += 1;
        p.clk->time += p.clk->dt;
    }
    if (e >= p.ne) return;
    double v0[3];
    load_node_v<3>(p, conn_at(p, 0, e), v0);
    float dv[3][3], sx[3], sy[3], sz[3];
#pragma unroll
    for (int i = 1; i < 4; ++i) {
        double vi[3];
        load_node_v<3>(p, conn_at(p, i, e), vi);
#pragma unroll
        for (int d = 0; d < 3; ++d) dv[i - 1][d] = (float)(vi[d] - v0[d]);
        sx[i - 1] = shp32_at(p, 0, i, e);
        sy[i - 1] = shp32_at(p, 1, i, e);
        sz[i - 1] = shp32_at(p, 2, i, e);
    }
    float s[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        s[0] += dv[i][0] * sx[i];
        s[1] += dv[i][1] * sy[i];
        s[2] += dv[i][2] * sz[i];
        s[3] += 0.5f * (dv[i][0] * sy[i] + dv[i][1] * sx[i]);
        s[4] += 0.5f * (dv[i][0] * sz[i] + dv[i][2] * sx[i]);
        s[5] += 0.5f * (dv[i][1] * sz[i] + dv[i][2] * sy[i]);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) p.srate[(size_t)c * p.ne + e] = (double)s[c];
}

// heat stencil on FP64 temperature differences (sum_j D_ij = 0), FP32
// products, FP64 nodal sum; dvoldt in FP64 (fields.cxx:99-146, geometry.cxx:111-155)
__global__ void __launch_bounds__(TPB_M) k_heat_dvoldt_mixed3(KP p, int heat, int do_dvoldt)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const double Tn = p.T[n];
    const bool k_const = (p.mat.nmat == 1) && !p.ef[DES_EF_THERM_COND];
    double tdot = 0, dvoldt = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        const int ent = p.sup_ent[q];
        const int e = ent >> 2, i = ent & 3;
        const double vol = p.vol[e];
        if (heat) {
            const float sxi = shp32_at(p, 0, i, e), syi = shp32_at(p, 1, i, e), szi = shp32_at(p, 2, i, e);
            float diffusion = 0.0f;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (j == i) continue;
                const float D = sxi * shp32_at(p, 0, j, e) + syi * shp32_at(p, 1, j, e)
                    + szi * shp32_at(p, 2, j, e);
                diffusion += D * (float)(p.T[conn_at(p, j, e)] - Tn);
            }
            const float volf = (float)vol;
            const float kv = (float)(k_const ? p.mat.therm_cond[0] : m_k(p, e)) * volf;
            const float rh = (float)((p.mat.nmat == 1) ? p.mat.hr_over_cp : (m_hr(p, e) / m_cp(p, e))) * volf;
            tdot += (double)(kv * diffusion - rh);
        }
        if (do_dvoldt) {
            const double dj = p.srate[e] + p.srate[(size_t)p.ne + e] + p.srate[2 * (size_t)p.ne + e];
            dvoldt += dj * vol;
        }
    }
    if (heat) p.tdot[n] = tdot;
    if (do_dvoldt) p.ntmp[n] = dvoldt / p.vol_n[n];
}

int launch_update_stress_mixed(const KP &p, cudaStream_t s, bool fused)
{
    k_update_stress_mixed3<<<nblocks_m(p.ne), TPB_M, 0, s>>>(p, (int)fused);
    return 1;
}

int launch_strain_rate_mixed(const KP &p, cudaStream_t s, bool begin_step)
{
    k_strain_rate_mixed3<<<nblocks_m(p.ne), TPB_M, 0, s>>>(p, (int)begin_step);
    return 1;
}

int launch_heat_and_dvoldt_mixed(const KP &p, cudaStream_t s, bool heat, bool dvoldt)
{
    k_heat_dvoldt_mixed3<<<nblocks_m(p.nn), TPB_M, 0, s>>>(p, (int)heat, (int)dvoldt);
    return 1;
}



}  // namespace des
