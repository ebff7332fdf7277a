// des_mixed.cu -- kernels of the mixed-precision step (DES_PREC_MIXED).
//
// On GB300 an FP64 instruction issues at 1/64 of the FP32 rate, and the FP64
// step is FP64-pipe-bound (update_stress keeps the FP64 pipe ~86% busy).
// The mixed step keeps every state variable, every stress and strain
// increment and every nodal sum in FP64, and moves to FP32 the expensive
// work whose result is a coefficient or a small correction:
//
// * the viscosity (Arrhenius power law: pow, exp; the harmonic mean over
//   the element's materials), evaluated to ~2e-7 with FP32 transcendentals
//   on an exact exponent split (visc_mixed);
// * the Mohr-Coulomb yield test: the DEVIATORIC trial stress is
//   diagonalised in FP32 (branch-free cyclic Jacobi) to screen out the
//   elements that are elastic by a margin above the FP32 error bound; the
//   others -- everything at or beyond yield -- run the FP64 return map
//   (FP64 eigen-solve), so plastic flow is never computed in FP32;
// * the shear strain rates, the spin and the heat stencil: sums of products
//   of shape function derivatives with nodal values whose sum over the
//   element vanishes, evaluated in FP32 on FP64 differences (v_i - v_0,
//   T_j - T_i); the Jaumann rotation increments.  The normal strain rates
//   stay FP64 (see k_strain_rate_mixed3).
// The elastic and Maxwell increments stay FP64: the quasi-static explicit
// scheme integrates their rounding without dissipating it (damping option 2
// only scales the force), and in FP32 they alone moved the stress by 4e-6
// (relative L2) after 2000 steps of the 998,400-tet workload.
// Element volumes, shape functions, forces and masses stay FP64.
#include "des_kernels.cuh"
#include "des_rheology.cuh"
#include "des_mixed.cuh"
#include "des_dw.cuh"
#include "des_mixed_elem.cuh"

namespace des {

constexpr int TPB_M = 256;

__device__ __forceinline__ float shp32_at(const KP &p, int k, int i, int e)
{
    return p.shpdw[((size_t)k * 4 + i) * p.ne + e].x;   // the pair's high part: the nearest float
}

static inline int nblocks_m(long long n)
{
    long long b = (n + TPB_M - 1) / TPB_M;
    return (int)(b < 1 ? 1 : b);
}

// exp(x) for |x| < 690 as 2^k exp(r): any integer k near x / ln 2 keeps |r|
// small, so k is rounded in FP32; r = x - k ln 2 is one FP64 fma; 2^k goes
// into the exponent field of expf(r) (in [0.7, 1.5], so the result stays
// normal).  Within ~1.5e-7 of exp(x).
__device__ __forceinline__ double exp_mixed(double x)
{
    const double LN2 = 0.6931471805599453;
    const float kf = fminf(fmaxf(rintf(f32_of(x) * 1.44269504f), -1000.0f), 1000.0f);
    const float rr = f32_of(fma(-f64_of(kf), LN2, x));
    const double m = f64_of(expf(rr));
    return __hiloint2double(__double2hiint(m) + ((int)kf << 20), __double2loint(m));
}

// ln visc_m of material m from ln(edot_II) and 1/T, clamped exactly to
// [visc_min, visc_max] on ln visc, then exp_mixed (visc_mixed's terms)
__device__ __forceinline__ double visc_law_mixed(const KP &p, int m, double ln_ed, double r)
{
    const double lnv = fma(p.mat.visc_qnr[m], r, fma(p.mat.visc_pw[m], ln_ed, p.mat.visc_lnc[m]));
    if (lnv <= p.mat.visc_lnmin) return p.mat.visc_min;
    if (!(lnv < p.mat.visc_lnmax)) return p.mat.visc_max;   // also T = 0 (1/T infinite), as the FP64 law
    return exp_mixed(lnv);
}

// visc_mixed over the element's markers.  One material present: its law
// (n / (n / visc) = visc).  Several: the harmonic mean.  Out of line: the
// registers of the blend stay out of the one-material kernels.
static __device__ __noinline__ double visc_blend_mixed(const KP &p, int e, double ln_ed, double r)
{
    int mone = -1, present = 0;
    for (int m = 0; m < p.mat.nmat; ++m)
        if (mcount(p, e, m)) {
            mone = m;
            ++present;
        }
    if (present == 1) return visc_law_mixed(p, mone, ln_ed, r);
    double result = 0;
    int n = 0;
    for (int m = 0; m < p.mat.nmat; ++m) {
        const int k = mcount(p, e, m);
        if (k == 0) continue;
        double lnv = fma(p.mat.visc_qnr[m], r, fma(p.mat.visc_pw[m], ln_ed, p.mat.visc_lnc[m]));
        lnv = fmin(fmax(lnv, p.mat.visc_lnmin - 50), p.mat.visc_lnmax + 50);
        result = fma((double)k, exp_mixed(-lnv), result);
        n += k;
    }
    return dmin_(dmax_(n / result, p.mat.visc_min), p.mat.visc_max);
}

// Arrhenius power-law viscosity (matprops.cxx:276-312), per material m
//   ln visc_m = ln(0.25e6 coef_m) + pw_m ln(edot_II) + Q_m / (n_m R T),
// with every term kept to ~1e-8 absolute at ~10 FP64 operations:
// ln(edot_II) = logf(mantissa) + exponent ln 2 (the FP32 log only sees
// [0.5, 1)); 1/T from an FP32 seed and one FP64 Newton step; exp by
// exp_mixed.  One material in the element: the clamps to [visc_min,
// visc_max] are exact on ln visc.  Several: the harmonic mean over the
// element's markers,
// n / sum_m k_m exp(-ln visc_m), over the materials it holds (each ln visc_m
// limited to 50 beyond the clamps, which moves no clamped mean), then the
// clamps.  The result is within ~2e-7 of the FP64 law.  Every FP64 <-> FP32
// conversion is f32_of / f64_of (integer instructions).
__device__ __forceinline__ double visc_mixed(const KP &p, int e, const double *edot, double T)
{
    if (p.ef[DES_EF_LOG10_VISC]) return m_visc<3>(p, e, edot);
    const double LN2 = 0.6931471805599453;
    float t[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = f32_of(edot[i]);
    const float a = (t[0] + t[1] + t[2]) * (1.0f / 3.0f);
    const float j2 = 0.5f * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a))
        + t[3] * t[3] + t[4] * t[4] + t[5] * t[5];
    const float ed = fmaxf(sqrtf(j2), 1e-30f);
    int ex;
    const float mant = frexpf(ed, &ex);
    const double ln_ed = fma(f64_of((float)ex), LN2, f64_of(logf(mant)));
    double r = f64_of(1.0f / f32_of(T));
    r = r * fma(-T, r, 2.0);
    if (p.mat.nmat == 1) return visc_law_mixed(p, 0, ln_ed, r);
    return visc_blend_mixed(p, e, ln_ed, r);
}

// maxwell (rheology.cxx:118-134).  The relaxation coefficients come from
// FP32: tmp = dt G / (2 visc) and f2 - 1 = -tmp / (1 + tmp), each within
// ~2^-22 of itself (the viscosity they scale is good to ~2e-7), so f1 =
// 1 - tmp and f2 are one FP64 addition each instead of two FP64 Newton
// reciprocals.  The updates are fused multiply-adds, and the mean stress
// and K dv are added to the deviator in one step.  The divisions by 3 are
// div3, bit-identical.
struct MaxwellCoef {
    double f1, f2;
};

__device__ __forceinline__ MaxwellCoef maxwell_coef(double shearm, double viscosity, double dt)
{
    const float tf = (0.5f * f32_of(dt) * f32_of(shearm)) / f32_of(viscosity);
    return {1 - f64_of(tf), 1 + f64_of(-tf / (1.0f + tf))};
}

// the update on the old normal deviator x_i = s_i - s0 and y_i = 2G (de_i -
// tr(de)/3); s0k = s0 + K dv; s and de for the shear components
__device__ __forceinline__ void maxwell_mixed_xy(const MaxwellCoef &c, double g2, double s0k, const double *x,
                                                 const double *y, const double *s, const double *de, double *out)
{
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = fma(fma(x[i], c.f1, y[i]), c.f2, s0k);
#pragma unroll
    for (int i = 3; i < 6; ++i) out[i] = fma(s[i], c.f1, g2 * de[i]) * c.f2;
}

__device__ __forceinline__ void maxwell_mixed(double bulkm, double shearm, double viscosity, double dt, double dv,
                                              const double *de, double *s)
{
    const double dev = div3(de[0] + de[1] + de[2]);
    const double s0 = div3(s[0] + s[1] + s[2]);
    const double g2 = 2 * shearm;
    double x[3], y[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        x[i] = s[i] - s0;
        y[i] = g2 * (de[i] - dev);
    }
    maxwell_mixed_xy(maxwell_coef(shearm, viscosity, dt), g2, s0 + bulkm * dv, x, y, s, de, s);
}

// elastic_ (rheology.cxx:13-40) with fused multiply-adds: 2G de_i + lambda tr(de)
// as one fma, each shear update as one fma (rounding an ulp from elastic_'s)
__device__ __forceinline__ void elastic_mixed(double bulkm, double shearm, const double *de, double *s)
{
    const double lambda = bulkm - 2. / 3 * shearm;
    const double ldev = lambda * (de[0] + de[1] + de[2]);
    const double g2 = 2 * shearm;
#pragma unroll
    for (int i = 0; i < 3; ++i) s[i] += fma(g2, de[i], ldev);
#pragma unroll
    for (int i = 3; i < 6; ++i) s[i] = fma(g2, de[i], s[i]);
}

// ------------------------------------------------------------------
// The mixed EVP branch in increment form.  Both candidates of the branch
// choice (rheology.cxx:594-634) are the old stress s plus an FP32 increment
// added in FP64:
//   Maxwell (rheology.cxx:118-134)  dv = c1 x + f2 y + K dv_vol   (normal),
//                                        c1 x + f2 y              (shear),
//   elastic trial (elastic_)        dp = y + K tr(de)             (normal),
//                                        y                        (shear),
// x the old deviator (s_i - s0 for the normal components, the old shear
// stress), y = 2G (de - tr(de)/3) (normal) and 2G de (shear) the trial's
// deviatoric increment, f2 = 1 / (1 + tmp), c1 = f1 f2 - 1 = -2 tmp f2
// with f1 = 1 - tmp and tmp = dt G / (2 visc): the Maxwell update
// (x f1 + y) f2 + s0 + K dv_vol less the old stress.  The increments are
// small against the stress (a few hundred Pa per step against ~1e8 Pa in
// the 998,400-tet workload), so their FP32 rounding (~2^-23 of themselves)
// moves the stress by ~1e-5 Pa per step, while the FP64 additions keep the
// state's own precision: 6 FP64 additions per candidate instead of the 16
// FP64 operations of the FP64-coefficient update.
// ------------------------------------------------------------------
struct MaxwellF {
    float c1, f2;
};

__device__ __forceinline__ MaxwellF maxwell_coef_f(double shearm, double viscosity, double dt)
{
    const float tf = (0.5f * f32_of(dt) * f32_of(shearm)) / f32_of(viscosity);
    const float f2 = 1.0f / (1.0f + tf);
    return {-2.0f * tf * f2, f2};
}

// relative volume change vol / vol_old - 1 in FP32 from the FP64 difference
// (exact for volumes within a factor 2 of each other)
__device__ __forceinline__ float dvol_f(const KP &p, int e)
{
    const double vo = p.vol_old[e];
    return f32_of(p.vol[e] - vo) / f32_of(vo);
}

// The branch choice svII < spII of the mixed step, decided from FP32 values
// where an identity allows.  The comparison it stands for is the FP64 one of
// the FP64 candidates (those the branch forms where the screen is
// undecided): the elastic trial sp = elastic_mixed(s, de) and the Maxwell
// update sv = maxwell_mixed_xy(x, y) with f1 = 1 - tmp, f2 = 1 / (1 + tmp).
// Their exact deviators are q = x + y and f2 (q - tmp x), so
//   J2(sv) - J2(sp) = -f2^2 tmp Q,  Q = (2 + tmp) J(q) + 2 <q, x> - tmp J(x),
// J(v) = (v0^2 + v1^2 + v2^2) / 2 + v3^2 + v4^2 + v5^2, <,> its bilinear
// form: the Maxwell candidate wins exactly when Q > 0.  Q carries no
// cancellation (for a small increment q ~ x and Q ~ 4 J(q)), so its FP32
// value decides the comparison wherever f2^2 tmp |Q| clears the FP64
// comparison's own roundings, even in cold elements whose relaxation tmp
// (~1e-8 per step) lies below FP32's resolution of the stress.
//   Inputs: xf, yf, qf the FP32 forms of x, y, q (per component, xf within
// 2^-24 |xf| of x plus 2^-50 S for the FP64 mean; yf, formed from FP32
// strain increments, within 2^-22 (|yf| + Y) of the FP64 y, Y = 2G sum
// |de_i|; qf within the sum of both plus 2^-24 |qf|).  The bound on
// |Q_est - Q| sums, per component with weights 1 (normal) and 2 (shear),
// the first-order terms of those errors in J(q), <q, x> and J(x) with their
// squares, and 2^-20 of the absolute terms for Q's own FP32 evaluation.
// R bounds the FP64 side: two second_invariant2_ evaluations (each within
// 12 u J + 12.25 u S sqrt(J) + 37.5 u^2 S^2, j2_est3's analysis) and the
// candidates' roundings (2 u S per component), taken as 2^-45 J + 2^-45 S
// sqrt(J) + (2^-46 S)^2 with J ~ Jq (margins of 8 and more), and the FP32 rounding of f2 - 1 in maxwell_coef
// (2^-23 tmp relative, times J(q) + 2 tmp |<q, x>| + tmp^2 J(x), taken as
// 2^-20 tmp of the absolute terms).  Returns 1 (Maxwell), 0 (elasto-
// plastic: not svII < spII, ties included) or -1 (undecided, or tmp not
// positive, or a non-finite input).
__device__ __forceinline__ int evp_choice_f(const float *xf, const float *yf, const float *qf, float tf, float Y,
                                            float S)
{
    const float e64 = 0x1p-50f * S;
    float jq2 = 0.0f, jx2 = 0.0f, c2 = 0.0f, Aqx = 0.0f, Eqq = 0.0f, Eqx = 0.0f, Exx = 0.0f;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const float wt = c < 3 ? 1.0f : 2.0f;
        const float aq = fabsf(qf[c]), ax = fabsf(xf[c]);
        jq2 += wt * qf[c] * qf[c];
        jx2 += wt * xf[c] * xf[c];
        c2 += wt * qf[c] * xf[c];
        Aqx += wt * aq * ax;
        const float ex = 0x1p-24f * ax + e64;
        const float eq = ex + 0x1p-22f * (fabsf(yf[c]) + Y) + 0x1p-24f * aq;
        Eqq += wt * eq * (2.0f * aq + eq);
        Eqx += wt * (eq * ax + ex * aq + eq * ex);
        Exx += wt * ex * (2.0f * ax + ex);
    }
    const float Q = 0.5f * (2.0f + tf) * jq2 + c2 - 0.5f * tf * jx2;
    const float absQ = (2.0f + tf) * jq2 + Aqx + tf * jx2;
    const float EQ = 0.5f * (2.0f + tf) * Eqq + Eqx + 0.5f * tf * Exx + 0x1p-20f * absQ;
    const float f2 = 1.0f / (1.0f + tf);
    const float G = f2 * f2 * tf;
    const float h = 0x1p-46f * S;
    const float R = 0x1p-46f * jq2 + 0x1p-46f * S * sqrtf(2.0f * jq2) + h * h + 0x1p-20f * tf * absQ + 0x1p-100f;
    if (!(tf > 0.0f)) return -1;
    if (G * (Q - EQ) > R) return 1;
    if (G * (Q + EQ) < -R) return 0;
    return -1;
}

// relative volume change (rheology.cxx:569,600: vol / vol_old - 1) as
// (vol - vol_old) (1 / vol_old): the difference is exact for volumes within a
// factor 2 of each other, and recip_newton's ~1e-14 relative error scales the
// ~1e-8 volume change, against the ~1e-16 absolute rounding of the quotient
// form; one FP64 division fewer
__device__ __forceinline__ double dvol_mixed(const KP &p, int e)
{
    const double vo = p.vol_old[e];
    return (p.vol[e] - vo) * recip_newton(vo);
}

// The mixed EVP branch where the FP32 screens leave it to FP64: the FP64
// candidates -- the trial as the EP branch forms it (through the return map
// unless the yield screen passed it) and the Maxwell update with FP64 terms
// -- and, for an undecided choice (vless < 0), their FP64 comparison.  Out
// of line: the elements that need it are few (yielding or near-tied), and
// the registers of the return map stay out of the common path.
__device__ __noinline__ unsigned evp_fp64_candidates(const KP &p, int e, double dt, double bulkm, double shearm,
                                                     double visc, double s0, bool elastic, int vless, double amc,
                                                     double anphi, double anpsi, double hardn, double ten_max,
                                                     const double *edot, double *s, double &pls, double &dpls)
{
    unsigned bits = 0;
    double de[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) de[i] = edot[i] * dt;
    const double dev = div3((de[0] + de[1]) + de[2]);
    const double g2 = 2 * shearm;
    double x[3], y[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        x[i] = s[i] - s0;
        y[i] = g2 * (de[i] - dev);
    }
    double sp[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) sp[i] = s[i];
    elastic_mixed(bulkm, shearm, de, sp);
    double depls = 0;
    if (!elastic && mc_return_<3>(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, depls, sp))
        bits |= DES_DEV_QL_NOCONV;
    double sv[6];
    if (vless < 0) {
        maxwell_mixed_xy(maxwell_coef(shearm, visc, dt), g2, s0 + bulkm * dvol_mixed(p, e), x, y, s, de, sv);
        vless = second_invariant2_<3>(sv) < second_invariant2_<3>(sp);
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = vless ? sv[i] : sp[i];
    if (!vless) {
        pls += depls;
        dpls = depls;
    }
    return bits;
}

// update_stress (rheology.cxx:510-646), 3D, mixed precision
// three blocks of 256 per SM (at most 85 registers; the spills stay in L1):
// 24 resident warps instead of 16 at 128 registers, 15 us less at 998,400 tets
__global__ void __launch_bounds__(TPB_M, 3) k_update_stress_mixed3(KP p, int fused)
{
    int e = p.e_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.e_hi) return;
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
        const double corr = div3(edv - div);   // as the FP64 step rounds it
#pragma unroll
        for (int i = 0; i < 3; ++i) edot[i] += corr;
    }
    const int rt = p.mat.rheol_type;
    double de[6];
    if (rt != DES_RH_EVP) {
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            de[i] = edot[i] * dt;
            es[i] += de[i];
        }
    }
    double dpv = 0;   // dpressure
    bool dp_set = false;
    const double bulkm = m_bulkm(p, e), shearm = m_shearm(p, e);
    const double T = elem_avg_T<4>(p, e);
    unsigned bits = 0;
    if (rt == DES_RH_ELASTIC) {
        elastic_mixed(bulkm, shearm, de, s);
    } else if (rt == DES_RH_VISCOUS) {
        viscous_<3>(bulkm, visc_mixed(p, e, edot, T), es[0] + es[1] + es[2], edot, s);
    } else if (rt == DES_RH_MAXWELL) {
        maxwell_mixed(bulkm, shearm, visc_mixed(p, e, edot, T), dt, dvol_mixed(p, e), de, s);
    } else if (rt == DES_RH_EP) {
        double amc, anphi, anpsi, hardn, ten_max;
        m_plastic_props(p, e, pls, amc, anphi, anpsi, hardn, ten_max);
        elastic_mixed(bulkm, shearm, de, s);
        const double am = div3(s[0] + s[1] + s[2]);
        const double q[3] = {s[0] - am, s[1] - am, s[2] - am};
        double depls = 0;
        if (!clearly_elastic3_dev(amc, anphi, ten_max, am, q, s)
            && mc_return_<3>(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, depls, s))
            bits |= DES_DEV_QL_NOCONV;
        pls += depls;
        dpls = depls;
    } else {   // EVP: the smaller second invariant wins (rheology.cxx:594-634)
        double amc, anphi, anpsi, hardn, ten_max;
        m_plastic_props(p, e, pls, amc, anphi, anpsi, hardn, ten_max);
        // FP32 strain increments; the strain accumulates them in FP64
        const float dtf = f32_of(dt);
        float def[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            def[i] = f32_of(edot[i]) * dtf;
            es[i] += f64_of(def[i]);
        }
        const double s0 = div3(old_s);
        const float g2f = 2.0f * f32_of(shearm), kf = f32_of(bulkm);
        const float trdef = (def[0] + def[1]) + def[2];
        const float devf = trdef * (1.0f / 3.0f);
        // x: the old deviator; y: the trial's deviatoric increment
        float xf[6], yf[6];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            xf[i] = f32_of(s[i] - s0);
            yf[i] = g2f * (def[i] - devf);
            xf[i + 3] = f32_of(s[i + 3]);
            yf[i + 3] = g2f * def[i + 3];
        }
        const double visc = visc_mixed(p, e, edot, T);
        const MaxwellF mc = maxwell_coef_f(shearm, visc, dt);
        const float tf = (0.5f * dtf * f32_of(shearm)) / f32_of(visc);
        const float dmp = kf * trdef;
        float qf[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) qf[c] = xf[c] + yf[c];
        // the yield screen on the trial deviator qf: against the deviator of
        // the FP64 trial elastic_mixed(s, de) it is off by xf's and qf's
        // roundings and by yf's distance from the FP64 y (2^-22 of
        // Lx + Ly + Y per component, taken as 2^-21 in the 2-norm) and by
        // the FP64 roundings of the mean (22 u S, taken as 2^-44 S)
        const float s0f = f32_of(s0);
        float Y = 0.0f, Sdev = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i) Y += fabsf(def[i]);
        Y *= g2f;
#pragma unroll
        for (int c = 0; c < 6; ++c) Sdev += fabsf(xf[c]) + fabsf(yf[c]);
        Sdev += Y;
        const float S = fabsf(s0f) + Sdev + 2.0f * fabsf(kf) * (Y / fmaxf(g2f, 1e-30f));
        const bool elastic = clearly_elastic3_f(f32_of(anphi), f32_of(amc), f32_of(ten_max), s0f + dmp,
                                                fabsf(s0f) + fabsf(dmp), qf, 0x1p-44f * S + 0x1p-21f * Sdev);
        int vless = elastic ? evp_choice_f(xf, yf, qf, tf, Y, S) : -1;
        if (vless == 1) {
            // the Maxwell update as the old stress plus its FP32 increment
            const float dmv = kf * dvol_f(p, e);
            float dn = 0.0f;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float d = fmaf(xf[i], mc.c1, fmaf(yf[i], mc.f2, dmv));
                s[i] += f64_of(d);
                dn += d;
                s[i + 3] += f64_of(fmaf(xf[i + 3], mc.c1, yf[i + 3] * mc.f2));
            }
            dpv = f64_of(dn);
            dp_set = true;
        } else {
            bits |= evp_fp64_candidates(p, e, dt, bulkm, shearm, visc, s0, elastic, vless, amc, anphi, anpsi, hardn,
                                        ten_max, edot, s, pls, dpls);
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
    const double dpf = dp_set ? dpv : (s[0] + s[1] + s[2]) - old_s;
    p.dp[e] = dpf;
    if (fused && p.pv) {   // the NMD gather's double-word dp vol, formed once per element instead of per node
        const dw w = dw_mul(dw_split(dpf), dw_split(p.vol[e]));
        p.pv[e] = make_float2(w.hi, w.lo);
    }
    if (fused && p.rho_e) {
        const double rho = m_rho_T(p, e, T);
        p.rho_e[e] = rho;
        if (p.buoy_e) p.buoy_e[e] = p.prm.gravity != 0 ? rho * p.prm.gravity / 4 : 0.0;
    }
    if (bits) set_err(p, bits);
}

// strain rate (fields.cxx:166-232) of one element, loaded from memory and
// formed by strain_rate_mixed_vals (des_mixed_elem.cuh)
__device__ __forceinline__ void strain_rate_mixed_elem(const KP &p, int e, double *out)
{
    const size_t ne = p.ne;
    dw v[4][3];
    float2 h[3][3];   // dN_i/dx_k of slots 1..3 as double-word pairs
    load_elem_v_dw(p, e, v);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 1; i < 4; ++i) h[k][i - 1] = p.shpdw[((size_t)k * 4 + i) * ne + e];
    strain_rate_mixed_vals(v, h, out);
#pragma unroll
    for (int c = 0; c < 6; ++c) p.srate[c * ne + e] = out[c];
}

__global__ void __launch_bounds__(TPB_M) k_strain_rate_mixed3(KP p, int begin_step)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (begin_step && e == 0) {
        p.clk->steps += 1;
        p.clk->time += p.clk->dt;
    }
    if (e >= p.ne) return;
    double sr[6];
    strain_rate_mixed_elem(p, e, sr);
}

// heat stencil on FP64 temperature differences (sum_j D_ij = 0), FP32
// products, a compensated FP32 nodal sum of the heat terms; dvoldt in FP64
// (fields.cxx:99-146, geometry.cxx:111-155)
__global__ void __launch_bounds__(TPB_M) k_heat_dvoldt_mixed3(KP p, int heat, int do_dvoldt)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const double Tn = p.T[n];
    const bool k_const = (p.mat.nmat == 1) && !p.ef[DES_EF_THERM_COND];
    dw_sum tsum;   // a compensated FP32 sum of the heat terms (des_dw.cuh)
    double dvoldt = 0;
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
                diffusion += D * f32_of(p.T[conn_at(p, j, e)] - Tn);
            }
            const float volf = f32_of(vol);
            const float kv = f32_of(k_const ? p.mat.therm_cond[0] : m_k(p, e)) * volf;
            const float rh = f32_of(m_hr_over_cp(p, e)) * volf;
            tsum.add(kv * diffusion - rh);
        }
        if (do_dvoldt) {
            const double dj = p.srate[e] + p.srate[(size_t)p.ne + e] + p.srate[2 * (size_t)p.ne + e];
            dvoldt += dj * vol;
        }
    }
    if (heat) p.tdot[n] = tsum.value();
    if (do_dvoldt) p.ntmp[n] = dvoldt / p.vol_n[n];
}

// ------------------------------------------------------------------
// Fused step: strain rate, heat, dvoldt and the temperature update as one
// element pass and one node pass.  The per-pair work of the node-centric
// gather above (k_heat_dvoldt_mixed3: the stencil row of the node's slot,
// four temperature differences and their FP32 conversions, which issue on
// the FP64 pipe) is done once per element: the element pass stores the
// four FP32 heat terms of the element and its dvoldt term, and the node
// pass sums them over the support list in ascending element order.  Each
// term is the very value the gather forms for that (node, element) pair,
// and the sums run in the same order, so the result is bit-identical to
// k_strain_rate_mixed3 + k_heat_dvoldt_mixed3 + k_temperature_update.
// ------------------------------------------------------------------
__global__ void __launch_bounds__(TPB_M) k_elem_pass_mixed3(KP p, int heat)
{
    int e = p.e_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 0) {   // var.steps++; var.time += var.dt (dynearthsol.cxx:325-326)
        p.clk->steps += 1;
        p.clk->time += p.clk->dt;
    }
    if (e >= p.e_hi) return;
    double sr[6];
    strain_rate_mixed_elem(p, e, sr);
    float s32[3][4];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) s32[k][i] = shp32_at(p, k, i, e);
    elem_terms_mixed(p, e, sr, p.vol[e], s32, heat);
}

// The node pass: heat and dvoldt sums, the temperature update.  In the
// chained step (mass_sums) it also forms the previous step's compute_mass
// sums (volume_n, mass, tmass) from the element records that the look-ahead
// geometry pass wrote (KP::ndpk), as k_mass_sum forms them, and (begin_step) starts the
// step's clock, which the look-ahead pass could not: the step's dt is final
// only after k_dt_finalize.
__global__ void __launch_bounds__(TPB_M) k_node_pass_mixed3(KP p, int heat, int mass_sums, int begin_step)
{
    if (begin_step && blockIdx.x == 0 && threadIdx.x == 0) {   // dynearthsol.cxx:325-326
        p.clk->steps += 1;
        p.clk->time += p.clk->dt;
    }
    int n = p.n_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.n_hi) return;
    const size_t ne = p.ne;
    const int q0 = p.sup_off[n], q1 = p.sup_off[n + 1];
    double vol_n, tmass = 0;
    // the heat terms in a compensated FP32 sum (des_dw.cuh), as
    // k_heat_dvoldt_mixed3 sums them; the dvoldt terms in FP64: they cancel
    // between a node's elements, and the 2^-47 of a double-word split of
    // each moved the volumetric rate enough to change the default damping's
    // copysign at some nodes within ten steps
    dw_sum tsum;
    double dvoldt = 0;
    if (mass_sums) {
        // one pass over the support: the mass sums in compensated FP32
        // (des_dw.cuh), as k_mass_sum's, from the look-ahead pass's records
        const bool thermal = p.prm.has_thermal_diffusion;
        dw_sum vs, mss, tms;
        for (int q = q0; q < q1; ++q) {
            const int ent = p.sup_ent[q];
            const int e = ent >> 2, i = ent & 3;
            const double4 r = p.ndpk[e];   // qv, vol, me, tme
            vs.add(dw_split(r.y));
            mss.add(dw_split(r.z));
            if (thermal) tms.add(dw_split(r.w));
            if (heat) tsum.add(p.hc[(size_t)i * ne + e]);
            dvoldt += r.x;
        }
        vol_n = vs.value();
        tmass = thermal ? tms.value() : 0.0;
        p.vol_n[n] = vol_n;
        p.mass[n] = mss.value();
        p.tmass[n] = tmass;
    } else {
        vol_n = p.vol_n[n];
        if (heat) tmass = p.tmass[n];
        for (int q = q0; q < q1; ++q) {
            const int ent = p.sup_ent[q];
            const int e = ent >> 2, i = ent & 3;
            if (heat) tsum.add(p.hc[(size_t)i * ne + e]);
            dvoldt += p.qv[e];
        }
    }
    const double tdot = tsum.value();
    p.ntmp[n] = dvoldt / vol_n;
    if (heat) {   // temperature update + Dirichlet BC (fields.cxx:151-162)
        const unsigned flag = p.bcflag[n];
        if (flag & BOUNDZ1) p.T[n] = p.prm.surface_temperature;
        else if ((flag & BOUNDZ0) && !p.prm.has_fixed_bottom_temperature) p.T[n] = p.prm.mantle_temperature;
        else p.T[n] -= tdot * p.clk->dt / tmass;
    }
}

int launch_update_stress_mixed(const KP &p, cudaStream_t s, bool fused)
{
    k_update_stress_mixed3<<<nblocks_m(p.e_hi - p.e_lo), TPB_M, 0, s>>>(p, (int)fused);
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



int launch_elem_pass_mixed(const KP &p, cudaStream_t s, bool heat)
{
    k_elem_pass_mixed3<<<nblocks_m(p.e_hi - p.e_lo), TPB_M, 0, s>>>(p, (int)heat);
    return 1;
}

int launch_node_pass_mixed(const KP &p, cudaStream_t s, bool heat, bool mass_sums, bool begin_step)
{
    k_node_pass_mixed3<<<nblocks_m(p.n_hi - p.n_lo), TPB_M, 0, s>>>(p, (int)heat, (int)mass_sums, (int)begin_step);
    return 1;
}

}  // namespace des
