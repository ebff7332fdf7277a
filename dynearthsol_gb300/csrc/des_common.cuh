// des_common.cuh -- device data layout and shared device helpers of the
// GB300 explicit-step library.
//
// Layout in HBM (structure of arrays, component-major):
//   node fields   x[d*nn + n], v[d*nn + n], f[d*nn + n], T[n], mass[n], ...
//   element fields stress[c*ne + e] (c = XX,YY,ZZ,XY,XZ,YZ; 2D: XX,ZZ,XZ),
//                  shp[(k*npe + i)*ne + e] (k = x,y,z derivative, i = local node)
//   connectivity   conn[i*ne + e]
//   support CSR    sup_off[nn+1], sup_ent[] = e*4 + local slot, ascending e
//                  (the reference's support lists, mesh.cxx:1707-1721, in the
//                  serial summation order of its element loops)
// Every node quantity the reference scatters element by element is gathered
// here per node in that same order: no atomics, reproducible results.
#pragma once

#include <cstdint>
#include <cfloat>
#include <cmath>

#include "../../include/desgpu.h"

#define DES_MAXMAT 8

namespace des {

constexpr unsigned BOUNDX0 = 1u << 0, BOUNDX1 = 1u << 1, BOUNDY0 = 1u << 2, BOUNDY1 = 1u << 3,
                   BOUNDZ0 = 1u << 4, BOUNDZ1 = 1u << 5, BOUND_ANY = 1023u;

// constants.hpp:73-74
constexpr double DEG2RAD = 3.1415926535897932384626433832795 / 180;

// device clock of a context (Variables::time, dt, steps)
struct Clock {
    double time;
    double dt;
    int steps;
    int pad;
    // compute_dt accumulators: min over elements as ordered bit patterns
    unsigned long long red_minh;
    unsigned long long red_maxwell;
    unsigned long long red_diffusion;   // unused: the diffusion time comes from red_minh
    double last_dt_terms[4];   // maxwell, diffusion, advection, elastic
};

// material table (MatProps, matprops.hpp:19-76) with nmat <= DES_MAXMAT
struct MatC {
    int rheol_type, nmat, is_plane_strain;
    unsigned scalar_mask;
    double visc_min, visc_max, tension_max, therm_diff_max;
    double rho0[DES_MAXMAT], alpha[DES_MAXMAT];
    double bulk_modulus[DES_MAXMAT], shear_modulus[DES_MAXMAT];
    double visc_exponent[DES_MAXMAT], visc_coefficient[DES_MAXMAT], visc_activation_energy[DES_MAXMAT];
    double heat_capacity[DES_MAXMAT], therm_cond[DES_MAXMAT], radiogenic_heating[DES_MAXMAT];
    double pls0[DES_MAXMAT], pls1[DES_MAXMAT];
    double cohesion0[DES_MAXMAT], cohesion1[DES_MAXMAT];
    double friction_angle0[DES_MAXMAT], friction_angle1[DES_MAXMAT];
    double dilation_angle0[DES_MAXMAT], dilation_angle1[DES_MAXMAT];
    // material constants hoisted out of the per-element work.  Each is
    // computed once with the very operation the per-element code would
    // perform on the same operands (on the device for the transcendental
    // ones), so using it changes no bit of the result.
    double visc_pw[DES_MAXMAT];      // 1 / n - 1               (matprops.cxx:298)
    double visc_pw1[DES_MAXMAT];     // -1 / n                  (matprops.cxx:299)
    double visc_coef[DES_MAXMAT];    // pow(0.75 * A, -1 / n)   (matprops.cxx:300)
    double rho_pseudo;               // bulkm / (v_max * inertial_scaling)^2 (geometry.cxx:348-349), nmat == 1
    double visc_lnc[DES_MAXMAT];     // ln(0.25e6 * visc_coef[m])   (mixed step)
    double visc_lnmin, visc_lnmax;   // ln(visc_min), ln(visc_max)  (mixed step)
    double visc_qnr[DES_MAXMAT];     // Q / (n R)                   (mixed step)
    // every material's viscosity law is positive wherever T > 0 (A > 0, Q >= 0,
    // n > 0), so a material without markers in the element adds exactly +0
    // to the harmonic sum of MatProps::visc and can be skipped
    int visc_skip_empty;
    double hr_over_cp;               // hr / cp (fields.cxx:118), nmat == 1
    // plastic_props at the material's start / saturated angles
    // (matprops.cxx:365-372): entry 2m at (phi0, psi0), 2m+1 at (phi1, psi1)
    int pt_n;
    double pt_phi[2 * DES_MAXMAT], pt_psi[2 * DES_MAXMAT];
    double pt_anphi[2 * DES_MAXMAT], pt_anpsi[2 * DES_MAXMAT];
    double pt_sqrt_anphi[2 * DES_MAXMAT], pt_tanphi[2 * DES_MAXMAT];
    double pt_coh_over_tan[2 * DES_MAXMAT];   // cohesion0 / tan(phi0), cohesion1 / tan(phi1)
    double hardening[DES_MAXMAT];             // (cohesion1 - cohesion0) / (pls1 - pls0)
};

// Everything a kernel needs, passed by value.
struct KP {
    int nd, npe, nstr, nn, ne, nbf;
    // index ranges of one launch of the fused step's kernels: elements
    // [e_lo, e_hi), nodes [n_lo, n_hi), boundary facets fac_order[f_lo, f_hi)
    // (fac_order null: the facet itself); the whole mesh outside the
    // slab-pipelined host step
    int e_lo, e_hi, n_lo, n_hi, f_lo, f_hi;
    const int *fac_order;
    // mesh
    const int *conn;
    const unsigned *bcflag;
    const int *sup_off, *sup_ent;
    const int *nf_off, *nf_ent;          // node -> boundary facets (ascending facet id)
    const int *fac_elem, *fac_f, *fac_bdry;
    const int *emark;                    // [nmat][ne] marker counts, or null
    // node fields
    double *x, *x0, *v, *f, *T, *mass, *tmass, *vol_n, *ntmp;
    // element fields
    double *stress, *strain, *srate, *pls, *dpls, *syy, *dp, *edvoldt, *vol, *vol_old, *shp;
    double *rho_e;                       // per-element density of the step (scratch), or null
    double *buoy_e;                      // per-element rho g / NPE of the step (scratch), or null
    double *tdot;                        // node scratch for the heat gather (ntmp outside the fused step)
    double *fv;                          // [nd][nbf] per-facet stress-BC force (scratch)
    // mixed 3D step (a mixed context is one with shpdw): the shape functions
    // as double-word pairs (hi, lo) at shp's indices, or null.  The hi parts
    // are the FP32 shape functions.  The mixed geometry writes these but not
    // shp, which downloads fill from them on demand.
    float2 *shpdw;
    float2 *vdw;                         // [3][nn] a mixed context's velocities as double-word pairs, from the force pass
    double4 *ndpk;                       // [ne] a mixed context's {qv, vol, me, tme}, from the look-ahead geometry pass
    float2 *pv;                          // [ne] a mixed context's double-word dp vol, from the fused stress pass
    float *hc;                           // [4][ne] per-element heat terms of the mixed step, or null
    double *qv;                          // [ne] per-element dvoldt term of the fused steps, or null
    double *hc64;                        // [NPE][ne] per-element heat terms of the FP64 step, or null
    // mixed 3D step: the element's share of its nodes' forces,
    // (sigma . dN_i/dx + buoyancy z) vol, as double-word triples, two float4
    // (hi (x, y, z, 0), lo) per support-list entry, at [2 q] for the entry q
    // of (element e, slot i): q = sup_pos[i ne + e], the inverse of sup_ent
    float4 *ft;
    const int *sup_pos;
    // set only by the reverse mode's forward recompute: the viscosity the
    // rheology used and the EVP branch it took (1: elasto-plastic), per element
    double *tape_visc;
    unsigned char *tape_evp;
    double *me, *tme;                    // [ne] per-element mass and tmass terms of the fused step
    // [EP_COUNT][ne] the element's marker-blended material properties
    // (k_elem_props), or null: formed once per marker change instead of per
    // use, with the very operations of hmean / amean
    const double *eprop;
    const double *ef[DES_EF_COUNT];      // per-element overrides or null
    Clock *clk;
    unsigned *err;
    // parameters
    des_params prm;
    MatC mat;
    double bnormals[DES_NBDRYTYPES][3];
    double edge_vectors[DES_NBDRYTYPES][DES_NBDRYTYPES][3];
};

__device__ __forceinline__ double dmax_(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double dmin_(double a, double b) { return (b < a) ? b : a; }  // std::min

template <int ND>
__device__ __forceinline__ double trace_(const double *s)
{
    if (ND == 3) return s[0] + s[1] + s[2];
    return s[0] + s[1];
}

// x / 3 correctly rounded, with one multiplication and one fma instead of a
// division (the method of Brisebarre, Muller and Raina, "Accelerating
// correctly rounded floating-point division when the divisor is known in
// advance", IEEE Trans. Computers 53(8), 2004).  With the two-term
// reciprocal YH + YL of 3, fma(x, YH, x * YL) lies within ~1e-32 (relative)
// of x / 3.  The exact quotient of a 53-bit significand by 3 has a
// fractional part, in units of the quotient's last place, of 0, 1/3 or 2/3,
// so it lies at least 1/6 ulp from every rounding midpoint, and the fma
// rounds to the IEEE quotient: the result is bit-identical to x / 3.  For a
// nonzero |x| below 2^-900, where x * YL could lose bits to underflow, it
// divides; +-0 takes the fma path, which returns it unchanged, as 0 / 3 does
// (the step divides exact zeros often: a pressure correction that vanishes).
// The tests read the exponent and mantissa bits with integer instructions,
// off the FP64 pipe.
__device__ __forceinline__ unsigned biased_exponent(double x)
{
    return ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
}

// the divisions of div3 and div6 for the rare operands where the product
// form does not apply, out of line: inlined, the compiler evaluates the
// division's whole FP64 sequence for every element and selects the result
static __device__ __noinline__ double div3_slow(double x) { return x / 3; }
static __device__ __noinline__ double div6_slow(double x) { return x / 6; }

__device__ __forceinline__ double div3(double x)
{
    constexpr double YH = 0x1.5555555555555p-2;    // RN(1/3)
    constexpr double YL = 0x1.5555555555555p-56;   // RN(1/3 - YH)
    const unsigned mag_hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
    if (mag_hi < (123u << 20) && (mag_hi | (unsigned)__double2loint(x)) != 0) return div3_slow(x);
    return fma(x, YH, x * YL);
}

// x / 6, bit-identical to the division: x / 2 is exact above the subnormal
// range, taken as exponent - 1 on the bits for finite |x| >= 2^-900, and
// div3 rounds (x / 2) / 3 = x / 6 correctly
__device__ __forceinline__ double div6(double x)
{
    const unsigned e = biased_exponent(x);
    if (e < 123u || e == 0x7ffu) return div6_slow(x);
    return div3(__hiloint2double(__double2hiint(x) - (1 << 20), __double2loint(x)));
}

// x / ND for ND = 2 or 3, bit-identical to the division
template <int ND>
__device__ __forceinline__ double divnd(double x)
{
    if (ND == 3) return div3(x);
    return x / ND;   // a power of two: the compiler multiplies by 0.5, exactly
}

// FP64 <-> FP32 conversions with integer instructions.  GB300 issues FP64
// instructions at 1/64 of the FP32 rate, and the conversion instructions
// occupy that same pipe: a conversion costs as much as an FP64 multiply.
// These forms move the exponent and mantissa bits with a few integer
// operations instead, which issue beside the FP64 work.
//
// f32_of(x): for |x| in [2^-126, 2^128), the nearest float, halfway cases
// rounded away from zero (IEEE's ties-to-even differs only when x lies
// exactly halfway between two floats); |x| < 2^-126 gives a signed zero;
// |x| >= 2^128 gives +-inf, and NaN gives NaN.
__device__ __forceinline__ float f32_of(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned mag = hi & 0x7fffffffu;
    // exponent 1023 -> 127 bias, the top 23 mantissa bits, plus the next bit
    // (a carry out of the mantissa correctly bumps the exponent)
    unsigned u = (((mag - (896u << 20)) << 3) | (lo >> 29)) + ((lo >> 28) & 1u);
    if (mag < (897u << 20)) u = 0;
    if (mag >= (1151u << 20)) u = (mag > 0x7ff00000u || (mag == 0x7ff00000u && lo)) ? 0x7fc00000u : 0x7f800000u;
    return __uint_as_float((hi & 0x80000000u) | u);
}

// f64_of(f): exact for every float but the subnormals, which give a signed
// zero; +-inf and NaN stay +-inf and NaN.
__device__ __forceinline__ double f64_of(float f)
{
    const unsigned u = __float_as_uint(f), mag = u & 0x7fffffffu;
    unsigned hi = (mag >> 3) + ((mag >= 0x7f800000u ? 1792u : 896u) << 20);
    unsigned lo = mag << 29;
    if (mag < 0x00800000u) hi = lo = 0;
    return __hiloint2double((int)((u & 0x80000000u) | hi), (int)lo);
}

// 1 / x from an FP32 seed and one FP64 Newton step (relative error ~1e-14,
// for |x| within the FP32 normal range), for the mixed step only; the FP64
// step divides
__device__ __forceinline__ double recip_newton(double x)
{
    const double r = f64_of(1.0f / f32_of(x));
    return fma(r, fma(-x, r, 1.0), r);   // r + r (1 - x r)
}

// utils.hpp:110-128
template <int ND>
__device__ __forceinline__ double second_invariant2_(const double *t)
{
    if (ND == 3) {
        double a = div3(t[0] + t[1] + t[2]);
        return (0.5 * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a))
                + t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
    }
    return 0.25 * (t[0] - t[1]) * (t[0] - t[1]) + t[2] * t[2];
}

template <int ND>
__device__ __forceinline__ double second_invariant_(const double *t)
{
    return sqrt(second_invariant2_<ND>(t));
}

// ------------------------------------------------------------------
// material properties (matprops.cxx:103-414)
// ------------------------------------------------------------------
__device__ __forceinline__ int mcount(const KP &p, int e, int m)
{
    if (p.emark) return p.emark[(size_t)m * p.ne + e];
    return m == 0 ? 1 : 0;
}

__device__ __forceinline__ double hmean(const KP &p, const double *s, int bit, int e)
{
    if (p.mat.nmat == 1 || ((p.mat.scalar_mask >> bit) & 1u)) return s[0];
    double result = 0;
    int m = 0;
    for (int i = 0; i < p.mat.nmat; i++) {
        int n = mcount(p, e, i);
        result += n / s[i];
        m += n;
    }
    return m / result;
}

__device__ __forceinline__ double amean(const KP &p, const double *s, int bit, int e)
{
    if (p.mat.nmat == 1 || ((p.mat.scalar_mask >> bit) & 1u)) return s[0];
    double result = 0;
    int m = 0;
    for (int i = 0; i < p.mat.nmat; i++) {
        int n = mcount(p, e, i);
        result += n * s[i];
        m += n;
    }
    return result / m;
}

// the blended properties that KP::eprop holds, in its component order
enum { EP_BULKM, EP_SHEARM, EP_CP, EP_HR, EP_K, EP_HR_OVER_CP, EP_COUNT };

__device__ __forceinline__ double m_bulkm(const KP &p, int e)
{
    if (p.eprop) return p.eprop[(size_t)EP_BULKM * p.ne + e];
    return hmean(p, p.mat.bulk_modulus, 0, e);
}
__device__ __forceinline__ double m_shearm(const KP &p, int e)
{
    if (p.ef[DES_EF_SHEAR_MODULUS]) return p.ef[DES_EF_SHEAR_MODULUS][e];
    if (p.eprop) return p.eprop[(size_t)EP_SHEARM * p.ne + e];
    return hmean(p, p.mat.shear_modulus, 1, e);
}
__device__ __forceinline__ double m_cp(const KP &p, int e)
{
    if (p.eprop) return p.eprop[(size_t)EP_CP * p.ne + e];
    return amean(p, p.mat.heat_capacity, 2, e);
}
__device__ __forceinline__ double m_hr(const KP &p, int e)
{
    if (p.eprop) return p.eprop[(size_t)EP_HR * p.ne + e];
    return amean(p, p.mat.radiogenic_heating, 3, e);
}
__device__ __forceinline__ double m_k(const KP &p, int e)
{
    if (p.ef[DES_EF_THERM_COND]) return p.ef[DES_EF_THERM_COND][e];
    if (p.eprop) return p.eprop[(size_t)EP_K * p.ne + e];
    return amean(p, p.mat.therm_cond, 4, e);
}
// hr / cp of the heat source term (fields.cxx:118,141)
__device__ __forceinline__ double m_hr_over_cp(const KP &p, int e)
{
    if (p.mat.nmat == 1) return p.mat.hr_over_cp;
    if (p.eprop) return p.eprop[(size_t)EP_HR_OVER_CP * p.ne + e];
    return m_hr(p, e) / m_cp(p, e);
}

template <int NPE>
__device__ __forceinline__ double elem_avg_T(const KP &p, int e)
{
    double t = 0;
#pragma unroll
    for (int i = 0; i < NPE; ++i) t += p.T[p.conn[(size_t)i * p.ne + e]];
    return t / NPE;
}

// MatProps::rho (matprops.cxx:376-397) given the element's mean temperature
__device__ __forceinline__ double m_rho_T(const KP &p, int e, double T)
{
    const double celsius0 = 273;
    double TinCelsius = T - celsius0;
    // one material, one marker: (x * 1) / 1 == x exactly
    if (p.mat.nmat == 1 && !p.emark) return p.mat.rho0[0] * (1 - p.mat.alpha[0] * TinCelsius);
    // a material without markers adds a signed zero (for finite T), which
    // leaves the sum unchanged; a division by n = 1 is exact
    const bool skip_empty = isfinite(TinCelsius);
    double result = 0;
    int n = 0;
    for (int m = 0; m < p.mat.nmat; m++) {
        int k = mcount(p, e, m);
        if (k == 0 && skip_empty) continue;
        result += p.mat.rho0[m] * (1 - p.mat.alpha[m] * TinCelsius) * k;
        n += k;
    }
    return n == 1 ? result : result / n;
}

template <int ND>
__device__ __forceinline__ double m_rho(const KP &p, int e)
{
    return m_rho_T(p, e, elem_avg_T<ND + 1>(p, e));
}

// MatProps::visc (matprops.cxx:276-312); edot = the element's strain rate
template <int ND>
__device__ double m_visc(const KP &p, int e, const double *edot)
{
    double v;
    if (p.ef[DES_EF_LOG10_VISC]) {
        v = pow(10.0, p.ef[DES_EF_LOG10_VISC][e]);
    } else {
        const double gas_constant = 8.3144;
        const double min_strain_rate = 1e-30;
        double T = elem_avg_T<ND + 1>(p, e);
        double ed = second_invariant_<ND>(edot);
        ed = dmax_(ed, min_strain_rate);
        double result = 0;
        int n = 0;
        const bool skip_empty = p.mat.visc_skip_empty && T > 0;
        for (int m = 0; m < p.mat.nmat; m++) {
            int k = mcount(p, e, m);
            if (k == 0 && skip_empty) continue;   // k / visc0 = +0 exactly
            const double pw = p.mat.visc_pw[m];
            const double visc0 = 0.25 * pow(ed, pw) * p.mat.visc_coef[m]
                * exp(p.mat.visc_activation_energy[m] / (p.mat.visc_exponent[m] * gas_constant * T)) * 1e6;
            result += k / visc0;
            n += k;
        }
        v = n / result;
    }
    return dmin_(dmax_(v, p.mat.visc_min), p.mat.visc_max);
}

// angle-dependent part of plastic_props (matprops.cxx:365-372)
__device__ inline void plastic_angles(double phi, double psi, double &anphi, double &anpsi, double &sq, double &tn)
{
    double sphi = sin(phi * DEG2RAD);
    double spsi = sin(psi * DEG2RAD);
    anphi = (1 + sphi) / (1 - sphi);
    anpsi = (1 + spsi) / (1 - spsi);
    sq = sqrt(anphi);
    tn = tan(phi * DEG2RAD);
}

// MatProps::plastic_weakening + plastic_props (matprops.cxx:315-373) for an
// element whose markers are all of material mone and number one (or, without
// markers, one material: mone = 0).  The general loop of plastic_props_blend
// then runs one iteration with k = 1, whose products and divisions by the
// marker count are exact identities (x*1 = x, x / 1 = x), and at the start /
// saturated angles the angle terms are the table entries of material mone
// (or entries of the same angles, which hold the same bits), so this returns
// the very bits of the general loop.
__device__ __forceinline__ void plastic_props_one(const KP &p, int e, int mone, double pls, double &amc,
                                                  double &anphi, double &anpsi, double &hardn, double &ten_max)
{
    const double l0 = p.mat.pls0[mone], l1 = p.mat.pls1[mone];
    const bool cov = p.ef[DES_EF_COHESION0] || p.ef[DES_EF_COHESION1];
    const double c0 = p.ef[DES_EF_COHESION0] ? p.ef[DES_EF_COHESION0][e] : p.mat.cohesion0[mone];
    const double c1 = p.ef[DES_EF_COHESION1] ? p.ef[DES_EF_COHESION1][e] : p.mat.cohesion1[mone];
    int k;
    double cohesion;
    if (pls < l0) {
        k = 2 * mone;
        cohesion = c0;
        hardn = 0;
    } else if (pls < l1) {
        hardn = cov ? (c1 - c0) / (l1 - l0) : p.mat.hardening[mone];
        if (pls == l0) {   // q = +0: c0 + 0*(c1-c0) == c0, phi0 + 0*(..) == phi0
            k = 2 * mone;
            cohesion = c0;
        } else {
            const double q = (pls - l0) / (l1 - l0);
            cohesion = c0 + q * (c1 - c0);
            const double phi = p.mat.friction_angle0[mone]
                + q * (p.mat.friction_angle1[mone] - p.mat.friction_angle0[mone]);
            const double psi = p.mat.dilation_angle0[mone]
                + q * (p.mat.dilation_angle1[mone] - p.mat.dilation_angle0[mone]);
            double sq, tn;
            plastic_angles(phi, psi, anphi, anpsi, sq, tn);
            amc = 2 * cohesion * sq;
            ten_max = (phi == 0) ? p.mat.tension_max : dmin_(p.mat.tension_max, cohesion / tn);
            return;
        }
    } else {
        k = 2 * mone + 1;
        cohesion = c1;
        hardn = 0;
    }
    anphi = p.mat.pt_anphi[k];
    anpsi = p.mat.pt_anpsi[k];
    amc = 2 * cohesion * p.mat.pt_sqrt_anphi[k];
    const double phi = p.mat.pt_phi[k];
    ten_max = (phi == 0) ? p.mat.tension_max
                         : dmin_(p.mat.tension_max, cov ? cohesion / p.mat.pt_tanphi[k] : p.mat.pt_coh_over_tan[k]);
}

// plastic_props over the element's markers: the one-marker branch where it
// applies, else the marker-weighted loop.  Out of line: the registers of the
// blend stay out of the one-material kernels.
static __device__ __noinline__ void plastic_props_blend(const KP &p, int e, double pls, double &amc, double &anphi,
                                                        double &anpsi, double &hardn, double &ten_max)
{
    if (p.emark && !p.ef[DES_EF_FRICTION0] && !p.ef[DES_EF_FRICTION1] && p.mat.pt_n >= 2) {
        int n = 0, mone = -1;
        for (int m = 0; m < p.mat.nmat; m++) {
            const int k = mcount(p, e, m);
            n += k;
            if (k) mone = m;
        }
        if (n == 1) {
            plastic_props_one(p, e, mone, pls, amc, anphi, anpsi, hardn, ten_max);
            return;
        }
    }
    double cc = 0, f = 0, d = 0, h = 0;
    int n = 0;
    for (int m = 0; m < p.mat.nmat; m++) {
        int k = mcount(p, e, m);
        if (k == 0) continue;
        n += k;
        double c0 = p.ef[DES_EF_COHESION0] ? p.ef[DES_EF_COHESION0][e] : p.mat.cohesion0[m];
        double c1 = p.ef[DES_EF_COHESION1] ? p.ef[DES_EF_COHESION1][e] : p.mat.cohesion1[m];
        double f0 = p.ef[DES_EF_FRICTION0] ? p.ef[DES_EF_FRICTION0][e] : p.mat.friction_angle0[m];
        double f1 = p.ef[DES_EF_FRICTION1] ? p.ef[DES_EF_FRICTION1][e] : p.mat.friction_angle1[m];
        double d0 = p.mat.dilation_angle0[m], d1 = p.mat.dilation_angle1[m];
        double l0 = p.mat.pls0[m], l1 = p.mat.pls1[m];
        if (pls < l0) {
            cc += c0 * k;
            f += f0 * k;
            d += d0 * k;
            h += 0;
        } else if (pls < l1) {
            double q = (pls - l0) / (l1 - l0);
            cc += (c0 + q * (c1 - c0)) * k;
            f += (f0 + q * (f1 - f0)) * k;
            d += (d0 + q * (d1 - d0)) * k;
            h += (c1 - c0) / (l1 - l0) * k;
        } else {
            cc += c1 * k;
            f += f1 * k;
            d += d1 * k;
            h += 0;
        }
    }
    // divisions by n = 1 (one marker) are exact
    double cohesion = n == 1 ? cc : cc / n, phi = n == 1 ? f : f / n, psi = n == 1 ? d : d / n;
    hardn = n == 1 ? h : h / n;
    int hit = -1;
    for (int k = 0; k < p.mat.pt_n; ++k)
        if (phi == p.mat.pt_phi[k] && psi == p.mat.pt_psi[k]) hit = k;
    double sq, tn;
    if (hit >= 0) {
        anphi = p.mat.pt_anphi[hit];
        anpsi = p.mat.pt_anpsi[hit];
        sq = p.mat.pt_sqrt_anphi[hit];
        tn = p.mat.pt_tanphi[hit];
    } else {
        plastic_angles(phi, psi, anphi, anpsi, sq, tn);
    }
    amc = 2 * cohesion * sq;
    ten_max = (phi == 0) ? p.mat.tension_max : dmin_(p.mat.tension_max, cohesion / tn);
}

// MatProps::plastic_weakening + plastic_props (matprops.cxx:315-373)
__device__ __forceinline__ void m_plastic_props(const KP &p, int e, double pls, double &amc, double &anphi,
                                                double &anpsi, double &hardn, double &ten_max)
{
    if (p.mat.nmat == 1 && !p.emark && !p.ef[DES_EF_FRICTION0] && !p.ef[DES_EF_FRICTION1] && p.mat.pt_n >= 2)
        plastic_props_one(p, e, 0, pls, amc, anphi, anpsi, hardn, ten_max);
    else
        plastic_props_blend(p, e, pls, amc, anphi, anpsi, hardn, ten_max);
}

// ref_pressure option 0 (matprops.cxx:190-202)
__device__ __forceinline__ double ref_pressure_(const KP &p, double z)
{
    double depth = -z;
    return p.mat.rho0[0] * p.prm.gravity * depth;
}

// ------------------------------------------------------------------
// mesh helpers
// ------------------------------------------------------------------
__device__ __forceinline__ int conn_at(const KP &p, int i, int e) { return p.conn[(size_t)i * p.ne + e]; }

__device__ __forceinline__ double shp_at(const KP &p, int k, int i, int e)
{
    return p.shp[((size_t)k * p.npe + i) * p.ne + e];
}

// tetrahedron_volume (geometry.cxx:29-49)
// the 18 coordinate differences of a tet that the volume and the shape
// functions share (xij = x_i - x_j)
struct TetEdges {
    double x01, x02, x03, x12, x13, x23;
    double y01, y02, y03, y12, y13, y23;
    double z01, z02, z03, z12, z13, z23;
};

__device__ __forceinline__ TetEdges tet_edges(const double *d0, const double *d1, const double *d2,
                                              const double *d3)
{
    TetEdges t;
    t.x01 = d0[0] - d1[0], t.x02 = d0[0] - d2[0], t.x03 = d0[0] - d3[0];
    t.x12 = d1[0] - d2[0], t.x13 = d1[0] - d3[0], t.x23 = d2[0] - d3[0];
    t.y01 = d0[1] - d1[1], t.y02 = d0[1] - d2[1], t.y03 = d0[1] - d3[1];
    t.y12 = d1[1] - d2[1], t.y13 = d1[1] - d3[1], t.y23 = d2[1] - d3[1];
    t.z01 = d0[2] - d1[2], t.z02 = d0[2] - d2[2], t.z03 = d0[2] - d3[2];
    t.z12 = d1[2] - d2[2], t.z13 = d1[2] - d3[2], t.z23 = d2[2] - d3[2];
    return t;
}

__device__ __forceinline__ double tet_volume(const TetEdges &t)
{
    return div6(t.x01 * (t.y23 * t.z12 - t.y12 * t.z23) + t.x12 * (t.y01 * t.z23 - t.y23 * t.z01)
                + t.x23 * (t.y12 * t.z01 - t.y01 * t.z12));
}

__device__ __forceinline__ double tet_volume(const double *d0, const double *d1, const double *d2,
                                             const double *d3)
{
    return tet_volume(tet_edges(d0, d1, d2, d3));
}

// triangle_area (geometry.cxx:53-83)
template <int ND>
__device__ __forceinline__ double tri_area(const double *a, const double *b, const double *c)
{
    double ab0 = b[0] - a[0], ab1 = b[1] - a[1];
    double ac0 = c[0] - a[0], ac1 = c[1] - a[1];
    if (ND == 2) return fabs(ab0 * ac1 - ab1 * ac0) / 2;
    double ab2 = b[2] - a[2], ac2 = c[2] - a[2];
    double d0 = ab1 * ac2 - ab2 * ac1;
    double d1 = ab2 * ac0 - ab0 * ac2;
    double d2 = ab0 * ac1 - ab1 * ac0;
    return sqrt(d0 * d0 + d1 * d1 + d2 * d2) / 2;
}

// (2 x area of triangle abc)^2 in 3D: tri_area<3> is sqrt of this over 2
__device__ __forceinline__ double tri_area2_3d(const double *a, const double *b, const double *c)
{
    double ab0 = b[0] - a[0], ab1 = b[1] - a[1], ab2 = b[2] - a[2];
    double ac0 = c[0] - a[0], ac1 = c[1] - a[1], ac2 = c[2] - a[2];
    double d0 = ab1 * ac2 - ab2 * ac1;
    double d1 = ab2 * ac0 - ab0 * ac2;
    double d2 = ab0 * ac1 - ab1 * ac0;
    return d0 * d0 + d1 * d1 + d2 * d2;
}

// the Maxwell time 0.5 visc_min / shearm is the same for every element: one
// material without markers or a per-element shear modulus
__device__ __forceinline__ bool uniform_maxwell_time(const KP &p)
{
    return p.mat.nmat == 1 && !p.emark && !p.ef[DES_EF_SHEAR_MODULUS];
}

template <int ND>
__device__ __forceinline__ void load_node_x(const KP &p, int n, double *c)
{
#pragma unroll
    for (int d = 0; d < ND; ++d) c[d] = p.x[(size_t)d * p.nn + n];
}

template <int ND>
__device__ __forceinline__ void load_node_v(const KP &p, int n, double *c)
{
#pragma unroll
    for (int d = 0; d < ND; ++d) c[d] = p.v[(size_t)d * p.nn + n];
}

__device__ __forceinline__ void set_err(const KP &p, unsigned bits) { atomicOr(p.err, bits); }

// positive doubles compare like their bit patterns
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ double bitsd(unsigned long long b) { return __longlong_as_double((long long)b); }

}  // namespace des
