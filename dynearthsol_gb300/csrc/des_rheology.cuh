// des_rheology.cuh -- per-element constitutive update (update_stress,
// rheology.cxx:510-646) and the 3x3 symmetric eigen-solver it needs.
//
// The eigen-solver is the hybrid method of J. Kopp, "Efficient numerical
// diagonalization of hermitian 3x3 matrices", Int. J. Mod. Phys. C 19 (2008)
// 523 (arXiv:physics/0610206), which the reference vendors as 3x3-C/dsyevh3.c:
// analytic (Cardano) eigenvalues, eigenvectors from cross products, and a
// Householder + QL fallback when a cross product is too small.  The branch
// criterion and the arithmetic order are kept as there, so that FP64 runs
// take the same branches as the reference.  Only the upper triangle of A is
// read.  The QL loop keeps the published 30-sweep cap; hitting it sets
// DES_DEV_QL_NOCONV instead of returning an unchecked -1.
//
// Notice for eig_cardano, eig_tridiag, eig_ql and eig_hybrid, which follow
// the arithmetic of Kopp's dsyevc3, dsytrd3, dsyevq3 and dsyevh3 step for
// step (the FP64 path must branch as the reference does):
//   Copyright (C) 2006 Joachim Kopp.  The original is free software; you
//   can redistribute it and/or modify it under the terms of the GNU Lesser
//   General Public License as published by the Free Software Foundation;
//   either version 2.1 of the License, or (at your option) any later
//   version.  It is distributed WITHOUT ANY WARRANTY; without even the
//   implied warranty of MERCHANTABILITY or FITNESS FOR A PARTICULAR PURPOSE.
//   See the GNU Lesser General Public License for more details.
#pragma once

#include "des_common.cuh"

namespace des {

__device__ __forceinline__ void eig_cardano(const double A[3][3], double w[3])
{
    const double inv_sqrt3 = 1.0 / 1.73205080756887729352744634151;
    double de = A[0][1] * A[1][2];
    double dd = A[0][1] * A[0][1];
    double ee = A[1][2] * A[1][2];
    double ff = A[0][2] * A[0][2];
    double m = A[0][0] + A[1][1] + A[2][2];
    double c1 = (A[0][0] * A[1][1] + A[0][0] * A[2][2] + A[1][1] * A[2][2]) - (dd + ee + ff);
    double c0 = A[2][2] * dd + A[0][0] * ee + A[1][1] * ff - A[0][0] * A[1][1] * A[2][2]
        - 2.0 * A[0][2] * de;
    double p = m * m - 3.0 * c1;
    double q = m * (p - (3.0 / 2.0) * c1) - (27.0 / 2.0) * c0;
    double sqrt_p = sqrt(fabs(p));
    double phi = 27.0 * (0.25 * (c1 * c1) * (p - c1) + c0 * (q + 27.0 / 4.0 * c0));
    phi = (1.0 / 3.0) * atan2(sqrt(fabs(phi)), q);
    double cc = sqrt_p * cos(phi);
    double ss = inv_sqrt3 * sqrt_p * sin(phi);
    double mid = (1.0 / 3.0) * (m - cc);
    w[2] = mid + ss;
    w[0] = mid + cc;
    w[1] = mid - ss;
}

__device__ __forceinline__ void eig_tridiag(const double A[3][3], double Q[3][3], double d[3], double e[3])
{
    double u[3], q[3];
    double omega, f, K, h, g;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        Q[i][i] = 1.0;
#pragma unroll
        for (int j = 0; j < i; j++) Q[i][j] = Q[j][i] = 0.0;
    }
    h = A[0][1] * A[0][1] + A[0][2] * A[0][2];
    g = (A[0][1] > 0) ? -sqrt(h) : sqrt(h);
    e[0] = g;
    f = g * A[0][1];
    u[1] = A[0][1] - g;
    u[2] = A[0][2];
    omega = h - f;
    if (omega > 0.0) {
        omega = 1.0 / omega;
        K = 0.0;
#pragma unroll
        for (int i = 1; i < 3; i++) {
            f = A[1][i] * u[1] + A[i][2] * u[2];
            q[i] = omega * f;
            K += u[i] * f;
        }
        K *= 0.5 * (omega * omega);
#pragma unroll
        for (int i = 1; i < 3; i++) q[i] = q[i] - K * u[i];
        d[0] = A[0][0];
        d[1] = A[1][1] - 2.0 * q[1] * u[1];
        d[2] = A[2][2] - 2.0 * q[2] * u[2];
#pragma unroll
        for (int j = 1; j < 3; j++) {
            f = omega * u[j];
#pragma unroll
            for (int i = 1; i < 3; i++) Q[i][j] = Q[i][j] - f * u[i];
        }
        e[1] = A[1][2] - q[1] * u[2] - u[1] * q[2];
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++) d[i] = A[i][i];
        e[1] = A[1][2];
    }
}

// returns 0, or -1 when a 30-sweep cap is hit
__device__ inline int eig_ql(const double A[3][3], double Q[3][3], double w[3])
{
    double e[3];
    double g, r, p, f, b, s, c, t;
    int m;
    eig_tridiag(A, Q, w, e);
    for (int l = 0; l < 2; l++) {
        int sweeps = 0;
        for (;;) {
            for (m = l; m <= 1; m++) {
                g = fabs(w[m]) + fabs(w[m + 1]);
                if (fabs(e[m]) + g == g) break;
            }
            if (m == l) break;
            if (sweeps++ >= 30) return -1;
            g = (w[l + 1] - w[l]) / (e[l] + e[l]);
            r = sqrt(g * g + 1.0);
            if (g > 0) g = w[m] - w[l] + e[l] / (g + r);
            else g = w[m] - w[l] + e[l] / (g - r);
            s = c = 1.0;
            p = 0.0;
            for (int i = m - 1; i >= l; i--) {
                f = s * e[i];
                b = c * e[i];
                if (fabs(f) > fabs(g)) {
                    c = g / f;
                    r = sqrt(c * c + 1.0);
                    e[i + 1] = f * r;
                    c *= (s = 1.0 / r);
                } else {
                    s = f / g;
                    r = sqrt(s * s + 1.0);
                    e[i + 1] = g * r;
                    s *= (c = 1.0 / r);
                }
                g = w[i + 1] - p;
                r = (w[i] - g) * s + 2.0 * c * b;
                p = s * r;
                w[i + 1] = g + p;
                g = c * r - b;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    t = Q[k][i + 1];
                    Q[k][i + 1] = s * Q[k][i] + c * t;
                    Q[k][i] = c * Q[k][i] - s * t;
                }
            }
            w[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    return 0;
}

__device__ inline int eig_hybrid(const double A[3][3], double Q[3][3], double w[3])
{
    double norm, error, t, u;
    eig_cardano(A, w);
    t = fabs(w[0]);
    if ((u = fabs(w[1])) > t) t = u;
    if ((u = fabs(w[2])) > t) t = u;
    if (t < 1.0) u = t;
    else u = t * t;
    error = 256.0 * DBL_EPSILON * (u * u);

    Q[0][1] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
    Q[1][1] = A[0][2] * A[0][1] - A[1][2] * A[0][0];
    Q[2][1] = A[0][1] * A[0][1];

    Q[0][0] = Q[0][1] + A[0][2] * w[0];
    Q[1][0] = Q[1][1] + A[1][2] * w[0];
    Q[2][0] = (A[0][0] - w[0]) * (A[1][1] - w[0]) - Q[2][1];
    norm = Q[0][0] * Q[0][0] + Q[1][0] * Q[1][0] + Q[2][0] * Q[2][0];
    if (norm <= error) return eig_ql(A, Q, w);
    norm = sqrt(1.0 / norm);
#pragma unroll
    for (int j = 0; j < 3; j++) Q[j][0] = Q[j][0] * norm;

    Q[0][1] = Q[0][1] + A[0][2] * w[1];
    Q[1][1] = Q[1][1] + A[1][2] * w[1];
    Q[2][1] = (A[0][0] - w[1]) * (A[1][1] - w[1]) - Q[2][1];
    norm = Q[0][1] * Q[0][1] + Q[1][1] * Q[1][1] + Q[2][1] * Q[2][1];
    if (norm <= error) return eig_ql(A, Q, w);
    norm = sqrt(1.0 / norm);
#pragma unroll
    for (int j = 0; j < 3; j++) Q[j][1] = Q[j][1] * norm;

    Q[0][2] = Q[1][0] * Q[2][1] - Q[2][0] * Q[1][1];
    Q[1][2] = Q[2][0] * Q[0][1] - Q[0][0] * Q[2][1];
    Q[2][2] = Q[0][0] * Q[1][1] - Q[1][0] * Q[0][1];
    return 0;
}

// principal_stresses3 (rheology.cxx:13-68)
__device__ __forceinline__ int principal_stresses3(const double *s, double p[3], double v[3][3])
{
    double a[3][3];
    a[0][0] = s[0];
    a[1][1] = s[1];
    a[2][2] = s[2];
    a[0][1] = s[3];
    a[0][2] = s[4];
    a[1][2] = s[5];
    a[1][0] = a[2][0] = a[2][1] = 0;
    int rc = eig_hybrid(a, v, p);
    // compare-and-swap on (0,1), (1,2), (0,1)
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int i = (k == 1) ? 1 : 0, j = i + 1;
        if (p[i] > p[j]) {
            double t = p[i];
            p[i] = p[j];
            p[j] = t;
#pragma unroll
            for (int r = 0; r < 3; r++) {
                double b = v[r][i];
                v[r][i] = v[r][j];
                v[r][j] = b;
            }
        }
    }
    return rc;
}

// principal_stresses2 (rheology.cxx:71-102)
__device__ __forceinline__ void principal_stresses2(const double *s, double p[2], double &cos2t, double &sin2t)
{
    double s0 = 0.5 * (s[0] + s[1]);
    double rad = second_invariant_<2>(s);
    p[0] = s0 - rad;
    p[1] = s0 + rad;
    const double eps = 1e-15;
    double a = 0.5 * (s[0] - s[1]);
    double b = -rad;
    if (b < -eps) {
        cos2t = a / b;
        sin2t = s[2] / b;
    } else {
        cos2t = 1;
        sin2t = 0;
    }
}

// elastic (rheology.cxx:105-115)
template <int ND>
__device__ __forceinline__ void elastic_(double bulkm, double shearm, const double *de, double *s)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    double lambda = bulkm - 2. / 3 * shearm;
    double dev = trace_<ND>(de);
#pragma unroll
    for (int i = 0; i < ND; ++i) s[i] += 2 * shearm * de[i] + lambda * dev;
#pragma unroll
    for (int i = ND; i < NSTR; ++i) s[i] += 2 * shearm * de[i];
}

// maxwell (rheology.cxx:118-134)
template <int ND>
__device__ __forceinline__ void maxwell_(double bulkm, double shearm, double viscosity, double dt,
                                         double dv, const double *de, double *s)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    double tmp = 0.5 * dt * shearm / viscosity;
    double f1 = 1 - tmp;
    double f2 = 1 / (1 + tmp);
    double dev = divnd<ND>(trace_<ND>(de));
    double s0 = divnd<ND>(trace_<ND>(s));
#pragma unroll
    for (int i = 0; i < ND; ++i) s[i] = ((s[i] - s0) * f1 + 2 * shearm * (de[i] - dev)) * f2 + s0 + bulkm * dv;
#pragma unroll
    for (int i = ND; i < NSTR; ++i) s[i] = (s[i] * f1 + 2 * shearm * de[i]) * f2;
}

// viscous (rheology.cxx:137-148)
template <int ND>
__device__ __forceinline__ void viscous_(double bulkm, double viscosity, double total_dv, const double *edot,
                                         double *s)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    double dev = divnd<ND>(trace_<ND>(edot));
#pragma unroll
    for (int i = 0; i < ND; ++i) s[i] = 2 * viscosity * (edot[i] - dev) + bulkm * total_dv;
#pragma unroll
    for (int i = ND; i < NSTR; ++i) s[i] = 2 * viscosity * edot[i];
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

// Screen of the Mohr-Coulomb yield test (rheology.cxx:163-178) in FP32, for
// 3D.  The deviatoric trial stress D is diagonalised in FP32 (eigenvalues
// only).  Each computed eigenvalue lies within ||E||_2 of the exact one
// (Weyl), E being the backward error of rounding D to FP32 and of twelve
// Jacobi rotations: a few tens of eps32 ||D||_F.  The principal stresses
// p = m + w and the yield functions fs = p0 - p2 anphi + amc, ft = p2 -
// ten_max are formed in FP32 too, from the FP64 mean stress m and material
// terms rounded to FP32: with P = |m| + ||D||, that adds at most
// 2^-21.6 (1 + anphi) P to fs and 2^-22 (P + |ten_max|) to ft.  The FP64
// principal stresses of the full stress (principal_stresses3) carry errors
// of a few eps64 P.  The screen passes an element only when both yield
// functions clear the surface by tol = 2^-12 ||D||_F + 2^-19 (|m| +
// ||D||_F) (~4000 eps32 ||D||_F plus four times the FP32 arithmetic's
// error), plus 2^-19 of the material term, plus 2^-100 for the conversions'
// flush of magnitudes below 2^-126 to zero, so a passed element is elastic
// in the FP64 test too: its output is its trial stress, bit for bit, and the
// eigen-solve is skipped.  Every other element takes the FP64 return map,
// including the choice of principal directions when two principal stresses
// (nearly) coincide, which FP32 cannot resolve.  Elements within ~2^-19 |m|
// of the yield surface fail the screen and take the return map; they are
// few, and the result does not depend on it.  A non-finite conversion makes
// a comparison false: such an element takes the return map.
// The screen on FP32 inputs: d the deviator (normal, then shear components),
// mf the mean stress, mag an FP32 bound on |m| that also covers the FP32
// rounding mf carries, dev_err a bound on the 2-norm distance of d (before
// its rounding to FP32) from the exact deviator of the FP64 stress.
__device__ __forceinline__ bool clearly_elastic3_f(float af, float cf, float tf, float mf, float mag,
                                                   const float d[6], float dev_err)
{
    float w[3], v[3][3];
    jacobi3f(d, w, v);
    const float nf = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
                           + 2.0f * (d[3] * d[3] + d[4] * d[4] + d[5] * d[5]));
    const float tol = 0x1p-12f * nf + 0x1p-19f * (mag + nf) + dev_err + 0x1p-100f;
    const float p0 = mf + w[0], p2 = mf + w[2];
    const float fs = p0 - p2 * af + cf;
    const float ft = p2 - tf;
    return fs > (1.0f + af) * tol + 0x1p-19f * fabsf(cf) && ft < -(tol + 0x1p-19f * fabsf(tf));
}

// The same screen given the mean stress m and the normal deviator q_i = s_i - m
// (any FP64 rounding of m is covered by tol).
__device__ __forceinline__ bool clearly_elastic3_dev(double amc, double anphi, double ten_max, double m,
                                                     const double *q, const double *s)
{
    const float d[6] = {f32_of(q[0]), f32_of(q[1]), f32_of(q[2]), f32_of(s[3]), f32_of(s[4]), f32_of(s[5])};
    const float mf = f32_of(m);
    return clearly_elastic3_f(f32_of(anphi), f32_of(amc), f32_of(ten_max), mf, fabsf(mf), d, 0.0f);
}

__device__ __forceinline__ bool clearly_elastic3(double amc, double anphi, double ten_max, const double *s)
{
    const double m = (s[0] + s[1] + s[2]) * (1.0 / 3);
    const double q[3] = {s[0] - m, s[1] - m, s[2] - m};
    return clearly_elastic3_dev(amc, anphi, ten_max, m, q, s);
}

// The EVP branch choice (rheology.cxx:594-634) compares second_invariant2_
// (utils.hpp:110-128) of two candidate stresses.  J2Est is an FP32 estimate
// j of that FP64 value with a bound tol on their distance; j2_less decides
// the comparison from two estimates where they are further apart than both
// bounds together, and otherwise leaves it to the FP64 evaluation.
struct J2Est {
    float j, tol;
};

// Estimate of second_invariant2_<3>(s).  Let u = 2^-53, S = max |s_i| over
// the normal components and J* the exact J2 of s.  The normal deviator
// enters through the FP64 pairwise differences s_i - s_j, each within u of
// itself: 0.5 sum_i (s_i - mean)^2 = (1/6) sum_{i<j} (s_i - s_j)^2, so no
// pressure cancels in FP32.  The FP32 evaluation (conversions, squares,
// sums, the constant 1/6) then lies within 9 * 2^-24 J* of J*.
// second_invariant2_'s mean lies within 2.7 u S of the exact mean and each
// of its deviator components within 5 u S of the exact one, which moves its
// J2 by at most 5 sqrt(6) u S sqrt(J*) + 37.5 u^2 S^2; its twelve roundings
// of nonnegative terms add at most 12 u J*.  tol = 2^-19 j + 2^-48 S
// sqrt(j) + (2^-50 S)^2 + 2^-100 covers these terms by factors of 1.7 and
// more, with its own FP32 rounding and the conversions' flush of magnitudes
// below 2^-126 to zero.  An infinite or NaN estimate gives an infinite or
// NaN tol, which decides nothing.
__device__ __forceinline__ J2Est j2_est3(const double *s)
{
    const float d01 = f32_of(s[0] - s[1]), d02 = f32_of(s[0] - s[2]), d12 = f32_of(s[1] - s[2]);
    const float t3 = f32_of(s[3]), t4 = f32_of(s[4]), t5 = f32_of(s[5]);
    const float j = (d01 * d01 + d02 * d02 + d12 * d12) * (1.0f / 6) + (t3 * t3 + t4 * t4 + t5 * t5);
    const float S = fmaxf(fmaxf(fabsf(f32_of(s[0])), fabsf(f32_of(s[1]))), fabsf(f32_of(s[2])));
    const float h = 0x1p-50f * S;
    return {j, 0x1p-19f * j + 0x1p-48f * S * sqrtf(j) + h * h + 0x1p-100f};
}

// Estimate of 0.5 (q0^2 + q1^2 + q2^2) + s3^2 + s4^2 + s5^2 evaluated in
// FP64 on these very q_i (a deviator formed as second_invariant2_ forms it)
// and shear components: the FP32 evaluation lies within 7 * 2^-24 of the
// exact value of the expression, the FP64 one within 12 u; tol = 2^-19 j +
// 2^-100 covers both and the flush below 2^-126.
__device__ __forceinline__ J2Est j2_est_dev3(const double *q, const double *s)
{
    const float q0 = f32_of(q[0]), q1 = f32_of(q[1]), q2 = f32_of(q[2]);
    const float t3 = f32_of(s[3]), t4 = f32_of(s[4]), t5 = f32_of(s[5]);
    const float j = 0.5f * (q0 * q0 + q1 * q1 + q2 * q2) + (t3 * t3 + t4 * t4 + t5 * t5);
    return {j, 0x1p-19f * j + 0x1p-100f};
}

// Estimate of second_invariant2_<3> of an FP64 stress s from a normal
// deviator qt that lies within 22 u S of the exact deviator of s in each
// component, and from the shear components of s itself (S an FP32 bound on
// the magnitudes behind both).  Against the exact J2 of s, J*, the FP32
// evaluation on qt is off by at most 7 * 2^-24 J + sqrt(6) 22 u S sqrt(J*)
// + 1.5 (22 u S)^2; second_invariant2_ by 12 u J* + 12.25 u S sqrt(J*) +
// 37.5 u^2 S^2 (j2_est3).  tol = 2^-19 j + 2^-44 S sqrt(j) + (2^-46 S)^2 +
// 2^-100 covers the sum by factors of 3.7 and more.
__device__ __forceinline__ J2Est j2_est_near3(const double *qt, const double *sh, float S)
{
    const float q0 = f32_of(qt[0]), q1 = f32_of(qt[1]), q2 = f32_of(qt[2]);
    const float t3 = f32_of(sh[0]), t4 = f32_of(sh[1]), t5 = f32_of(sh[2]);
    const float j = 0.5f * (q0 * q0 + q1 * q1 + q2 * q2) + (t3 * t3 + t4 * t4 + t5 * t5);
    const float h = 0x1p-46f * S;
    return {j, 0x1p-19f * j + 0x1p-44f * S * sqrtf(j) + h * h + 0x1p-100f};
}

// 1 when the FP64 J2 behind a is certainly below that behind b, 0 when it
// certainly is not (equal included), -1 when the estimates are too close
__device__ __forceinline__ int j2_less(const J2Est &a, const J2Est &b)
{
    const float gap = b.j - a.j, tol = a.tol + b.tol;
    return gap > tol ? 1 : (-gap > tol ? 0 : -1);
}

// Mohr-Coulomb return map in principal space of the elastic trial stress s
// (rheology.cxx:163-299).  Returns nonzero when the QL fallback of the
// eigen-solver hit its sweep cap.
template <int ND>
__device__ int mc_return_(double bulkm, double shearm, double amc, double anphi, double anpsi, double hardn,
                          double ten_max, double &depls, double *s)
{
    depls = 0;
    double p[3];
    double v[3][3];
    double cos2t = 1, sin2t = 0;
    int rc = 0;
    if (ND == 3) rc = principal_stresses3(s, p, v);
    else principal_stresses2(s, p, cos2t, sin2t);
    constexpr int last = ND - 1;
    double fs = p[0] - p[last] * anphi + amc;
    double ft = p[last] - ten_max;
    if (fs > 0 && ft < 0) return rc;

    double pa = sqrt(1 + anphi * anphi) + anphi;
    double ps = ten_max * anphi - amc;
    double h = p[last] - ten_max + pa * (p[0] - ps);
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double alam;
    if (h < 0) {
        alam = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2 * sqrt(anphi) * hardn);
        p[0] -= alam * (a1 - a2 * anpsi);
        if (ND == 3) p[1] -= alam * (a2 - a2 * anpsi);
        p[last] -= alam * (a2 - a1 * anpsi);
        if (ND == 3) depls = fabs(alam) * sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18);
        else depls = fabs(alam) * sqrt((3 + 2 * anpsi + 3 * anpsi * anpsi) / 8);
    } else {
        alam = ft / a1;
        p[0] -= alam * a2;
        if (ND == 3) p[1] -= alam * a2;
        p[last] -= alam * a1;
        if (ND == 3) depls = fabs(alam) * sqrt(7. / 18);
        else depls = fabs(alam) * sqrt(3. / 8);
    }
    if (ND == 3) {
        double ss[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int m = 0; m < 3; m++)
#pragma unroll
            for (int n = m; n < 3; n++)
#pragma unroll
                for (int k = 0; k < 3; k++) ss[m][n] += v[m][k] * v[n][k] * p[k];
        s[0] = ss[0][0];
        s[1] = ss[1][1];
        s[2] = ss[2][2];
        s[3] = ss[0][1];
        s[4] = ss[0][2];
        s[5] = ss[1][2];
    } else {
        double dc2 = (p[0] - p[1]) * cos2t;
        double dss = p[0] + p[1];
        s[0] = 0.5 * (dss + dc2);
        s[1] = 0.5 * (dss - dc2);
        s[2] = 0.5 * (p[0] - p[1]) * sin2t;
    }
    return rc;
}

// elasto_plastic (rheology.cxx:151-299): elastic trial stress, then the
// return map; in 3D the FP32 screen first skips the eigen-solve of the
// elements that are elastic beyond its error bound (same result, bit for bit)
template <int ND>
__device__ int elasto_plastic_(double bulkm, double shearm, double amc, double anphi, double anpsi,
                               double hardn, double ten_max, const double *de, double &depls, double *s)
{
    elastic_<ND>(bulkm, shearm, de, s);
    if (ND == 3 && clearly_elastic3(amc, anphi, ten_max, s)) {
        depls = 0;
        return 0;
    }
    return mc_return_<ND>(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, depls, s);
}

// elasto_plastic2d: plane-strain Mohr-Coulomb (rheology.cxx:302-507)
__device__ inline void elasto_plastic2d_(double bulkm, double shearm, double amc, double anphi, double anpsi,
                                  double hardn, double ten_max, const double *de, double &depls,
                                  double *s, double &syy)
{
    depls = 0;
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double sxx = s[0] + de[1] * a2 + de[0] * a1;
    double szz = s[1] + de[0] * a2 + de[1] * a1;
    double sxz = s[2] + de[2] * 2 * shearm;
    syy += (de[0] + de[1]) * a2;

    double p[3];
    double cos2t, sin2t;
    int n1, n2, n3;
    {
        double s0 = 0.5 * (sxx + szz);
        double rad = 0.5 * sqrt((sxx - szz) * (sxx - szz) + 4 * sxz * sxz);
        double si = s0 - rad;
        double sii = s0 + rad;
        const double eps = 1e-15;
        if (rad > eps) {
            cos2t = 0.5 * (szz - sxx) / rad;
            sin2t = -sxz / rad;
        } else {
            cos2t = 1;
            sin2t = 0;
        }
        if (syy > sii) {
            n1 = 0; n2 = 1; n3 = 2;
            p[0] = si; p[1] = sii; p[2] = syy;
        } else if (syy < si) {
            n1 = 1; n2 = 2; n3 = 0;
            p[0] = syy; p[1] = si; p[2] = sii;
        } else {
            n1 = 0; n2 = 2; n3 = 1;
            p[0] = si; p[1] = syy; p[2] = sii;
        }
    }
    if (p[0] >= ten_max) {
        s[0] = s[1] = syy = ten_max;
        s[2] = 0.0;
        return;
    }
    if (p[1] >= ten_max) {
        p[1] = p[2] = ten_max;
    } else if (p[2] >= ten_max) {
        p[2] = ten_max;
    }
    double fs = p[0] - p[2] * anphi + amc;
    if (fs >= 0.0) {
        s[0] = sxx;
        s[1] = szz;
        s[2] = sxz;
        return;
    }
    const double alams = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + hardn);
    p[0] -= alams * (a1 - a2 * anpsi);
    p[1] -= alams * (a2 - a2 * anpsi);
    p[2] -= alams * (a2 - a1 * anpsi);
    depls = 0.5 * fabs(alams + alams * anpsi);
    if (p[0] >= ten_max) {
        s[0] = s[1] = syy = ten_max;
        s[2] = 0.0;
        return;
    }
    if (p[1] >= ten_max) {
        p[1] = p[2] = ten_max;
    } else if (p[2] >= ten_max) {
        p[2] = ten_max;
    }
    double pn1 = (n1 == 0) ? p[0] : p[1];
    double pn2 = (n2 == 1) ? p[1] : p[2];
    double pn3 = (n3 == 0) ? p[0] : ((n3 == 1) ? p[1] : p[2]);
    double dc2 = (pn1 - pn2) * cos2t;
    double dss = pn1 + pn2;
    s[0] = 0.5 * (dss + dc2);
    s[1] = 0.5 * (dss - dc2);
    s[2] = 0.5 * (pn1 - pn2) * sin2t;
    syy = pn3;
}

// One element of update_stress (rheology.cxx:510-646).  In/out arrays are
// the element's own values; dt = Variables::dt.  Returns a DES_DEV_* bit set.
template <int ND>
__device__ unsigned update_stress_elem(const KP &p, int e, double dt, double *s, double &syy, double *es,
                                       double *edot, double &pls, double &dpls, double edvoldt, double vol,
                                       double vol_old, double &dpressure)
{
    constexpr int NSTR = ND * (ND + 1) / 2;
    unsigned bits = 0;
    double old_s = trace_<ND>(s);
    {
        double div = trace_<ND>(edot);
#pragma unroll
        for (int i = 0; i < ND; ++i) edot[i] += divnd<ND>(edvoldt - div);
    }
#pragma unroll
    for (int i = 0; i < NSTR; ++i) es[i] += edot[i] * dt;
    double de[NSTR];
#pragma unroll
    for (int i = 0; i < NSTR; ++i) de[i] = edot[i] * dt;

    const int rt = p.mat.rheol_type;
    if (rt == DES_RH_ELASTIC) {
        elastic_<ND>(m_bulkm(p, e), m_shearm(p, e), de, s);
    } else if (rt == DES_RH_VISCOUS) {
        viscous_<ND>(m_bulkm(p, e), m_visc<ND>(p, e, edot), trace_<ND>(es), edot, s);
    } else if (rt == DES_RH_MAXWELL) {
        double dv = vol / vol_old - 1;
        const double viscosity = m_visc<ND>(p, e, edot);
        if (p.tape_visc) p.tape_visc[e] = viscosity;
        maxwell_<ND>(m_bulkm(p, e), m_shearm(p, e), viscosity, dt, dv, de, s);
    } else if (rt == DES_RH_EP) {
        double depls = 0, amc, anphi, anpsi, hardn, ten_max;
        double bulkm = m_bulkm(p, e), shearm = m_shearm(p, e);
        m_plastic_props(p, e, pls, amc, anphi, anpsi, hardn, ten_max);
        if (p.mat.is_plane_strain)
            elasto_plastic2d_(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, s, syy);
        else if (elasto_plastic_<ND>(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, s))
            bits |= DES_DEV_QL_NOCONV;
        pls += depls;
        dpls = depls;
    } else if (rt == DES_RH_EVP) {
        double depls = 0;
        double bulkm = m_bulkm(p, e), shearm = m_shearm(p, e);
        double viscosity = m_visc<ND>(p, e, edot);
        if (p.tape_visc) p.tape_visc[e] = viscosity;
        double dv = vol / vol_old - 1;
        double sv[NSTR];
#pragma unroll
        for (int i = 0; i < NSTR; ++i) sv[i] = s[i];
        maxwell_<ND>(bulkm, shearm, viscosity, dt, dv, de, sv);
        double amc, anphi, anpsi, hardn, ten_max;
        m_plastic_props(p, e, pls, amc, anphi, anpsi, hardn, ten_max);
        double sp[NSTR], spyy = syy;
#pragma unroll
        for (int i = 0; i < NSTR; ++i) sp[i] = s[i];
        if (p.mat.is_plane_strain)
            elasto_plastic2d_(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, sp, spyy);
        else if (elasto_plastic_<ND>(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, sp))
            bits |= DES_DEV_QL_NOCONV;
        // svII < spII, decided in FP32 where the two are clearly apart
        int vless = -1;
        if constexpr (ND == 3) vless = j2_less(j2_est3(sv), j2_est3(sp));
        if (vless < 0) vless = second_invariant2_<ND>(sv) < second_invariant2_<ND>(sp);
        if (p.tape_evp) p.tape_evp[e] = vless ? 0 : 1;
        if (vless) {
#pragma unroll
            for (int i = 0; i < NSTR; ++i) s[i] = sv[i];
        } else {
#pragma unroll
            for (int i = 0; i < NSTR; ++i) s[i] = sp[i];
            pls += depls;
            dpls = depls;
            // rheology.cxx:632 copies spyy, which is initialised only in plane
            // strain; elsewhere stressyy is left unchanged.
            if (p.mat.is_plane_strain) syy = spyy;
        }
    }
    dpressure = trace_<ND>(s) - old_s;
    return bits;
}

}  // namespace des
