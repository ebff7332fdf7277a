/*
 * des_oracle.c -- CPU restatement (oracle) of the reference's explicit
 * time-step hot path.  TEST INFRASTRUCTURE ONLY (see des_oracle.h): parity
 * tests, the smoke check and bench.py's CPU-baseline leg call it; the
 * product library never does.
 *
 * Each function cites the reference file:line whose arithmetic it restates.
 * Expression order is kept as in the reference so that, compiled without
 * FP contraction (-ffp-contract=off), a 1-thread run reproduces the
 * reference's serial results.  With nthreads > 1 the loops use OpenMP in the
 * reference's pattern (element-parallel loops; two-colour element bands for
 * scatters, utils.hpp:18-44 and mesh.cxx:1724-1817).
 */
#include "des_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef DES_ORACLE_PERTURB_LIBM
/* Sensitivity probe (a separate build, liboracle_pert.so): every libm
 * transcendental result is moved by -1, 0 or +1 ulp, pseudo-randomly, to
 * measure how far the reference's own algorithm drifts when its libm
 * differs in the last bit -- the envelope inside which any other faithful
 * implementation (another libm, another processor) must land. */
/* One xorshift stream per thread: thread t starts from seed ^ (t * golden
 * ratio) -- thread 0 from the seed itself -- whenever a new seed was set, so
 * an OpenMP run (static schedule, fixed thread count) is reproducible and
 * free of data races, and a one-thread run draws the single stream. */
static unsigned long long pert_seed = 88172645463325252ull;
static int pert_epoch = 1;
static __thread unsigned long long pert_state;
static __thread int pert_seen;
void oracle_perturb_seed(unsigned long long s)
{
    pert_seed = s ? s : 88172645463325252ull;
    ++pert_epoch;
}
static double pert_(double x)
{
    if (pert_seen != pert_epoch) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        pert_state = pert_seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)tid);
        if (!pert_state) pert_state = 88172645463325252ull;
        pert_seen = pert_epoch;
    }
    pert_state ^= pert_state << 13;
    pert_state ^= pert_state >> 7;
    pert_state ^= pert_state << 17;
    int r = (int)(pert_state % 3);
    if (r == 0) return nextafter(x, INFINITY);
    if (r == 1) return nextafter(x, -INFINITY);
    return x;
}
#define sin(x) pert_(sin(x))
#define cos(x) pert_(cos(x))
#define tan(x) pert_(tan(x))
#define pow(a, b) pert_(pow(a, b))
#define exp(x) pert_(exp(x))
#define atan2(a, b) pert_(atan2(a, b))
#endif

#define MAXND 3
#define MAXNPE 4
#define MAXNSTR 6

/* NODE_OF_FACET (constants.hpp:59-71) */
static const int FACET3[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
static const int FACET2[3][2] = {{1, 2}, {2, 0}, {0, 1}};

#define BOUNDX0 (1u << 0)
#define BOUNDX1 (1u << 1)
#define BOUNDY0 (1u << 2)
#define BOUNDY1 (1u << 3)
#define BOUNDZ0 (1u << 4)
#define BOUNDZ1 (1u << 5)
#define BOUND_ANY 1023u

static const double DEG2RAD_ = 3.1415926535897932384626433832795 / 180;

struct oracle_ctx {
    const des_mesh *mesh;
    const des_params *param;
    const des_material *mat;
    des_host_state *st;
    int nd, npe, nstr, nn, ne;
    int nthreads;
    int *egroups;     /* element band boundaries, size ngroups+1 */
    int ngroups;
    double *tmp_nn;   /* used when st->ntmp is NULL */
    const double *ef[DES_EF_COUNT];
};

/* ------------------------------------------------------------------ */
/* small tensor helpers (utils.hpp:100-128)                            */
/* ------------------------------------------------------------------ */
static double trace_(int nd, const double *s)
{
    return nd == 3 ? s[0] + s[1] + s[2] : s[0] + s[1];
}

static double second_invariant2_(int nd, const double *t)
{
    if (nd == 3) {
        double a = (t[0] + t[1] + t[2]) / 3;
        return (0.5 * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a))
                + t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
    }
    return 0.25 * (t[0] - t[1]) * (t[0] - t[1]) + t[2] * t[2];
}

static double second_invariant_(int nd, const double *t) { return sqrt(second_invariant2_(nd, t)); }

static double dmax_(double a, double b) { return (a < b) ? b : a; } /* std::max */
static double dmin_(double a, double b) { return (b < a) ? b : a; } /* std::min */

/* ------------------------------------------------------------------ */
/* material properties (matprops.cxx)                                  */
/* ------------------------------------------------------------------ */
static int mcount(const oracle_ctx *c, int e, int m)
{
    if (c->mat->elemmarkers) return c->mat->elemmarkers[(size_t)e * c->mat->nmat + m];
    return m == 0 ? 1 : 0;
}

/* harmonic_mean (matprops.cxx:117-128) */
static double hmean(const oracle_ctx *c, const double *s, int bit, int e)
{
    const des_material *mt = c->mat;
    if (mt->nmat == 1 || (mt->scalar_mask >> bit & 1u)) return s[0];
    double result = 0;
    int m = 0;
    for (int i = 0; i < mt->nmat; i++) {
        int n = mcount(c, e, i);
        result += n / s[i];
        m += n;
    }
    return m / result;
}

/* arithmetic_mean (matprops.cxx:103-114) */
static double amean(const oracle_ctx *c, const double *s, int bit, int e)
{
    const des_material *mt = c->mat;
    if (mt->nmat == 1 || (mt->scalar_mask >> bit & 1u)) return s[0];
    double result = 0;
    int m = 0;
    for (int i = 0; i < mt->nmat; i++) {
        int n = mcount(c, e, i);
        result += n * s[i];
        m += n;
    }
    return result / m;
}

static double m_bulkm(const oracle_ctx *c, int e) { return hmean(c, c->mat->bulk_modulus, 0, e); }   /* :264-267 */
static double m_shearm(const oracle_ctx *c, int e)                                                     /* :270-273 */
{
    if (c->ef[DES_EF_SHEAR_MODULUS]) return c->ef[DES_EF_SHEAR_MODULUS][e];
    return hmean(c, c->mat->shear_modulus, 1, e);
}
static double m_cp(const oracle_ctx *c, int e) { return amean(c, c->mat->heat_capacity, 2, e); }      /* :400-403 */
static double m_hr(const oracle_ctx *c, int e) { return amean(c, c->mat->radiogenic_heating, 3, e); } /* :405-408 */
static double m_k(const oracle_ctx *c, int e)                                                          /* :411-414 */
{
    if (c->ef[DES_EF_THERM_COND]) return c->ef[DES_EF_THERM_COND][e];
    return amean(c, c->mat->therm_cond, 4, e);
}

static double elem_avg_T(const oracle_ctx *c, int e)
{
    const int *conn = c->mesh->connectivity + (size_t)e * c->npe;
    const double *T = c->st->temperature;
    double t = 0;
    for (int i = 0; i < c->npe; ++i) t += T[conn[i]];
    return t / c->npe;
}

/* MatProps::visc (matprops.cxx:276-312) */
static double m_visc(const oracle_ctx *c, int e)
{
    const des_material *mt = c->mat;
    double v;
    if (c->ef[DES_EF_LOG10_VISC]) {
        v = pow(10.0, c->ef[DES_EF_LOG10_VISC][e]);
    } else {
        const double gas_constant = 8.3144;
        const double min_strain_rate = 1e-30;
        double T = elem_avg_T(c, e);
        double edot = second_invariant_(c->nd, c->st->strain_rate + (size_t)e * c->nstr);
        edot = dmax_(edot, min_strain_rate);
        double result = 0;
        int n = 0;
        for (int m = 0; m < mt->nmat; m++) {
            double pw = 1 / mt->visc_exponent[m] - 1;
            double pw1 = -1 / mt->visc_exponent[m];
            double visc0 = 0.25 * pow(edot, pw) * pow(0.75 * mt->visc_coefficient[m], pw1)
                * exp(mt->visc_activation_energy[m] / (mt->visc_exponent[m] * gas_constant * T)) * 1e6;
            int k = mcount(c, e, m);
            result += k / visc0;
            n += k;
        }
        v = n / result;
    }
    return dmin_(dmax_(v, mt->visc_min), mt->visc_max);
}

/* MatProps::plastic_weakening (matprops.cxx:315-353) */
static void m_plastic_weakening(const oracle_ctx *c, int e, double pls, double *cohesion,
                                double *friction_angle, double *dilation_angle, double *hardening)
{
    const des_material *mt = c->mat;
    double cc = 0, f = 0, d = 0, h = 0;
    int n = 0;
    for (int m = 0; m < mt->nmat; m++) {
        int k = mcount(c, e, m);
        if (k == 0) continue;
        n += k;
        double c0 = c->ef[DES_EF_COHESION0] ? c->ef[DES_EF_COHESION0][e] : mt->cohesion0[m];
        double c1 = c->ef[DES_EF_COHESION1] ? c->ef[DES_EF_COHESION1][e] : mt->cohesion1[m];
        double f0 = c->ef[DES_EF_FRICTION0] ? c->ef[DES_EF_FRICTION0][e] : mt->friction_angle0[m];
        double f1 = c->ef[DES_EF_FRICTION1] ? c->ef[DES_EF_FRICTION1][e] : mt->friction_angle1[m];
        double d0 = mt->dilation_angle0[m], d1 = mt->dilation_angle1[m];
        if (pls < mt->pls0[m]) {
            cc += c0 * k;
            f += f0 * k;
            d += d0 * k;
            h += 0;
        } else if (pls < mt->pls1[m]) {
            double p = (pls - mt->pls0[m]) / (mt->pls1[m] - mt->pls0[m]);
            cc += (c0 + p * (c1 - c0)) * k;
            f += (f0 + p * (f1 - f0)) * k;
            d += (d0 + p * (d1 - d0)) * k;
            h += (c1 - c0) / (mt->pls1[m] - mt->pls0[m]) * k;
        } else {
            cc += c1 * k;
            f += f1 * k;
            d += d1 * k;
            h += 0;
        }
    }
    *cohesion = cc / n;
    *friction_angle = f / n;
    *dilation_angle = d / n;
    *hardening = h / n;
}

/* MatProps::plastic_props (matprops.cxx:356-373) */
static void m_plastic_props(const oracle_ctx *c, int e, double pls, double *amc, double *anphi,
                            double *anpsi, double *hardn, double *ten_max)
{
    double cohesion, phi, psi;
    m_plastic_weakening(c, e, pls, &cohesion, &phi, &psi, hardn);
    double sphi = sin(phi * DEG2RAD_);
    double spsi = sin(psi * DEG2RAD_);
    *anphi = (1 + sphi) / (1 - sphi);
    *anpsi = (1 + spsi) / (1 - spsi);
    *amc = 2 * cohesion * sqrt(*anphi);
    *ten_max = (phi == 0) ? c->mat->tension_max : dmin_(c->mat->tension_max, cohesion / tan(phi * DEG2RAD_));
}

/* MatProps::rho (matprops.cxx:376-397) */
static double m_rho(const oracle_ctx *c, int e)
{
    const double celsius0 = 273;
    double T = elem_avg_T(c, e);
    double TinCelsius = T - celsius0;
    double result = 0;
    int n = 0;
    for (int m = 0; m < c->mat->nmat; m++) {
        int k = mcount(c, e, m);
        result += c->mat->rho0[m] * (1 - c->mat->alpha[m] * TinCelsius) * k;
        n += k;
    }
    return result / n;
}

/* ref_pressure (matprops.cxx:190-202), option 0 (lithostatic with rho0[0]) */
static double ref_pressure_(const oracle_ctx *c, double z)
{
    double depth = -z;
    return c->mat->rho0[0] * c->param->gravity * depth;
}

/* ------------------------------------------------------------------ */
/* 3x3 symmetric eigen-solver: J. Kopp, "Efficient numerical           */
/* diagonalization of hermitian 3x3 matrices", Int. J. Mod. Phys. C 19 */
/* (2008) 523 (arXiv:physics/0610206).  Hybrid method as vendored in   */
/* 3x3-C/dsyevh3.c:31-134: analytic (Cardano) eigenvalues              */
/* (dsyevc3.c:31-80), eigenvectors from cross products, falling back   */
/* to Householder tridiagonalisation (dsytrd3.c:28-105) + QL          */
/* (dsyevq3.c:29-134) when a cross product is too small.               */
/* Only the upper triangle a[0..2][i>=j] of A is read.                  */
/* ------------------------------------------------------------------ */
static void eig_cardano(const double A[3][3], double w[3])
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

static void eig_tridiag(const double A[3][3], double Q[3][3], double d[3], double e[2])
{
    double u[3], q[3];
    double omega, f, K, h, g;
    for (int i = 0; i < 3; i++) {
        Q[i][i] = 1.0;
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
        for (int i = 1; i < 3; i++) {
            f = A[1][i] * u[1] + A[i][2] * u[2];
            q[i] = omega * f;
            K += u[i] * f;
        }
        K *= 0.5 * (omega * omega);
        for (int i = 1; i < 3; i++) q[i] = q[i] - K * u[i];
        d[0] = A[0][0];
        d[1] = A[1][1] - 2.0 * q[1] * u[1];
        d[2] = A[2][2] - 2.0 * q[2] * u[2];
        for (int j = 1; j < 3; j++) {
            f = omega * u[j];
            for (int i = 1; i < 3; i++) Q[i][j] = Q[i][j] - f * u[i];
        }
        e[1] = A[1][2] - q[1] * u[2] - u[1] * q[2];
    } else {
        for (int i = 0; i < 3; i++) d[i] = A[i][i];
        e[1] = A[1][2];
    }
}

static int eig_ql(const double A[3][3], double Q[3][3], double w[3])
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

static int eig_hybrid(const double A[3][3], double Q[3][3], double w[3], int *used_ql)
{
    double norm, error, t, u;
    *used_ql = 0;
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
    if (norm <= error) {
        *used_ql = 1;
        return eig_ql(A, Q, w);
    }
    norm = sqrt(1.0 / norm);
    for (int j = 0; j < 3; j++) Q[j][0] = Q[j][0] * norm;

    Q[0][1] = Q[0][1] + A[0][2] * w[1];
    Q[1][1] = Q[1][1] + A[1][2] * w[1];
    Q[2][1] = (A[0][0] - w[1]) * (A[1][1] - w[1]) - Q[2][1];
    norm = Q[0][1] * Q[0][1] + Q[1][1] * Q[1][1] + Q[2][1] * Q[2][1];
    if (norm <= error) {
        *used_ql = 1;
        return eig_ql(A, Q, w);
    }
    norm = sqrt(1.0 / norm);
    for (int j = 0; j < 3; j++) Q[j][1] = Q[j][1] * norm;

    Q[0][2] = Q[1][0] * Q[2][1] - Q[2][0] * Q[1][1];
    Q[1][2] = Q[2][0] * Q[0][1] - Q[0][0] * Q[2][1];
    Q[2][2] = Q[0][0] * Q[1][1] - Q[1][0] * Q[0][1];
    return 0;
}

int oracle_eigen3(const double a6[6], double w[3], double q[9], int *used_ql)
{
    double A[3][3] = {{a6[0], a6[3], a6[4]}, {0, a6[1], a6[5]}, {0, 0, a6[2]}};
    double Q[3][3];
    int rc = eig_hybrid(A, Q, w, used_ql);
    memcpy(q, Q, sizeof Q);
    return rc;
}

/* principal_stresses3 (rheology.cxx:13-68): eigen-solve, then sort ascending */
static void principal_stresses3_(const double *s, double p[3], double v[3][3])
{
    double a[3][3] = {{s[0], s[3], s[4]}, {0, s[1], s[5]}, {0, 0, s[2]}};
    int ql;
    eig_hybrid(a, v, p, &ql);
    /* three compare-and-swap passes on (0,1), (1,2), (0,1) */
    const int pairs[3][2] = {{0, 1}, {1, 2}, {0, 1}};
    for (int k = 0; k < 3; k++) {
        int i = pairs[k][0], j = pairs[k][1];
        if (p[i] > p[j]) {
            double t = p[i];
            p[i] = p[j];
            p[j] = t;
            for (int r = 0; r < 3; r++) {
                double b = v[r][i];
                v[r][i] = v[r][j];
                v[r][j] = b;
            }
        }
    }
}

void oracle_principal_stresses3(const double s[6], double p[3], double v[9])
{
    double vv[3][3];
    principal_stresses3_(s, p, vv);
    memcpy(v, vv, sizeof vv);
}

/* principal_stresses2 (rheology.cxx:71-102) */
static void principal_stresses2_(const double *s, double p[2], double *cos2t, double *sin2t)
{
    double s0 = 0.5 * (s[0] + s[1]);
    double rad = second_invariant_(2, s);
    p[0] = s0 - rad;
    p[1] = s0 + rad;
    const double eps = 1e-15;
    double a = 0.5 * (s[0] - s[1]);
    double b = -rad;
    if (b < -eps) {
        *cos2t = a / b;
        *sin2t = s[2] / b;
    } else {
        *cos2t = 1;
        *sin2t = 0;
    }
}

/* ------------------------------------------------------------------ */
/* constitutive updates (rheology.cxx:105-507)                         */
/* ------------------------------------------------------------------ */
static void elastic_(int nd, double bulkm, double shearm, const double *de, double *s)
{
    int nstr = nd == 3 ? 6 : 3;
    double lambda = bulkm - 2. / 3 * shearm;
    double dev = trace_(nd, de);
    for (int i = 0; i < nd; ++i) s[i] += 2 * shearm * de[i] + lambda * dev;
    for (int i = nd; i < nstr; ++i) s[i] += 2 * shearm * de[i];
}

static void maxwell_(int nd, double bulkm, double shearm, double viscosity, double dt, double dv,
                     const double *de, double *s)
{
    int nstr = nd == 3 ? 6 : 3;
    double tmp = 0.5 * dt * shearm / viscosity;
    double f1 = 1 - tmp;
    double f2 = 1 / (1 + tmp);
    double dev = trace_(nd, de) / nd;
    double s0 = trace_(nd, s) / nd;
    for (int i = 0; i < nd; ++i)
        s[i] = ((s[i] - s0) * f1 + 2 * shearm * (de[i] - dev)) * f2 + s0 + bulkm * dv;
    for (int i = nd; i < nstr; ++i) s[i] = (s[i] * f1 + 2 * shearm * de[i]) * f2;
}

static void viscous_(int nd, double bulkm, double viscosity, double total_dv, const double *edot,
                     double *s)
{
    int nstr = nd == 3 ? 6 : 3;
    double dev = trace_(nd, edot) / nd;
    for (int i = 0; i < nd; ++i) s[i] = 2 * viscosity * (edot[i] - dev) + bulkm * total_dv;
    for (int i = nd; i < nstr; ++i) s[i] = 2 * viscosity * edot[i];
}

/* elasto_plastic (rheology.cxx:151-299) */
static void elasto_plastic_(int nd, double bulkm, double shearm, double amc, double anphi,
                            double anpsi, double hardn, double ten_max, const double *de,
                            double *depls, double *s, int *failure_mode)
{
    elastic_(nd, bulkm, shearm, de, s);
    *depls = 0;
    *failure_mode = 0;
    double p[3];
    double v[3][3];
    double cos2t = 1, sin2t = 0;
    if (nd == 3) principal_stresses3_(s, p, v);
    else principal_stresses2_(s, p, &cos2t, &sin2t);
    const int last = nd - 1;
    double fs = p[0] - p[last] * anphi + amc;
    double ft = p[last] - ten_max;
    if (fs > 0 && ft < 0) return;

    double pa = sqrt(1 + anphi * anphi) + anphi;
    double ps = ten_max * anphi - amc;
    double h = p[last] - ten_max + pa * (p[0] - ps);
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double alam;
    if (h < 0) {
        *failure_mode = 10;
        alam = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2 * sqrt(anphi) * hardn);
        p[0] -= alam * (a1 - a2 * anpsi);
        if (nd == 3) p[1] -= alam * (a2 - a2 * anpsi);
        p[last] -= alam * (a2 - a1 * anpsi);
        if (nd == 3) *depls = fabs(alam) * sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18);
        else *depls = fabs(alam) * sqrt((3 + 2 * anpsi + 3 * anpsi * anpsi) / 8);
    } else {
        *failure_mode = 1;
        alam = ft / a1;
        p[0] -= alam * a2;
        if (nd == 3) p[1] -= alam * a2;
        p[last] -= alam * a1;
        if (nd == 3) *depls = fabs(alam) * sqrt(7. / 18);
        else *depls = fabs(alam) * sqrt(3. / 8);
    }

    if (nd == 3) {
        double ss[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int m = 0; m < 3; m++)
            for (int n = m; n < 3; n++)
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
}

/* elasto_plastic2d: plane-strain Mohr-Coulomb (rheology.cxx:302-507) */
static void elasto_plastic2d_(double bulkm, double shearm, double amc, double anphi, double anpsi,
                              double hardn, double ten_max, const double *de, double *depls,
                              double *s, double *syy, int *failure_mode)
{
    *depls = 0;
    *failure_mode = 0;
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double sxx = s[0] + de[1] * a2 + de[0] * a1;
    double szz = s[1] + de[0] * a2 + de[1] * a1;
    double sxz = s[2] + de[2] * 2 * shearm;
    *syy += (de[0] + de[1]) * a2;

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
        if (*syy > sii) { /* syy is the minor principal stress */
            n1 = 0; n2 = 1; n3 = 2;
            p[0] = si; p[1] = sii; p[2] = *syy;
        } else if (*syy < si) { /* syy is the major one */
            n1 = 1; n2 = 2; n3 = 0;
            p[0] = *syy; p[1] = si; p[2] = sii;
        } else { /* intermediate */
            n1 = 0; n2 = 2; n3 = 1;
            p[0] = si; p[1] = *syy; p[2] = sii;
        }
    }

    if (p[0] >= ten_max) {
        s[0] = s[1] = *syy = ten_max;
        s[2] = 0.0;
        *failure_mode = 1;
        return;
    }
    if (p[1] >= ten_max) {
        p[1] = p[2] = ten_max;
        *failure_mode = 2;
    } else if (p[2] >= ten_max) {
        p[2] = ten_max;
        *failure_mode = 3;
    }

    double fs = p[0] - p[2] * anphi + amc;
    if (fs >= 0.0) {
        s[0] = sxx;
        s[1] = szz;
        s[2] = sxz;
        return;
    }
    *failure_mode += 10;
    const double alams = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + hardn);
    p[0] -= alams * (a1 - a2 * anpsi);
    p[1] -= alams * (a2 - a2 * anpsi);
    p[2] -= alams * (a2 - a1 * anpsi);
    *depls = 0.5 * fabs(alams + alams * anpsi);

    if (p[0] >= ten_max) {
        s[0] = s[1] = *syy = ten_max;
        s[2] = 0.0;
        *failure_mode += 20;
        return;
    }
    if (p[1] >= ten_max) {
        p[1] = p[2] = ten_max;
        *failure_mode += 20;
    } else if (p[2] >= ten_max) {
        p[2] = ten_max;
        *failure_mode += 20;
    }
    {
        double dc2 = (p[n1] - p[n2]) * cos2t;
        double dss = p[n1] + p[n2];
        s[0] = 0.5 * (dss + dc2);
        s[1] = 0.5 * (dss - dc2);
        s[2] = 0.5 * (p[n1] - p[n2]) * sin2t;
        *syy = p[n3];
    }
}

/* ------------------------------------------------------------------ */
/* loop helpers: loop_all_elem (utils.hpp:18-44)                       */
/* ------------------------------------------------------------------ */
typedef void (*elem_fn)(oracle_ctx *c, int e, void *arg);

static void loop_all_elem(oracle_ctx *c, elem_fn fn, void *arg)
{
#ifdef _OPENMP
    if (c->nthreads > 1) {
        const int *eg = c->egroups;
        int ng = c->ngroups;
#pragma omp parallel for num_threads(c->nthreads) schedule(static)
        for (int i = 0; i < ng; i += 2)
            for (int e = eg[i]; e < eg[i + 1]; ++e) fn(c, e, arg);
#pragma omp parallel for num_threads(c->nthreads) schedule(static)
        for (int i = 1; i < ng; i += 2)
            for (int e = eg[i]; e < eg[i + 1]; ++e) fn(c, e, arg);
        return;
    }
#endif
    for (int e = 0; e < c->ne; ++e) fn(c, e, arg);
}

#ifdef _OPENMP
#define PFOR _Pragma("omp parallel for num_threads(c->nthreads) schedule(static) if(c->nthreads > 1)")
#else
#define PFOR
#endif

/* ------------------------------------------------------------------ */
/* geometry (geometry.cxx)                                             */
/* ------------------------------------------------------------------ */
static double dist2_(int nd, const double *a, const double *b)
{
    double sum = 0;
    for (int i = 0; i < nd; ++i) {
        double d = b[i] - a[i];
        sum += d * d;
    }
    return sum;
}

/* tetrahedron_volume (geometry.cxx:29-49) */
static double tet_volume(const double *d0, const double *d1, const double *d2, const double *d3)
{
    double x01 = d0[0] - d1[0], x12 = d1[0] - d2[0], x23 = d2[0] - d3[0];
    double y01 = d0[1] - d1[1], y12 = d1[1] - d2[1], y23 = d2[1] - d3[1];
    double z01 = d0[2] - d1[2], z12 = d1[2] - d2[2], z23 = d2[2] - d3[2];
    return (x01 * (y23 * z12 - y12 * z23) + x12 * (y01 * z23 - y23 * z01) + x23 * (y12 * z01 - y01 * z12)) / 6;
}

/* triangle_area (geometry.cxx:53-83) */
static double tri_area(int nd, const double *a, const double *b, const double *c)
{
    double ab0 = b[0] - a[0], ab1 = b[1] - a[1];
    double ac0 = c[0] - a[0], ac1 = c[1] - a[1];
    if (nd == 2) return fabs(ab0 * ac1 - ab1 * ac0) / 2;
    double ab2 = b[2] - a[2], ac2 = c[2] - a[2];
    double d0 = ab1 * ac2 - ab2 * ac1;
    double d1 = ab2 * ac0 - ab0 * ac2;
    double d2 = ab0 * ac1 - ab1 * ac0;
    return sqrt(d0 * d0 + d1 * d1 + d2 * d2) / 2;
}

#define CO(n) (st->coord + (size_t)(n) * nd)

void oracle_compute_volume(oracle_ctx *c) /* geometry.cxx:86-108 */
{
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe, ne = c->ne;
    const int *cn = c->mesh->connectivity;
    PFOR
    for (int e = 0; e < ne; ++e) {
        const int *k = cn + (size_t)e * npe;
        if (nd == 3) st->volume[e] = tet_volume(CO(k[0]), CO(k[1]), CO(k[2]), CO(k[3]));
        else st->volume[e] = tri_area(2, CO(k[0]), CO(k[1]), CO(k[2]));
    }
}

static void dvoldt_elem(oracle_ctx *c, int e, void *arg)
{
    double *dvoldt = (double *)arg;
    const int *k = c->mesh->connectivity + (size_t)e * c->npe;
    double dj = trace_(c->nd, c->st->strain_rate + (size_t)e * c->nstr);
    for (int i = 0; i < c->npe; ++i) dvoldt[k[i]] += dj * c->st->volume[e];
}

static double *ntmp_(oracle_ctx *c) { return c->st->ntmp ? c->st->ntmp : c->tmp_nn; }

void oracle_compute_dvoldt(oracle_ctx *c) /* geometry.cxx:111-155 */
{
    double *dvoldt = ntmp_(c);
    memset(dvoldt, 0, sizeof(double) * c->nn);
    loop_all_elem(c, dvoldt_elem, dvoldt);
    const double *vn = c->st->volume_n;
    PFOR
    for (int n = 0; n < c->nn; ++n) dvoldt[n] /= vn[n];
}

void oracle_compute_edvoldt(oracle_ctx *c) /* geometry.cxx:158-179 */
{
    const double *dvoldt = ntmp_(c);
    double *edvoldt = c->st->edvoldt;
    const int *cn = c->mesh->connectivity;
    const int npe = c->npe;
    PFOR
    for (int e = 0; e < c->ne; ++e) {
        const int *k = cn + (size_t)e * npe;
        double dj = 0;
        for (int i = 0; i < npe; ++i) dj += dvoldt[k[i]];
        edvoldt[e] = dj / npe;
    }
}

static void nmd_elem(oracle_ctx *c, int e, void *arg)
{
    double *dp_nd = (double *)arg;
    const int *k = c->mesh->connectivity + (size_t)e * c->npe;
    double dp = c->st->dpressure[e];
    for (int i = 0; i < c->npe; ++i) dp_nd[k[i]] += dp * c->st->volume[e];
}

void oracle_NMD_stress(oracle_ctx *c) /* geometry.cxx:182-236 */
{
    des_host_state *st = c->st;
    double *dp_nd = ntmp_(c);
    memset(dp_nd, 0, sizeof(double) * c->nn);
    loop_all_elem(c, nmd_elem, dp_nd);
    PFOR
    for (int n = 0; n < c->nn; ++n) dp_nd[n] /= st->volume_n[n];
    const int *cn = c->mesh->connectivity;
    const int npe = c->npe, nd = c->nd, nstr = c->nstr;
    PFOR
    for (int e = 0; e < c->ne; ++e) {
        const int *k = cn + (size_t)e * npe;
        double dp = 0;
        for (int i = 0; i < npe; ++i) dp += dp_nd[k[i]];
        double dp_el = dp / npe;
        double *s = st->stress + (size_t)e * nstr;
        double dp_orig = st->dpressure[e];
        for (int i = 0; i < nd; ++i) s[i] += (-dp_orig + dp_el) / nd;
    }
}

int oracle_compute_dt(oracle_ctx *c, double *dt_out) /* geometry.cxx:239-310 */
{
    const des_params *pr = c->param;
    if (pr->fixed_dt != 0) {
        *dt_out = pr->fixed_dt;
        return 0;
    }
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe;
    double dt_maxwell = DBL_MAX, dt_diffusion = DBL_MAX, minl = DBL_MAX;
    for (int e = 0; e < c->ne; ++e) {
        const int *k = c->mesh->connectivity + (size_t)e * npe;
        const double *a = CO(k[0]), *b = CO(k[1]), *cc = CO(k[2]);
        double minh;
        if (nd == 3) {
            const double *d = CO(k[3]);
            double maxa = dmax_(dmax_(tri_area(3, a, b, cc), tri_area(3, a, b, d)),
                                dmax_(tri_area(3, cc, d, a), tri_area(3, cc, d, b)));
            minh = 3 * st->volume[e] / maxa;
        } else {
            double maxl = sqrt(dmax_(dmax_(dist2_(2, a, b), dist2_(2, b, cc)), dist2_(2, a, cc)));
            minh = 2 * st->volume[e] / maxl;
        }
        dt_maxwell = dmin_(dt_maxwell, 0.5 * c->mat->visc_min / (1e-40 + m_shearm(c, e)));
        if (pr->has_thermal_diffusion)
            dt_diffusion = dmin_(dt_diffusion, 0.5 * minh * minh / c->mat->therm_diff_max);
        minl = dmin_(minl, minh);
    }
    double dt_advection = 0.5 * minl / pr->max_vbc_val;
    double dt_elastic = pr->is_quasi_static
        ? 0.5 * minl / (pr->max_vbc_val * pr->inertial_scaling)
        : 0.5 * minl / sqrt(m_bulkm(c, 0) / m_rho(c, 0));
    double dt = dmin_(dmin_(dt_elastic, dt_maxwell), dmin_(dt_advection, dt_diffusion)) * pr->dt_fraction;
    *dt_out = dt;
    if (dt <= 0) return DES_ERUNTIME; /* geometry.cxx:304-308 (NaN passes, as there) */
    return 0;
}

struct mass_arg {
    double pseudo_speed;
};

static void mass_elem(oracle_ctx *c, int e, void *arg)
{
    des_host_state *st = c->st;
    const des_params *pr = c->param;
    double pseudo_speed = ((struct mass_arg *)arg)->pseudo_speed;
    double rho = pr->is_quasi_static ? m_bulkm(c, e) / (pseudo_speed * pseudo_speed) : m_rho(c, e);
    double m = rho * st->volume[e] / c->npe;
    double tm = m_rho(c, e) * m_cp(c, e) * st->volume[e] / c->npe;
    const int *k = c->mesh->connectivity + (size_t)e * c->npe;
    for (int i = 0; i < c->npe; ++i) {
        st->volume_n[k[i]] += st->volume[e];
        st->mass[k[i]] += m;
        if (pr->has_thermal_diffusion) st->tmass[k[i]] += tm;
    }
}

void oracle_compute_mass(oracle_ctx *c) /* geometry.cxx:313-365 */
{
    des_host_state *st = c->st;
    memset(st->volume_n, 0, sizeof(double) * c->nn);
    memset(st->mass, 0, sizeof(double) * c->nn);
    memset(st->tmass, 0, sizeof(double) * c->nn);
    struct mass_arg a = {c->param->max_vbc_val * c->param->inertial_scaling};
    loop_all_elem(c, mass_elem, &a);
}

static void shape_elem(oracle_ctx *c, int e, void *arg)
{
    (void)arg;
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe;
    const int *k = c->mesh->connectivity + (size_t)e * npe;
    const double *d0 = CO(k[0]), *d1 = CO(k[1]), *d2 = CO(k[2]);
    double *sx = st->shpdx + (size_t)e * npe;
    double *sz = st->shpdz + (size_t)e * npe;
    if (nd == 3) {
        const double *d3 = CO(k[3]);
        double *sy = st->shpdy + (size_t)e * npe;
        double iv = 1 / (6 * st->volume[e]);
        double x01 = d0[0] - d1[0], x02 = d0[0] - d2[0], x03 = d0[0] - d3[0];
        double x12 = d1[0] - d2[0], x13 = d1[0] - d3[0], x23 = d2[0] - d3[0];
        double y01 = d0[1] - d1[1], y02 = d0[1] - d2[1], y03 = d0[1] - d3[1];
        double y12 = d1[1] - d2[1], y13 = d1[1] - d3[1], y23 = d2[1] - d3[1];
        double z01 = d0[2] - d1[2], z02 = d0[2] - d2[2], z03 = d0[2] - d3[2];
        double z12 = d1[2] - d2[2], z13 = d1[2] - d3[2], z23 = d2[2] - d3[2];
        sx[0] = iv * (y13 * z12 - y12 * z13);
        sx[1] = iv * (y02 * z23 - y23 * z02);
        sx[2] = iv * (y13 * z03 - y03 * z13);
        sx[3] = iv * (y01 * z02 - y02 * z01);
        sy[0] = iv * (z13 * x12 - z12 * x13);
        sy[1] = iv * (z02 * x23 - z23 * x02);
        sy[2] = iv * (z13 * x03 - z03 * x13);
        sy[3] = iv * (z01 * x02 - z02 * x01);
        sz[0] = iv * (x13 * y12 - x12 * y13);
        sz[1] = iv * (x02 * y23 - x23 * y02);
        sz[2] = iv * (x13 * y03 - x03 * y13);
        sz[3] = iv * (x01 * y02 - x02 * y01);
    } else {
        double iv = 1 / (2 * st->volume[e]);
        sx[0] = iv * (d1[1] - d2[1]);
        sx[1] = iv * (d2[1] - d0[1]);
        sx[2] = iv * (d0[1] - d1[1]);
        sz[0] = iv * (d2[0] - d1[0]);
        sz[1] = iv * (d0[0] - d2[0]);
        sz[2] = iv * (d1[0] - d0[0]);
    }
}

void oracle_compute_shape_fn(oracle_ctx *c) /* geometry.cxx:368-455 */
{
    loop_all_elem(c, shape_elem, NULL);
}

/* elem_quality / worst_elem_quality (geometry.cxx:458-512) */
double oracle_worst_elem_quality(oracle_ctx *c, int *worst)
{
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe;
    double q = 1;
    *worst = 0;
    for (int e = 0; e < c->ne; e++) {
        const int *k = c->mesh->connectivity + (size_t)e * npe;
        const double *a = CO(k[0]), *b = CO(k[1]), *cc = CO(k[2]);
        double vol = st->volume[e], quality;
        if (nd == 3) {
            const double *d = CO(k[3]);
            double normalization_factor = 216 * sqrt(3);
            double area_sum = (tri_area(3, a, b, cc) + tri_area(3, a, b, d) + tri_area(3, cc, d, a)
                               + tri_area(3, cc, d, b));
            quality = normalization_factor * vol * vol / (area_sum * area_sum * area_sum);
        } else {
            double normalization_factor = 4 * sqrt(3);
            double dist2_sum = dist2_(2, a, b) + dist2_(2, b, cc) + dist2_(2, a, cc);
            quality = normalization_factor * vol / dist2_sum;
        }
        if (quality < q) {
            q = quality;
            *worst = e;
        }
    }
    return q;
}

/* ------------------------------------------------------------------ */
/* fields (fields.cxx)                                                 */
/* ------------------------------------------------------------------ */
static void temperature_elem(oracle_ctx *c, int e, void *arg)
{
    double *tdot = (double *)arg;
    des_host_state *st = c->st;
    const int npe = c->npe;
    const int *k = c->mesh->connectivity + (size_t)e * npe;
    double D[MAXNPE][MAXNPE];
    double kv = m_k(c, e) * st->volume[e];
    double rh = (m_hr(c, e) / m_cp(c, e)) * st->volume[e];
    const double *sx = st->shpdx + (size_t)e * npe;
    const double *sz = st->shpdz + (size_t)e * npe;
    const double *sy = (c->nd == 3) ? st->shpdy + (size_t)e * npe : NULL;
    for (int i = 0; i < npe; ++i)
        for (int j = 0; j < npe; ++j)
            D[i][j] = sy ? (sx[i] * sx[j] + sy[i] * sy[j] + sz[i] * sz[j]) : (sx[i] * sx[j] + sz[i] * sz[j]);
    for (int i = 0; i < npe; ++i) {
        double diffusion = 0;
        for (int j = 0; j < npe; ++j) diffusion += D[i][j] * st->temperature[k[j]];
        tdot[k[i]] += diffusion * kv - rh;
    }
}

void oracle_update_temperature(oracle_ctx *c) /* fields.cxx:96-163 */
{
    des_host_state *st = c->st;
    const des_params *pr = c->param;
    double *tdot = ntmp_(c);
    memset(tdot, 0, sizeof(double) * c->nn);
    loop_all_elem(c, temperature_elem, tdot);
    const unsigned *bcflag = c->mesh->bcflag;
    PFOR
    for (int n = 0; n < c->nn; ++n) {
        if (bcflag[n] & BOUNDZ1) st->temperature[n] = pr->surface_temperature;
        else if ((bcflag[n] & BOUNDZ0) && !pr->has_fixed_bottom_temperature)
            st->temperature[n] = pr->mantle_temperature;
        else st->temperature[n] -= tdot[n] * st->dt / st->tmass[n];
    }
}

void oracle_update_strain_rate(oracle_ctx *c) /* fields.cxx:166-232 */
{
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe, nstr = c->nstr;
    PFOR
    for (int e = 0; e < c->ne; ++e) {
        const int *k = c->mesh->connectivity + (size_t)e * npe;
        const double *sx = st->shpdx + (size_t)e * npe;
        const double *sz = st->shpdz + (size_t)e * npe;
        double *s = st->strain_rate + (size_t)e * nstr;
        const double *v[MAXNPE];
        for (int i = 0; i < npe; ++i) v[i] = st->vel + (size_t)k[i] * nd;
        if (nd == 3) {
            const double *sy = st->shpdy + (size_t)e * npe;
            s[0] = 0;
            for (int i = 0; i < npe; ++i) s[0] += v[i][0] * sx[i];
            s[1] = 0;
            for (int i = 0; i < npe; ++i) s[1] += v[i][1] * sy[i];
            s[2] = 0;
            for (int i = 0; i < npe; ++i) s[2] += v[i][2] * sz[i];
            s[3] = 0;
            for (int i = 0; i < npe; ++i) s[3] += 0.5 * (v[i][0] * sy[i] + v[i][1] * sx[i]);
            s[4] = 0;
            for (int i = 0; i < npe; ++i) s[4] += 0.5 * (v[i][0] * sz[i] + v[i][2] * sx[i]);
            s[5] = 0;
            for (int i = 0; i < npe; ++i) s[5] += 0.5 * (v[i][1] * sz[i] + v[i][2] * sy[i]);
        } else {
            s[0] = 0;
            for (int i = 0; i < npe; ++i) s[0] += v[i][0] * sx[i];
            s[1] = 0;
            for (int i = 0; i < npe; ++i) s[1] += v[i][1] * sz[i];
            s[2] = 0;
            for (int i = 0; i < npe; ++i) s[2] += 0.5 * (v[i][0] * sz[i] + v[i][1] * sx[i]);
        }
    }
}

/* apply_damping (fields.cxx:235-288) */
static void apply_damping_(oracle_ctx *c)
{
    double *ff = c->st->force;
    const double *v = c->st->vel;
    const double small_vel = 1e-13;
    const double df = c->param->damping_factor;
    const int n = c->nn * c->nd;
    switch (c->param->damping_option) {
    case 1:
        PFOR
        for (int i = 0; i < n; ++i)
            if (fabs(v[i]) > small_vel) ff[i] -= df * copysign(ff[i], v[i]);
        break;
    case 2:
        PFOR
        for (int i = 0; i < n; ++i) ff[i] -= df * ff[i];
        break;
    case 3:
        PFOR
        for (int i = 0; i < n; ++i) {
            if ((ff[i] < 0) == (v[i] < 0)) ff[i] -= df * ff[i];
            else ff[i] += (1 - df) * ff[i];
        }
        break;
    default:
        break;
    }
}

/* normal_vector_of_facet (bc.cxx:12-47) */
static void facet_normal(const oracle_ctx *c, int f, const int *conn, double *normal, double *zcenter)
{
    const des_host_state *st = c->st;
    const int nd = c->nd;
    if (nd == 3) {
        int n0 = conn[FACET3[f][0]], n1 = conn[FACET3[f][1]], n2 = conn[FACET3[f][2]];
        double v01[3], v02[3];
        for (int i = 0; i < 3; ++i) {
            v01[i] = CO(n1)[i] - CO(n0)[i];
            v02[i] = CO(n2)[i] - CO(n0)[i];
        }
        normal[0] = (v01[1] * v02[2] - v01[2] * v02[1]) / 2;
        normal[1] = (v01[2] * v02[0] - v01[0] * v02[2]) / 2;
        normal[2] = (v01[0] * v02[1] - v01[1] * v02[0]) / 2;
        *zcenter = (CO(n0)[2] + CO(n1)[2] + CO(n2)[2]) / 3;
    } else {
        int n0 = conn[FACET2[f][0]], n1 = conn[FACET2[f][1]];
        double v01[2];
        for (int i = 0; i < 2; ++i) v01[i] = CO(n1)[i] - CO(n0)[i];
        normal[0] = v01[1];
        normal[1] = -v01[0];
        *zcenter = (CO(n0)[1] + CO(n1)[1]) / 2;
    }
}

/* apply_stress_bcs (bc.cxx:493-566) */
static void apply_stress_bcs_(oracle_ctx *c)
{
    const des_params *pr = c->param;
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe, npf = nd;
    if (pr->gravity == 0) return;
    for (int i = 0; i < DES_NBDRYTYPES; i++) {
        int t = pr->vbc_types[i];
        if (t != 0 && t != 2 && t != 4) continue;
        if (i == 4 && !pr->has_winkler_foundation) continue;
        if (i == 5 && !pr->has_water_loading) continue;
        for (int q = c->mesh->bfacet_offsets[i]; q < c->mesh->bfacet_offsets[i + 1]; ++q) {
            int e = c->mesh->bfacets[2 * q], f = c->mesh->bfacets[2 * q + 1];
            const int *conn = c->mesh->connectivity + (size_t)e * npe;
            double normal[3], zcenter;
            facet_normal(c, f, conn, normal, &zcenter);
            double p;
            if (i == 4 && pr->has_winkler_foundation) {
                p = pr->compensation_pressure
                    - (m_rho(c, e) + pr->winkler_delta_rho) * pr->gravity * (zcenter + pr->zlength);
            } else if (i == 5 && pr->has_water_loading) {
                const double sea_level = 0;
                p = 0;
                if (zcenter < sea_level) {
                    const double sea_water_density = 1030;
                    p = sea_water_density * pr->gravity * (sea_level - zcenter);
                }
            } else {
                p = ref_pressure_(c, zcenter);
            }
            for (int j = 0; j < npf; ++j) {
                int n = conn[nd == 3 ? FACET3[f][j] : FACET2[f][j]];
                for (int d = 0; d < nd; ++d) st->force[(size_t)n * nd + d] -= p * normal[d] / npf;
            }
        }
    }
    if (pr->has_elastic_foundation) {
        for (int n = 0; n < c->nn; ++n) {
            if (!(c->mesh->bcflag[n] & BOUNDZ0)) continue;
            st->force[(size_t)n * nd + nd - 1] -= pr->elastic_foundation_constant
                * (st->coord[(size_t)n * nd + nd - 1] - st->coord0[(size_t)n * nd + nd - 1]);
        }
    }
}

static void force_elem(oracle_ctx *c, int e, void *arg)
{
    des_host_state *st = c->st;
    double gravity = *(const double *)arg;
    const int nd = c->nd, npe = c->npe;
    const int *k = c->mesh->connectivity + (size_t)e * npe;
    const double *sx = st->shpdx + (size_t)e * npe;
    const double *sz = st->shpdz + (size_t)e * npe;
    const double *s = st->stress + (size_t)e * c->nstr;
    double vol = st->volume[e];
    double buoy = 0;
    if (gravity != 0) buoy = m_rho(c, e) * gravity / npe;
    if (nd == 3) {
        const double *sy = st->shpdy + (size_t)e * npe;
        for (int i = 0; i < npe; ++i) {
            double *f = st->force + (size_t)k[i] * 3;
            f[0] -= (s[0] * sx[i] + s[3] * sy[i] + s[4] * sz[i]) * vol;
            f[1] -= (s[3] * sx[i] + s[1] * sy[i] + s[5] * sz[i]) * vol;
            f[2] -= (s[4] * sx[i] + s[5] * sy[i] + s[2] * sz[i] + buoy) * vol;
        }
    } else {
        for (int i = 0; i < npe; ++i) {
            double *f = st->force + (size_t)k[i] * 2;
            f[0] -= (s[0] * sx[i] + s[2] * sz[i]) * vol;
            f[1] -= (s[2] * sx[i] + s[1] * sz[i] + buoy) * vol;
        }
    }
}

void oracle_update_force(oracle_ctx *c) /* fields.cxx:291-340 */
{
    memset(c->st->force, 0, sizeof(double) * c->nn * c->nd);
    double g = c->param->gravity;
    loop_all_elem(c, force_elem, &g);
    apply_stress_bcs_(c);
    if (c->param->is_quasi_static) apply_damping_(c);
}

void oracle_update_velocity(oracle_ctx *c) /* fields.cxx:343-355 */
{
    des_host_state *st = c->st;
    const int nd = c->nd, n = c->nn * nd;
    PFOR
    for (int i = 0; i < n; ++i) st->vel[i] += st->dt * st->force[i] / st->mass[i / nd];
}

void oracle_update_coordinate(oracle_ctx *c) /* fields.cxx:358-368 */
{
    des_host_state *st = c->st;
    const int n = c->nn * c->nd;
    PFOR
    for (int i = 0; i < n; ++i) st->coord[i] += st->vel[i] * st->dt;
}

/* jaumann_rate_3d / _2d (fields.cxx:375-404) */
static void jaumann3(double *s, double dt, double w3, double w4, double w5)
{
    double si[6];
    si[0] = -2.0 * s[3] * w3 - 2.0 * s[4] * w4;
    si[1] = 2.0 * s[3] * w3 - 2.0 * s[5] * w5;
    si[2] = 2.0 * s[4] * w4 + 2.0 * s[5] * w5;
    si[3] = s[0] * w3 - s[1] * w3 - s[4] * w5 - s[5] * w4;
    si[4] = s[0] * w4 - s[2] * w4 + s[3] * w5 - s[5] * w3;
    si[5] = s[1] * w5 - s[2] * w5 + s[3] * w4 + s[4] * w3;
    for (int i = 0; i < 6; ++i) s[i] += dt * si[i];
}

static void jaumann2(double *s, double dt, double w2)
{
    double si[3];
    si[0] = -2.0 * s[2] * w2;
    si[1] = 2.0 * s[2] * w2;
    si[2] = s[0] * w2 - s[1] * w2;
    for (int i = 0; i < 3; ++i) s[i] += dt * si[i];
}

void oracle_rotate_stress(oracle_ctx *c) /* fields.cxx:411-483 */
{
    des_host_state *st = c->st;
    const int nd = c->nd, npe = c->npe, nstr = c->nstr;
    PFOR
    for (int e = 0; e < c->ne; ++e) {
        const int *k = c->mesh->connectivity + (size_t)e * npe;
        const double *sx = st->shpdx + (size_t)e * npe;
        const double *sz = st->shpdz + (size_t)e * npe;
        const double *v[MAXNPE];
        for (int i = 0; i < npe; ++i) v[i] = st->vel + (size_t)k[i] * nd;
        if (nd == 3) {
            const double *sy = st->shpdy + (size_t)e * npe;
            double w3 = 0, w4 = 0, w5 = 0;
            for (int i = 0; i < npe; ++i) w3 += 0.5 * (v[i][0] * sy[i] - v[i][1] * sx[i]);
            for (int i = 0; i < npe; ++i) w4 += 0.5 * (v[i][0] * sz[i] - v[i][2] * sx[i]);
            for (int i = 0; i < npe; ++i) w5 += 0.5 * (v[i][1] * sz[i] - v[i][2] * sy[i]);
            jaumann3(st->stress + (size_t)e * nstr, st->dt, w3, w4, w5);
            jaumann3(st->strain + (size_t)e * nstr, st->dt, w3, w4, w5);
        } else {
            double w2 = 0;
            for (int i = 0; i < npe; ++i) w2 += 0.5 * (v[i][1] * sx[i] - v[i][0] * sz[i]);
            jaumann2(st->stress + (size_t)e * nstr, st->dt, w2);
            jaumann2(st->strain + (size_t)e * nstr, st->dt, w2);
        }
    }
}

void oracle_swap_volume(oracle_ctx *c) /* dynearthsol.cxx:226 */
{
    memcpy(c->st->volume_old, c->st->volume, sizeof(double) * c->ne);
}

/* ------------------------------------------------------------------ */
/* velocity boundary conditions (bc.cxx:179-490)                       */
/* ------------------------------------------------------------------ */
static void vbc_x(int type, double val, int nd, double *v)
{
    switch (type) {
    case 1: v[0] = val; break;
    case 2: v[1] = 0; if (nd == 3) v[2] = 0; break;
    case 3: v[0] = val; v[1] = 0; if (nd == 3) v[2] = 0; break;
    case 4: if (nd == 3) { v[1] = val; v[2] = 0; } break;
    case 5: if (nd == 3) { v[0] = 0; v[1] = val; v[2] = 0; } break;
    case 7: if (nd == 3) { v[0] = val; v[1] = 0; } break;
    default: break;
    }
}

static void vbc_y0(int type, double val, double *v)
{
    switch (type) {
    case 1: v[1] = val; break;
    case 2: v[0] = 0; v[2] = 0; break;
    case 3: v[0] = 0; v[1] = val; v[2] = 0; break;
    case 4: v[0] = val; v[2] = 0; break;
    case 5: v[0] = val; v[1] = 0; v[2] = 0; break;
    case 7: v[0] = 0; v[1] = val; break;
    default: break;
    }
}

/* the y1 side differs from y0 in case 3 (bc.cxx:325-329) */
static void vbc_y1(int type, double val, double *v)
{
    switch (type) {
    case 1: v[1] = val; break;
    case 2: v[0] = 0; v[2] = 0; break;
    case 3: v[0] = val; v[1] = 0; v[2] = 0; break;
    case 4: v[0] = val; v[2] = 0; break;
    case 5: v[0] = val; v[1] = 0; v[2] = 0; break;
    case 7: v[0] = 0; v[1] = val; break;
    default: break;
    }
}

static void vbc_z(int type, double val, int nd, double *v)
{
    switch (type) {
    case 1: v[nd - 1] = val; break;
    case 2: v[0] = 0; if (nd == 3) v[1] = 0; break;
    case 3: v[0] = 0; if (nd == 3) v[1] = 0; v[nd - 1] = val; break;
    default: break;
    }
}

void oracle_apply_vbcs(oracle_ctx *c)
{
    const des_params *pr = c->param;
    const des_mesh *mh = c->mesh;
    des_host_state *st = c->st;
    const int nd = c->nd;
    PFOR
    for (int i = 0; i < c->nn; ++i) {
        unsigned flag = mh->bcflag[i];
        if (!(flag & BOUND_ANY)) continue;
        double *v = st->vel + (size_t)i * nd;
        if (flag & BOUNDX0) vbc_x(pr->vbc_types[0], pr->vbc_values[0], nd, v);
        if (flag & BOUNDX1) vbc_x(pr->vbc_types[1], pr->vbc_values[1], nd, v);
        if (nd == 3) {
            if (flag & BOUNDY0) vbc_y0(pr->vbc_types[2], pr->vbc_values[2], v);
            if (flag & BOUNDY1) vbc_y1(pr->vbc_types[3], pr->vbc_values[3], v);
        }
        for (int ib = 6; ib <= 9; ib++) {
            const double *n = mh->bnormals[ib];
            if (!(flag & (1u << ib))) continue;
            double fac = 0;
            switch (pr->vbc_types[ib]) {
            case 1:
                if (flag == (1u << ib)) {
                    double vn = 0;
                    for (int d = 0; d < nd; d++) vn += v[d] * n[d];
                    for (int d = 0; d < nd; d++) v[d] += (pr->vbc_values[ib] - vn) * n[d];
                } else {
                    for (int ic = 0; ic < ib; ic++) {
                        if (!(flag & (1u << ic))) continue;
                        if (pr->vbc_types[ic] == 0) {
                            double vn = 0;
                            for (int d = 0; d < nd; d++) vn += v[d] * n[d];
                            for (int d = 0; d < nd; d++) v[d] += (pr->vbc_values[ib] - vn) * n[d];
                        } else if (pr->vbc_types[ic] == 1) {
                            const double *edge = mh->edge_vectors[ic][ib];
                            double ve = 0;
                            for (int d = 0; d < nd; d++) ve += v[d] * edge[d];
                            for (int d = 0; d < nd; d++) v[d] = ve * edge[d];
                        }
                    }
                }
                break;
            case 3:
                for (int d = 0; d < nd; d++) v[d] = pr->vbc_values[ib] * n[d];
                break;
            case 11:
                fac = 1 / sqrt(1 - n[nd - 1] * n[nd - 1]);
                if (flag == (1u << ib)) {
                    double vn = 0;
                    for (int d = 0; d < nd - 1; d++) vn += v[d] * n[d];
                    for (int d = 0; d < nd - 1; d++) v[d] += (pr->vbc_values[ib] * fac - vn) * n[d];
                } else {
                    for (int ic = 0; ic < ib; ic++) {
                        if (!(flag & (1u << ic))) continue;
                        if (pr->vbc_types[ic] == 0) {
                            double vn = 0;
                            for (int d = 0; d < nd - 1; d++) vn += v[d] * n[d];
                            for (int d = 0; d < nd - 1; d++) v[d] += (pr->vbc_values[ib] * fac - vn) * n[d];
                        } else if (pr->vbc_types[ic] == 1) {
                            const double *edge = mh->edge_vectors[ic][ib];
                            double ve = 0;
                            for (int d = 0; d < nd; d++) ve += v[d] * edge[d];
                            for (int d = 0; d < nd; d++) v[d] = ve * edge[d];
                        }
                    }
                }
                break;
            case 13:
                fac = 1 / sqrt(1 - n[nd - 1] * n[nd - 1]);
                for (int d = 0; d < nd - 1; d++) v[d] = pr->vbc_values[ib] * fac * n[d];
                v[nd - 1] = 0;
                break;
            default:
                break;
            }
        }
        if (pr->vbc_types[4] == 0 && pr->vbc_types[5] == 0) continue;
        if (flag & BOUNDZ0) vbc_z(pr->vbc_types[4], pr->vbc_values[4], nd, v);
        if (flag & BOUNDZ1) vbc_z(pr->vbc_types[5], pr->vbc_values[5], nd, v);
    }
}

/* ------------------------------------------------------------------ */
/* update_stress (rheology.cxx:510-646)                                */
/* ------------------------------------------------------------------ */
int oracle_update_stress(oracle_ctx *c)
{
    des_host_state *st = c->st;
    const des_material *mt = c->mat;
    const int nd = c->nd, nstr = c->nstr;
    const int rheol_type = mt->rheol_type;
    int bad = 0;
    PFOR
    for (int e = 0; e < c->ne; ++e) {
        double *s = st->stress + (size_t)e * nstr;
        double *syy = &st->stressyy[e];
        double *es = st->strain + (size_t)e * nstr;
        double *edot = st->strain_rate + (size_t)e * nstr;
        double old_s = trace_(nd, s);
        {
            double div = trace_(nd, edot);
            for (int i = 0; i < nd; ++i) edot[i] += (st->edvoldt[e] - div) / nd;
        }
        for (int i = 0; i < nstr; ++i) es[i] += edot[i] * st->dt;
        double de[MAXNSTR];
        for (int i = 0; i < nstr; ++i) de[i] = edot[i] * st->dt;

        switch (rheol_type) {
        case DES_RH_ELASTIC:
            elastic_(nd, m_bulkm(c, e), m_shearm(c, e), de, s);
            break;
        case DES_RH_VISCOUS:
            viscous_(nd, m_bulkm(c, e), m_visc(c, e), trace_(nd, es), edot, s);
            break;
        case DES_RH_MAXWELL: {
            double dv = st->volume[e] / st->volume_old[e] - 1;
            maxwell_(nd, m_bulkm(c, e), m_shearm(c, e), m_visc(c, e), st->dt, dv, de, s);
            break;
        }
        case DES_RH_EP: {
            double depls = 0, amc, anphi, anpsi, hardn, ten_max;
            double bulkm = m_bulkm(c, e), shearm = m_shearm(c, e);
            m_plastic_props(c, e, st->plstrain[e], &amc, &anphi, &anpsi, &hardn, &ten_max);
            int fm;
            if (mt->is_plane_strain)
                elasto_plastic2d_(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, &depls, s, syy, &fm);
            else
                elasto_plastic_(nd, bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, &depls, s, &fm);
            st->plstrain[e] += depls;
            st->delta_plstrain[e] = depls;
            break;
        }
        case DES_RH_EVP: {
            double depls = 0;
            double bulkm = m_bulkm(c, e), shearm = m_shearm(c, e);
            double viscosity = m_visc(c, e);
            double dv = st->volume[e] / st->volume_old[e] - 1;
            double sv[MAXNSTR];
            for (int i = 0; i < nstr; ++i) sv[i] = s[i];
            maxwell_(nd, bulkm, shearm, viscosity, st->dt, dv, de, sv);
            double svII = second_invariant2_(nd, sv);
            double amc, anphi, anpsi, hardn, ten_max;
            m_plastic_props(c, e, st->plstrain[e], &amc, &anphi, &anpsi, &hardn, &ten_max);
            double sp[MAXNSTR], spyy = *syy;
            for (int i = 0; i < nstr; ++i) sp[i] = s[i];
            int fm;
            if (mt->is_plane_strain)
                elasto_plastic2d_(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, &depls, sp, &spyy, &fm);
            else
                elasto_plastic_(nd, bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, &depls, sp, &fm);
            double spII = second_invariant2_(nd, sp);
            if (svII < spII) {
                for (int i = 0; i < nstr; ++i) s[i] = sv[i];
            } else {
                for (int i = 0; i < nstr; ++i) s[i] = sp[i];
                st->plstrain[e] += depls;
                st->delta_plstrain[e] = depls;
                /* rheology.cxx:632 copies spyy, which is only initialised in
                 * plane strain; elsewhere stressyy is left unchanged here. */
                if (mt->is_plane_strain) *syy = spyy;
            }
            break;
        }
        default:
            bad = 1;
            break;
        }
        st->dpressure[e] = trace_(nd, s) - old_s;
    }
    return bad ? DES_EINPUT : 0;
}

/* ------------------------------------------------------------------ */
/* create_boundary_normals (bc.cxx:87-176)                             */
/* ------------------------------------------------------------------ */
int oracle_boundary_normals(const des_mesh *mesh, const double *coord,
                            double bnormals[DES_NBDRYTYPES][3],
                            double edge_vectors[DES_NBDRYTYPES][DES_NBDRYTYPES][3])
{
    const int nd = mesh->ndims, npe = nd + 1;
    oracle_ctx tmp;
    des_host_state st;
    memset(&tmp, 0, sizeof tmp);
    memset(&st, 0, sizeof st);
    st.coord = (double *)coord;
    tmp.st = &st;
    tmp.nd = nd;
    for (int i = 0; i < DES_NBDRYTYPES; i++) {
        double normal[3] = {0, 0, 0};
        int b = mesh->bfacet_offsets[i], end = mesh->bfacet_offsets[i + 1];
        if (b == end) continue;
        for (int q = b; q < end; ++q) {
            int e = mesh->bfacets[2 * q], f = mesh->bfacets[2 * q + 1];
            double zc;
            facet_normal(&tmp, f, mesh->connectivity + (size_t)e * npe, normal, &zc);
            double len = 0;
            for (int d = 0; d < nd; d++) len += normal[d] * normal[d];
            len = sqrt(len);
            for (int d = 0; d < nd; d++) normal[d] = normal[d] / len;
            if (q == b) {
                for (int d = 0; d < nd; d++) bnormals[i][d] = normal[d];
                if (i < 6) break;
            } else {
                const double eps2 = 1e-12;
                double diff2 = 0;
                for (int d = 0; d < nd; d++)
                    diff2 += (bnormals[i][d] - normal[d]) * (bnormals[i][d] - normal[d]);
                if (diff2 > eps2) return 1;
            }
        }
    }
    for (int i = 0; i < DES_NBDRYTYPES; i++) {
        if (mesh->bfacet_offsets[i] == mesh->bfacet_offsets[i + 1]) continue;
        const double eps = 1e-15;
        for (int j = i + 1; j < DES_NBDRYTYPES; j++) {
            if (mesh->bfacet_offsets[j] == mesh->bfacet_offsets[j + 1]) continue;
            double *s = edge_vectors[i][j];
            if (nd == 3) {
                if (fabs(bnormals[i][2]) < eps && fabs(bnormals[j][2]) < eps) {
                    s[0] = s[1] = 0;
                    s[2] = 1;
                } else {
                    s[0] = bnormals[i][1] * bnormals[j][2] - bnormals[i][2] * bnormals[j][1];
                    s[1] = bnormals[i][2] * bnormals[j][0] - bnormals[i][0] * bnormals[j][2];
                    s[2] = bnormals[i][0] * bnormals[j][1] - bnormals[i][1] * bnormals[j][0];
                }
            } else {
                s[0] = 0;
                s[1] = 1;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* context and driver                                                  */
/* ------------------------------------------------------------------ */
/* no node has elements in two bands of one colour (bands b and b' with
 * |b - b'| >= 2) */
static int bands_share_no_node(const des_mesh *mesh, const int *eg, int ng)
{
    const int nn = mesh->nnode, npe = mesh->ndims + 1;
    int *lo = (int *)malloc(sizeof(int) * (size_t)nn), *hi = (int *)malloc(sizeof(int) * (size_t)nn);
    for (int n = 0; n < nn; ++n) lo[n] = ng, hi[n] = -1;
    for (int b = 0; b < ng; ++b)
        for (int e = eg[b]; e < eg[b + 1]; ++e)
            for (int i = 0; i < npe; ++i) {
                const int n = mesh->connectivity[(size_t)e * npe + i];
                if (b < lo[n]) lo[n] = b;
                if (b > hi[n]) hi[n] = b;
            }
    int ok = 1;
    for (int n = 0; n < nn && ok; ++n)
        if (hi[n] - lo[n] >= 2) ok = 0;
    free(lo);
    free(hi);
    return ok;
}

oracle_ctx *oracle_create(const des_mesh *mesh, const des_params *param, const des_material *mat,
                          int nthreads)
{
    if (!mesh || !param || !mat || (mesh->ndims != 2 && mesh->ndims != 3)) return NULL;
    oracle_ctx *c = (oracle_ctx *)calloc(1, sizeof *c);
    c->mesh = mesh;
    c->param = param;
    c->mat = mat;
    c->nd = mesh->ndims;
    c->npe = c->nd + 1;
    c->nstr = c->nd == 3 ? 6 : 3;
    c->nn = mesh->nnode;
    c->ne = mesh->nelem;
    if (nthreads < 1) nthreads = 1;
#ifndef _OPENMP
    nthreads = 1;
#endif
    /* create_elem_groups (mesh.cxx:1724-1817): 2T contiguous bands, run as
     * two colours.  Two bands of one colour must share no node, or the
     * element scatters race: a node whose elements lie in bands two or more
     * apart breaks that, and then the thread count is halved (down to one). */
    c->egroups = (int *)malloc(sizeof(int) * (2 * (size_t)nthreads + 1));
    for (;;) {
        c->ngroups = nthreads > 1 ? 2 * nthreads : 1;
        int per = c->ne / c->ngroups;
        for (int i = 0; i < c->ngroups; i++) c->egroups[i] = i * per;
        c->egroups[c->ngroups] = c->ne;
        if (nthreads == 1 || bands_share_no_node(mesh, c->egroups, c->ngroups)) break;
        nthreads /= 2;
    }
    c->nthreads = nthreads;
    c->tmp_nn = (double *)calloc((size_t)c->nn, sizeof(double));
    return c;
}

void oracle_destroy(oracle_ctx *c)
{
    if (!c) return;
    free(c->egroups);
    free(c->tmp_nn);
    free(c);
}

int oracle_threads(const oracle_ctx *c) { return c->nthreads; }

int oracle_bind_state(oracle_ctx *c, des_host_state *st)
{
    c->st = st;
    return 0;
}

int oracle_set_elem_field(oracle_ctx *c, int field, const double *values)
{
    if (field < 0 || field >= DES_EF_COUNT) return DES_EINPUT;
    c->ef[field] = values;
    return 0;
}

int oracle_init_fields(oracle_ctx *c)
{
    des_host_state *st = c->st;
    if (st->coord0) memcpy(st->coord0, st->coord, sizeof(double) * c->nn * c->nd);
    oracle_compute_volume(c);
    memcpy(st->volume_old, st->volume, sizeof(double) * c->ne);
    /* init() computes the masses before initial_temperature runs
     * (dynearthsol.cxx:88-96), so tmass sees a zero temperature field. */
    double *T = st->temperature;
    double *zeroT = (double *)calloc((size_t)c->nn, sizeof(double));
    st->temperature = zeroT;
    oracle_compute_mass(c);
    st->temperature = T;
    free(zeroT);
    oracle_compute_shape_fn(c);
    oracle_apply_vbcs(c);
    double dt;
    int rc = oracle_compute_dt(c, &dt);
    st->dt = dt;
    return rc;
}

int oracle_run(oracle_ctx *c, int nsteps)
{
    des_host_state *st = c->st;
    for (int it = 0; it < nsteps; ++it) {
        st->steps++;
        st->time += st->dt;
        if (c->param->has_thermal_diffusion) oracle_update_temperature(c);
        oracle_update_strain_rate(c);
        oracle_compute_dvoldt(c);
        oracle_compute_edvoldt(c);
        int rc = oracle_update_stress(c);
        if (rc) return rc;
        oracle_NMD_stress(c);
        oracle_update_force(c);
        oracle_update_velocity(c);
        oracle_apply_vbcs(c);
        /* update_mesh (dynearthsol.cxx:221-232), surface_process_option 0 */
        oracle_update_coordinate(c);
        oracle_swap_volume(c);
        oracle_compute_volume(c);
        oracle_compute_mass(c);
        oracle_compute_shape_fn(c);
        if (c->mat->rheol_type & DES_RH_ELASTIC) oracle_rotate_stress(c);
        if (st->steps % 10 == 0) {
            double dt;
            rc = oracle_compute_dt(c, &dt);
            st->dt = dt;
            if (rc) return rc;
        }
    }
    return 0;
}
