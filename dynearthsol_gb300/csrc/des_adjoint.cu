// des_adjoint.cu -- hand-written reverse mode of the 3D FP64 step.
//
// Every kernel here is the adjoint (transpose of the derivative) of one
// forward stage of des_kernels.cu, evaluated at the forward values recorded
// on the tape.  Branches (yield, EVP choice, clamps, damping signs, Dirichlet
// and velocity BCs) follow the forward's decisions, so each adjoint is the
// derivative of the branch the forward took: a subgradient at the kinks.
// Where the forward's map is discontinuous in its input -- the eigenbasis
// of repeated principal stresses, the sign of a zero force under damping --
// the term of the discontinuity is dropped.  Adjoints are checked against
// finite differences, not bit for bit: divisions by 3 are div3, and the
// reciprocals of the common paths are recip_newton (~1e-14 relative), each
// a few FP64 instructions instead of an FP64 division.
#include <cfloat>

#include "des_adjoint.cuh"
#include "des_bc.cuh"
#include "des_kernels.cuh"
#include "des_rheology.cuh"

namespace des {

constexpr int TPB_A = 128;

static inline int nblk(long long n, int tpb = TPB_A)
{
    long long b = (n + tpb - 1) / tpb;
    return (int)(b < 1 ? 1 : b);
}

__device__ __forceinline__ double tshp(const TapeStep &t, size_t ne, int k, int i, int e)
{
    return t.shp[((size_t)k * 4 + i) * ne + e];
}

// the stress after NMD_stress (geometry.cxx:182-236), as k_nmd_correct forms
// it, from the tape's stress after update_stress and its pressure changes:
// the same operations in the same order, so the same bits (the division by
// 4 is exact, with or without a fused multiply-add)
__device__ __forceinline__ void tape_sss(const KP &p, const TapeStep &t, int e, double *s)
{
    const size_t ne = p.ne;
    double dpn = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) dpn += t.dpn[conn_at(p, i, e)];
    const double corr = divnd<3>(-t.dp[e] + dpn / 4);
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) s[cc] = t.sstar[cc * ne + e];
#pragma unroll
    for (int i = 0; i < 3; ++i) s[i] += corr;
}

__device__ __forceinline__ void tload3(const double *a, size_t nn, int n, double *o)
{
    o[0] = a[n];
    o[1] = a[nn + n];
    o[2] = a[2 * nn + n];
}

// ------------------------------------------------------------------
// geometry: volume (geometry.cxx:29-49) and shape functions
// (geometry.cxx:368-455) of one tet, reversed.  Given the adjoints gvol of
// the volume and gs[k][i] of dN_i/dx_k, adds the coordinate adjoints to gc.
// dN_i/dx_k = (P_a Q_b - P_b Q_a) / (6V), with (P, Q) = (y, z), (z, x),
// (x, y) for k = 0, 1, 2 and the differences P_ij = P_i - P_j over the
// pairs a, b listed below -- the forward's expressions, regrouped.
// ------------------------------------------------------------------
__device__ void geom_reverse(const double (*c)[3], double vol, const double (*gs)[4], double gvol,
                             double (*gc)[3])
{
    const int PA[4][2] = {{1, 3}, {0, 2}, {1, 3}, {0, 1}};
    const int PB[4][2] = {{1, 2}, {2, 3}, {0, 3}, {0, 2}};
    const double iv = recip_newton(6 * vol);
    double giv = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int P = (k + 1) % 3, Q = (k + 2) % 3;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int a0 = PA[i][0], a1 = PA[i][1], b0 = PB[i][0], b1 = PB[i][1];
            const double Pa = c[a0][P] - c[a1][P], Qa = c[a0][Q] - c[a1][Q];
            const double Pb = c[b0][P] - c[b1][P], Qb = c[b0][Q] - c[b1][Q];
            const double g = gs[k][i];
            giv += g * (Pa * Qb - Pb * Qa);
            const double gt = g * iv;
            // d/dPa = Qb, d/dQb = Pa, d/dPb = -Qa, d/dQa = -Pb
            gc[a0][P] += gt * Qb;
            gc[a1][P] -= gt * Qb;
            gc[b0][Q] += gt * Pa;
            gc[b1][Q] -= gt * Pa;
            gc[b0][P] -= gt * Qa;
            gc[b1][P] += gt * Qa;
            gc[a0][Q] -= gt * Pb;
            gc[a1][Q] += gt * Pb;
        }
    }
    gvol += giv * (-6 * iv * iv);   // d/dvol 1/(6 vol) = -6 iv^2
    // V = [x01 (y23 z12 - y12 z23) + x12 (y01 z23 - y23 z01) + x23 (y12 z01 - y01 z12)] / 6
    const double g6 = div6(gvol);
    const double x01 = c[0][0] - c[1][0], x12 = c[1][0] - c[2][0], x23 = c[2][0] - c[3][0];
    const double y01 = c[0][1] - c[1][1], y12 = c[1][1] - c[2][1], y23 = c[2][1] - c[3][1];
    const double z01 = c[0][2] - c[1][2], z12 = c[1][2] - c[2][2], z23 = c[2][2] - c[3][2];
    const double gx01 = g6 * (y23 * z12 - y12 * z23), gx12 = g6 * (y01 * z23 - y23 * z01),
                 gx23 = g6 * (y12 * z01 - y01 * z12);
    const double gy01 = g6 * (x12 * z23 - x23 * z12), gy12 = g6 * (x23 * z01 - x01 * z23),
                 gy23 = g6 * (x01 * z12 - x12 * z01);
    const double gz01 = g6 * (x23 * y12 - x12 * y23), gz12 = g6 * (x01 * y23 - x23 * y01),
                 gz23 = g6 * (x12 * y01 - x01 * y12);
    const double gd[3][3] = {{gx01, gx12, gx23}, {gy01, gy12, gy23}, {gz01, gz12, gz23}};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        gc[0][d] += gd[d][0];
        gc[1][d] += gd[d][1] - gd[d][0];
        gc[2][d] += gd[d][2] - gd[d][1];
        gc[3][d] -= gd[d][2];
    }
}

// mass, tmass and volume_n of the element's four nodes (geometry.cxx:313-365),
// reversed: adds to gvol and returns the element density adjoint
__device__ __forceinline__ double mass_reverse(const KP &p, int e, const double *gm, const double *gtm,
                                               const double *gvn, double vol, double rho_e, double &gvol)
{
    const bool quasi = p.prm.is_quasi_static, thermal = p.prm.has_thermal_diffusion;
    const double rho = quasi ? p.mat.rho_pseudo : rho_e;
    const double cp = m_cp(p, e);
    double grho = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        gvol += rho / 4 * gm[i] + gvn[i];
        if (!quasi) grho += vol / 4 * gm[i];
        if (thermal) {
            gvol += rho_e * cp / 4 * gtm[i];
            grho += cp * vol / 4 * gtm[i];
        }
    }
    return grho;
}

// ------------------------------------------------------------------
// end of the step: mass (at the new volumes), rotate_stress
// (fields.cxx:411-483, Jaumann rate with the new velocities and shape
// functions) and the geometry of the new coordinates, reversed.
// In: as = adjoint of the rotated stress, avol/ashp = adjoints of the new
// volume and shape functions, am/atm/avn = adjoints of the new nodal mass,
// tmass, volume_n.  Out: as = adjoint of the stress before the rotation,
// arho = element density adjoint (mass share), slot3 = new-velocity
// contributions, slotx = new-coordinate contributions.
// ------------------------------------------------------------------
__global__ void __launch_bounds__(TPB_A) k_adj_end_geometry(KP p, AdjBufs a, TapeStep t, TapeStep t1, double dt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne, nn = p.nn;
    int nodes[4];
    double c[4][3], v[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        nodes[i] = conn_at(p, i, e);
        tload3(t1.x, nn, nodes[i], c[i]);
        tload3(t1.v, nn, nodes[i], v[i]);
    }
    const double vol = t1.vol[e];
    double gvol = a.avol[e];
    double gs[3][4];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) gs[k][i] = a.ashp[((size_t)k * 4 + i) * ne + e];
    {
        double gm[4], gtm[4], gvn[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            gm[i] = a.am[nodes[i]];
            gtm[i] = a.atm[nodes[i]];
            gvn[i] = a.avn[nodes[i]];
        }
        a.arho[e] = mass_reverse(p, e, gm, gtm, gvn, vol, t.rho[e], gvol);
    }
    double gv[4][3] = {};
    if (p.mat.rheol_type & DES_RH_ELASTIC) {
        double s[6], g[6];
        tape_sss(p, t, e, s);
#pragma unroll
        for (int cc = 0; cc < 6; ++cc) g[cc] = a.as[cc * ne + e];
        double sh[3][4];
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int i = 0; i < 4; ++i) sh[k][i] = tshp(t1, ne, k, i, e);
        double w3 = 0, w4 = 0, w5 = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) w3 += 0.5 * (v[i][0] * sh[1][i] - v[i][1] * sh[0][i]);
#pragma unroll
        for (int i = 0; i < 4; ++i) w4 += 0.5 * (v[i][0] * sh[2][i] - v[i][2] * sh[0][i]);
#pragma unroll
        for (int i = 0; i < 4; ++i) w5 += 0.5 * (v[i][1] * sh[2][i] - v[i][2] * sh[1][i]);
        // s_out = s + dt * si(s, w) (jaumann3), bilinear in s and w
        double gsin[6];
        gsin[0] = g[0] + dt * (g[3] * w3 + g[4] * w4);
        gsin[1] = g[1] + dt * (-g[3] * w3 + g[5] * w5);
        gsin[2] = g[2] + dt * (-g[4] * w4 - g[5] * w5);
        gsin[3] = g[3] + dt * (-2 * g[0] * w3 + 2 * g[1] * w3 + g[4] * w5 + g[5] * w4);
        gsin[4] = g[4] + dt * (-2 * g[0] * w4 + 2 * g[2] * w4 - g[3] * w5 + g[5] * w3);
        gsin[5] = g[5] + dt * (-2 * g[1] * w5 + 2 * g[2] * w5 - g[3] * w4 - g[4] * w3);
        const double gw3 = dt * (-2 * s[3] * g[0] + 2 * s[3] * g[1] + (s[0] - s[1]) * g[3] - s[5] * g[4] + s[4] * g[5]);
        const double gw4 = dt * (-2 * s[4] * g[0] + 2 * s[4] * g[2] - s[5] * g[3] + (s[0] - s[2]) * g[4] + s[3] * g[5]);
        const double gw5 = dt * (-2 * s[5] * g[1] + 2 * s[5] * g[2] - s[4] * g[3] + s[3] * g[4] + (s[1] - s[2]) * g[5]);
#pragma unroll
        for (int cc = 0; cc < 6; ++cc) a.as[cc * ne + e] = gsin[cc];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            gv[i][0] += 0.5 * (gw3 * sh[1][i] + gw4 * sh[2][i]);
            gv[i][1] += 0.5 * (-gw3 * sh[0][i] + gw5 * sh[2][i]);
            gv[i][2] += 0.5 * (-gw4 * sh[0][i] - gw5 * sh[1][i]);
            gs[0][i] += 0.5 * (-gw3 * v[i][1] - gw4 * v[i][2]);
            gs[1][i] += 0.5 * (gw3 * v[i][0] - gw5 * v[i][2]);
            gs[2][i] += 0.5 * (gw4 * v[i][0] + gw5 * v[i][1]);
        }
    }
    double gc[4][3] = {};
    geom_reverse(c, vol, gs, gvol, gc);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a.slot3[((size_t)d * 4 + i) * ne + e] = gv[i][d];
            a.slotx[((size_t)d * 4 + i) * ne + e] = gc[i][d];
        }
}

int launch_adj_end_geometry(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                            cudaStream_t s)
{
    k_adj_end_geometry<<<nblk(p.ne), TPB_A, 0, s>>>(p, a, t, t1, dt);
    return 1;
}

// derivative of the damped force with respect to the undamped one
// (fields.cxx:235-288); the force keeps the sign of the undamped force, and
// the velocity enters only through signs (derivative zero)
__device__ __forceinline__ double damp_deriv(const KP &p, double f, double v)
{
    const double df = p.prm.damping_factor;
    switch (p.prm.damping_option) {
    case 1:
        if (fabs(v) > 1e-13) {
            const double sf = (f > 0) ? 1.0 : ((f < 0) ? -1.0 : 0.0);
            return 1 - df * sf * ((v > 0) ? 1.0 : -1.0);
        }
        return 1;
    case 2: return 1 - df;
    case 3: return ((f < 0) == (v < 0)) ? (1 - df) : (2 - df);
    default: return 1;
    }
}

// ------------------------------------------------------------------
// nodes: gather the end-of-step contributions, then reverse
// update_coordinate (x' = x + v' dt), apply_vbcs (affine in v and the
// prescribed values: its transpose is read off by probing the forward map
// with unit vectors), update_velocity (v' = v + dt f / m), the elastic
// foundation and the damping.  Writes ax (coordinate adjoint, start of the
// step), av (velocity adjoint, before the strain-rate share), af (adjoint
// of the undamped force), am (mass adjoint of the start), clears atm and
// avn, and adds the per-block sums of the prescribed-value adjoints to gvbc.
// ------------------------------------------------------------------
__global__ void __launch_bounds__(TPB_A) k_adj_motion(KP p, AdjBufs a, TapeStep t, TapeStep t1, double dt)
{
    __shared__ double red[DES_NBDRYTYPES][TPB_A];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t ne = p.ne, nn = p.nn;
    double gva[DES_NBDRYTYPES];
#pragma unroll
    for (int ib = 0; ib < DES_NBDRYTYPES; ++ib) gva[ib] = 0;
    if (n < p.nn) {
        double gx[3], gv[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            gx[d] = a.ax[d * nn + n];
            gv[d] = a.av[d * nn + n];
        }
        for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
            const int ent = p.sup_ent[q];
            const int e = ent >> 2, i = ent & 3;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                gx[d] += a.slotx[((size_t)d * 4 + i) * ne + e];
                gv[d] += a.slot3[((size_t)d * 4 + i) * ne + e];
            }
        }
        // x' = x + v' dt
#pragma unroll
        for (int d = 0; d < 3; ++d) gv[d] += dt * gx[d];
        // v' = BC(pre): gpre = A^T gv, gva = B^T gv
        const unsigned flag = p.bcflag[n];
        double gpre[3] = {gv[0], gv[1], gv[2]};
        if (flag & BOUND_ANY) {
            double zero[DES_NBDRYTYPES];
#pragma unroll
            for (int ib = 0; ib < DES_NBDRYTYPES; ++ib) zero[ib] = 0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double col[3] = {0, 0, 0};
                col[d] = 1;
                apply_vbcs_node_va<3>(p, flag, col, zero);
                gpre[d] = col[0] * gv[0] + col[1] * gv[1] + col[2] * gv[2];
            }
            for (int ib = 0; ib < DES_NBDRYTYPES; ++ib) {
                double col[3] = {0, 0, 0};
                zero[ib] = 1;
                apply_vbcs_node_va<3>(p, flag, col, zero);
                zero[ib] = 0;
                gva[ib] = col[0] * gv[0] + col[1] * gv[1] + col[2] * gv[2];
            }
        }
        const double im = recip_newton(t.mass[n]);
        double gm = 0, gf[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double f = t.f[d * nn + n];
            a.av[d * nn + n] = gpre[d];
            gf[d] = dt * gpre[d] * im;
            gm -= gf[d] * f * im;
            double dd = 1;
            if (p.prm.is_quasi_static) dd = damp_deriv(p, f, t.v[d * nn + n]);
            gf[d] *= dd;
            a.af[d * nn + n] = gf[d];
        }
        if (p.prm.has_elastic_foundation && (flag & BOUNDZ0)) gx[2] -= p.prm.elastic_foundation_constant * gf[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) a.ax[d * nn + n] = gx[d];
        a.am[n] = gm;
        a.atm[n] = 0;
        a.avn[n] = 0;
    }
    // fixed-order block sums of the prescribed-value adjoints
#pragma unroll
    for (int ib = 0; ib < DES_NBDRYTYPES; ++ib) red[ib][threadIdx.x] = gva[ib];
    __syncthreads();
    for (int w = TPB_A / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
#pragma unroll
            for (int ib = 0; ib < DES_NBDRYTYPES; ++ib) red[ib][threadIdx.x] += red[ib][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < DES_NBDRYTYPES) a.gvbc[(size_t)blockIdx.x * DES_NBDRYTYPES + threadIdx.x] += red[threadIdx.x][0];
}

int launch_adj_motion(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                      cudaStream_t s)
{
    k_adj_motion<<<nblk(p.nn), TPB_A, 0, s>>>(p, a, t, t1, dt);
    return 1;
}

int adj_vbc_blocks(const KP &p) { return nblk(p.nn); }

// ------------------------------------------------------------------
// stress BCs of one boundary facet (bc.cxx:493-566), reversed.  The facet
// force fv = pr(zcenter, rho) * normal / 3 is subtracted at each of the
// facet's nodes, so its adjoint is minus the sum of their force adjoints.
// Writes the coordinate adjoints of the facet's three nodes to fslot and
// the element density adjoint (Winkler foundation) to frho.
// ------------------------------------------------------------------
__global__ void __launch_bounds__(TPB_A) k_adj_facets(KP p, AdjBufs a, TapeStep t)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= p.nbf) return;
    const size_t nn = p.nn, nbf = p.nbf;
    const int i = p.fac_bdry[q];
    const int ty = p.prm.vbc_types[i];
    const bool active = p.prm.gravity != 0 && (ty == 0 || ty == 2 || ty == 4) &&
                        !(i == 4 && !p.prm.has_winkler_foundation) && !(i == 5 && !p.prm.has_water_loading);
    double gc[3][3] = {};
    double grho = 0;
    if (active) {
        const int e = p.fac_elem[q], f = p.fac_f[q];
        const int F[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
        int nd[3];
        double c[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            nd[j] = conn_at(p, F[f][j], e);
            tload3(t.x, nn, nd[j], c[j]);
        }
        double gfv[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
            gfv[d] = -(a.af[d * nn + nd[0]] + a.af[d * nn + nd[1]] + a.af[d * nn + nd[2]]);
        double va[3], vb[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            va[d] = c[1][d] - c[0][d];
            vb[d] = c[2][d] - c[0][d];
        }
        const double nrm[3] = {(va[1] * vb[2] - va[2] * vb[1]) / 2, (va[2] * vb[0] - va[0] * vb[2]) / 2,
                               (va[0] * vb[1] - va[1] * vb[0]) / 2};
        const double zc = div3(c[0][2] + c[1][2] + c[2][2]);
        double pr, gzc_per_gpr, grho_per_gpr = 0;
        if (i == 4 && p.prm.has_winkler_foundation) {
            const double rho = t.rho[e];
            pr = p.prm.compensation_pressure - (rho + p.prm.winkler_delta_rho) * p.prm.gravity * (zc + p.prm.zlength);
            gzc_per_gpr = -(rho + p.prm.winkler_delta_rho) * p.prm.gravity;
            grho_per_gpr = -p.prm.gravity * (zc + p.prm.zlength);
        } else if (i == 5 && p.prm.has_water_loading) {
            pr = (zc < 0) ? 1030 * p.prm.gravity * (0 - zc) : 0;
            gzc_per_gpr = (zc < 0) ? -1030 * p.prm.gravity : 0;
        } else {
            pr = ref_pressure_(p, zc);
            gzc_per_gpr = -p.mat.rho0[0] * p.prm.gravity;
        }
        double gpr = 0, gn[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            gpr += div3(gfv[d] * nrm[d]);
            gn[d] = div3(gfv[d] * pr);
        }
        grho = gpr * grho_per_gpr;
        const double gzc = gpr * gzc_per_gpr;
        const double ga[3] = {(-gn[1] * vb[2] + gn[2] * vb[1]) / 2, (gn[0] * vb[2] - gn[2] * vb[0]) / 2,
                              (-gn[0] * vb[1] + gn[1] * vb[0]) / 2};
        const double gb[3] = {(gn[1] * va[2] - gn[2] * va[1]) / 2, (-gn[0] * va[2] + gn[2] * va[0]) / 2,
                              (gn[0] * va[1] - gn[1] * va[0]) / 2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            gc[0][d] = -ga[d] - gb[d];
            gc[1][d] = ga[d];
            gc[2][d] = gb[d];
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) gc[j][2] += div3(gzc);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int j = 0; j < 3; ++j) a.fslot[((size_t)d * 3 + j) * nbf + q] = gc[j][d];
    a.frho[q] = grho;
}

// ------------------------------------------------------------------
// update_force element terms (fields.cxx:291-340), reversed: per element,
// the four nodes' undamped force adjoints give the adjoints of the NMD
// stress, the start shape functions and volume, and the element density
// (buoyancy; Winkler facets from frho).  Also the first half of NMD_stress
// reversed (geometry.cxx:182-236): the trace of the stress adjoint feeds
// dp directly and, through the nodal average, every node of the element.
// Out: as (stress after update_stress), ashp and avol (start of the step;
// avol also takes the adjoint of volume_old of the next state), arho,
// adp (direct part), slot1[e] = the element's share of the NMD nodal sum.
// ------------------------------------------------------------------
__global__ void __launch_bounds__(TPB_A) k_adj_force(KP p, AdjBufs a, TapeStep t)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne, nn = p.nn;
    double s[6], gsig[6];
    tape_sss(p, t, e, s);
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) gsig[cc] = a.as[cc * ne + e];
    const double vol = t.vol[e];
    const double gravity = p.prm.gravity;
    const double buoy = (gravity != 0) ? t.rho[e] * gravity / 4 : 0.0;
    double gvol = a.avolo[e];
    a.avolo[e] = 0;
    double grho = a.arho[e], gbuoy = 0;
    for (int q = a.e2f_off[e]; q < a.e2f_off[e + 1]; ++q) grho += a.frho[a.e2f_ent[q]];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int n = conn_at(p, i, e);
        double gf[3];
        tload3(a.af, nn, n, gf);
        const double sx = tshp(t, ne, 0, i, e), sy = tshp(t, ne, 1, i, e), sz = tshp(t, ne, 2, i, e);
        const double t0 = s[0] * sx + s[3] * sy + s[4] * sz;
        const double t1 = s[3] * sx + s[1] * sy + s[5] * sz;
        const double t2 = s[4] * sx + s[5] * sy + s[2] * sz + buoy;
        gvol -= gf[0] * t0 + gf[1] * t1 + gf[2] * t2;
        const double g0 = -gf[0] * vol, g1 = -gf[1] * vol, g2 = -gf[2] * vol;
        gsig[0] += g0 * sx;
        gsig[1] += g1 * sy;
        gsig[2] += g2 * sz;
        gsig[3] += g0 * sy + g1 * sx;
        gsig[4] += g0 * sz + g2 * sx;
        gsig[5] += g1 * sz + g2 * sy;
        a.ashp[((size_t)0 * 4 + i) * ne + e] = g0 * s[0] + g1 * s[3] + g2 * s[4];
        a.ashp[((size_t)1 * 4 + i) * ne + e] = g0 * s[3] + g1 * s[1] + g2 * s[5];
        a.ashp[((size_t)2 * 4 + i) * ne + e] = g0 * s[4] + g1 * s[5] + g2 * s[2];
        gbuoy += g2;
    }
    if (gravity != 0) grho += gbuoy * gravity / 4;
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) a.as[cc * ne + e] = gsig[cc];
    a.avol[e] = gvol;
    a.arho[e] = grho;
    // NMD: stress_ii += (-dp + mean_i dpn_i) / 3
    const double tr = gsig[0] + gsig[1] + gsig[2];
    a.adp[e] = -div3(tr);
    a.slot1[e] = div3(tr) / 4;
}

// nodes: NMD nodal sum reversed (dpn = sum_e dp_e vol_e / volume_n), and the
// facets' coordinate adjoints added to ax
__global__ void __launch_bounds__(TPB_A) k_adj_nmd_nodes(KP p, AdjBufs a, TapeStep t)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const size_t nn = p.nn, nbf = p.nbf;
    double acc = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) acc += a.slot1[p.sup_ent[q] >> 2];
    const double ivn = recip_newton(t.voln[n]);
    a.adpn[n] = acc * ivn;
    a.avn[n] -= acc * t.dpn[n] * ivn;
    if (p.nf_off[n] < p.nf_off[n + 1]) {
        const int F[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
        double gx[3] = {0, 0, 0};
        for (int k = p.nf_off[n]; k < p.nf_off[n + 1]; ++k) {
            const int q = p.nf_ent[k];
            const int e = p.fac_elem[q], f = p.fac_f[q];
#pragma unroll
            for (int j = 0; j < 3; ++j)
                if (conn_at(p, F[f][j], e) == n)
#pragma unroll
                    for (int d = 0; d < 3; ++d) gx[d] += a.fslot[((size_t)d * 3 + j) * nbf + q];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) a.ax[d * nn + n] += gx[d];
    }
}

int launch_adj_force(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s)
{
    int n = 0;
    if (p.nbf > 0) {
        k_adj_facets<<<nblk(p.nbf), TPB_A, 0, s>>>(p, a, t);
        ++n;
    }
    k_adj_force<<<nblk(p.ne), TPB_A, 0, s>>>(p, a, t);
    return n + 1;
}

int launch_adj_nmd_nodes(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s)
{
    k_adj_nmd_nodes<<<nblk(p.nn), TPB_A, 0, s>>>(p, a, t);
    return 1;
}

// ------------------------------------------------------------------
// rheology, reversed (rheology.cxx:105-299, matprops.cxx:264-373).  Each
// *_reverse adds to the adjoints it is given; forward values are recomputed
// with the forward's own functions, so every branch matches the forward.
// ------------------------------------------------------------------
// elastic: out = s + E(de), out_i = s_i + 2G de_i + (K - 2G/3) tr(de), out_c = s_c + 2G de_c
__device__ __forceinline__ void elastic_reverse(double K, double G, const double *de, const double *go, double *gs,
                                                double *gde, double &gG)
{
    const double lambda = K - 2. / 3 * G;
    const double trde = de[0] + de[1] + de[2], tg = go[0] + go[1] + go[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gs[i] += go[i];
        gde[i] += 2 * G * go[i] + lambda * tg;
        gG += 2 * de[i] * go[i];
    }
    gG -= 2. / 3 * trde * tg;
#pragma unroll
    for (int c = 3; c < 6; ++c) {
        gs[c] += go[c];
        gde[c] += 2 * G * go[c];
        gG += 2 * de[c] * go[c];
    }
}

// maxwell: out_i = ((s_i - s0) f1 + 2G (de_i - dev)) f2 + s0 + K dv, out_c = (s_c f1 + 2G de_c) f2,
// f1 = 1 - tmp, f2 = 1 / (1 + tmp), tmp = dt G / (2 visc)
__device__ __forceinline__ void maxwell_reverse(double K, double G, double visc, double dt, const double *de,
                                                const double *s, const double *go, double *gs, double *gde,
                                                double &gG, double &gvisc, double &gdv)
{
    const double ivisc = recip_newton(visc);
    const double tmp = 0.5 * dt * G * ivisc;
    const double f1 = 1 - tmp, f2 = recip_newton(1 + tmp);
    const double dev = div3(de[0] + de[1] + de[2]), s0 = div3(s[0] + s[1] + s[2]);
    double gf1 = 0, gf2 = 0, gs0 = 0, gdev = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double u = (s[i] - s0) * f1 + 2 * G * (de[i] - dev);
        gf2 += go[i] * u;
        const double gu = go[i] * f2;
        gs0 += go[i] - gu * f1;
        gdv += K * go[i];
        gs[i] += gu * f1;
        gf1 += gu * (s[i] - s0);
        gG += gu * 2 * (de[i] - dev);
        gde[i] += 2 * G * gu;
        gdev -= 2 * G * gu;
    }
#pragma unroll
    for (int c = 3; c < 6; ++c) {
        const double u = s[c] * f1 + 2 * G * de[c];
        gf2 += go[c] * u;
        const double gu = go[c] * f2;
        gs[c] += gu * f1;
        gf1 += gu * s[c];
        gG += 2 * gu * de[c];
        gde[c] += 2 * G * gu;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gs[i] += div3(gs0);
        gde[i] += div3(gdev);
    }
    const double gtmp = -gf1 - gf2 * f2 * f2;
    gG += gtmp * 0.5 * dt * ivisc;
    gvisc -= gtmp * tmp * ivisc;
}

// MatProps::visc for one material without markers, at an explicit mean
// temperature T (the forward reads it from the nodes at that time)
__device__ double visc_eval(const KP &p, int e, const double *edot, double T, double &raw, double &ed)
{
    ed = 0;
    if (p.ef[DES_EF_LOG10_VISC]) {
        raw = pow(10.0, p.ef[DES_EF_LOG10_VISC][e]);
    } else {
        const double gas_constant = 8.3144;
        ed = dmax_(second_invariant_<3>(edot), 1e-30);
        const double visc0 = 0.25 * pow(ed, p.mat.visc_pw[0]) * p.mat.visc_coef[0]
            * exp(p.mat.visc_activation_energy[0] / (p.mat.visc_exponent[0] * gas_constant * T)) * 1e6;
        raw = 1 / (1 / visc0);
    }
    return dmin_(dmax_(raw, p.mat.visc_min), p.mat.visc_max);
}

// adjoint of the viscosity -> strain rate (corrected), mean temperature, log10
// viscosity; raw is the unclamped viscosity and ed the strain-rate invariant
// of visc_eval for the same element (ed < 0: not known yet)
__device__ void visc_reverse(const KP &p, int e, const double *edot, double T, double raw, double ed, double gvisc,
                             double *gedot, double &gT, double &glv)
{
    if (!(raw > p.mat.visc_min && raw < p.mat.visc_max)) return;   // clamped: no sensitivity
    if (p.ef[DES_EF_LOG10_VISC]) {
        glv += gvisc * raw * 2.302585092994046;   // d 10^x / dx = 10^x ln 10
        return;
    }
    const double gas_constant = 8.3144;
    const double q = p.mat.visc_activation_energy[0] / (p.mat.visc_exponent[0] * gas_constant);
    const double iT = recip_newton(T);
    gT -= gvisc * raw * q * iT * iT;
    if (ed < 0) ed = dmax_(second_invariant_<3>(edot), 1e-30);   // as visc_eval forms it
    if (ed > 1e-30) {
        const double ied = recip_newton(ed);
        const double ged = gvisc * raw * p.mat.visc_pw[0] * ied;
        const double gj2 = 0.5 * ged * ied;
        const double a = div3(edot[0] + edot[1] + edot[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) gedot[i] += gj2 * (edot[i] - a);
#pragma unroll
        for (int c = 3; c < 6; ++c) gedot[c] += gj2 * 2 * edot[c];
    }
}

// MatProps::plastic_weakening + plastic_props for one material without
// markers, reversed from the adjoints of (amc, anphi, anpsi, hardn,
// ten_max) to the per-element cohesion and friction angles and plstrain
__device__ void plastic_props_reverse(const KP &p, int e, double pls, double gamc, double ganphi, double ganpsi,
                                      double ghardn, double gtmax, double *gpar, double &gpls)
{
    // an element whose return map was inactive passes zero adjoints: its
    // contributions below are all zero, and the transcendentals are skipped
    if (gamc == 0 && ganphi == 0 && ganpsi == 0 && ghardn == 0 && gtmax == 0) return;
    const double c0 = p.ef[DES_EF_COHESION0] ? p.ef[DES_EF_COHESION0][e] : p.mat.cohesion0[0];
    const double c1 = p.ef[DES_EF_COHESION1] ? p.ef[DES_EF_COHESION1][e] : p.mat.cohesion1[0];
    const double f0 = p.ef[DES_EF_FRICTION0] ? p.ef[DES_EF_FRICTION0][e] : p.mat.friction_angle0[0];
    const double f1 = p.ef[DES_EF_FRICTION1] ? p.ef[DES_EF_FRICTION1][e] : p.mat.friction_angle1[0];
    const double d0 = p.mat.dilation_angle0[0], d1 = p.mat.dilation_angle1[0];
    const double l0 = p.mat.pls0[0], l1 = p.mat.pls1[0];
    int seg;
    double q = 0, c, phi, psi;
    if (pls < l0) {
        seg = 0;
        c = c0; phi = f0; psi = d0;
    } else if (pls < l1) {
        seg = 1;
        q = (pls - l0) / (l1 - l0);
        c = c0 + q * (c1 - c0); phi = f0 + q * (f1 - f0); psi = d0 + q * (d1 - d0);
    } else {
        seg = 2;
        c = c1; phi = f1; psi = d1;
    }
    const double sphi = sin(phi * DEG2RAD), spsi = sin(psi * DEG2RAD);
    const double anphi = (1 + sphi) / (1 - sphi);
    const double sq = sqrt(anphi), tn = tan(phi * DEG2RAD);
    double gc = 2 * sq * gamc;
    ganphi += 2 * c * gamc / (2 * sq);
    double gtn = 0;
    if (phi != 0 && c / tn < p.mat.tension_max) {
        gc += gtmax / tn;
        gtn = -gtmax * c / (tn * tn);
    }
    const double gphi = ganphi * 2 / ((1 - sphi) * (1 - sphi)) * cos(phi * DEG2RAD) * DEG2RAD
        + gtn * (1 + tn * tn) * DEG2RAD;
    const double gpsi = ganpsi * 2 / ((1 - spsi) * (1 - spsi)) * cos(psi * DEG2RAD) * DEG2RAD;
    if (seg == 0) {
        gpar[DES_EF_COHESION0] += gc;
        gpar[DES_EF_FRICTION0] += gphi;
    } else if (seg == 1) {
        const double il = 1 / (l1 - l0);
        gpar[DES_EF_COHESION0] += gc * (1 - q) - ghardn * il;
        gpar[DES_EF_COHESION1] += gc * q + ghardn * il;
        gpar[DES_EF_FRICTION0] += gphi * (1 - q);
        gpar[DES_EF_FRICTION1] += gphi * q;
        gpls += (gc * (c1 - c0) + gphi * (f1 - f0) + gpsi * (d1 - d0)) * il;
    } else {
        gpar[DES_EF_COHESION1] += gc;
        gpar[DES_EF_FRICTION1] += gphi;
    }
}

// Mohr-Coulomb return map in principal space (rheology.cxx:163-299),
// reversed.  S' = sum_k (p_k - alpha c_k) v_k v_k^T = S - alpha M.  With G_o
// the symmetric matrix of the output adjoint and g_ab = v_a^T G_o v_b, the
// adjoint of the trial stress is
//   H = G_o + sum_k dp_k v_k v_k^T - sum_{a<b} g_ab alpha (c_a - c_b) / (p_a - p_b) (v_a v_b^T + v_b v_a^T),
// (first-order perturbation of the eigenvalues, v_k^T dS v_k, and of the
// eigenprojectors), dp_k being the eigenvalue adjoints that alpha's
// dependence on the principal stresses contributes.  The identity part is
// applied directly: the analytic eigenvectors of near-repeated principal
// stresses are not orthonormal to working precision, so only the plastic
// correction goes through them, and an element that does not yield takes
// the identity exactly.  When p_a and p_b (nearly) coincide the eigenbasis,
// and with it the direction of the correction, is discontinuous in S: the
// term of that pair is dropped (a subgradient).
__device__ void mc_return_reverse(double K, double G, double amc, double anphi, double anpsi, double hardn,
                                  double tmax, const double *S, const double *go, double gdepls, double *gS,
                                  double &gG, double &gamc, double &ganphi, double &ganpsi, double &ghardn,
                                  double &gtmax)
{
    if (clearly_elastic3(amc, anphi, tmax, S)) {   // S' = S (the forward skipped the eigen-solve too)
#pragma unroll
        for (int cc = 0; cc < 6; ++cc) gS[cc] += go[cc];
        return;
    }
    double pr[3], v[3][3];
    principal_stresses3(S, pr, v);
    const double fs = pr[0] - pr[2] * anphi + amc;
    const double ft = pr[2] - tmax;
    double alpha = 0, c[3] = {0, 0, 0}, r = 0, D = 1;
    bool yield = !(fs > 0 && ft < 0), shear = false;
    const double a1 = K + 4. / 3 * G, a2 = K - 2. / 3 * G;
    if (!yield) {   // S' = S
#pragma unroll
        for (int cc = 0; cc < 6; ++cc) gS[cc] += go[cc];
        return;
    }
    {
        const double pa = sqrt(1 + anphi * anphi) + anphi;
        const double ps = tmax * anphi - amc;
        const double h = pr[2] - tmax + pa * (pr[0] - ps);
        shear = h < 0;
        if (shear) {
            D = a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2 * sqrt(anphi) * hardn;
            alpha = fs / D;
            c[0] = a1 - a2 * anpsi;
            c[1] = a2 - a2 * anpsi;
            c[2] = a2 - a1 * anpsi;
            r = sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18);
        } else {
            alpha = ft / a1;
            c[0] = a2;
            c[1] = a2;
            c[2] = a1;
            r = sqrt(7. / 18);
        }
    }
    // G_o and its eigenbasis components
    const double Go[3][3] = {{go[0], go[3] / 2, go[4] / 2}, {go[3] / 2, go[1], go[5] / 2}, {go[4] / 2, go[5] / 2, go[2]}};
    double gv[3][3];   // G_o v_k
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int m = 0; m < 3; ++m) gv[m][k] = Go[m][0] * v[0][k] + Go[m][1] * v[1][k] + Go[m][2] * v[2][k];
    double g[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) g[a][b] = v[0][a] * gv[0][b] + v[1][a] * gv[1][b] + v[2][a] * gv[2][b];
    double pb[3] = {g[0][0], g[1][1], g[2][2]};   // adjoints of p'_k, then of p_k
    double w[3][3] = {};   // projector terms beyond the identity
    const double scale = fabs(pr[0]) + fabs(pr[1]) + fabs(pr[2]) + 1e-300;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = a + 1; b < 3; ++b) {
            const double gap = pr[a] - pr[b];
            if (c[a] != c[b] && fabs(gap) > 1e-12 * scale) w[a][b] = -g[a][b] * alpha * (c[a] - c[b]) / gap;
        }
    {
        double galpha = -(pb[0] * c[0] + pb[1] * c[1] + pb[2] * c[2]);
        galpha += gdepls * ((alpha > 0) ? r : ((alpha < 0) ? -r : 0.0));
        double gc[3] = {-alpha * pb[0], -alpha * pb[1], -alpha * pb[2]};
        double ga1 = 0, ga2 = 0;
        if (shear) {
            const double gfs = galpha / D, gD = -galpha * alpha / D;
            pb[0] += gfs;
            pb[2] -= anphi * gfs;
            ganphi -= pr[2] * gfs;
            gamc += gfs;
            const double sqa = sqrt(anphi);
            ga1 += gD * (1 + anphi * anpsi);
            ga2 += gD * (-anpsi - anphi);
            ganpsi += gD * (-a2 + a1 * anphi);
            ganphi += gD * (a1 * anpsi - a2 + hardn / sqa);
            ghardn += gD * 2 * sqa;
            ga1 += gc[0] - gc[2] * anpsi;
            ga2 += -gc[0] * anpsi + gc[1] * (1 - anpsi) + gc[2];
            ganpsi += -gc[0] * a2 - gc[1] * a2 - gc[2] * a1;
            if (alpha != 0) ganpsi += gdepls * fabs(alpha) * (4 + 14 * anpsi) / (36 * r);
        } else {
            const double gft = galpha / a1;
            ga1 -= galpha * alpha / a1;
            pb[2] += gft;
            gtmax -= gft;
            ga2 += gc[0] + gc[1];
            ga1 += gc[2];
        }
        gG += ga1 * 4. / 3 - ga2 * 2. / 3;
    }
    // H - G_o in components (diagonal H_mm, off-diagonal 2 H_mn), plus G_o
    const double dpb[3] = {pb[0] - g[0][0], pb[1] - g[1][1], pb[2] - g[2][2]};
    const int cm[6] = {0, 1, 2, 0, 0, 1}, cn[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) {
        const int m = cm[cc], n = cn[cc];
        double h = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) h += dpb[k] * v[m][k] * v[n][k];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = a + 1; b < 3; ++b) h += w[a][b] * (v[m][a] * v[n][b] + v[m][b] * v[n][a]);
        gS[cc] += go[cc] + ((cc < 3) ? h : 2 * h);
    }
}

// ------------------------------------------------------------------
// update_stress (rheology.cxx:510-646) of one element, reversed, plus the
// second half of NMD_stress (the dp adjoint gathered from the element's
// nodes) and the element density rho(T) of the step.
// In: as = adjoint of the stress after update_stress, apls = of plstrain
// after the step, adp/adpn/arho/avol.  Out: as, apls = adjoints at the
// start of the step; aedot = adjoint of the strain rate before the
// anti-locking correction; aedv; avol, avolo; slot1 = T' contributions of
// the four nodes; g += the parameter gradients of the element.
// ------------------------------------------------------------------
__global__ void __launch_bounds__(TPB_A) k_adj_stress(KP p, AdjBufs a, TapeStep t, TapeStep t1, double dt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne;
    int nodes[4];
    double sacc = 0, Tsum = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        nodes[i] = conn_at(p, i, e);
        sacc += a.adpn[nodes[i]];
        Tsum += t1.T[nodes[i]];
    }
    const double T = Tsum / 4;   // elem_avg_T of the updated temperature
    const double vol = t.vol[e], volo = t.volo[e];
    const double gdp = a.adp[e] + vol * sacc;
    double gvol = a.avol[e] + t.dp[e] * sacc, gvolo = 0;
    double s0[6], edot[6], go[6];
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) {
        s0[cc] = t.s[cc * ne + e];
        edot[cc] = t.edot[cc * ne + e];
        go[cc] = a.as[cc * ne + e];
    }
    const double pls = t.pls[e];
    // anti-locking correction (rheology.cxx:527-534) and increments
    {
        const double div = edot[0] + edot[1] + edot[2];
        const double corr = divnd<3>(t.edv[e] - div);
#pragma unroll
        for (int i = 0; i < 3; ++i) edot[i] += corr;
    }
    double de[6];
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) de[cc] = edot[cc] * dt;
    const double K = m_bulkm(p, e), G = m_shearm(p, e);
    // dp = tr(s_out) - tr(s0)
#pragma unroll
    for (int i = 0; i < 3; ++i) go[i] += gdp;
    double gs[6] = {-gdp, -gdp, -gdp, 0, 0, 0};
    double gde[6] = {0, 0, 0, 0, 0, 0}, gec[6] = {0, 0, 0, 0, 0, 0};
    double gG = 0, gvisc = 0, gdv = 0, gT = 0, glv = 0, gpls_props = 0;
    double gpar[DES_EF_COUNT] = {};
    const int rt = p.mat.rheol_type;
    // the viscosity and the EVP branch: the forward recompute's, from the
    // tape (else evaluated again, as the forward does)
    double visc = 0, raw = 0, ed = -1;
    const bool viscous = (rt & DES_RH_VISCOUS) != 0;
    if (viscous) {
        if (t.visc) raw = visc = t.visc[e];   // unclamped: raw == visc; clamped: no sensitivity either way
        else visc = visc_eval(p, e, edot, T, raw, ed);
    }
    if (rt == DES_RH_ELASTIC) {
        elastic_reverse(K, G, de, go, gs, gde, gG);
    } else if (rt == DES_RH_MAXWELL) {
        maxwell_reverse(K, G, visc, dt, de, s0, go, gs, gde, gG, gvisc, gdv);
    } else {   // EP or EVP
        double amc, anphi, anpsi, hardn, tmax;
        m_plastic_props(p, e, pls, amc, anphi, anpsi, hardn, tmax);
        bool plastic = true;
        if (rt == DES_RH_EVP) {
            if (t.evp) {
                plastic = t.evp[e] != 0;
            } else {
                const double dv = vol / volo - 1;
                double sv[6], sp[6];
#pragma unroll
                for (int cc = 0; cc < 6; ++cc) sv[cc] = sp[cc] = s0[cc];
                elastic_<3>(K, G, de, sp);
                maxwell_<3>(K, G, visc, dt, dv, de, sv);
                double depls;
                if (!clearly_elastic3(amc, anphi, tmax, sp))
                    mc_return_<3>(K, G, amc, anphi, anpsi, hardn, tmax, depls, sp);
                plastic = !(second_invariant2_<3>(sv) < second_invariant2_<3>(sp));
            }
        }
        if (plastic) {
            double S[6];   // the elastic trial stress
#pragma unroll
            for (int cc = 0; cc < 6; ++cc) S[cc] = s0[cc];
            elastic_<3>(K, G, de, S);
            double gS[6] = {0, 0, 0, 0, 0, 0};
            double gamc = 0, ganphi = 0, ganpsi = 0, ghardn = 0, gtmax = 0;
            mc_return_reverse(K, G, amc, anphi, anpsi, hardn, tmax, S, go, a.apls[e], gS, gG, gamc, ganphi, ganpsi,
                              ghardn, gtmax);
            elastic_reverse(K, G, de, gS, gs, gde, gG);
            plastic_props_reverse(p, e, pls, gamc, ganphi, ganpsi, ghardn, gtmax, gpar, gpls_props);
        } else {
            maxwell_reverse(K, G, visc, dt, de, s0, go, gs, gde, gG, gvisc, gdv);
        }
    }
    if (viscous && gvisc != 0) visc_reverse(p, e, edot, T, raw, ed, gvisc, gec, gT, glv);
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) gec[cc] += dt * gde[cc];
    const double ivo = recip_newton(volo);
    gvol += gdv * ivo;
    gvolo -= gdv * vol * ivo * ivo;
    // corrected strain rate -> strain rate before the correction, edvoldt
    const double tg = gec[0] + gec[1] + gec[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) a.aedot[i * ne + e] = gec[i] - div3(tg);
#pragma unroll
    for (int cc = 3; cc < 6; ++cc) a.aedot[cc * ne + e] = gec[cc];
    a.aedv[e] = div3(tg);
    // element density of the step: rho0 (1 - alpha (T - 273))
    gT += a.arho[e] * (-p.mat.rho0[0] * p.mat.alpha[0]);
#pragma unroll
    for (int i = 0; i < 4; ++i) a.slot1[(size_t)i * ne + e] = gT / 4;
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) a.as[cc * ne + e] = gs[cc];
    a.apls[e] += gpls_props;
    a.avol[e] = gvol;
    a.avolo[e] = gvolo;
    gpar[DES_EF_LOG10_VISC] += glv;
    gpar[DES_EF_SHEAR_MODULUS] += gG;
#pragma unroll
    for (int k = 0; k < DES_EF_COUNT; ++k)
        if (gpar[k] != 0) a.g[(size_t)k * ne + e] += gpar[k];
}

// nodes: adjoint of the updated temperature (state + the stress kernel's
// T' terms), nodal dvoldt (ntmp = sum_e tr(edot) vol / volume_n, edvoldt =
// mean of ntmp), and the temperature update with its Dirichlet BCs
// (fields.cxx:151-162): T' = T - tdot dt / tmass
__global__ void __launch_bounds__(TPB_A) k_adj_nodes_heat(KP p, AdjBufs a, TapeStep t, TapeStep t1, double dt)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const size_t ne = p.ne;
    double gTp = a.aT[n], gnt = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        const int ent = p.sup_ent[q];
        const int e = ent >> 2, i = ent & 3;
        gTp += a.slot1[(size_t)i * ne + e];
        gnt += a.aedv[e] / 4;
    }
    const double vn = t.voln[n];
    a.antmp[n] = gnt / vn;
    a.avn[n] -= gnt * t.ntmp[n] / vn;
    double gT = gTp, gtd = 0;
    if (p.prm.has_thermal_diffusion) {
        const unsigned flag = p.bcflag[n];
        if ((flag & BOUNDZ1) || ((flag & BOUNDZ0) && !p.prm.has_fixed_bottom_temperature)) {
            gT = 0;
        } else {
            const double tm = t.tmass[n];
            gtd = -gTp * dt / tm;
            a.atm[n] += gTp * t.tdot[n] * dt / (tm * tm);
        }
    }
    a.aT[n] = gT;
    a.atdot[n] = gtd;
}

// elements: dvoldt terms, the heat stencil (fields.cxx:99-146) and the
// strain rate (fields.cxx:166-232), reversed, at the start of the step.
// Out: ashp, avol (+=), slot3 = velocity contributions, slot1 = temperature
// contributions, g[therm_cond].
__global__ void __launch_bounds__(TPB_A) k_adj_kinematics(KP p, AdjBufs a, TapeStep t)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne, nn = p.nn;
    int nodes[4];
    double sh[3][4], gsh[3][4], v[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        nodes[i] = conn_at(p, i, e);
        tload3(t.v, nn, nodes[i], v[i]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sh[k][i] = tshp(t, ne, k, i, e);
            gsh[k][i] = a.ashp[((size_t)k * 4 + i) * ne + e];
        }
    }
    const double vol = t.vol[e];
    double gvol = a.avol[e];
    double g[6];
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) g[cc] = a.aedot[cc * ne + e];
    // dvoldt: sum_e tr(edot) vol
    {
        double sant = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) sant += a.antmp[nodes[i]];
        const double tr = t.edot[e] + t.edot[ne + e] + t.edot[2 * ne + e];
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] += vol * sant;
        gvol += tr * sant;
    }
    double gTn[4] = {0, 0, 0, 0};
    if (p.prm.has_thermal_diffusion) {
        double Tn[4], gtd[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            Tn[i] = t.T[nodes[i]];
            gtd[i] = a.atdot[nodes[i]];
        }
        const double k = m_k(p, e), kv = k * vol, hrcp = p.mat.hr_over_cp;
        double gkv = 0, grh = 0;
        // tdot_i = kv sum_j D_ij T_j - rh with the symmetric D_ij = dN_i . dN_j:
        // D is formed once (10 entries), and the adjoints of D_ij and D_ji,
        // kg_i T_j and kg_j T_i (kg = kv gtd), are folded into one symmetric
        // H_mk, so that d/d dN_m = sum_k H_mk dN_k
        double D[4][4], kg[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            kg[i] = kv * gtd[i];
#pragma unroll
            for (int j = i; j < 4; ++j) {
                D[i][j] = sh[0][i] * sh[0][j] + sh[1][i] * sh[1][j] + sh[2][i] * sh[2][j];
                D[j][i] = D[i][j];
            }
        }
        double H[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            double diffusion = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                diffusion += D[i][j] * Tn[j];
                gTn[i] += D[i][j] * kg[j];
            }
            gkv += gtd[i] * diffusion;
            grh -= gtd[i];
#pragma unroll
            for (int j = i; j < 4; ++j) {
                H[i][j] = kg[i] * Tn[j] + kg[j] * Tn[i];
                H[j][i] = H[i][j];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                double acc = 0;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) acc += H[m][kk] * sh[c][kk];
                gsh[c][m] += acc;
            }
        a.g[(size_t)DES_EF_THERM_COND * ne + e] += gkv * vol;
        gvol += gkv * k + grh * hrcp;
    }
    // strain rate
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double sx = sh[0][i], sy = sh[1][i], sz = sh[2][i];
        const double gv0 = g[0] * sx + 0.5 * g[3] * sy + 0.5 * g[4] * sz;
        const double gv1 = g[1] * sy + 0.5 * g[3] * sx + 0.5 * g[5] * sz;
        const double gv2 = g[2] * sz + 0.5 * g[4] * sx + 0.5 * g[5] * sy;
        gsh[0][i] += g[0] * v[i][0] + 0.5 * g[3] * v[i][1] + 0.5 * g[4] * v[i][2];
        gsh[1][i] += g[1] * v[i][1] + 0.5 * g[3] * v[i][0] + 0.5 * g[5] * v[i][2];
        gsh[2][i] += g[2] * v[i][2] + 0.5 * g[4] * v[i][0] + 0.5 * g[5] * v[i][1];
        a.slot3[((size_t)0 * 4 + i) * ne + e] = gv0;
        a.slot3[((size_t)1 * 4 + i) * ne + e] = gv1;
        a.slot3[((size_t)2 * 4 + i) * ne + e] = gv2;
        a.slot1[(size_t)i * ne + e] = gTn[i];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) a.ashp[((size_t)k * 4 + i) * ne + e] = gsh[k][i];
    a.avol[e] = gvol;
}

// nodes: add the element contributions to the velocity and temperature adjoints
__global__ void __launch_bounds__(TPB_A) k_adj_gather_vT(KP p, AdjBufs a)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const size_t ne = p.ne, nn = p.nn;
    double gv[3] = {0, 0, 0}, gT = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        const int ent = p.sup_ent[q];
        const int e = ent >> 2, i = ent & 3;
#pragma unroll
        for (int d = 0; d < 3; ++d) gv[d] += a.slot3[((size_t)d * 4 + i) * ne + e];
        gT += a.slot1[(size_t)i * ne + e];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) a.av[d * nn + n] += gv[d];
    a.aT[n] += gT;
}

// window start: adjoints of the derived fields (volume, shape functions,
// mass, tmass, volume_n) -> coordinates and temperature (tmass through
// rho(T) of the start temperature)
__global__ void __launch_bounds__(TPB_A) k_adj_start_geometry(KP p, AdjBufs a, TapeStep t)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.ne) return;
    const size_t ne = p.ne, nn = p.nn;
    int nodes[4];
    double c[4][3], Tsum = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        nodes[i] = conn_at(p, i, e);
        tload3(t.x, nn, nodes[i], c[i]);
        Tsum += t.T[nodes[i]];
    }
    const double rho_e = m_rho_T(p, e, Tsum / 4);
    double gvol = a.avol[e];
    double gm[4], gtm[4], gvn[4], gs[3][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        gm[i] = a.am[nodes[i]];
        gtm[i] = a.atm[nodes[i]];
        gvn[i] = a.avn[nodes[i]];
#pragma unroll
        for (int k = 0; k < 3; ++k) gs[k][i] = a.ashp[((size_t)k * 4 + i) * ne + e];
    }
    const double grho = mass_reverse(p, e, gm, gtm, gvn, t.vol[e], rho_e, gvol);
    const double gT = grho * (-p.mat.rho0[0] * p.mat.alpha[0]);
    double gc[4][3] = {};
    geom_reverse(c, t.vol[e], gs, gvol, gc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int d = 0; d < 3; ++d) a.slotx[((size_t)d * 4 + i) * ne + e] = gc[i][d];
        a.slot1[(size_t)i * ne + e] = gT / 4;
    }
}

__global__ void __launch_bounds__(TPB_A) k_adj_gather_xT(KP p, AdjBufs a)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.nn) return;
    const size_t ne = p.ne, nn = p.nn;
    double gx[3] = {0, 0, 0}, gT = 0;
    for (int q = p.sup_off[n]; q < p.sup_off[n + 1]; ++q) {
        const int ent = p.sup_ent[q];
        const int e = ent >> 2, i = ent & 3;
#pragma unroll
        for (int d = 0; d < 3; ++d) gx[d] += a.slotx[((size_t)d * 4 + i) * ne + e];
        gT += a.slot1[(size_t)i * ne + e];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) a.ax[d * nn + n] += gx[d];
    a.aT[n] += gT;
}

int launch_adj_stress(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                      cudaStream_t s)
{
    k_adj_stress<<<nblk(p.ne), TPB_A, 0, s>>>(p, a, t, t1, dt);
    return 1;
}

int launch_adj_nodes_heat(const KP &p, const AdjBufs &a, const TapeStep &t, const TapeStep &t1, double dt,
                          cudaStream_t s)
{
    k_adj_nodes_heat<<<nblk(p.nn), TPB_A, 0, s>>>(p, a, t, t1, dt);
    return 1;
}

int launch_adj_kinematics(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s)
{
    k_adj_kinematics<<<nblk(p.ne), TPB_A, 0, s>>>(p, a, t);
    return 1;
}

int launch_adj_gather_vT(const KP &p, const AdjBufs &a, cudaStream_t s)
{
    k_adj_gather_vT<<<nblk(p.nn), TPB_A, 0, s>>>(p, a);
    return 1;
}

int launch_adj_start_geometry(const KP &p, const AdjBufs &a, const TapeStep &t, cudaStream_t s)
{
    k_adj_start_geometry<<<nblk(p.ne), TPB_A, 0, s>>>(p, a, t);
    return 1;
}

int launch_adj_gather_xT(const KP &p, const AdjBufs &a, cudaStream_t s)
{
    k_adj_gather_xT<<<nblk(p.nn), TPB_A, 0, s>>>(p, a);
    return 1;
}

}  // namespace des
