// des_bc.cuh -- velocity boundary conditions of one node (bc.cxx:179-490).
#pragma once
#include "des_common.cuh"

namespace des {

// ==================================================================
// velocity boundary conditions (bc.cxx:179-490), one node
// ==================================================================
template <int ND>
__device__ __forceinline__ void vbc_x(int type, double val, double *v)
{
    switch (type) {
    case 1: v[0] = val; break;
    case 2: v[1] = 0; if (ND == 3) v[ND - 1] = 0; break;
    case 3: v[0] = val; v[1] = 0; if (ND == 3) v[ND - 1] = 0; break;
    case 4: if (ND == 3) { v[1] = val; v[ND - 1] = 0; } break;
    case 5: if (ND == 3) { v[0] = 0; v[1] = val; v[ND - 1] = 0; } break;
    case 7: if (ND == 3) { v[0] = val; v[1] = 0; } break;
    default: break;
    }
}

__device__ __forceinline__ void vbc_y(int type, double val, double *v, bool y1)
{
    switch (type) {
    case 1: v[1] = val; break;
    case 2: v[0] = 0; v[2] = 0; break;
    case 3:
        if (y1) { v[0] = val; v[1] = 0; v[2] = 0; }   // bc.cxx:325-329
        else { v[0] = 0; v[1] = val; v[2] = 0; }      // bc.cxx:294-298
        break;
    case 4: v[0] = val; v[2] = 0; break;
    case 5: v[0] = val; v[1] = 0; v[2] = 0; break;
    case 7: v[0] = 0; v[1] = val; break;
    default: break;
    }
}

template <int ND>
__device__ __forceinline__ void vbc_z(int type, double val, double *v)
{
    switch (type) {
    case 1: v[ND - 1] = val; break;
    case 2: v[0] = 0; if (ND == 3) v[1] = 0; break;
    case 3: v[0] = 0; if (ND == 3) v[1] = 0; v[ND - 1] = val; break;
    default: break;
    }
}

// va = the boundaries' prescribed values (Variables::vbc_values); the map
// is affine in (v, va), which the adjoint uses to transpose it
template <int ND>
__device__ void apply_vbcs_node_va(const KP &p, unsigned flag, double *v, const double *va)
{
    if (!(flag & BOUND_ANY)) return;
    const int *ty = p.prm.vbc_types;
    if (flag & BOUNDX0) vbc_x<ND>(ty[0], va[0], v);
    if (flag & BOUNDX1) vbc_x<ND>(ty[1], va[1], v);
    if (ND == 3) {
        if (flag & BOUNDY0) vbc_y(ty[2], va[2], v, false);
        if (flag & BOUNDY1) vbc_y(ty[3], va[3], v, true);
    }
    for (int ib = 6; ib <= 9; ib++) {
        if (!(flag & (1u << ib))) continue;
        const double *n = p.bnormals[ib];
        double fac = 0;
        switch (ty[ib]) {
        case 1:
            if (flag == (1u << ib)) {
                double vn = 0;
                for (int d = 0; d < ND; d++) vn += v[d] * n[d];
                for (int d = 0; d < ND; d++) v[d] += (va[ib] - vn) * n[d];
            } else {
                for (int ic = 0; ic < ib; ic++) {
                    if (!(flag & (1u << ic))) continue;
                    if (ty[ic] == 0) {
                        double vn = 0;
                        for (int d = 0; d < ND; d++) vn += v[d] * n[d];
                        for (int d = 0; d < ND; d++) v[d] += (va[ib] - vn) * n[d];
                    } else if (ty[ic] == 1) {
                        const double *edge = p.edge_vectors[ic][ib];
                        double ve = 0;
                        for (int d = 0; d < ND; d++) ve += v[d] * edge[d];
                        for (int d = 0; d < ND; d++) v[d] = ve * edge[d];
                    }
                }
            }
            break;
        case 3:
            for (int d = 0; d < ND; d++) v[d] = va[ib] * n[d];
            break;
        case 11:
            fac = 1 / sqrt(1 - n[ND - 1] * n[ND - 1]);
            if (flag == (1u << ib)) {
                double vn = 0;
                for (int d = 0; d < ND - 1; d++) vn += v[d] * n[d];
                for (int d = 0; d < ND - 1; d++) v[d] += (va[ib] * fac - vn) * n[d];
            } else {
                for (int ic = 0; ic < ib; ic++) {
                    if (!(flag & (1u << ic))) continue;
                    if (ty[ic] == 0) {
                        double vn = 0;
                        for (int d = 0; d < ND - 1; d++) vn += v[d] * n[d];
                        for (int d = 0; d < ND - 1; d++) v[d] += (va[ib] * fac - vn) * n[d];
                    } else if (ty[ic] == 1) {
                        const double *edge = p.edge_vectors[ic][ib];
                        double ve = 0;
                        for (int d = 0; d < ND; d++) ve += v[d] * edge[d];
                        for (int d = 0; d < ND; d++) v[d] = ve * edge[d];
                    }
                }
            }
            break;
        case 13:
            fac = 1 / sqrt(1 - n[ND - 1] * n[ND - 1]);
            for (int d = 0; d < ND - 1; d++) v[d] = va[ib] * fac * n[d];
            v[ND - 1] = 0;
            break;
        default:
            break;
        }
    }
    if (ty[4] == 0 && ty[5] == 0) return;
    if (flag & BOUNDZ0) vbc_z<ND>(ty[4], va[4], v);
    if (flag & BOUNDZ1) vbc_z<ND>(ty[5], va[5], v);
}

template <int ND>
__device__ __forceinline__ void apply_vbcs_node(const KP &p, unsigned flag, double *v)
{
    apply_vbcs_node_va<ND>(p, flag, v, p.prm.vbc_values);
}

}  // namespace des
