// drd_ops.cuh — device forms of the momentum operator shared by the per-step kernels
// (drd_kernels.cu) and the batched solver (drd_batch.cu): the ghost-aware fetch of the packed
// unknowns, one row of MatrixVector_uv_2_CG and the Jacobi diagonal of PSolve_uv_2_CG
// (microfluidics_complex_domain/VeloSolve_2_combined.f90:515-711).
#pragma once

#include "drd_kernels.cuh"

namespace drd {

// Values of the unknown fields at any index the operator reads, with the ghost values
// MatrixVector_uv_2_CG assigns (:533-553; TP lr_bd_type 'n': copies instead of reflections).
template <typename T, bool CG = false>
struct UVFetch {
    const T* x; int nr, nz; long mn; int neumann;
    __device__ __forceinline__ T ld(long q) const {
        if constexpr (CG) return __ldcg(x + q);
        return x[q];
    }
    __device__ __forceinline__ T U(int i, int k) const {
        if (k < 0) return -Uc(i, 0);
        if (k > nz - 1) return -Uc(i, nz - 1);
        return Uc(i, k);
    }
    __device__ __forceinline__ T Uc(int i, int k) const {  // k in [0, nz-1]
        if (i < 0) return neumann ? ld(1 + (long)(nr + 1) * k) : -ld(1 + (long)(nr + 1) * k);
        if (i > nr) return neumann ? ld((nr - 1) + (long)(nr + 1) * k) : -ld((nr - 1) + (long)(nr + 1) * k);
        return ld(i + (long)(nr + 1) * k);
    }
    __device__ __forceinline__ T V(int i, int k) const {
        if (k <= 0 || k >= nz) return T(0);
        const int ii = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
        return ld(mn + ii + (long)nr * (k - 1));
    }
};

// Row q of MatrixVector_uv_2_CG (:515-646) / MatrixVector_uv_CG: (A x)_q.  The FP64 form keeps
// the reference's expression; the FP32 form (the mixed mode's inner operator) takes differences
// before scaling and multiplies by the reciprocals of dr^2, dz^2 and dr dz instead of dividing.
// DIFF selects the difference form with reciprocal multiplies (the FP32 form) for either T; the
// default keeps the reference's expression in FP64.
template <typename T, class FX, bool DIFF = (sizeof(T) == 4)>
__device__ __forceinline__ T uv_apply(const OpScal<T>& o, const T* __restrict__ rho, const T* __restrict__ eta,
                                      const T* __restrict__ pen, const FX& F, long q) {
    const int nr = o.nr;
    const long mn = F.mn;
    const T h = T(0.5), q4 = T(0.25);
    const T mcoef = (o.bdf == 2) ? T(1.5) * o.re : o.re;
    T val;
#define E_(i, k) eta[cidx(nr, i, k)]
    if (q < mn) {
        const int qi = (int)q, k = qi / (nr + 1), i = qi - k * (nr + 1);
        const T f1 = F.ld(q);
        if (o.bdf == 2)
            val = f1 * mcoef * (rho[cidx(nr, i, k)] + rho[cidx(nr, i - 1, k)]) * h +
                  f1 * o.pk * (pen[cidx(nr, i, k)] + pen[cidx(nr, i - 1, k)]) * h * o.dt;
        else
            val = f1 * mcoef * (rho[cidx(nr, i, k)] + rho[cidx(nr, i - 1, k)]) * h;
        T cr = E_(i, k), cl = E_(i - 1, k);
        if constexpr (DIFF)
            val = val - T(2) * o.dt * (cr * (F.Uc(i + 1, k) - f1) + cl * (F.Uc(i - 1, k) - f1)) * o.idr2;
        else
            val = val - T(2) * o.dt * (cr * F.Uc(i + 1, k) + cl * F.Uc(i - 1, k) - (cl + cr) * f1) / o.dr2;
        cr = (E_(i, k + 1) + E_(i - 1, k + 1) + E_(i, k) + E_(i - 1, k)) * q4;
        cl = (E_(i, k) + E_(i - 1, k) + E_(i, k - 1) + E_(i - 1, k - 1)) * q4;
        if constexpr (DIFF) {
            val = val - o.dt * (cr * (F.U(i, k + 1) - f1) + cl * (F.U(i, k - 1) - f1)) * o.idz2;
            val = val - o.dt * (cr * (F.V(i, k + 1) - F.V(i - 1, k + 1)) - cl * (F.V(i, k) - F.V(i - 1, k))) * o.idrdz;
        } else {
            val = val - o.dt * (cr * F.U(i, k + 1) + cl * F.U(i, k - 1) - (cl + cr) * f1) / o.dz2;
            val = val - o.dt * (cr * (F.V(i, k + 1) - F.V(i - 1, k + 1)) - cl * (F.V(i, k) - F.V(i - 1, k))) / o.dr / o.dz;
        }
    } else {
        const int qv = (int)(q - mn), kv = qv / nr, i = qv - kv * nr, k = kv + 1;
        const T f2 = F.ld(q);
        if (o.bdf == 2)
            val = f2 * mcoef * (rho[cidx(nr, i, k)] + rho[cidx(nr, i, k - 1)]) * h +
                  f2 * o.pk * (pen[cidx(nr, i, k)] + pen[cidx(nr, i, k - 1)]) * h * o.dt;
        else
            val = f2 * mcoef * (rho[cidx(nr, i, k)] + rho[cidx(nr, i, k - 1)]) * h;
        T cr = E_(i, k), cl = E_(i, k - 1);
        if constexpr (DIFF)
            val = val - T(2) * o.dt * (cr * (F.V(i, k + 1) - f2) + cl * (F.V(i, k - 1) - f2)) * o.idz2;
        else
            val = val - T(2) * o.dt * (cr * F.V(i, k + 1) + cl * F.V(i, k - 1) - (cl + cr) * f2) / o.dz2;
        cr = (E_(i + 1, k) + E_(i, k) + E_(i + 1, k - 1) + E_(i, k - 1)) * q4;
        cl = (E_(i, k) + E_(i - 1, k) + E_(i, k - 1) + E_(i - 1, k - 1)) * q4;
        if constexpr (DIFF) {
            val = val - o.dt * (cr * (F.V(i + 1, k) - f2) + cl * (F.V(i - 1, k) - f2)) * o.idr2;
            val = val - o.dt * (cr * (F.Uc(i + 1, k) - F.Uc(i + 1, k - 1)) - cl * (F.Uc(i, k) - F.Uc(i, k - 1))) * o.idrdz;
        } else {
            val = val - o.dt * (cr * F.V(i + 1, k) + cl * F.V(i - 1, k) - (cl + cr) * f2) / o.dr2;
            val = val - o.dt * (cr * (F.Uc(i + 1, k) - F.Uc(i + 1, k - 1)) - cl * (F.Uc(i, k) - F.Uc(i, k - 1))) / o.dr / o.dz;
        }
    }
#undef E_
    return val;
}

// The Jacobi diagonal of PSolve_uv_2_CG (:649-711) / PSolve_uv_CG for row q: 1.5 re rho-bar (re
// for bdf 1) plus the eta stencil's diagonal, boundary-aware, without the penalty; the v rows
// average rho(i,j) and rho(i-1,j) as the reference does (:690).
// UNIT: the same diagonal with rho = eta = 1 (the arrays are not read).
template <typename T, bool UNIT = false>
__device__ __forceinline__ T uv_diag(const OpScal<T>& o, const T* __restrict__ rho, const T* __restrict__ eta, long q) {
    const int nr = o.nr, nz = o.nz;
    const long mn = (long)(nr + 1) * nz;
    const T mcoef = (o.bdf == 2) ? T(1.5) * o.re : o.re;
    const T h = T(0.5), q4 = T(0.25);
#define E_(i, k) (UNIT ? T(1) : eta[cidx(nr, i, k)])
    T tmp;
    if (q < mn) {
        const int i = (int)(q % (nr + 1)), j = (int)(q / (nr + 1));
        tmp = mcoef * (UNIT ? T(2) : rho[cidx(nr, i, j)] + rho[cidx(nr, i - 1, j)]) * h;
        T cr = E_(i, j), cl = E_(i - 1, j);
        tmp = tmp + T(2) * o.dt * (cl + cr) / o.dr2;
        cr = (E_(i, j + 1) + E_(i - 1, j + 1) + E_(i, j) + E_(i - 1, j)) * q4;
        cl = (E_(i, j) + E_(i - 1, j) + E_(i, j - 1) + E_(i - 1, j - 1)) * q4;
        if (j == 0) tmp = tmp + o.dt * (cl + (cl + cr)) / o.dz2;
        else if (j == nz - 1) tmp = tmp + o.dt * (cr + (cl + cr)) / o.dz2;
        else tmp = tmp + o.dt * (cl + cr) / o.dz2;
    } else {
        const long qv = q - mn;
        const int i = (int)(qv % nr), j = (int)(qv / nr) + 1;
        tmp = mcoef * (UNIT ? T(2) : rho[cidx(nr, i, j)] + rho[cidx(nr, i - 1, j)]) * h;
        T cr = E_(i, j), cl = E_(i, j - 1);
        tmp = tmp + T(2) * o.dt * (cl + cr) / o.dz2;
        cr = (E_(i + 1, j) + E_(i, j) + E_(i + 1, j - 1) + E_(i, j - 1)) * q4;
        cl = (E_(i, j) + E_(i - 1, j) + E_(i, j - 1) + E_(i - 1, j - 1)) * q4;
        if (i == 0) tmp = tmp + o.dt * cr / o.dr2;
        else if (i == nr - 1) tmp = tmp + o.dt * cl / o.dr2;
        else tmp = tmp + o.dt * (cl + cr) / o.dr2;
    }
#undef E_
    return tmp;
}

}  // namespace drd
