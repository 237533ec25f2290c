// drd_kernels.cu — sm_103a kernels of the DRD-Micro per-time-step solver core.
//
// Every kernel is written against the reference line it replaces (cited at the kernel).
// Floating-point expressions keep the reference's left-to-right evaluation order so that
// the FP64 path agrees with the FP64 CPU restatement to rounding (FMA contraction aside).
// Kernels that take a Krylov state `ks` and a gate return immediately when the solve has
// left the state they belong to, so a fixed launch sequence (a captured CUDA graph) can
// express BiCGSTAB's early exits.
#include <cooperative_groups.h>
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched at run time)
#include <math.h>
#include <cstdlib>

#include "drd_kernels.cuh"
#include "drd_ops.cuh"

namespace cg = cooperative_groups;

namespace drd {

static __device__ __forceinline__ bool gate_closed(const KState* ks, int gate) {
    if (gate == G_ALWAYS || ks == nullptr) return false;
    const int ph = *((volatile const int*)&ks->phase);
    if (gate == G_RUNNING) return ph != PH_RUNNING;
    if (gate == G_XNZ) return ph != PH_RUNNING || ks->x_nonzero == 0;
    if (gate == G_EARLY_OR_RUNNING) return ph == PH_DONE;
    return false;
}

static inline int grid_for(long n, int per_thread = 2) {
    long b = (n + (long)DRD_TPB * per_thread - 1) / ((long)DRD_TPB * per_thread);
    if (b < 1) b = 1;
    if (b > 4096) b = 4096;
    return (int)b;
}

// ======================================================================================
// op_double_gradient_Neum (microfluidics_complex_domain/matrix_tool.f90:178-219) at (i,k):
// variable-coefficient 5-point operator with face mobility (M_i + M_nb)/2 and zero flux
// through the domain faces.  Reads interior values only.
// ======================================================================================
//
// FP64 keeps the reference's form moL*x(i-1) + moR*x(i+1) - (moL+moR)*x(i).  FP32 (the inner
// operators of the mixed mode) evaluates the same sum as moR*(x(i+1)-x(i)) - moL*(x(i)-x(i-1)):
// for smooth fields the neighbour differences are exact in FP32 while the reference form
// cancels, and iterative refinement only converges if the FP32 operator stays close to the
// FP64 one on those fields.
template <typename T, class XA, class MA>
__device__ __forceinline__ T op_dgn(int i, int k, int nr, int nz, T idx2, T idz2, const XA& x, const MA& mo) {
    const T h = T(0.5);
    T acc = T(0);
    const T m0 = mo(i, k), x0 = x(i, k);
    if constexpr (sizeof(T) == 4) {
        T sx = T(0), sz = T(0);
        if (i > 0) sx -= (mo(i - 1, k) + m0) * h * (x0 - x(i - 1, k));
        if (i < nr - 1) sx += (m0 + mo(i + 1, k)) * h * (x(i + 1, k) - x0);
        if (k > 0) sz -= (mo(i, k - 1) + m0) * h * (x0 - x(i, k - 1));
        if (k < nz - 1) sz += (m0 + mo(i, k + 1)) * h * (x(i, k + 1) - x0);
        return idx2 * sx + idz2 * sz;
    }
    T moL, moR;
    if (i == 0) {
        moL = (m0 + m0) * h;
        moR = (m0 + mo(i + 1, k)) * h;
        acc = acc + idx2 * (moL * x0 + moR * x(i + 1, k) - (moL + moR) * x0);
    } else if (i == nr - 1) {
        moL = (mo(i - 1, k) + m0) * h;
        moR = (m0 + m0) * h;
        acc = acc + idx2 * (moL * x(i - 1, k) + moR * x0 - (moL + moR) * x0);
    } else {
        moL = (mo(i - 1, k) + m0) * h;
        moR = (m0 + mo(i + 1, k)) * h;
        acc = acc + idx2 * (moL * x(i - 1, k) + moR * x(i + 1, k) - (moL + moR) * x0);
    }
    if (k == 0) {
        moL = (m0 + m0) * h;
        moR = (m0 + mo(i, k + 1)) * h;
        acc = acc + idz2 * (moL * x0 + moR * x(i, k + 1) - (moL + moR) * x0);
    } else if (k == nz - 1) {
        moL = (mo(i, k - 1) + m0) * h;
        moR = (m0 + m0) * h;
        acc = acc + idz2 * (moL * x(i, k - 1) + moR * x0 - (moL + moR) * x0);
    } else {
        moL = (mo(i, k - 1) + m0) * h;
        moR = (m0 + mo(i, k + 1)) * h;
        acc = acc + idz2 * (moL * x(i, k - 1) + moR * x(i, k + 1) - (moL + moR) * x0);
    }
    return acc;
}

template <typename T>
struct PackedA {
    const T* p; int nr;
    __device__ __forceinline__ T operator()(int i, int k) const { return p[i + (long)nr * k]; }
};
template <typename T>
struct CellA {
    const T* p; int nr;
    __device__ __forceinline__ T operator()(int i, int k) const { return p[cidx(nr, i, k)]; }
};

// Block-level accumulation of up to two dot products into the partials buffer.
template <int NT>
__device__ __forceinline__ void emit_partials(double a1, double a2, int n1, int n2, const Dots& d, int slot1) {
    __shared__ double sm[32];
    if (n1) {
        double r = block_sum<NT>(a1, sm);
        if (threadIdx.x == 0) d.part[slot1 * DRD_MAXB + blockIdx.x] = r;
    }
    if (n2) {
        double r = block_sum<NT>(a2, sm);
        if (threadIdx.x == 0) d.part[(slot1 + 1) * DRD_MAXB + blockIdx.x] = r;
    }
}

// ======================================================================================
// CH (microfluidics_complex_domain/PhSolve.f90)
// ======================================================================================

// f2 = ph - dt u.grad(ph) (:26-34) on the whole CELL array (ghosts keep ph).
__global__ void k_ch_f2(DevParams P, const double* __restrict__ u, const double* __restrict__ v,
                        const double* __restrict__ ph, double* __restrict__ f2, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long cs = (long)(nr + 2) * (nz + 2);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        double val = ph[q];
        if (i >= 0 && i < nr && k >= 0 && k < nz) {
            val = val - P.dt * (u[uidx(nr, i + 1, k)] + u[uidx(nr, i, k)]) / 2.0 *
                            (ph[cidx(nr, i + 1, k)] - ph[cidx(nr, i - 1, k)]) / 2.0 / P.dr -
                  P.dt * (v[vidx(nr, i, k + 1)] + v[vidx(nr, i, k)]) / 2.0 *
                      (ph[cidx(nr, i, k + 1)] - ph[cidx(nr, i, k - 1)]) / 2.0 / P.dz;
        }
        f2[q] = val;
    }
}

// ch_bulk_energy (microfluidics_complex_domain/ch_bulk_energy.f90:20-22).
__device__ __forceinline__ double bulk_mf(double phi, double psi) {
    double aa = (phi * phi) * ((1.0 - phi) * (1.0 - phi));
    aa = 1.0 - sqrt(aa / (aa + 1.0E-2)) * psi;
    return 0.5 * phi * (1.0 - phi) * (1.0 - 2.0 * phi) * aa;
}

// rhs = -f1 + s f2/eps - eps L_Mi(f2) (:37-48) packed by Atob; x0 = Atob(rmu) (:62-63).
// With rmu_pre non-NULL the guess is extrapolated: 2 rmu - rmu_pre; with rmu_pre2 too,
// quadratically: 3 rmu - 3 rmu_pre + rmu_pre2; with rmu_pre3, cubically.
__global__ void k_ch_rhs(DevParams P, const double* __restrict__ ph, const double* __restrict__ rmu,
                         const double* __restrict__ rmu_pre, const double* __restrict__ rmu_pre2,
                         const double* __restrict__ rmu_pre3, const double* __restrict__ bdr,
                         const double* __restrict__ grad, const double* __restrict__ Mi,
                         const double* __restrict__ f2, double* __restrict__ b, double* __restrict__ x, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long n = (long)nr * nz;
    CellA<double> F{f2, nr}, M{Mi, nr};
    const double sq2 = sqrt(2.0);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const long c = cidx(nr, i, k);
        const double p0 = ph[c];
        double f1 = P.s * p0 / P.eps - bulk_mf(p0, bdr[c]) / P.eps - p0 * (p0 - 1.0) * grad[c] * P.cang / sq2;
        const double ff = op_dgn<double>(i, k, nr, nz, P.idr2, P.idz2, F, M);
        b[q] = -f1 + P.s * f2[c] / P.eps - P.eps * ff;
        x[q] = rmu_pre3   ? 4.0 * (rmu[c] + rmu_pre2[c]) - 6.0 * rmu_pre[c] - rmu_pre3[c]
               : rmu_pre2 ? 3.0 * (rmu[c] - rmu_pre[c]) + rmu_pre2[c]
               : rmu_pre  ? 2.0 * rmu[c] - rmu_pre[c]
                          : rmu[c];
    }
}

// MATRIX_VECTOR_CG (:240-292), first half: ff1 = -(dt xld) L_M0(x).
template <typename T>
__global__ void k_ch_mv1(OpScal<T> o, const T* __restrict__ M0, const T* __restrict__ x, T* __restrict__ ff1,
                         const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz;
    const long n = (long)nr * nz;
    PackedA<T> X{x, nr};
    CellA<T> M{M0, nr};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        ff1[q] = -(o.dtxld * op_dgn<T>(i, k, nr, nz, o.idr2, o.idz2, X, M));
    }
}

// Second half: y = alpha (x + s ff1/eps - eps L_Mi(ff1)) + beta y, with optional partial dots.
template <typename T>
__global__ void k_ch_mv2(OpScal<T> o, const T* __restrict__ Mi, const T* __restrict__ x, const T* __restrict__ ff1,
                         T alpha, T beta, T* y, const T* dot1, int self2, Dots d, int slot1, const KState* ks,
                         int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz;
    const long n = (long)nr * nz;
    PackedA<T> F{ff1, nr};
    CellA<T> M{Mi, nr};
    double a1 = 0.0, a2 = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const T f = ff1[q];
        const T a = o.s * f / o.eps - o.eps * op_dgn<T>(i, k, nr, nz, o.idr2, o.idz2, F, M);
        const T av = x[q] + a;
        const T yn = (beta == T(0)) ? alpha * av : alpha * av + beta * y[q];
        y[q] = yn;
        if (dot1) a1 += (double)dot1[q] * (double)yn;
        if (self2) a2 += (double)yn * (double)yn;
    }
    if (dot1 != nullptr || self2) emit_partials<DRD_TPB>(a1, a2, dot1 != nullptr, self2, d, slot1);
}

// The FP32 CH operator in one pass over 64 x 8 cell tiles (the mixed mode's inner operator):
// x and M0 for the tile with a halo of two cells, Mi with a halo of one, staged in shared
// memory; ff1 = -(dt xld) L_M0(x) on the tile and its one-cell halo into shared memory; then
// y = alpha (x + s ff1/eps - eps L_Mi(ff1)) + beta y on the tile, with the same op_dgn
// expressions as k_ch_mv1 / k_ch_mv2 (read through shared-memory accessors), so y is the same
// bit for bit; ff1 never goes to global memory.  Blocks loop over the tiles; each block emits one
// partial per dot product.
constexpr int kChTX = 64, kChTY = 8;
constexpr int kChXW = kChTX + 4, kChXH = kChTY + 4;  // x, M0: tile + 2
constexpr int kChFW = kChTX + 2, kChFH = kChTY + 2;  // ff1, Mi: tile + 1
struct ChSm {  // a shared-memory rectangle of a field addressed by global cell (i, k)
    const float* p; int i0, k0, w;
    __device__ __forceinline__ float operator()(int i, int k) const { return p[(k - k0) * w + (i - i0)]; }
};
__global__ void __launch_bounds__(DRD_TPB) k_ch_mv_tile(OpScal<float> o, const float* __restrict__ M0,
                                                        const float* __restrict__ Mi, const float* __restrict__ x,
                                                        float alpha, float beta, float* y, const float* dot1, int self2,
                                                        Dots d, int slot1, const KState* ks, int gate, ull* ctr) {
    __shared__ float sx[kChXH * kChXW], sm0[kChXH * kChXW], smi[kChFH * kChFW], sf[kChFH * kChFW];
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz, tid = threadIdx.x;
    const int tx = (nr + kChTX - 1) / kChTX, ntiles = tx * ((nz + kChTY - 1) / kChTY);
    double a1 = 0.0, a2 = 0.0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i0 = (tile % tx) * kChTX, k0 = (tile / tx) * kChTY;
        // stage (cells outside the domain are never read by op_dgn: 0)
        for (int e = tid; e < kChXH * kChXW; e += DRD_TPB) {
            const int i = i0 - 2 + e % kChXW, k = k0 - 2 + e / kChXW;
            const bool in = i >= 0 && i < nr && k >= 0 && k < nz;
            sx[e] = in ? x[i + (long)nr * k] : 0.f;
            sm0[e] = in ? M0[cidx(nr, i, k)] : 0.f;
        }
        for (int e = tid; e < kChFH * kChFW; e += DRD_TPB) {
            const int i = i0 - 1 + e % kChFW, k = k0 - 1 + e / kChFW;
            smi[e] = (i >= 0 && i < nr && k >= 0 && k < nz) ? Mi[cidx(nr, i, k)] : 0.f;
        }
        __syncthreads();
        const ChSm X{sx, i0 - 2, k0 - 2, kChXW}, M{sm0, i0 - 2, k0 - 2, kChXW};
        for (int e = tid; e < kChFH * kChFW; e += DRD_TPB) {
            const int i = i0 - 1 + e % kChFW, k = k0 - 1 + e / kChFW;
            sf[e] = (i >= 0 && i < nr && k >= 0 && k < nz)
                        ? -(o.dtxld * op_dgn<float>(i, k, nr, nz, o.idr2, o.idz2, X, M))
                        : 0.f;
        }
        __syncthreads();
        const ChSm F{sf, i0 - 1, k0 - 1, kChFW}, MI{smi, i0 - 1, k0 - 1, kChFW};
        for (int e = tid; e < kChTX * kChTY; e += DRD_TPB) {
            const int i = i0 + e % kChTX, k = k0 + e / kChTX;
            if (i >= nr || k >= nz) continue;
            const long q = i + (long)nr * k;
            const float f = F(i, k);
            const float a = o.s * f / o.eps - o.eps * op_dgn<float>(i, k, nr, nz, o.idr2, o.idz2, F, MI);
            const float av = X(i, k) + a;
            const float yn = (beta == 0.f) ? alpha * av : alpha * av + beta * y[q];
            y[q] = yn;
            if (dot1) a1 += (double)dot1[q] * (double)yn;
            if (self2) a2 += (double)yn * (double)yn;
        }
        __syncthreads();
    }
    if (dot1 != nullptr || self2) emit_partials<DRD_TPB>(a1, a2, dot1 != nullptr, self2, d, slot1);
}

// rmu_after interior (:85) and ph_after = f2 + dt xld L_M0(rmu_after) interior (:100-101).
__global__ void k_ch_fin(DevParams P, const double* __restrict__ x, const double* __restrict__ f2,
                         const double* __restrict__ M0, double* __restrict__ rmu_after, double* __restrict__ ph_after,
                         ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long n = (long)nr * nz;
    PackedA<double> X{x, nr};
    CellA<double> M{M0, nr};
    const double dtxld = P.dt * P.xld;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const long c = cidx(nr, i, k);
        rmu_after[c] = x[q];
        ph_after[c] = f2[c] + dtxld * op_dgn<double>(i, k, nr, nz, P.idr2, P.idz2, X, M);
    }
}

// ======================================================================================
// PhSolve_ori (microfluidics_complex_domain/PhSolve_ori.f90): phi in [-1,1], unit mobility,
// wall-energy rows at k = 0 and nz-1; finit repeats it to smooth the wall indicator.  Neumann
// left/right (laplace_nn, :463-487) and the non-dynamic wall branch (:71-78, :110-118).
// ======================================================================================

// laplace_nn at (i,k) of a field read through `a` with Neumann ghosts (clamped neighbours).
// FP64: the reference's (a+ + a- - 2 a0)/h^2; FP32: ((a+ - a0) - (a0 - a-))/h^2.
template <typename T, class A>
__device__ __forceinline__ T lap_nn(int i, int k, int nr, int nz, T dr2, T dz2, const A& a) {
    const T a0 = a(i, k);
    const T xl = a(i > 0 ? i - 1 : 0, k), xr = a(i < nr - 1 ? i + 1 : nr - 1, k);
    const T zl = a(i, k > 0 ? k - 1 : 0), zr = a(i, k < nz - 1 ? k + 1 : nz - 1);
    if constexpr (sizeof(T) == 4) return ((xr - a0) - (a0 - xl)) / dr2 + ((zr - a0) - (a0 - zl)) / dz2;
    return (xr + xl - 2 * a0) / dr2 + (zr + zl - 2 * a0) / dz2;
}

// pnb(i) / pnt(i) of the non-dynamic wall branch: (cf cos(tmp pi/2) + alpha_s tmp) / tmp1,
// tmp the wall-face mean of ph (:44-49, :71-78; :84-89, :110-118).
__device__ __forceinline__ double ori_wall(double cf, double p_in, double p_gh, double alpha_s, double tmp1) {
    const double tmp = (p_gh + p_in) / 2.0;
    double pn = cf * cos(tmp * 3.14159265358979323846264338327950288 / 2) + alpha_s * tmp;
    return pn / tmp1;
}

struct OriF1 {  // f1 of :35-39 plus the wall rows, read with Neumann ghosts
    const double* ph; const double* cfb; const double* cft; int nr, nz; double s, eps, dz2, alpha_s, tmp1;
    __device__ __forceinline__ double operator()(int i, int k) const {
        const double p0 = ph[cidx(nr, i, k)];
        double f = ((1. + s) * p0 - p0 * p0 * p0) / eps;
        if (k == 0) f = f + ori_wall(cfb[i], p0, ph[cidx(nr, i, -1)], alpha_s, tmp1) * eps / dz2;
        if (k == nz - 1) f = f + ori_wall(cft[i], p0, ph[cidx(nr, i, nz)], alpha_s, tmp1) * eps / dz2;
        return f;
    }
};

// rhs = Atob(f2 - dt xld laplace_nn(f1)) and x0 = Atob(ph) (:126-138); pnb / pnt stored for
// the ghost rows of the result.
__global__ void k_ori_rhs(DevParams P, const double* __restrict__ ph, const double* __restrict__ f2,
                          const double* __restrict__ cfb, const double* __restrict__ cft, double alpha_s,
                          double* __restrict__ b, double* __restrict__ x, double* __restrict__ pnb,
                          double* __restrict__ pnt, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long n = (long)nr * nz;
    const double tmp1 = P.eps / P.dz + 0.5 * alpha_s;
    const OriF1 F{ph, cfb, cft, nr, nz, P.s, P.eps, P.dz2, alpha_s, tmp1};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const long c = cidx(nr, i, k);
        const double ff = lap_nn<double>(i, k, nr, nz, P.dr2, P.dz2, F);
        b[q] = f2[c] - P.dt * P.xld * ff;
        x[q] = ph[c];
        if (k == 0) pnb[i] = ori_wall(cfb[i], ph[c], ph[cidx(nr, i, -1)], alpha_s, tmp1);
        if (k == nz - 1) pnt[i] = ori_wall(cft[i], ph[c], ph[cidx(nr, i, nz)], alpha_s, tmp1);
    }
}

// MATRIX_VECTOR_CG_ori (:368-421), first half: ff1 = -eps laplace_nn(x) + wall rows + s x/eps.
template <typename T>
__global__ void k_ori_mv1(OpScal<T> o, const T* __restrict__ x, T* __restrict__ ff1, const KState* ks, int gate,
                          ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz;
    const long n = (long)nr * nz;
    PackedA<T> X{x, nr};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const T x0 = x[q];
        T f = -o.eps * lap_nn<T>(i, k, nr, nz, o.dr2, o.dz2, X);
        if (k == 0) f = f + o.eps / o.dz2 * (x0 - o.cb * x0);       // the ghost equals x(i,0) here
        if (k == nz - 1) f = f + o.eps / o.dz2 * (x0 - o.ct * x0);
        ff1[q] = f + x0 * o.s / o.eps;
    }
}

// Second half: y = alpha (x - dt xld laplace_nn(ff1)) + beta y, with optional partial dots.
template <typename T>
__global__ void k_ori_mv2(OpScal<T> o, const T* __restrict__ x, const T* __restrict__ ff1, T alpha, T beta, T* y,
                          const T* dot1, int self2, Dots d, int slot1, const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz;
    const long n = (long)nr * nz;
    PackedA<T> F{ff1, nr};
    double a1 = 0.0, a2 = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const T ff2 = -(o.dtxld * lap_nn<T>(i, k, nr, nz, o.dr2, o.dz2, F));
        const T av = x[q] + ff2;
        const T yn = (beta == T(0)) ? alpha * av : alpha * av + beta * y[q];
        y[q] = yn;
        if (dot1) a1 += (double)dot1[q] * (double)yn;
        if (self2) a2 += (double)yn * (double)yn;
    }
    if (dot1 != nullptr || self2) emit_partials<DRD_TPB>(a1, a2, dot1 != nullptr, self2, d, slot1);
}

// ph_after with its ghost rows (:156-173) and rmu_after (:178-201) on the whole CELL array.
struct OriPh {
    const double* x; const double* pnb; const double* pnt; int nr, nz; double cb, ct;
    __device__ __forceinline__ double operator()(int i, int k) const {
        i = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);  // left/right ghost columns copy columns 0 / nr-1
        if (k < 0) return x[i] * cb + pnb[i];
        if (k > nz - 1) return x[i + (long)nr * (nz - 1)] * ct + pnt[i];
        return x[i + (long)nr * k];
    }
};
__global__ void k_ori_fin(DevParams P, const double* __restrict__ x, const double* __restrict__ pnb,
                          const double* __restrict__ pnt, double cb, double ct, double* __restrict__ ph_after,
                          double* __restrict__ rmu_after, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long cs = (long)(nr + 2) * (nz + 2);
    const OriPh A{x, pnb, pnt, nr, nz, cb, ct};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        ph_after[q] = A(i, k);
        const int si = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
        const int sk = k < 0 ? 0 : (k > nz - 1 ? nz - 1 : k);
        const double p0 = A(si, sk);
        rmu_after[q] = -P.eps * ((A(si + 1, sk) + A(si - 1, sk) - 2 * p0) / P.dr2 +
                                 (A(si, sk + 1) + A(si, sk - 1) - 2 * p0) / P.dz2) -
                       p0 / P.eps + p0 * p0 * p0 / P.eps;
    }
}

// finit.f90:163-169: rmu from ph and its ghosts on the interior (ghosts left as they are).
__global__ void k_ori_rmu0(DevParams P, const double* __restrict__ ph, double* __restrict__ rmu, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long n = (long)nr * nz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const double p0 = ph[cidx(nr, i, k)];
        rmu[cidx(nr, i, k)] = -P.eps * ((ph[cidx(nr, i + 1, k)] + ph[cidx(nr, i - 1, k)] - 2 * p0) / P.dr2 +
                                        (ph[cidx(nr, i, k + 1)] + ph[cidx(nr, i, k - 1)] - 2 * p0) / P.dz2) -
                              p0 / P.eps + p0 * p0 * p0 / P.eps;
    }
}

// finit.f90:178-189: bdr_ph = (ph + 1)/2 everywhere, clipped to [0, 1] on the interior.
__global__ void k_ori_bdr(int nr, int nz, const double* __restrict__ ph, double* __restrict__ bdr, ull* ctr) {
    count_launch(ctr);
    const long cs = (long)(nr + 2) * (nz + 2);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        double b = (ph[q] + 1.0) / 2.0;
        if (i >= 0 && i < nr && k >= 0 && k < nz) {
            if (b >= 1.0) b = 1.0;
            else if (b <= 0.0) b = 0.0;
        }
        bdr[q] = b;
    }
}

// ======================================================================================
// ESOLP_x tridiagonal stage (Precipitation_dynamics/ESOLP.f90:23-41 with rfords): for every
// x mode k of a block of `rows` rows of `len` values (row j, mode k at w[k + len*j]), solve
// the tridiagonal system along j in place.  The elimination multipliers r_j = -a_j/b'_{j-1}
// and the pivots b'_j depend only on the coefficients and come precomputed, like c_j, at
// [k + len*j]: thread k's loads are coalesced across the warp.  The two blocks of a momentum
// vector (u, then v) are one launch.  The sweep is a chain of dependent steps, so each thread
// loads TRI_CH rows ahead before it runs the chain through them.
// ======================================================================================
constexpr int TRI_CH = 16;
template <typename T>
__global__ void k_tridiag(TriBlock<T> b0, TriBlock<T> b1, const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool second = k >= b0.len;
    const TriBlock<T>& B = second ? b1 : b0;
    if (second) k -= b0.len;
    if (k >= B.len) return;
    const long L = B.len;
    T* __restrict__ w = B.w + k;
    const T* __restrict__ rm = B.rm + k;
    const T* __restrict__ bp = B.bp + k;
    const T* __restrict__ cc = B.cc + k;
    const int R = B.rows;
    // forward elimination f_j = f_j + r_j f_{j-1} (f_0 = w_0)
    T f = T(0);
    for (int j0 = 0; j0 < R; j0 += TRI_CH) {
        T wv[TRI_CH], rv[TRI_CH];
#pragma unroll
        for (int q = 0; q < TRI_CH; ++q)
            if (j0 + q < R) { wv[q] = w[L * (j0 + q)]; rv[q] = rm[L * (j0 + q)]; }
#pragma unroll
        for (int q = 0; q < TRI_CH; ++q)
            if (j0 + q < R) {
                f = (j0 + q == 0) ? wv[q] : wv[q] + rv[q] * f;
                w[L * (j0 + q)] = f;
            }
    }
    // back substitution ff_{R-1} = f/b' (0 when |b'| <= 1e-12), ff_j = (f_j - c_j ff_{j+1}) / b'_j
    const T bl = bp[L * (R - 1)];
    T nxt = (fabs((double)bl) <= 1.0E-12) ? T(0) : f / bl;
    w[L * (R - 1)] = nxt;
    for (int j1 = R - 2; j1 >= 0; j1 -= TRI_CH) {
        T fv[TRI_CH], cv[TRI_CH], bv[TRI_CH];
#pragma unroll
        for (int q = 0; q < TRI_CH; ++q)
            if (j1 - q >= 0) { fv[q] = w[L * (j1 - q)]; cv[q] = cc[L * (j1 - q)]; bv[q] = bp[L * (j1 - q)]; }
#pragma unroll
        for (int q = 0; q < TRI_CH; ++q)
            if (j1 - q >= 0) {
                nxt = (fv[q] - cv[q] * nxt) / bv[q];
                w[L * (j1 - q)] = nxt;
            }
    }
}

// Neumann ghost copies of CELL fields: the ghost takes the nearest interior value, which is
// the net effect of the reference's two loops (e.g. PhSolve.f90:88-96, dct_fftw.f90:41-51).
__global__ void k_fill_neumann(int nr, int nz, double* a, double* b, ull* ctr) {
    count_launch(ctr);
    const long ng = 2L * (nr + 2) + 2L * nz;
    for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < ng; g += (long)gridDim.x * blockDim.x) {
        int i, k;
        if (g < nr + 2) { i = (int)g - 1; k = -1; }
        else if (g < 2L * (nr + 2)) { i = (int)(g - (nr + 2)) - 1; k = nz; }
        else {
            const long h = g - 2L * (nr + 2);
            k = (int)(h >> 1);
            i = (h & 1) ? nr : -1;
        }
        const int si = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
        const int sk = k < 0 ? 0 : (k > nz - 1 ? nz - 1 : k);
        const long dst = cidx(nr, i, k), src = cidx(nr, si, sk);
        a[dst] = a[src];
        if (b) b[dst] = b[src];
    }
}

// ======================================================================================
// Coupled CH (two_phase_flow_complex_domain/ph_mu_solve.f90)
// ======================================================================================

// M0 = (1-bdr) W(ph) (:31-35) and f2 = ph (used + adjust) - dt u.grad(ph used) (:40-51).
__global__ void k_phmu_prep(DevParams P, const double* __restrict__ u, const double* __restrict__ v,
                            const double* __restrict__ ph, const double* __restrict__ bdr,
                            const double* __restrict__ used, double* __restrict__ M0, double* __restrict__ f2,
                            ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long cs = (long)(nr + 2) * (nz + 2);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        const double p0 = ph[q];
        if (P.phi_mode == 1) M0[q] = (1.0 - bdr[q]) * (p0 * p0) * ((p0 - 1.0) * (p0 - 1.0));
        else M0[q] = (1.0 - bdr[q]) * ((p0 * p0 - 1.0) * (p0 * p0 - 1.0));
        double val = p0 * (used[q] + P.adjust);
        if (i >= 0 && i < nr && k >= 0 && k < nz) {
            val = val -
                  P.dt * (u[uidx(nr, i + 1, k)] + u[uidx(nr, i, k)]) / 2.0 *
                      (ph[cidx(nr, i + 1, k)] * used[cidx(nr, i + 1, k)] - ph[cidx(nr, i - 1, k)] * used[cidx(nr, i - 1, k)]) /
                      2.0 / P.dr -
                  P.dt * (v[vidx(nr, i, k + 1)] + v[vidx(nr, i, k)]) / 2.0 *
                      (ph[cidx(nr, i, k + 1)] * used[cidx(nr, i, k + 1)] - ph[cidx(nr, i, k - 1)] * used[cidx(nr, i, k - 1)]) /
                      2.0 / P.dz;
        }
        f2[q] = val;
    }
}

// ch_bulk_energy (two_phase_flow_complex_domain/ch_bulk_energy.f90:39-58).
__device__ __forceinline__ double bulk_tp(double phi, double psi, int mode) {
    if (mode == 1) return 0.5 * phi * (1.0 - phi) * (1.0 - 2.0 * phi) * (1 - psi);
    return (phi * phi * phi - phi) * (1 - psi);
}

// rhs [f1; f2] (:55-153) with the wall terms of ch_bdr_condition (:108-149); cfB/cfT hold
// cos(angle pi/180)/sqrt(2) per column.
__global__ void k_phmu_rhs(DevParams P, const double* __restrict__ ph, const double* __restrict__ rmu,
                           const double* __restrict__ ph_pre, const double* __restrict__ rmu_pre,
                           const double* __restrict__ bdr, const double* __restrict__ grad,
                           const double* __restrict__ f2, const double* __restrict__ cfB,
                           const double* __restrict__ cfT, double* __restrict__ b, double* __restrict__ x,
                           double* __restrict__ pnb, double* __restrict__ pnt, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz, mode = P.phi_mode;
    const long n = (long)nr * nz;
    const double sq2 = sqrt(2.0);
    const double tmp = P.eps / P.dz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const long c = cidx(nr, i, k);
        const double p0 = ph[c];
        const double wet = (mode == 1) ? p0 * (p0 - 1.0) : (p0 * p0 - 1.0);
        double f1 = P.s * p0 / P.eps - bulk_tp(p0, bdr[c], mode) / P.eps - wet * grad[c] * P.cang / sq2;
        if (k == 0) {
            const double pb = (ph[cidx(nr, i, -1)] + ph[cidx(nr, i, 0)]) / 2.0;
            double val = (mode == 1) ? cfB[i] * (1.0 - pb) * pb : cfB[i] * (1.0 - pb * pb);
            val = val / tmp;
            pnb[i] = val;
            f1 = f1 + val * P.eps / P.dz2;
        }
        if (k == nz - 1) {
            const double pt = (ph[cidx(nr, i, nz - 1)] + ph[cidx(nr, i, nz)]) / 2.0;
            double val = (mode == 1) ? cfT[i] * (1.0 - pt) * pt : cfT[i] * (1.0 - pt * pt);
            val = val / tmp;
            pnt[i] = val;
            f1 = f1 + val * P.eps / P.dz2;
        }
        b[q] = f1;
        b[q + n] = f2[c];
        x[q] = ph_pre ? 2.0 * p0 - ph_pre[c] : p0;
        x[q + n] = rmu_pre ? 2.0 * rmu[c] - rmu_pre[c] : rmu[c];
    }
}

// MATRIX_VECTOR_PH_MU_CG (:203-299).  The ghost rows of phi are the Neumann copies of
// btoA_ph_mu (matrix_tool.f90:120-126).
template <typename T>
__global__ void k_phmu_mv(OpScal<T> o, const T* __restrict__ M0, const T* __restrict__ Mi,
                          const T* __restrict__ used, const T* __restrict__ x, T alpha, T beta, T* y, const T* dot1,
                          int self2, Dots d, int slot1, const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz;
    const long n = (long)nr * nz;
    PackedA<T> F1{x, nr}, F2{x + n, nr};
    CellA<T> MI{Mi, nr}, MO{M0, nr};
    const T epsdz2 = o.eps / o.dz2;
    double a1 = 0.0, a2 = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < 2 * n; q += (long)gridDim.x * blockDim.x) {
        const long qq = q < n ? q : q - n;
        const int i = (int)(qq % nr), k = (int)(qq / nr);
        const long c = cidx(nr, i, k);
        T val;
        if (q < n) {
            const T f1 = x[qq];
            val = o.s * f1 / o.eps - o.eps * op_dgn<T>(i, k, nr, nz, o.idr2, o.idz2, F1, MI) - x[qq + n] * used[c];
            if (k == 0) val = val + epsdz2 * (f1 - o.cb * f1);
            if (k == nz - 1) val = val + epsdz2 * (f1 - o.ct * f1);
        } else {
            val = x[qq] * (used[c] + o.adjust) - o.dtxld * op_dgn<T>(i, k, nr, nz, o.idr2, o.idz2, F2, MO);
        }
        const T yn = (beta == T(0)) ? alpha * val : alpha * val + beta * y[q];
        y[q] = yn;
        if (dot1) a1 += (double)dot1[q] * (double)yn;
        if (self2) a2 += (double)yn * (double)yn;
    }
    if (dot1 != nullptr || self2) emit_partials<DRD_TPB>(a1, a2, dot1 != nullptr, self2, d, slot1);
}

// Diagonal of PSolve_PH_MU_CG (:321-353) with its index tests exactly as written there.
template <typename T>
__global__ void k_phmu_diag(OpScal<T> o, T* __restrict__ diag, ull* ctr) {
    count_launch(ctr);
    const int nr = o.nr, nz = o.nz;
    const long n = (long)nr * nz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), j = (int)(q / nr);
        const T tmpx = (i == 0 || j == nr - 1) ? T(1) / o.dr2 : T(2) / o.dr2;
        const T tmpz = (i == 0 || j == nz - 1) ? T(1) / o.dz2 : T(2) / o.dz2;
        diag[q] = (tmpx + tmpz) * o.eps + o.s / o.eps;
        diag[q + n] = o.dtxld * (tmpx + tmpz);
    }
}

// btoA_ph_mu + ghost rows of phi (:173-177).
__global__ void k_phmu_fin(DevParams P, const double* __restrict__ x, const double* __restrict__ pnb,
                           const double* __restrict__ pnt, double cb, double ct, double* __restrict__ ph_after,
                           double* __restrict__ rmu_after, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long n = (long)nr * nz;
    const long cs = (long)(nr + 2) * (nz + 2);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        const int si = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
        const int sk = k < 0 ? 0 : (k > nz - 1 ? nz - 1 : k);
        const long s = si + (long)nr * sk;
        double pv = x[s];
        if (i >= 0 && i < nr && k == -1) pv = x[i] * cb + pnb[i];
        if (i >= 0 && i < nr && k == nz) pv = x[i + (long)nr * (nz - 1)] * ct + pnt[i];
        ph_after[q] = pv;
        rmu_after[q] = x[s + n];
    }
}

// ======================================================================================
// Momentum (microfluidics_complex_domain/VeloSolve_2_combined.f90, VeloSolve_combined.f90,
// two_phase_flow_complex_domain/VeloSolve_2_combined.f90)
// ======================================================================================

// RHS fu/fv (:62-295, :377-385) packed by Atob_uv (:388-389); x0 = Atob_uv(u, v).
__global__ void k_uv_rhs(DevParams P, int bdf, const CallArgs* __restrict__ ca, const double* __restrict__ psi1,
                         const double* __restrict__ psi2, const double* __restrict__ u_pre,
                         const double* __restrict__ u, const double* __restrict__ v_pre,
                         const double* __restrict__ v, const double* __restrict__ p, const double* __restrict__ rho,
                         const double* __restrict__ eta, const double* __restrict__ bdr,
                         const double* __restrict__ used, const double* __restrict__ ph,
                         const double* __restrict__ rmu, const double* __restrict__ pf1,
                         const double* __restrict__ pf2, double* __restrict__ b, double* __restrict__ x,
                         double* __restrict__ uL, int extrap, const double* __restrict__ u_pre2,
                         const double* __restrict__ v_pre2, const double* __restrict__ u_pre3,
                         const double* __restrict__ v_pre3, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long mn = (long)(nr + 1) * nz, N = mn + (long)nr * (nz - 1);
    const bool tp = P.variant == DRD_VARIANT_TP;
    const bool dirichlet = !(tp && P.lr_neumann);
    const double dr = P.dr, dz = P.dz, dt = P.dt, re = P.re, ca_ = P.ca;
    const double cf = ca->cf;
#define UT(i, k) (bdf == 2 ? 2.0 * u[uidx(nr, i, k)] - u_pre[uidx(nr, i, k)] : u[uidx(nr, i, k)])
#define VT(i, k) (bdf == 2 ? 2.0 * v[vidx(nr, i, k)] - v_pre[vidx(nr, i, k)] : v[vidx(nr, i, k)])
#define TPR(i, k) (bdf == 2 ? p[cidx(nr, i, k)] + 4 * psi2[cidx(nr, i, k)] / 3.0 - psi1[cidx(nr, i, k)] / 3.0 : p[cidx(nr, i, k)])
#define C_(a, i, k) a[cidx(nr, i, k)]
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        if (q < mn) {
            const int i = (int)(q % (nr + 1)), k = (int)(q / (nr + 1));
            double fu;
            if (!tp)
                fu = ca_ * (C_(rmu, i, k) + C_(rmu, i - 1, k)) / 2.0 * (C_(ph, i, k) - C_(ph, i - 1, k)) / dr *
                     (1.0 - (C_(bdr, i, k) + C_(bdr, i - 1, k)) / 2.0);
            else
                fu = ca_ * (C_(rmu, i, k) + C_(rmu, i - 1, k)) / 2.0 *
                     (C_(ph, i, k) * C_(used, i, k) - C_(ph, i - 1, k) * C_(used, i - 1, k)) / dr;
            fu = fu - re * (C_(rho, i, k) + C_(rho, i - 1, k)) / 2.0 *
                          (UT(i, k) * (UT(i + 1, k) - UT(i - 1, k)) / 2.0 / dr +
                           (VT(i, k) + VT(i - 1, k) + VT(i, k + 1) + VT(i - 1, k + 1)) / 4.0 * (UT(i, k + 1) - UT(i, k - 1)) / 2.0 / dz);
            const double g = (tp && bdf == 2) ? (C_(ph, i, k) + C_(ph, i - 1, k)) / 2.0 * P.ggx : P.ggx;
            const double uu = u[uidx(nr, i, k)];
            const double mass = (bdf == 2) ? 2.0 * uu * re / dt - u_pre[uidx(nr, i, k)] * re / 2.0 / dt + g : uu * re / dt + g;
            fu = fu - (TPR(i, k) - TPR(i - 1, k)) / dr + (C_(rho, i, k) + C_(rho, i - 1, k)) / 2.0 * mass;
            fu = fu + (C_(pf1, i, k) + C_(pf1, i - 1, k)) / 2.0;
            fu = fu * dt;
            if (dirichlet && (i == 0 || i == nr)) {
                const double hig = P.bdr_upp - P.bdr_low;
                const double z = (k + 0.5) * dz;
                double ul = 0.0;
                if (z > P.bdr_low && z < P.bdr_upp) {
                    const double dd = z - P.bdr_low - hig / 2;
                    ul = P.UU * (-(dd * dd) / hig / hig * 4 + 1) * cf;
                }
                if (i == 0 && uL != nullptr) uL[k] = ul;
                fu = fu + 2.0 * ul * C_(eta, i, k) * 2.0 * dt / P.dr2;
            }
            if (k == 0) {
                const double etay = (C_(eta, i, k) + C_(eta, i - 1, k) + C_(eta, i, k - 1) + C_(eta, i - 1, k - 1)) / 4.0;
                fu = fu + dt * (2.0 * P.uwB / P.dz2 * etay);
            }
            if (k == nz - 1) {
                const double etay = (C_(eta, i, k + 1) + C_(eta, i - 1, k + 1) + C_(eta, i, k) + C_(eta, i - 1, k)) / 4.0;
                fu = fu + dt * (2.0 * P.uwT / P.dz2 * etay);
            }
            b[q] = fu;
            const long ui = uidx(nr, i, k);
            x[q] = extrap == 3 ? 4.0 * (uu + u_pre2[ui]) - 6.0 * u_pre[ui] - u_pre3[ui]
                   : extrap == 2 ? 3.0 * (uu - u_pre[ui]) + u_pre2[ui]
                   : extrap ? 2.0 * uu - u_pre[ui] : uu;
        } else {
            const long qv = q - mn;
            const int i = (int)(qv % nr), k = (int)(qv / nr) + 1;
            double fv;
            if (!tp)
                fv = ca_ * (C_(rmu, i, k) + C_(rmu, i, k - 1)) / 2.0 * (C_(ph, i, k) - C_(ph, i, k - 1)) / dz *
                     (1.0 - (C_(bdr, i, k) + C_(bdr, i, k - 1)) / 2.0);
            else
                fv = ca_ * (C_(rmu, i, k) + C_(rmu, i, k - 1)) / 2.0 *
                     (C_(ph, i, k) * C_(used, i, k) - C_(ph, i, k - 1) * C_(used, i, k - 1)) / dz;
            fv = fv - re * (C_(rho, i, k) + C_(rho, i, k - 1)) / 2.0 *
                          ((UT(i, k) + UT(i + 1, k) + UT(i, k - 1) + UT(i + 1, k - 1)) / 4.0 * (VT(i + 1, k) - VT(i - 1, k)) / 2.0 / dr +
                           VT(i, k) * (VT(i, k + 1) - VT(i, k - 1)) / 2.0 / dz);
            const double g = (tp && bdf == 2) ? (C_(ph, i, k) + C_(ph, i - 1, k)) / 2.0 * P.ggz : P.ggz;
            const double vv = v[vidx(nr, i, k)];
            const double mass = (bdf == 2) ? 2.0 * vv * re / dt - v_pre[vidx(nr, i, k)] * re / 2.0 / dt + g : vv * re / dt + g;
            fv = fv - (TPR(i, k) - TPR(i, k - 1)) / dz + (C_(rho, i, k) + C_(rho, i, k - 1)) / 2.0 * mass;
            fv = fv + (C_(pf2, i, k) + C_(pf2, i, k - 1)) / 2.0;
            fv = fv * dt;
            b[q] = fv;
            const long vi = vidx(nr, i, k);
            x[q] = extrap == 3 ? 4.0 * (vv + v_pre2[vi]) - 6.0 * v_pre[vi] - v_pre3[vi]
                   : extrap == 2 ? 3.0 * (vv - v_pre[vi]) + v_pre2[vi]
                   : extrap ? 2.0 * vv - v_pre[vi] : vv;
        }
    }
#undef UT
#undef VT
#undef TPR
#undef C_
}

// MatrixVector_uv_2_CG (:515-646) / MatrixVector_uv_CG: y = alpha A x + beta y.
template <typename T>
__global__ void k_uv_mv(OpScal<T> o, const T* __restrict__ rho, const T* __restrict__ eta,
                        const T* __restrict__ pen, const T* __restrict__ x, T alpha, T beta, T* y, const T* dot1,
                        int self2, Dots d, int slot1, const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    const int nr = o.nr, nz = o.nz;
    const long mn = (long)(nr + 1) * nz, N = mn + (long)nr * (nz - 1);
    UVFetch<T> F{x, nr, nz, mn, o.lr_neumann};
    double a1 = 0.0, a2 = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const T val = uv_apply<T>(o, rho, eta, pen, F, q);
        const T yn = (beta == T(0)) ? alpha * val : alpha * val + beta * y[q];
        y[q] = yn;
        if (dot1) a1 += (double)dot1[q] * (double)yn;
        if (self2) a2 += (double)yn * (double)yn;
    }
    if (dot1 != nullptr || self2) emit_partials<DRD_TPB>(a1, a2, dot1 != nullptr, self2, d, slot1);
}

// The FP32 momentum operator, tiled: a block stages the unknowns (with MatrixVector_uv_2_CG's
// ghost values, :533-553) and the cell coefficients eta, rho and pen for a tile of
// kUvTI x kUvTK cells plus a one-cell halo in shared memory, then evaluates the u and v rows
// of the tile branch-free with the expressions of uv_apply<float>.  Same arguments and
// partial sums as k_uv_mv; blocks walk the tiles with a grid stride.
constexpr int kUvTI = 64;
constexpr int kUvSI = kUvTI + 2;

template <int kUvTK>
__global__ void __launch_bounds__(DRD_TPB) k_uv_mv_tile(OpScal<float> o, const float* __restrict__ rho,
                                                        const float* __restrict__ eta, const float* __restrict__ pen,
                                                        const float* __restrict__ x, float alpha, float beta, float* y,
                                                        const float* dot1, int self2, Dots d, int slot1,
                                                        const KState* ks, int gate, ull* ctr) {
    constexpr int kUvSK = kUvTK + 2;
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    __shared__ float sU[kUvSK][kUvSI], sV[kUvSK][kUvSI], sE[kUvSK][kUvSI], sR[kUvSK][kUvSI], sP[kUvSK][kUvSI];
    const int nr = o.nr, nz = o.nz;
    const long mn = (long)(nr + 1) * nz;
    const int nti = (nr + 1 + kUvTI - 1) / kUvTI, ntk = (nz + kUvTK - 1) / kUvTK;
    const float h = 0.5f, q4 = 0.25f;
    const float mcoef = (o.bdf == 2) ? 1.5f * o.re : o.re;
    const float refl = o.lr_neumann ? 1.f : -1.f;
    double a1 = 0.0, a2 = 0.0;
    for (int tile = blockIdx.x; tile < nti * ntk; tile += gridDim.x) {
        const int i0 = (tile % nti) * kUvTI, k0 = (tile / nti) * kUvTK;
        __syncthreads();  // the previous tile's reads are done
        // a tile whose halo lies inside the unknowns' and the cells' ranges needs no ghost rules
        const bool interior = i0 >= 1 && i0 + kUvTI <= nr - 1 && k0 >= 2 && k0 + kUvTK <= nz - 1;
        if (interior) {
            for (int e = threadIdx.x; e < kUvSI * kUvSK; e += DRD_TPB) {
                const int li = e % kUvSI, lk = e / kUvSI;
                const int i = i0 - 1 + li, k = k0 - 1 + lk;
                sU[lk][li] = x[i + (long)(nr + 1) * k];
                sV[lk][li] = x[mn + i + (long)nr * (k - 1)];
                const long c = cidx(nr, i, k);
                sE[lk][li] = eta[c];
                sR[lk][li] = rho[c];
                sP[lk][li] = pen[c];
            }
        } else
        for (int e = threadIdx.x; e < kUvSI * kUvSK; e += DRD_TPB) {
            const int li = e % kUvSI, lk = e / kUvSI;
            const int i = i0 - 1 + li, k = k0 - 1 + lk;
            // U(i, k): k reflected with a sign change, then i by the side rule (UVFetch)
            const int kc = k < 0 ? 0 : (k > nz - 1 ? nz - 1 : k);
            const float ks_ = (k < 0 || k > nz - 1) ? -1.f : 1.f;
            float u;
            if (i < 0) u = refl * x[1 + (long)(nr + 1) * kc];
            else if (i > nr) u = refl * x[(nr - 1) + (long)(nr + 1) * kc];
            else u = x[i + (long)(nr + 1) * kc];
            sU[lk][li] = ks_ * u;
            const int ic = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
            sV[lk][li] = (k <= 0 || k >= nz) ? 0.f : x[mn + ic + (long)nr * (k - 1)];
            const bool cell = i >= -1 && i <= nr && k >= -1 && k <= nz;
            const long c = cidx(nr, i, k);
            sE[lk][li] = cell ? eta[c] : 0.f;
            sR[lk][li] = cell ? rho[c] : 0.f;
            sP[lk][li] = cell ? pen[c] : 0.f;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < kUvTI * kUvTK; r += DRD_TPB) {
            const int li = r % kUvTI + 1, lk = r / kUvTI + 1;  // staged coordinates of (i, k)
            const int i = i0 + li - 1, k = k0 + lk - 1;
#define E_(di, dk) sE[lk + (dk)][li + (di)]
            if (i <= nr && k <= nz - 1) {  // u row
                const long q = i + (long)(nr + 1) * k;
                const float f1 = sU[lk][li];
                float val;
                if (o.bdf == 2)
                    val = f1 * mcoef * (sR[lk][li] + sR[lk][li - 1]) * h + f1 * o.pk * (sP[lk][li] + sP[lk][li - 1]) * h * o.dt;
                else
                    val = f1 * mcoef * (sR[lk][li] + sR[lk][li - 1]) * h;
                float cr = E_(0, 0), cl = E_(-1, 0);
                val = val - 2.f * o.dt * (cr * (sU[lk][li + 1] - f1) + cl * (sU[lk][li - 1] - f1)) * o.idr2;
                cr = (E_(0, 1) + E_(-1, 1) + E_(0, 0) + E_(-1, 0)) * q4;
                cl = (E_(0, 0) + E_(-1, 0) + E_(0, -1) + E_(-1, -1)) * q4;
                val = val - o.dt * (cr * (sU[lk + 1][li] - f1) + cl * (sU[lk - 1][li] - f1)) * o.idz2;
                val = val - o.dt * (cr * (sV[lk + 1][li] - sV[lk + 1][li - 1]) - cl * (sV[lk][li] - sV[lk][li - 1])) * o.idrdz;
                const float yn = (beta == 0.f) ? alpha * val : alpha * val + beta * y[q];
                y[q] = yn;
                if (dot1) a1 += (double)dot1[q] * (double)yn;
                if (self2) a2 += (double)yn * (double)yn;
            }
            if (i <= nr - 1 && k >= 1 && k <= nz - 1) {  // v row
                const long q = mn + i + (long)nr * (k - 1);
                const float f2 = sV[lk][li];
                float val;
                if (o.bdf == 2)
                    val = f2 * mcoef * (sR[lk][li] + sR[lk - 1][li]) * h + f2 * o.pk * (sP[lk][li] + sP[lk - 1][li]) * h * o.dt;
                else
                    val = f2 * mcoef * (sR[lk][li] + sR[lk - 1][li]) * h;
                float cr = E_(0, 0), cl = E_(0, -1);
                val = val - 2.f * o.dt * (cr * (sV[lk + 1][li] - f2) + cl * (sV[lk - 1][li] - f2)) * o.idz2;
                cr = (E_(1, 0) + E_(0, 0) + E_(1, -1) + E_(0, -1)) * q4;
                cl = (E_(0, 0) + E_(-1, 0) + E_(0, -1) + E_(-1, -1)) * q4;
                val = val - o.dt * (cr * (sV[lk][li + 1] - f2) + cl * (sV[lk][li - 1] - f2)) * o.idr2;
                val = val - o.dt * (cr * (sU[lk][li + 1] - sU[lk - 1][li + 1]) - cl * (sU[lk][li] - sU[lk - 1][li])) * o.idrdz;
                const float yn = (beta == 0.f) ? alpha * val : alpha * val + beta * y[q];
                y[q] = yn;
                if (dot1) a1 += (double)dot1[q] * (double)yn;
                if (self2) a2 += (double)yn * (double)yn;
            }
#undef E_
        }
    }
    if (dot1 != nullptr || self2) emit_partials<DRD_TPB>(a1, a2, dot1 != nullptr, self2, d, slot1);
}

// Jacobi diagonal of PSolve_uv_2_CG (:662-709) / PSolve_uv_CG, including rho(i-1,j) in the
// v block as written at :690.
template <typename T>
__global__ void k_uv_diag(OpScal<T> o, const T* __restrict__ rho, const T* __restrict__ eta, T* __restrict__ diag,
                          ull* ctr) {
    count_launch(ctr);
    const long N = (long)(o.nr + 1) * o.nz + (long)o.nr * (o.nz - 1);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x)
        diag[q] = uv_diag<T>(o, rho, eta, q);
}

// btoA_uv (matrix_tool.f90:32-75) followed by the ghost assignments of :411-436 (TP :428-441).
__global__ void k_uv_fin(DevParams P, const double* __restrict__ x, const double* __restrict__ uL,
                         double* __restrict__ u_after, double* __restrict__ v_after, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long mn = (long)(nr + 1) * nz;
    const bool dirichlet = !(P.variant == DRD_VARIANT_TP && P.lr_neumann);
    const long us = (long)(nr + 3) * (nz + 2), vs = (long)(nr + 2) * (nz + 1);
    auto xu = [&](int i, int k) { return x[i + (long)(nr + 1) * k]; };
    auto ucol = [&](int i, int k) -> double {  // value at column i (-1..nr+1), row k (0..nz-1)
        if (i < 0) return dirichlet ? 2.0 * uL[k] - xu(1, k) : xu(1, k);
        if (i > nr) return dirichlet ? 2.0 * uL[k] - xu(nr - 1, k) : xu(nr - 1, k);
        return xu(i, k);
    };
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < us + vs; q += (long)gridDim.x * blockDim.x) {
        if (q < us) {
            const int i = (int)(q % (nr + 3)) - 1, k = (int)(q / (nr + 3)) - 1;
            double val;
            if (k == -1) val = P.uwB * 2.0 - ucol(i, 0);
            else if (k == nz) val = P.uwT * 2.0 - ucol(i, nz - 1);
            else val = ucol(i, k);
            u_after[q] = val;
        } else {
            const long qv = q - us;
            const int i = (int)(qv % (nr + 2)) - 1, k = (int)(qv / (nr + 2));
            double val = 0.0;
            if (k > 0 && k < nz) {
                const int ii = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
                val = x[mn + ii + (long)nr * (k - 1)];
            }
            v_after[qv] = val;
        }
    }
}

// ======================================================================================
// Pressure (microfluidics_complex_domain/PreSolve_2.f90:16-21), interpolate_coef, mass
// ======================================================================================
__global__ void k_pre_div(DevParams P, const double* __restrict__ u, const double* __restrict__ v,
                          double* __restrict__ w, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long n = (long)nr * nz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        w[q] = (u[uidx(nr, i + 1, k)] - u[uidx(nr, i, k)]) / P.dr + (v[vidx(nr, i, k + 1)] - v[vidx(nr, i, k)]) / P.dz;
    }
}

__global__ void k_cell_add(long n, const double* __restrict__ x, double* __restrict__ y, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        y[q] = x[q] + y[q];
}

// interpolate_coef (interpolate_coef.f90:55-89): fpd = (tanh(-d/(sqrt2 eps))+1)/2 + bdr,
// Neumann ghosts, rho/eta linear in fpd.
__global__ void k_interp_coef(DevParams P, const double* __restrict__ dist, const double* __restrict__ bdr,
                              double* __restrict__ fpd, double* __restrict__ rho, double* __restrict__ eta, ull* ctr) {
    count_launch(ctr);
    const int nr = P.nr, nz = P.nz;
    const long cs = (long)(nr + 2) * (nz + 2);
    const double sq2 = sqrt(2.0);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        const int si = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
        const int sk = k < 0 ? 0 : (k > nz - 1 ? nz - 1 : k);
        double f = tanh(-1.0 * dist[si + (long)nr * sk] / sq2 / P.eps);
        f = (f + 1.0) / 2.0;
        f = f + bdr[cidx(nr, si, sk)];
        fpd[q] = f;
        rho[q] = 1.0 + (P.lambda_rho - 1.0) * f;
        eta[q] = 1.0 + (P.lambda_eta - 1.0) * f;
    }
}

// y = 1 where x > t, else 0 (reinint_by_PhSolve.f90:78-86's bdr_ph_penalty).
__global__ void k_threshold(long n, const double* __restrict__ x, double t, double* __restrict__ y, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        y[q] = x[q] > t ? 1.0 : 0.0;
}

// The two-fluid form of interpolate_coef that two_phase_flow_complex_domain/
// interpolate_coef.f90:91-112 keeps commented out: rho and eta_ph piecewise linear in ph (1 at
// ph <= -1, the ratio at ph >= 1), eta = max(eta(fpd), eta_ph).  Products and sums are rounded
// separately (no contraction), as the host evaluates them.  FP32 copies are written for the
// mixed mode's operators (may be null).
__global__ void k_two_phase_coef(DevParams P, long cs, const double* __restrict__ fpd, const double* __restrict__ ph,
                                 double* __restrict__ rho, double* __restrict__ eta, float* __restrict__ rho32,
                                 float* __restrict__ eta32, ull* ctr) {
    count_launch(ctr);
    const double lr = P.lambda_rho - 1.0, le = P.lambda_eta - 1.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const double x = ph[q];
        double r, e;
        if (x <= -1.0) {
            r = 1.0; e = 1.0;
        } else if (x >= 1.0) {
            r = P.lambda_rho; e = P.lambda_eta;
        } else {
            r = __dadd_rn(1.0, __dmul_rn(lr, x));
            e = __dadd_rn(1.0, __dmul_rn(le, x));
        }
        const double es = __dadd_rn(1.0, __dmul_rn(le, fpd[q]));
        e = fmax(es, e);
        rho[q] = r;
        eta[q] = e;
        if (rho32) { rho32[q] = (float)r; eta32[q] = (float)e; }
    }
}

__global__ void k_mass_partial(int nr, int nz, const double* __restrict__ ph, Dots d, int slot, ull* ctr) {
    count_launch(ctr);
    const long n = (long)nr * nz;
    double a = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        a += ph[cidx(nr, i, k)];
    }
    __shared__ double sm[32];
    double r = block_sum<DRD_TPB>(a, sm);
    if (threadIdx.x == 0) d.part[slot * DRD_MAXB + blockIdx.x] = r;
}

__global__ void k_mass_final(Dots d, int slot, double drdz, double* out, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    double r = reduce_partials<DRD_TPB>(d.part + slot * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) *out = r * drdz;
}

// dissipation() (microfluidics_complex_domain/dissipation.f90:1-122): per-block partial sums of
// e1 (|grad rmu|^2 over interior cells), e2 (the wall rows' contact-angle residual), e3 (the
// velocity-gradient terms at the nodes 0..nr x 0..nz with the trapezoid weights) and the mass.
// Derivatives use setup's coefficients xa1 = -1/(2dr), xb1 = 0, xc1 = 1/(2dr) in dif1x's
// expression ua u(i-1) + ub u(i) + uc u(i+1) (setup.f90:9-19, :269-307).  v's derivatives are
// taken on v's own grid (the reference hands v to dif1x through u's shape), one-sided at i = nr
// and, like u_z, in the wall rows (:68-77).
__device__ __forceinline__ double dfdx3(double a, double b, double c, double h) {
    const double ua = -1.0 / 2.0 / h, ub = 0.0, uc = -ua;
    return ua * a + ub * b + uc * c;
}
__global__ void k_dissip_partial(DissipArgs a, const double* __restrict__ u, const double* __restrict__ v,
                                 const double* __restrict__ ph, const double* __restrict__ rmu,
                                 const double* __restrict__ angB, const double* __restrict__ angT, Dots d, ull* ctr) {
    count_launch(ctr);
    const int nr = a.nr, nz = a.nz;
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x, nt = (long)gridDim.x * blockDim.x;
    const double pi = 3.14159265358979323846264338327950288;
    double s1 = 0.0, s2 = 0.0, s3 = 0.0, sm_ = 0.0;
    const long nc = (long)nr * nz;
    for (long q = tid; q < nc; q += nt) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const double gx = (rmu[cidx(nr, i + 1, k)] - rmu[cidx(nr, i - 1, k)]) / 2.0 / a.dr;
        const double gz = (rmu[cidx(nr, i, k + 1)] - rmu[cidx(nr, i, k - 1)]) / 2.0 / a.dz;
        s1 += gx * gx + gz * gz;
        sm_ += ph[cidx(nr, i, k)];
    }
    for (long i = tid; i < nr; i += nt) {
        const double aT = angT ? angT[i] : a.angle, aB = angB ? angB[i] : a.angle;
        double cf = sqrt(2.0) * cos(aT * pi / 180.0) / 3.0 * pi / 2. / a.eps;
        const double pt = ph[cidx(nr, (int)i, nz)], pt1 = ph[cidx(nr, (int)i, nz - 1)];
        const double gt = (pt - pt1) / a.dz - cf * cos(pi * (pt + pt1) / 2.0 / 2.);
        cf = sqrt(2.0) * cos(aB * pi / 180.0) / 3.0 * pi / 2. / a.eps;
        const double pb = ph[cidx(nr, (int)i, -1)], pb0 = ph[cidx(nr, (int)i, 0)];
        const double gb = (pb - pb0) / a.dz - cf * cos(pi * (pb0 + pb) / 2.0 / 2.);
        s2 += gt * gt + gb * gb;
    }
    const long nn = (long)(nr + 1) * (nz + 1);
    for (long q = tid; q < nn; q += nt) {
        const int i = (int)(q % (nr + 1)), k = (int)(q / (nr + 1));
        const double uua = dfdx3(u[uidx(nr, i - 1, k)], u[uidx(nr, i, k)], u[uidx(nr, i + 1, k)], a.dr);
        double uub, vvb, vva;
        if (k == 0) {
            uub = (u[uidx(nr, i, 1)] - u[uidx(nr, i, 0)]) / a.dz;
            vvb = (v[vidx(nr, i, 1)] - v[vidx(nr, i, 0)]) / a.dz;
        } else if (k == nz) {
            uub = (u[uidx(nr, i, nz)] - u[uidx(nr, i, nz - 1)]) / a.dz;
            vvb = (v[vidx(nr, i, nz)] - v[vidx(nr, i, nz - 1)]) / a.dz;
        } else {
            uub = dfdx3(u[uidx(nr, i, k - 1)], u[uidx(nr, i, k)], u[uidx(nr, i, k + 1)], a.dz);
            vvb = dfdx3(v[vidx(nr, i, k - 1)], v[vidx(nr, i, k)], v[vidx(nr, i, k + 1)], a.dz);
        }
        if (i < nr) vva = dfdx3(v[vidx(nr, i - 1, k)], v[vidx(nr, i, k)], v[vidx(nr, i + 1, k)], a.dr);
        else vva = (v[vidx(nr, nr, k)] - v[vidx(nr, nr - 1, k)]) / a.dr;
        const double cx = (i == 0 || i == nr) ? 0.5 : 1.0, cz = (k == 0 || k == nz) ? 0.5 : 1.0;
        s3 += cx * cz * ((uua * uua + vvb * vvb) + uub * uub + vva * vva);
    }
    __shared__ double sh[32];
    double r = block_sum<DRD_TPB>(s1, sh);
    if (threadIdx.x == 0) d.part[0 * DRD_MAXB + blockIdx.x] = r;
    r = block_sum<DRD_TPB>(s2, sh);
    if (threadIdx.x == 0) d.part[1 * DRD_MAXB + blockIdx.x] = r;
    r = block_sum<DRD_TPB>(s3, sh);
    if (threadIdx.x == 0) d.part[2 * DRD_MAXB + blockIdx.x] = r;
    r = block_sum<DRD_TPB>(sm_, sh);
    if (threadIdx.x == 0) d.part[3 * DRD_MAXB + blockIdx.x] = r;
}

// Fixed-order sums of the partials and the reference's scalings (dissipation.f90:47, :57, :88,
// :101, :122): out = e1, e2, e3, e4, dissip, mass.
__global__ void k_dissip_final(DissipArgs a, Dots d, double* out, ull* ctr) {
    count_launch(ctr);
    __shared__ double sh[32];
    const double s1 = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sh);
    const double s2 = reduce_partials<DRD_TPB>(d.part + 1 * DRD_MAXB, d.G, sh);
    const double s3 = reduce_partials<DRD_TPB>(d.part + 2 * DRD_MAXB, d.G, sh);
    const double sm_ = reduce_partials<DRD_TPB>(d.part + 3 * DRD_MAXB, d.G, sh);
    if (threadIdx.x == 0) {
        const double e1 = s1 * a.xld * a.ca * a.dr * a.dz;
        const double e2 = s2 * a.vs * a.ca * (a.eps * a.eps) * a.dr;
        const double e3 = s3 * a.dr * a.dz;
        const double e4 = 0.0;
        out[0] = e1; out[1] = e2; out[2] = e3; out[3] = e4;
        out[4] = e1 + e2 + e3 + e4;
        out[5] = sm_ * a.dr * a.dz;
    }
}

// ======================================================================================
// Transforms as GEMMs: C = A B (row-major), the 2-D DCT-I / DCT-II / DCT-III of the
// preconditioner and the pressure solve applied one axis at a time.  Tiles BM x BN x BK,
// each thread TM x TN outputs strided by the thread grid (coalesced loads and stores).
// ======================================================================================
// Operand loads and output placement shared by the transform GEMMs (see GemmArgs::fold).
template <typename T>
struct GemmView {
    const T* A; const T* B; int M, N, par;
    __device__ __forceinline__ GemmView(const GemmArgs<T>& a, int p) : par(p) {
        A = (a.fold == FOLD_B && p) ? a.A_odd : a.A;
        B = (a.fold == FOLD_A && p) ? a.B_odd : a.B;
        M = (a.fold == FOLD_B && p) ? a.M_odd : a.M;
        N = (a.fold == FOLD_A && p) ? a.N_odd : a.N;
    }
    __device__ __forceinline__ T loadA(const GemmArgs<T>& a, int m, int k, int kend) const {
        if (m >= M || k >= kend) return T(0);
        if (a.fold != FOLD_A) return A[(long)m * a.lda + k];
        const T* row = A + (long)m * a.lda;
        if (2 * k == a.Lf) return par ? T(0) : row[k];
        return par ? row[k] - row[a.Lf - k] : row[k] + row[a.Lf - k];
    }
    __device__ __forceinline__ T loadB(const GemmArgs<T>& a, int k, int n, int kend) const {
        if (n >= N || k >= kend) return T(0);
        if (a.fold != FOLD_B) return B[(long)k * a.ldb + n];
        if (2 * k == a.Lf) return par ? T(0) : B[(long)k * a.ldb + n];
        const T x0 = B[(long)k * a.ldb + n], x1 = B[(long)(a.Lf - k) * a.ldb + n];
        return par ? x0 - x1 : x0 + x1;
    }
    __device__ __forceinline__ int orow(const GemmArgs<T>& a, int m) const { return a.fold == FOLD_B ? 2 * m + par : m; }
    __device__ __forceinline__ int ocol(const GemmArgs<T>& a, int n) const { return a.fold == FOLD_A ? 2 * n + par : n; }
};

template <typename T, int EPI>
__device__ __forceinline__ void gemm_store(const GemmArgs<T>& a, int gm, int gn, T v, double coef) {
    if (EPI == EPI_STORE) a.C[(long)gm * a.ldc + gn] = v;
    else if (EPI == EPI_DIV_TAB) a.C[(long)gm * a.ldc + gn] = v / a.tab[(long)gm * a.ldt + gn];
    else if (EPI == EPI_SCALE) a.C[(long)gm * a.ldc + gn] = v * (T)a.scale;
    else a.C[cidx(a.nr, gn, gm)] = (T)(((double)v / a.scale) * coef);
}

template <typename T, int BM, int BN, int BK, int TM, int TN, int EPI>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_gemm(GemmArgs<T> a) {
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int TX = BN / TN, TY = BM / TM;
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    count_launch(a.ctr);
    if (gate_closed(a.ks, a.gate)) return;
    const GemmView<T> g(a, a.fold ? (int)blockIdx.z : 0);
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    if (m0 >= g.M || n0 >= g.N) return;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
    for (int k0 = 0; k0 < a.K; k0 += BK) {
#pragma unroll
        for (int e = tid; e < BM * BK; e += NT) {
            const int r = e / BK, c = e % BK;
            As[c][r] = g.loadA(a, m0 + r, k0 + c, a.K);
        }
#pragma unroll
        for (int e = tid; e < BK * BN; e += NT) {
            const int r = e / BN, c = e % BN;
            Bs[r][c] = g.loadB(a, k0 + r, n0 + c, a.K);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T av[TM], bv[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) av[i] = As[kk][ty + i * TY];
#pragma unroll
            for (int j = 0; j < TN; ++j) bv[j] = Bs[kk][tx + j * TX];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
    const double coef = (EPI == EPI_PRE_FINAL) ? a.ca->coef : 0.0;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int gm = m0 + ty + i * TY;
        if (gm >= g.M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int gn = n0 + tx + j * TX;
            if (gn >= g.N) continue;
            gemm_store<T, EPI>(a, g.orow(a, gm), g.ocol(a, gn), acc[i][j], coef);
        }
    }
}

// Split-K variant: the KS CTAs of a thread-block cluster (cluster dims 1 x 1 x KS) each
// accumulate one slice of K for the same output tile; the partial tiles are then summed
// through distributed shared memory in a fixed rank order (deterministic, no atomics), each
// CTA reducing and storing BM/KS of the tile's rows.  Small-M transforms get KS times more
// CTAs this way, enough to occupy all SMs.
template <typename T, int BM, int BN, int BK, int TM, int TN, int KS, int EPI>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_gemm_sk(GemmArgs<T> a) {
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int TX = BN / TN, TY = BM / TM;
    static_assert(BM % KS == 0, "rows split over the cluster");
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    __shared__ T Cs[BM][BN + 1];
    count_launch(a.ctr);
    if (gate_closed(a.ks, a.gate)) return;  // uniform over the cluster: the state is not written here
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const GemmView<T> g(a, a.fold ? (int)(blockIdx.z / KS) : 0);
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const bool live = m0 < g.M && n0 < g.N;  // uniform over the cluster (same tile, same parity)
    const int kchunk = ((a.K + KS * BK - 1) / (KS * BK)) * BK;
    const int kbeg = rank * kchunk, kend = min(a.K, kbeg + kchunk);
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
    constexpr int LA = (BM * BK + NT - 1) / NT, LB = (BK * BN + NT - 1) / NT;
    T ra[LA], rb[LB];
    auto gload = [&](int k0) {
#pragma unroll
        for (int l = 0; l < LA; ++l) {
            const int e = tid + l * NT;
            ra[l] = (e < BM * BK) ? g.loadA(a, m0 + e / BK, k0 + e % BK, kend) : T(0);
        }
#pragma unroll
        for (int l = 0; l < LB; ++l) {
            const int e = tid + l * NT;
            rb[l] = (e < BK * BN) ? g.loadB(a, k0 + e / BN, n0 + e % BN, kend) : T(0);
        }
    };
    if (live && kbeg < kend) gload(kbeg);
    for (int k0 = kbeg; live && k0 < kend; k0 += BK) {
#pragma unroll
        for (int l = 0; l < LA; ++l) {
            const int e = tid + l * NT;
            if (e < BM * BK) As[e % BK][e / BK] = ra[l];
        }
#pragma unroll
        for (int l = 0; l < LB; ++l) {
            const int e = tid + l * NT;
            if (e < BK * BN) Bs[e / BN][e % BN] = rb[l];
        }
        __syncthreads();
        if (k0 + BK < kend) gload(k0 + BK);  // prefetch the next slice while computing this one
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T av[TM], bv[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) av[i] = As[kk][ty + i * TY];
#pragma unroll
            for (int j = 0; j < TN; ++j) bv[j] = Bs[kk][tx + j * TX];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) Cs[ty + i * TY][tx + j * TX] = acc[i][j];
    cluster.sync();
    const double coef = (EPI == EPI_PRE_FINAL) ? a.ca->coef : 0.0;
    constexpr int RB = BM / KS;
    for (int e = tid; live && e < RB * BN; e += NT) {
        const int r = rank * RB + e / BN, c = e % BN;
        const int gm = m0 + r, gn = n0 + c;
        T v = T(0);
#pragma unroll
        for (int q = 0; q < KS; ++q) v += cluster.map_shared_rank(&Cs[0][0], q)[r * (BN + 1) + c];
        if (gm < g.M && gn < g.N) gemm_store<T, EPI>(a, g.orow(a, gm), g.ocol(a, gn), v, coef);
    }
    cluster.sync();  // keep every CTA's partial tile alive until all readers are done
}

// FP64 transforms in double-float arithmetic on the FP32 pipes.  GB300 issues FP64 at a small
// fraction of its FP32 rate, and the FP64 transform GEMMs were the larger part of an FP64 CH
// iteration.  Each FP64 operand is split into hi + lo FP32 values (hi = fl32(x), lo = fl32(x -
// hi): 48 significant bits).  A product is hi*hi, taken exactly as p + e with one FMA, plus the
// cross terms hi*lo + lo*hi (lo*lo, about 2^-48 of the product, is dropped).  The running sum is
// a double-float (sh, sl): sh += p by an exact two-sum (Knuth), and its error joins e and the
// cross terms in sl.  The result is sh + sl in FP64: about 2^-44 of sum |a b|, where FP64
// accumulation gives about 2^-50.  The error-free steps use the _rn intrinsics, which the
// compiler never contracts into FMAs.
__device__ __forceinline__ void df_split(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}
__device__ __forceinline__ void df_mac(float ah, float al, float bh, float bl, float& sh, float& sl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);  // ah*bh = p + e exactly
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float s = __fadd_rn(sh, p);  // two-sum: sh + p = s + err exactly
    const float bv = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bv)), __fsub_rn(p, bv));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

template <int BM, int BN, int BK, int TM, int TN, int EPI>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_gemm_df(GemmArgs<double> a) {
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int TX = BN / TN, TY = BM / TM;
    __shared__ float Ah[BK][BM + 1], Al[BK][BM + 1];
    __shared__ float Bh[BK][BN], Bl[BK][BN];
    count_launch(a.ctr);
    if (gate_closed(a.ks, a.gate)) return;
    const GemmView<double> g(a, a.fold ? (int)blockIdx.z : 0);
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    if (m0 >= g.M || n0 >= g.N) return;
    float sh[TM][TN], sl[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) sh[i][j] = sl[i][j] = 0.f;
    for (int k0 = 0; k0 < a.K; k0 += BK) {
        for (int e = tid; e < BM * BK; e += NT) {
            const int r = e / BK, c = e % BK;
            df_split(g.loadA(a, m0 + r, k0 + c, a.K), Ah[c][r], Al[c][r]);
        }
        for (int e = tid; e < BK * BN; e += NT) {
            const int r = e / BN, c = e % BN;
            df_split(g.loadB(a, k0 + r, n0 + c, a.K), Bh[r][c], Bl[r][c]);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float ah[TM], al[TM], bh[TN], bl[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) { ah[i] = Ah[kk][ty + i * TY]; al[i] = Al[kk][ty + i * TY]; }
#pragma unroll
            for (int j = 0; j < TN; ++j) { bh[j] = Bh[kk][tx + j * TX]; bl[j] = Bl[kk][tx + j * TX]; }
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) df_mac(ah[i], al[i], bh[j], bl[j], sh[i][j], sl[i][j]);
        }
        __syncthreads();
    }
    const double coef = (EPI == EPI_PRE_FINAL) ? a.ca->coef : 0.0;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int gm = m0 + ty + i * TY;
        if (gm >= g.M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int gn = n0 + tx + j * TX;
            if (gn >= g.N) continue;
            gemm_store<double, EPI>(a, g.orow(a, gm), g.ocol(a, gn), (double)sh[i][j] + (double)sl[i][j], coef);
        }
    }
}

template <int BM, int BN, int TM, int TN>
static void gemm_df_dispatch(int epi, const GemmArgs<double>& a, cudaStream_t s) {
    dim3 grid((a.N + BN - 1) / BN, (a.M + BM - 1) / BM, a.fold ? 2 : 1);
    constexpr int NT = (BM / TM) * (BN / TN);
    switch (epi) {
        case EPI_STORE: k_gemm_df<BM, BN, 16, TM, TN, EPI_STORE><<<grid, NT, 0, s>>>(a); break;
        case EPI_DIV_TAB: k_gemm_df<BM, BN, 16, TM, TN, EPI_DIV_TAB><<<grid, NT, 0, s>>>(a); break;
        case EPI_SCALE: k_gemm_df<BM, BN, 16, TM, TN, EPI_SCALE><<<grid, NT, 0, s>>>(a); break;
        default: k_gemm_df<BM, BN, 16, TM, TN, EPI_PRE_FINAL><<<grid, NT, 0, s>>>(a); break;
    }
}

struct GemmCfg { const char* name; };
static const GemmCfg kGemmCfgs[] = {{"64x64x16/4x4"},         {"32x64x16/2x4"},         {"32x32x16/2x2"},
                                    {"16x32x16/1x2"},         {"sk4 32x64x16/4x4"},     {"sk4 32x32x16/4x4"},
                                    {"sk4 16x64x16/2x4"},     {"sk8 32x32x16/2x2"},     {"sk2 32x64x16/4x4"},
                                    {"df 64x64x16/4x4"},      {"df 32x64x16/2x4"},      {"df 32x32x16/2x2"},
                                    {"df 16x32x16/1x2"},      {"df 16x16x16/1x1"}};

// Configurations 9-13 are the double-float kernels: FP64 only.  The small tiles give the
// unfolded pressure passes at 420x180 four to eight times the blocks of 32x64 tiles.
// ---- the transform GEMM on the fifth-generation tensor cores (FP32 data, 3xTF32) -------------
// C = A B for the folded DCT passes (FOLD_A or FOLD_B, epilogue EPI_STORE or EPI_DIV_TAB): a
// 128 x 128 output tile per CTA, K in chunks of 32.  Each operand is split into high and low
// TF32 parts as it is staged (x = hi + lo, both rounded to TF32), and every K step issues
// tcgen05.mma kind::tf32 three times into one FP32 accumulator in TMEM: lo(A) hi(B),
// hi(A) lo(B), hi(A) hi(B), the products of FP32 operands up to the lo lo term.  One thread
// issues the MMAs; the operands are in shared memory in the K-major, unswizzled core-matrix
// layout (8 rows x 16 bytes, i.e. 4 TF32 values), in stages tracked by mbarriers that
// tcgen05.commit arrives on.  Two kernels: k_gemm_tc_tma (data operand by TMA boxes,
// warp-specialised) where the data rows are 16-byte aligned, k_gemm_tc (data operand staged
// through registers by all threads) otherwise.  Waits are bounded: a wait that gives up sets
// *err and the tile's outputs are written as NaN, which the solve's FP64 residual then reports.
constexpr int kGtcThreads = 512;  // 16 warps: all stage; warp w reads TMEM lanes 32 (w % 4), columns 32 (w / 4)
constexpr int kGtcM = 128, kGtcN = 128, kGtcK = 32;
constexpr uint32_t kGtcOp = kGtcM * kGtcK * 4;        // bytes of one operand part (hi or lo), 16 KB
constexpr uint32_t kGtcStage = 4 * kGtcOp;            // A hi, A lo, B hi, B lo
constexpr int kGtcStages = 3;
constexpr int kGtcSmem = kGtcStages * kGtcStage + 1024;  // three stages, 1 KB for alignment
constexpr int kGtcSpin = 1 << 22;

__device__ __forceinline__ uint64_t gtc_desc(uint32_t addr) {
    // start >> 4; leading byte offset (K-direction core stride, 16 rows of cores x 128 B = 2048)
    // >> 4; stride byte offset (8-row group stride, 128) >> 4; descriptor version 1; no swizzle
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((2048u >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((128u >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
__device__ __forceinline__ bool gtc_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < kGtcSpin; ++it) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ float gtc_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
// byte offset of element (row r, k) of a 128-row K-major operand part
__device__ __forceinline__ uint32_t gtc_off(int r, int k) {
    return (uint32_t)((k >> 2) * 2048 + (r >> 3) * 128 + (r & 7) * 16 + (k & 3) * 4);
}
__device__ __forceinline__ void gtc_put4(unsigned char* hi, unsigned char* lo, int r, int kg, const float (&v)[4]) {
    float4 h, l;
    h.x = gtc_tf32(v[0]); l.x = gtc_tf32(v[0] - h.x);
    h.y = gtc_tf32(v[1]); l.y = gtc_tf32(v[1] - h.y);
    h.z = gtc_tf32(v[2]); l.z = gtc_tf32(v[2] - h.z);
    h.w = gtc_tf32(v[3]); l.w = gtc_tf32(v[3] - h.w);
    const uint32_t o = gtc_off(r, 4 * kg);
    *reinterpret_cast<float4*>(hi + o) = h;
    *reinterpret_cast<float4*>(lo + o) = l;
}

// Loads chunk k0 of the data operand(s) of the tensor-core GEMM into registers: 128 rows /
// columns x 8 groups of 4 K values, GTC_NI (row, group) items of each operand per thread
// (row = item % 128, so a warp's later float4 stores are contiguous).  The packed constant
// operand is skipped (its values stay 0).
constexpr int GTC_NI = kGtcM * (kGtcK / 4) / kGtcThreads;
__device__ __forceinline__ void gtc_load(const GemmArgs<float>& a, const GemmView<float>& g, bool pk, bool const_b,
                                         bool a_vec, int m0, int n0, int k0, float (&va)[GTC_NI][4],
                                         float (&vb)[GTC_NI][4]) {
    const int tid = threadIdx.x, K = a.K, L = a.Lf;
#pragma unroll
    for (int it = 0; it < GTC_NI; ++it) {
        const int item = tid + it * kGtcThreads, r = item % kGtcM, kg = item / kGtcM;
        const int m = m0 + r, n = n0 + r, kb = k0 + 4 * kg, kbb = kb;
        // A as float4 (and its mirrored half, reversed) where a whole group lies before the
        // middle of the fold and the rows are 16-byte aligned
        if (pk && !const_b) {
            va[it][0] = va[it][1] = va[it][2] = va[it][3] = 0.f;  // A comes packed
        } else if (a_vec && m < g.M && kb + 3 < K && (a.fold != FOLD_A || 2 * (kb + 3) < L)) {
            const float* row = g.A + (long)m * a.lda;
            const float4 x0 = *reinterpret_cast<const float4*>(row + kb);
            if (a.fold == FOLD_A) {
                const float4 x1 = *reinterpret_cast<const float4*>(row + L - kb - 3);
                const float sg = g.par ? -1.f : 1.f;
                va[it][0] = fmaf(sg, x1.w, x0.x);
                va[it][1] = fmaf(sg, x1.z, x0.y);
                va[it][2] = fmaf(sg, x1.y, x0.z);
                va[it][3] = fmaf(sg, x1.x, x0.w);
            } else {
                va[it][0] = x0.x; va[it][1] = x0.y; va[it][2] = x0.z; va[it][3] = x0.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = kb + j;
                float x = 0.f;
                if (m < g.M && k < K) {
                    if (a.fold == FOLD_A) {
                        const float* row = g.A + (long)m * a.lda;
                        const float x0 = row[k], x1 = (2 * k == L) ? 0.f : row[L - k];
                        x = (2 * k == L) ? (g.par ? 0.f : x0) : (g.par ? x0 - x1 : x0 + x1);
                    } else {
                        x = g.A[(long)m * a.lda + k];
                    }
                }
                va[it][j] = x;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = kbb + j;
            float y = 0.f;
            if (!(pk && const_b) && n < g.N && k < K) {
                if (a.fold == FOLD_B) {
                    const float y0 = g.B[(long)k * a.ldb + n];
                    const float y1 = (2 * k == L) ? 0.f : g.B[(long)(L - k) * a.ldb + n];
                    y = (2 * k == L) ? (g.par ? 0.f : y0) : (g.par ? y0 - y1 : y0 + y1);
                } else {
                    y = g.B[(long)k * a.ldb + n];
                }
            }
            vb[it][j] = y;
        }
    }
}

// One packed block per (parity, 128-row tile, 32-K chunk): hi part then lo part, each in the
// core-matrix layout of gtc_off, zeros past the matrix.
__global__ void k_gtc_pack(const float* __restrict__ ev, const float* __restrict__ od, int re, int ro, int K, long ld,
                           int b_style, int tiles, int chunks, float* __restrict__ out) {
    const long tot = 2L * tiles * chunks * (kGtcM * kGtcK);
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot; e += (long)gridDim.x * blockDim.x) {
        const int kl = (int)(e % kGtcK), rl = (int)((e / kGtcK) % kGtcM);
        const long blk = e / (kGtcM * kGtcK);
        const int ch = (int)(blk % chunks), tl = (int)((blk / chunks) % tiles), par = (int)(blk / ((long)chunks * tiles));
        const int r = tl * kGtcM + rl, k = ch * kGtcK + kl;
        const float* src = par ? od : ev;
        const int rows = par ? ro : re;
        float x = 0.f;
        if (r < rows && k < K) x = b_style ? src[(long)k * ld + r] : src[(long)r * ld + k];
        const float hi = gtc_tf32(x), lo = gtc_tf32(x - hi);
        float* base = out + blk * (2 * kGtcM * kGtcK);
        const uint32_t o = gtc_off(rl, kl) / 4;
        base[o] = hi;
        base[kGtcM * kGtcK + o] = lo;
    }
}
long gemm_tc_pack(const float* even, const float* odd, int rows_e, int rows_o, int K, long ld, int b_style,
                  float* out, int* tiles_out, int* chunks_out, cudaStream_t s) {
    const int rows = rows_e > rows_o ? rows_e : rows_o;
    const int tiles = (rows + kGtcM - 1) / kGtcM, chunks = (K + kGtcK - 1) / kGtcK;
    const long n = 2L * tiles * chunks * 2 * kGtcM * kGtcK;
    if (tiles_out) *tiles_out = tiles;
    if (chunks_out) *chunks_out = chunks;
    if (out) k_gtc_pack<<<256, 256, 0, s>>>(even, odd, rows_e, rows_o, K, ld, b_style, tiles, chunks, out);
    return n;
}

// Epilogue of the tensor-core GEMM: warp w reads TMEM lanes 32 (w % 4) (tile rows) and
// columns 32 (w / 4) (tile columns) into a 128 x 129 shared-memory tile (`tile`, 66 KB of the
// CTA's stages, free once every MMA is done), and the warps then store the tile row by row,
// lanes along the tile's columns (consecutive output columns for FOLD_B, every other one for
// FOLD_A); a tile that gave up is stored as NaN.  Frees the TMEM.
template <int EPI>
__device__ __forceinline__ void gtc_epilogue(const GemmArgs<float>& a, const GemmView<float>& g, uint32_t tbase, int m0,
                                             int n0, bool poison, float* tile) {
    constexpr int TP = kGtcN + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int q = warp & 3, cq = warp >> 2;  // TMEM lane quarter, column quarter (warps 0-15)
#pragma unroll 1
    for (int col = 32 * cq; warp < 16 && col < 32 * cq + 32; col += 16) {
        uint32_t r[16];
        const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)col;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                       "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                     : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        float* trow = tile + (32 * q + lane) * TP + col;
#pragma unroll
        for (int j = 0; j < 16; ++j) trow[j] = __uint_as_float(r[j]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(128) : "memory");
    const int nw = blockDim.x >> 5;
#pragma unroll 1
    for (int rr = warp; rr < kGtcM; rr += nw) {
        const int m = m0 + rr;
        if (m >= g.M) break;
#pragma unroll
        for (int i = 0; i < kGtcN / 32; ++i) {
            const int cl = lane + 32 * i, n = n0 + cl;
            if (n < g.N)
                gemm_store<float, EPI>(a, g.orow(a, m), g.ocol(a, n), poison ? __int_as_float(0x7fc00000) : tile[rr * TP + cl], 0.0);
        }
    }
}

// The twelve MMAs of one 32-K chunk, A and B each given as its hi part followed by its lo part
// (16 KB each): per K = 8 step lo(A) hi(B), hi(A) lo(B), hi(A) hi(B); the first of the tile
// overwrites D.
__device__ __forceinline__ void gtc_mma_chunk(uint32_t opa, uint32_t opb, uint32_t tbase, uint32_t idesc, bool first) {
    const uint32_t aH = opa, aL = aH + kGtcOp, bH = opb, bL = bH + kGtcOp;
#pragma unroll
    for (int t = 0; t < kGtcK / 8; ++t) {  // K = 8 per MMA: two core columns, 4096 bytes
        const uint32_t off = (uint32_t)t * 4096u;
        const uint64_t dAH = gtc_desc(aH + off), dAL = gtc_desc(aL + off);
        const uint64_t dBH = gtc_desc(bH + off), dBL = gtc_desc(bL + off);
        const uint32_t acc0 = (!first || t > 0) ? 1u : 0u;
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                     ::"r"(tbase), "l"(dAL), "l"(dBH), "r"(idesc), "r"(acc0) : "memory");
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                     ::"r"(tbase), "l"(dAH), "l"(dBL), "r"(idesc), "r"(1u) : "memory");
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                     ::"r"(tbase), "l"(dAH), "l"(dBH), "r"(idesc), "r"(1u) : "memory");
    }
}

template <int EPI>
__global__ void __launch_bounds__(kGtcThreads) k_gemm_tc(GemmArgs<float> a) {
    extern __shared__ __align__(1024) unsigned char gsm_raw[];
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t mbar[kGtcStages];
    __shared__ __align__(8) uint64_t lbar[kGtcStages];  // bulk copies of the packed constant operand
    __shared__ int bad;
    count_launch(a.ctr);
    if (gate_closed(a.ks, a.gate)) return;
    const GemmView<float> g(a, a.fold ? (int)blockIdx.z : 0);
    const bool pk = a.packed != nullptr;  // the constant operand comes packed (B of FOLD_A, A of FOLD_B)
    const bool const_b = a.fold == FOLD_A;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.y * kGtcM, n0 = blockIdx.x * kGtcN;
    if (m0 >= g.M || n0 >= g.N) return;
    unsigned char* gsm = gsm_raw + ((1024u - ((uint32_t)__cvta_generic_to_shared(gsm_raw) & 1023u)) & 1023u);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(gsm);
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tmem_base);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(128) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < kGtcStages; ++i) {
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[i]);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
            const uint32_t lb = (uint32_t)__cvta_generic_to_shared(&lbar[i]);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(lb) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        bad = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tbase = tmem_base;
    const int ctile = const_b ? (int)blockIdx.x : (int)blockIdx.y;  // the packed operand's row tile
    // D F32, A TF32, B TF32, both K-major, N = 128, M = 128
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kGtcN >> 3) << 17) | ((uint32_t)(kGtcM >> 4) << 24);
    const int K = a.K, nchunks = (K + kGtcK - 1) / kGtcK;
    const int L = a.Lf;
    // float4 loads of A: 16-byte aligned rows, and for FOLD_A mirrored groups that start on a
    // multiple of 4 as well (row length L + 1 a multiple of 4)
    const bool a_vec = (a.lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(g.A) & 15) == 0) &&
                       (a.fold != FOLD_A || (L + 1) % 4 == 0);
    // Pipeline over the K chunks, three stages (chunk c in stage c % 3).  Chunk c: store its data
    // operand (loaded into registers during chunk c - 1) and issue chunk c + 1's loads; after the
    // barrier thread 0 waits for chunk c's bulk copy (issued two chunks earlier), issues its
    // MMAs, waits for chunk c - 1's MMAs and issues the bulk copy of chunk c + 2 into the stage
    // they read.  Use k of stage s completes phase k of lbar[s] and of mbar[s].
    auto bulk = [&](int cc) {  // thread 0: the packed constant operand of chunk cc
        const int sc = cc % kGtcStages;
        const uint32_t lb = (uint32_t)__cvta_generic_to_shared(&lbar[sc]);
        const uint32_t dst = sbase + sc * kGtcStage + (const_b ? 2 * kGtcOp : 0);
        const float* src = a.packed + ((long)(g.par * a.pk_tiles + ctile) * a.pk_chunks + cc) * (2 * kGtcM * kGtcK);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(lb), "r"(2u * kGtcOp) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(dst), "l"(src), "r"(2u * kGtcOp), "r"(lb) : "memory");
    };
    float cva[GTC_NI][4], cvb[GTC_NI][4];
    if (nchunks > 0) gtc_load(a, g, pk, const_b, a_vec, m0, n0, 0, cva, cvb);
    if (pk && tid == 0) {
        for (int cc = 0; cc < 2 && cc < nchunks; ++cc) bulk(cc);
    }
    for (int c = 0; c < nchunks; ++c) {
        const int st = c % kGtcStages, use = c / kGtcStages;
        unsigned char* sA = gsm + st * kGtcStage;
        unsigned char* sB = sA + 2 * kGtcOp;
        __syncthreads();  // every thread reads the same `bad`; stage st is free (chunk c - 3 done)
        if (bad) break;
#pragma unroll
        for (int it = 0; it < GTC_NI; ++it) {
            const int item = tid + it * kGtcThreads, r = item % kGtcM, kg = item / kGtcM;
            if (!(pk && !const_b)) gtc_put4(sA, sA + kGtcOp, r, kg, cva[it]);
            if (!(pk && const_b)) gtc_put4(sB, sB + kGtcOp, r, kg, cvb[it]);
        }
        if (c + 1 < nchunks) gtc_load(a, g, pk, const_b, a_vec, m0, n0, (c + 1) * kGtcK, cva, cvb);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            if (pk) {  // the bulk copy of this chunk has landed
                const uint32_t lb = (uint32_t)__cvta_generic_to_shared(&lbar[st]);
                if (!bad && !gtc_wait(lb, (uint32_t)(use & 1))) {
                    bad = 1;
                    if (a.err) atomicExch(a.err, 1);
                }
            }
            if (!bad) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                gtc_mma_chunk(sbase + st * kGtcStage, sbase + st * kGtcStage + 2 * kGtcOp, tbase, idesc, c == 0);
                const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[st]);
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb) : "memory");
            }
            // chunk c - 1's MMAs done: its stage takes chunk c + 2 (and, with chunk c - 2's, the
            // next chunk's stores may overwrite stage (c + 1) % 3)
            if (!bad && c >= 1) {
                const int pc = c - 1;
                const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[pc % kGtcStages]);
                if (!gtc_wait(mb, (uint32_t)((pc / kGtcStages) & 1))) {
                    bad = 1;
                    if (a.err) atomicExch(a.err, 1);
                }
            }
            if (!bad && pk && c + 2 < nchunks) bulk(c + 2);
        }
    }
    // the last chunk's commit covers every MMA of the CTA; after a give-up, wait (bounded) for
    // every stage's MMAs and bulk copy so that nothing still writes or reads the stages or TMEM
    if (tid == 0 && nchunks > 0) {
        if (!bad) {
            const int lc = nchunks - 1;
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[lc % kGtcStages]);
            if (!gtc_wait(mb, (uint32_t)((lc / kGtcStages) & 1))) {
                bad = 1;
                if (a.err) atomicExch(a.err, 1);
            }
        }
        if (bad) {
            for (int i = 0; i < kGtcStages; ++i) {
                const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[i]);
                gtc_wait(mb, 0u);
                gtc_wait(mb, 1u);
                if (pk) {
                    const uint32_t lb = (uint32_t)__cvta_generic_to_shared(&lbar[i]);
                    gtc_wait(lb, 0u);
                    gtc_wait(lb, 1u);
                }
            }
        }
    }
    __syncthreads();
    gtc_epilogue<EPI>(a, g, tbase, m0, n0, bad != 0, reinterpret_cast<float*>(gsm));
}

// The tensor-core GEMM with TMA staging of the data operand.  Per 32-K chunk the data tile and
// its fold mirror arrive as two 16 KB boxes of a 2-D tensor map (cp.async.bulk.tensor, one
// thread issues, an expect-tx mbarrier tracks them), two chunks ahead in a ring of raw stages;
// the threads fold each (row, 4-K group) from shared memory, split it into TF32 high and low
// parts and write the data operand stage (two stages).  The packed constant operand has its
// own ring of three 32 KB stages, filled two chunks ahead by one bulk copy per chunk.  FOLD_A: the boxes are 32 K x 128
// rows of X at (k0, m0) and (L - k0 - 31, m0), 128-byte swizzled (16-byte chunk j of box row r
// sits at chunk j ^ (r & 7)); FOLD_B: 128 columns x 32 K rows of X at (n0, k0) and
// (n0, L - k0 - 31), unswizzled.  Shared memory: data stages (2 x 32 KB: hi, lo), constant
// stages (3 x 32 KB: hi, lo), raw stages (2 x 32 KB: box, mirror box).
constexpr int kGtrRaw = 2;                                  // raw stages
constexpr int kGtrCst = 3;                                  // constant operand stages
constexpr uint32_t kGtrBox = kGtcM * kGtcK * 4;             // one box, 16 KB
constexpr uint32_t kGtrRawStage = 2 * kGtrBox;              // the data box and its mirror
constexpr uint32_t kGtrOpStage = 2 * kGtcOp;                // hi and lo parts of one operand, 32 KB
constexpr uint32_t kGtrCst0 = 2 * kGtrOpStage;              // offset of the constant stages
constexpr uint32_t kGtrRaw0 = kGtrCst0 + kGtrCst * kGtrOpStage;  // offset of the raw stages
constexpr int kGtrSmem = kGtrRaw0 + kGtrRaw * kGtrRawStage + 1024;

__device__ __forceinline__ void gtr_box(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar) : "memory");
}

constexpr int kGtrThreads = kGtcThreads + 32;  // 16 converter warps and the copy / MMA warp

// gtc_wait that also gives up as soon as *flag is set (another thread gave up)
__device__ __forceinline__ bool gtr_wait(uint32_t bar, uint32_t parity, const volatile int* flag) {
    for (int it = 0; it < kGtcSpin; ++it) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if (*flag) return false;
    }
    return false;
}

// Warp roles: warps 0-15 convert (chunk c: wait until the MMAs of chunk c - 2 have released data
// stage c & 1 and chunk c's boxes have landed, fold and split into the stage, arrive on its
// `full` barrier); warp 16's first lane issues every copy and MMA (chunk c: wait for `full`,
// refill the consumed raw stage with chunk c + 2, wait for the constant operand, issue the
// twelve MMAs and commit them, wait for chunk c - 1's MMAs and refill their constant stage with
// chunk c + 2).  No block-wide barrier inside the K loop: conversion of chunk c + 1 overlaps
// the MMAs of chunk c.
// PF (pre-folded, FOLD_A only): the tensor map addresses the folded even operand in rows
// [0, M) and the odd one in rows [M, 2M) (gtr_prefold), one box per chunk and no fold here.
template <int EPI, bool PF>
__global__ void __launch_bounds__(kGtrThreads) k_gemm_tc_tma(GemmArgs<float> a, const __grid_constant__ CUtensorMap tm) {
    extern __shared__ __align__(1024) unsigned char gsm_raw[];
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t mbar[2];        // MMAs of chunk c (data stage c & 1) are done
    __shared__ __align__(8) uint64_t fbar[2];        // data stage s converted (kGtcThreads arrivals)
    __shared__ __align__(8) uint64_t lbar[kGtrCst];  // packed constant operand of stage s landed
    __shared__ __align__(8) uint64_t rbar[kGtrRaw];  // data boxes of raw stage s landed
    __shared__ volatile int bad;
    count_launch(a.ctr);
    if (gate_closed(a.ks, a.gate)) return;
    const GemmView<float> g(a, a.fold ? (int)blockIdx.z : 0);
    const bool fa = a.fold == FOLD_A;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.y * kGtcM, n0 = blockIdx.x * kGtcN;
    if (m0 >= g.M || n0 >= g.N) return;
    unsigned char* gsm = gsm_raw + ((1024u - ((uint32_t)__cvta_generic_to_shared(gsm_raw) & 1023u)) & 1023u);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(gsm);
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tmem_base);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(128) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&mbar[i])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(&fbar[i])),
                         "r"(kGtcThreads) : "memory");
        }
        for (int i = 0; i < kGtrCst; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&lbar[i])) : "memory");
        for (int i = 0; i < kGtrRaw; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&rbar[i])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        bad = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tbase = tmem_base;
    const int K = a.K, L = a.Lf, nchunks = (K + kGtcK - 1) / kGtcK;
    auto fail = [&]() {
        bad = 1;
        if (a.err) atomicExch(a.err, 1);
    };
    if (warp < kGtcThreads / 32) {
        // ---- converters ----
        const float sg = g.par ? -1.f : 1.f;
        const unsigned char* rawp = gsm + kGtrRaw0;
        for (int c = 0; c < nchunks; ++c) {
            if (bad) break;
            const int st = c & 1, rs = c % kGtrRaw;
            if (c >= 2 && !gtr_wait((uint32_t)__cvta_generic_to_shared(&mbar[st]), (uint32_t)(((c - 2) >> 1) & 1), &bad)) {
                fail();
                break;
            }
            if (!gtr_wait((uint32_t)__cvta_generic_to_shared(&rbar[rs]), (uint32_t)((c / kGtrRaw) & 1), &bad)) {
                fail();
                break;
            }
            const unsigned char* r0 = rawp + rs * kGtrRawStage;
            const unsigned char* r1 = r0 + kGtrBox;
            unsigned char* op = gsm + st * kGtrOpStage;
            const int k0 = c * kGtcK;
            // a chunk past K's end or holding the middle point k = L / 2 takes the masked fold
            const bool edge = (k0 + kGtcK > K) || ((L & 1) == 0 && 2 * k0 <= L && L < 2 * (k0 + kGtcK));
#pragma unroll
            for (int it = 0; it < GTC_NI; ++it) {
                const int item = tid + it * kGtcThreads, r = item % kGtcM, kg = item / kGtcM;
                float a0[4], a1[4], v[4];
                if (PF) {  // the folded value itself (zeros past K)
                    const float4 x0 = *reinterpret_cast<const float4*>(r0 + r * 128 + ((kg ^ (r & 7)) << 4));
                    v[0] = x0.x; v[1] = x0.y; v[2] = x0.z; v[3] = x0.w;
                    gtc_put4(op, op + kGtcOp, r, kg, v);
                    continue;
                }
                if (fa) {
                    const float4 x0 = *reinterpret_cast<const float4*>(r0 + r * 128 + ((kg ^ (r & 7)) << 4));
                    const float4 x1 = *reinterpret_cast<const float4*>(r1 + r * 128 + (((7 - kg) ^ (r & 7)) << 4));
                    a0[0] = x0.x; a0[1] = x0.y; a0[2] = x0.z; a0[3] = x0.w;
                    a1[0] = x1.w; a1[1] = x1.z; a1[2] = x1.y; a1[3] = x1.x;
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        a0[j] = *reinterpret_cast<const float*>(r0 + (4 * kg + j) * 512 + r * 4);
                        a1[j] = *reinterpret_cast<const float*>(r1 + (kGtcK - 1 - 4 * kg - j) * 512 + r * 4);
                    }
                }
                if (!edge) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) v[j] = fmaf(sg, a1[j], a0[j]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int k = k0 + 4 * kg + j;
                        v[j] = (k >= K) ? 0.f : (2 * k == L) ? (g.par ? 0.f : a0[j]) : fmaf(sg, a1[j], a0[j]);
                    }
                }
                gtc_put4(op, op + kGtcOp, r, kg, v);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"((uint32_t)__cvta_generic_to_shared(&fbar[st])) : "memory");
        }
    } else if ((tid & 31) == 0) {
        // ---- copies and MMAs ----
        const int ctile = fa ? (int)blockIdx.x : (int)blockIdx.y;  // the packed operand's row tile
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kGtcN >> 3) << 17) | ((uint32_t)(kGtcM >> 4) << 24);
        const uint32_t raw0 = sbase + kGtrRaw0;
        // chunks [0, n_tma) have their boxes issued, [0, n_bulk) their packed operand, [0, n_mma)
        // their MMAs committed; [0, w_bulk) and [0, w_mma) were waited for
        int n_tma = 0, n_bulk = 0, n_mma = 0, w_bulk = 0, w_mma = 0;
        auto issue_tma = [&](int cc) {
            const int rs = cc % kGtrRaw;
            const uint32_t rb = (uint32_t)__cvta_generic_to_shared(&rbar[rs]);
            const uint32_t dst = raw0 + rs * kGtrRawStage;
            const int k0 = cc * kGtcK, k1 = L - k0 - (kGtcK - 1);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(rb),
                         "r"(PF ? kGtrBox : kGtrRawStage) : "memory");
            if (PF) {
                gtr_box(dst, &tm, k0, g.par * a.M + m0, rb);
            } else if (fa) {
                gtr_box(dst, &tm, k0, m0, rb);
                gtr_box(dst + kGtrBox, &tm, k1, m0, rb);
            } else {
                gtr_box(dst, &tm, n0, k0, rb);
                gtr_box(dst + kGtrBox, &tm, n0, k1, rb);
            }
            n_tma = cc + 1;
        };
        auto issue_bulk = [&](int cc) {  // the packed constant operand of chunk cc into stage cc % 3
            const int cs = cc % kGtrCst;
            const uint32_t lb = (uint32_t)__cvta_generic_to_shared(&lbar[cs]);
            const uint32_t dst = sbase + kGtrCst0 + cs * kGtrOpStage;
            const float* src = a.packed + ((long)(g.par * a.pk_tiles + ctile) * a.pk_chunks + cc) * (2 * kGtcM * kGtcK);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(lb), "r"(2u * kGtcOp) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         ::"r"(dst), "l"(src), "r"(2u * kGtcOp), "r"(lb) : "memory");
            n_bulk = cc + 1;
        };
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tm)) : "memory");
        for (int cc = 0; cc < kGtrRaw && cc < nchunks; ++cc) issue_tma(cc);
        for (int cc = 0; cc < kGtrCst - 1 && cc < nchunks; ++cc) issue_bulk(cc);
        for (int c = 0; c < nchunks; ++c) {
            const int st = c & 1, cs = c % kGtrCst;
            // chunk c converted: its raw stage takes chunk c + 2
            if (!gtr_wait((uint32_t)__cvta_generic_to_shared(&fbar[st]), (uint32_t)((c >> 1) & 1), &bad) || bad) {
                fail();
                break;
            }
            if (c + kGtrRaw < nchunks) issue_tma(c + kGtrRaw);
            if (!gtr_wait((uint32_t)__cvta_generic_to_shared(&lbar[cs]), (uint32_t)((c / kGtrCst) & 1), &bad)) {
                fail();
                break;
            }
            w_bulk = c + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t dop = sbase + st * kGtrOpStage, cop = sbase + kGtrCst0 + cs * kGtrOpStage;
            gtc_mma_chunk(fa ? dop : cop, fa ? cop : dop, tbase, idesc, c == 0);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"((uint32_t)__cvta_generic_to_shared(&mbar[st])) : "memory");
            n_mma = c + 1;
            // chunk c - 1's MMAs done: its constant stage takes chunk c + 2
            if (c >= 1) {
                if (!gtr_wait((uint32_t)__cvta_generic_to_shared(&mbar[st ^ 1]), (uint32_t)(((c - 1) >> 1) & 1), &bad)) {
                    fail();
                    break;
                }
                w_mma = c;
            }
            if (c + kGtrCst - 1 < nchunks) issue_bulk(c + kGtrCst - 1);
        }
        if (!bad) {  // the last commit covers every MMA of the tile
            const int lc = nchunks - 1;
            if (gtc_wait((uint32_t)__cvta_generic_to_shared(&mbar[lc & 1]), (uint32_t)((lc >> 1) & 1))) w_mma = nchunks;
            else fail();
        }
        if (bad) {
            // drain (bounded, in issue order) what may still be in flight, so that no copy lands
            // in and no MMA reads this CTA's shared memory after it has exited: the boxes of the
            // last two chunks issued (a stage is refilled only after every converter has passed
            // its wait), the packed operands and the MMAs not yet waited for.  Each is the oldest
            // pending phase of its barrier, or already complete.
            for (int cc = n_tma > kGtrRaw ? n_tma - kGtrRaw : 0; cc < n_tma; ++cc)
                gtc_wait((uint32_t)__cvta_generic_to_shared(&rbar[cc % kGtrRaw]), (uint32_t)((cc / kGtrRaw) & 1));
            for (int cc = w_bulk; cc < n_bulk; ++cc)
                gtc_wait((uint32_t)__cvta_generic_to_shared(&lbar[cc % kGtrCst]), (uint32_t)((cc / kGtrCst) & 1));
            for (int cc = w_mma; cc < n_mma; ++cc)
                gtc_wait((uint32_t)__cvta_generic_to_shared(&mbar[cc & 1]), (uint32_t)((cc >> 1) & 1));
        }
    }
    __syncthreads();
    gtc_epilogue<EPI>(a, g, tbase, m0, n0, bad != 0, reinterpret_cast<float*>(gsm));
}

__global__ void k_host_copies(HostCopies h, ull* ctr) {
    count_launch(ctr);
    const int i = blockIdx.y;
    const double* __restrict__ src = h.src[i];
    double* __restrict__ dst = h.dst[i];
    const long n = h.len[i];
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) dst[j] = src[j];
}
void launch_host_copies(const HostCopies& h, ull* ctr, cudaStream_t s) {
    if (h.n <= 0) return;
    long mx = 0;
    for (int i = 0; i < h.n; ++i) mx = h.len[i] > mx ? h.len[i] : mx;
    const int bx = (int)std::min<long>((mx + 255) / 256, 96);  // about 2 MB in flight per copy row
    k_host_copies<<<dim3(bx, h.n), 256, 0, s>>>(h, ctr);
}

// cuTensorMapEncodeTiled, fetched from the driver once (no link against libcuda)
typedef CUresult (*GtrEncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static GtrEncodeFn gtr_encoder() {
    static GtrEncodeFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<GtrEncodeFn>(p);
    }
    return fn;
}

// The tensor map of the data operand for k_gemm_tc_tma, or false when the pass does not meet
// TMA's alignment rules (16-byte base and row stride; for FOLD_A the mirror box's x = L - k0 - 31
// must be a multiple of 4, i.e. L + 1 a multiple of 4) or has no packed constant operand.
static bool gtr_map(const GemmArgs<float>& a, CUtensorMap* tm) {
    if (!a.packed || (a.fold != FOLD_A && a.fold != FOLD_B) || a.Lf < 2 * kGtcK + 1) return false;
    GtrEncodeFn enc = gtr_encoder();
    if (!enc) return false;
    const bool fa = a.fold == FOLD_A;
    const float* X = fa ? a.A : a.B;
    const long ld = fa ? a.lda : a.ldb;
    if ((reinterpret_cast<uintptr_t>(X) & 15) || (ld % 4) || (fa && (a.Lf + 1) % 4)) return false;
    cuuint64_t dim[2], stride[1] = {(cuuint64_t)ld * 4};
    cuuint32_t box[2], es[2] = {1, 1};
    if (fa) {  // X is M rows of L + 1 values
        dim[0] = (cuuint64_t)a.Lf + 1; dim[1] = (cuuint64_t)a.M;
        box[0] = kGtcK; box[1] = kGtcM;
    } else {   // X is L + 1 rows of N values
        dim[0] = (cuuint64_t)a.N; dim[1] = (cuuint64_t)a.Lf + 1;
        box[0] = kGtcN; box[1] = kGtcK;
    }
    if ((long)dim[0] > ld) return false;
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(X), dim, stride, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, fa ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Pre-pass of the pre-folded tensor-core GEMM (FOLD_A rows that TMA cannot address): rows
// [0, M) of `out` receive the even-folded operand x[j] + x[L - j] (x[j] at the middle point
// j = L / 2), rows [M, 2M) the odd one x[j] - x[L - j] (0 at the middle point), for j < K, and
// zeros in [K, ld): the values GemmView::loadA and the TMA kernel's fold form.
__global__ void k_gtr_prefold(const float* __restrict__ X, long lda, int M, int L, int K, int ld,
                              float* __restrict__ out) {
    const long tot = (long)M * ld;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < tot; e += (long)gridDim.x * blockDim.x) {
        const int m = (int)(e / ld), j = (int)(e % ld);
        float ev = 0.f, od = 0.f;
        if (j < K) {
            const float* row = X + (long)m * lda;
            const float x0 = row[j];
            if (2 * j == L) {
                ev = x0;
            } else {
                const float x1 = row[L - j];
                ev = x0 + x1;
                od = x0 - x1;
            }
        }
        out[e] = ev;
        out[tot + e] = od;
    }
}

// The pre-folded form for a FOLD_A pass that gtr_map refuses: runs the pre-pass into a.pad and
// encodes the tensor map of its 2M rows of ld = K rounded up to 4 values; false when there is no
// scratch (or too little), no packed operand or no encoder.
static bool gtr_prefold(const GemmArgs<float>& a, CUtensorMap* tm, cudaStream_t s) {
    if (a.fold != FOLD_A || !a.packed || !a.pad) return false;
    GtrEncodeFn enc = gtr_encoder();
    if (!enc) return false;
    const int ld = (a.K + 3) & ~3;
    if (2L * a.M * ld > a.pad_cap || (reinterpret_cast<uintptr_t>(a.pad) & 15)) return false;
    cuuint64_t dim[2] = {(cuuint64_t)ld, 2 * (cuuint64_t)a.M}, stride[1] = {(cuuint64_t)ld * 4};
    cuuint32_t box[2] = {kGtcK, kGtcM}, es[2] = {1, 1};
    if (enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, a.pad, dim, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const long tot = (long)a.M * ld;
    const int blocks = (int)std::min<long>((tot + 255) / 256, 152L * 8);
    k_gtr_prefold<<<blocks, 256, 0, s>>>(a.A, a.lda, a.M, a.Lf, a.K, ld, a.pad);
    return true;
}

static void gemm_tc_launch(int epi, const GemmArgs<float>& a, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_gemm_tc<EPI_STORE>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGtcSmem);
        cudaFuncSetAttribute(k_gemm_tc<EPI_DIV_TAB>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGtcSmem);
        cudaFuncSetAttribute(k_gemm_tc_tma<EPI_STORE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGtrSmem);
        cudaFuncSetAttribute(k_gemm_tc_tma<EPI_DIV_TAB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGtrSmem);
        cudaFuncSetAttribute(k_gemm_tc_tma<EPI_STORE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGtrSmem);
        cudaFuncSetAttribute(k_gemm_tc_tma<EPI_DIV_TAB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGtrSmem);
        attr = true;
    }
    const int M = a.fold == FOLD_B ? (a.M > a.M_odd ? a.M : a.M_odd) : a.M;
    const int N = a.fold == FOLD_A ? (a.N > a.N_odd ? a.N : a.N_odd) : a.N;
    dim3 grid((N + kGtcN - 1) / kGtcN, (M + kGtcM - 1) / kGtcM, a.fold ? 2 : 1);
    alignas(64) CUtensorMap tm;
    if (!std::getenv("DRD_GEMM_TC_NOTMA")) {  // the variable selects the register-staged fallback (tests)
        if (gtr_map(a, &tm)) {
            if (epi == EPI_DIV_TAB) k_gemm_tc_tma<EPI_DIV_TAB, false><<<grid, kGtrThreads, kGtrSmem, s>>>(a, tm);
            else k_gemm_tc_tma<EPI_STORE, false><<<grid, kGtrThreads, kGtrSmem, s>>>(a, tm);
            return;
        }
        if (gtr_prefold(a, &tm, s)) {
            if (epi == EPI_DIV_TAB) k_gemm_tc_tma<EPI_DIV_TAB, true><<<grid, kGtrThreads, kGtrSmem, s>>>(a, tm);
            else k_gemm_tc_tma<EPI_STORE, true><<<grid, kGtrThreads, kGtrSmem, s>>>(a, tm);
            return;
        }
    }
    if (epi == EPI_DIV_TAB) k_gemm_tc<EPI_DIV_TAB><<<grid, kGtcThreads, kGtcSmem, s>>>(a);
    else k_gemm_tc<EPI_STORE><<<grid, kGtcThreads, kGtcSmem, s>>>(a);
}

int gemm_config_count(int fp64) { return fp64 ? 14 : 9; }
const char* gemm_config_name(int cfg) { return kGemmCfgs[cfg].name; }

template <typename T, int BM, int BN, int TM, int TN, int KS, int EPI>
static void gemm_sk_launch(const GemmArgs<T>& a, cudaStream_t s) {
    constexpr int NT = (BM / TM) * (BN / TN);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((a.N + BN - 1) / BN, (a.M + BM - 1) / BM, KS * (a.fold ? 2 : 1));
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = KS;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_gemm_sk<T, BM, BN, 16, TM, TN, KS, EPI>, a);
}

template <typename T, int BM, int BN, int TM, int TN, int KS>
static void gemm_sk_dispatch(int epi, const GemmArgs<T>& a, cudaStream_t s) {
    switch (epi) {
        case EPI_STORE: gemm_sk_launch<T, BM, BN, TM, TN, KS, EPI_STORE>(a, s); break;
        case EPI_DIV_TAB: gemm_sk_launch<T, BM, BN, TM, TN, KS, EPI_DIV_TAB>(a, s); break;
        case EPI_SCALE: gemm_sk_launch<T, BM, BN, TM, TN, KS, EPI_SCALE>(a, s); break;
        default: gemm_sk_launch<T, BM, BN, TM, TN, KS, EPI_PRE_FINAL>(a, s); break;
    }
}

template <typename T, int BM, int BN, int TM, int TN>
static void gemm_dispatch_epi(int epi, const GemmArgs<T>& a, cudaStream_t s) {
    dim3 grid((a.N + BN - 1) / BN, (a.M + BM - 1) / BM, a.fold ? 2 : 1);
    constexpr int NT = (BM / TM) * (BN / TN);
    switch (epi) {
        case EPI_STORE: k_gemm<T, BM, BN, 16, TM, TN, EPI_STORE><<<grid, NT, 0, s>>>(a); break;
        case EPI_DIV_TAB: k_gemm<T, BM, BN, 16, TM, TN, EPI_DIV_TAB><<<grid, NT, 0, s>>>(a); break;
        case EPI_SCALE: k_gemm<T, BM, BN, 16, TM, TN, EPI_SCALE><<<grid, NT, 0, s>>>(a); break;
        default: k_gemm<T, BM, BN, 16, TM, TN, EPI_PRE_FINAL><<<grid, NT, 0, s>>>(a); break;
    }
}

template <typename T>
void launch_gemm(int cfg, int epi, const GemmArgs<T>& a, cudaStream_t s) {
    switch (cfg) {
        case 0: gemm_dispatch_epi<T, 64, 64, 4, 4>(epi, a, s); break;
        case 1: gemm_dispatch_epi<T, 32, 64, 2, 4>(epi, a, s); break;
        case 2: gemm_dispatch_epi<T, 32, 32, 2, 2>(epi, a, s); break;
        case 3: gemm_dispatch_epi<T, 16, 32, 1, 2>(epi, a, s); break;
        case 4: gemm_sk_dispatch<T, 32, 64, 4, 4, 4>(epi, a, s); break;
        case 5: gemm_sk_dispatch<T, 32, 32, 4, 4, 4>(epi, a, s); break;
        case 6: gemm_sk_dispatch<T, 16, 64, 2, 4, 4>(epi, a, s); break;
        case 7: gemm_sk_dispatch<T, 32, 32, 2, 2, 8>(epi, a, s); break;
        case 8: gemm_sk_dispatch<T, 32, 64, 4, 4, 2>(epi, a, s); break;
        default:
            if constexpr (sizeof(T) == 8) {
                if (cfg == 9) gemm_df_dispatch<64, 64, 4, 4>(epi, a, s);
                else if (cfg == 10) gemm_df_dispatch<32, 64, 2, 4>(epi, a, s);
                else if (cfg == 11) gemm_df_dispatch<32, 32, 2, 2>(epi, a, s);
                else if (cfg == 12) gemm_df_dispatch<16, 32, 1, 2>(epi, a, s);
                else gemm_df_dispatch<16, 16, 1, 1>(epi, a, s);
            } else {
                // kGemmTcCfg: the tensor-core GEMM for the folded passes it covers
                if (cfg == kGemmTcCfg && a.fold != FOLD_NONE && (epi == EPI_STORE || epi == EPI_DIV_TAB))
                    gemm_tc_launch(epi, reinterpret_cast<const GemmArgs<float>&>(a), s);
                else
                    gemm_dispatch_epi<T, 64, 64, 4, 4>(epi, a, s);
            }
            break;
    }
}
template void launch_gemm<double>(int, int, const GemmArgs<double>&, cudaStream_t);
template void launch_gemm<float>(int, int, const GemmArgs<float>&, cudaStream_t);

// ======================================================================================
// BiCGSTAB (lib/BiCGSTABREVCOM.f:150-418, lib/STOPTEST2.f:281-290) as element-wise kernels
// with fused partial dot products and one-block scalar kernels.  Dot products are summed in
// FP64 in a fixed order (deterministic for a fixed grid).
// Partials slots (a kernel never reads a slot it writes, since other blocks may still be
// reading it): 0 = ||r||^2 (and init/residual norms), 1 = (rtld, r), 3 = ||b||^2,
// 4 = (rtld, v), 5 = ||s||^2, 6 = (t, s), 7 = (t, t).  RHO, ALPHA and OMEGA are computed
// redundantly by every block of the vector kernel that needs them, from the partials in a
// fixed order, so all blocks agree and no one-block scalar kernel is launched for them.
// ======================================================================================
static __device__ const double kBreakTol = 1.2325951644078309e-32;  // DLAMCH('E')**2 (getbreak.f)
// Mixed mode: a refinement sweep that reduces the FP64 residual by less than 10 % tightens the
// inner FP32 solves' tolerance tenfold, down to this floor; a stall at the floor ends the solve.
static __device__ const double kMixedItolFloor = 1.5e-4;

template <typename T>
__global__ void k_bi_init1(long n, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ r, Dots d,
                           ull* ctr) {
    count_launch(ctr);
    double ax = 0.0, ab = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const T bv = b[q], xv = x[q];
        r[q] = bv;
        ax += (double)xv * (double)xv;
        ab += (double)bv * (double)bv;
    }
    __shared__ double sm[32];
    double r1 = block_sum<DRD_TPB>(ax, sm);
    if (threadIdx.x == 0) d.part[0 * DRD_MAXB + blockIdx.x] = r1;
    double r2 = block_sum<DRD_TPB>(ab, sm);
    if (threadIdx.x == 0) d.part[3 * DRD_MAXB + blockIdx.x] = r2;
}

// Start of BICGSTABREVCOM (:153-255) up to the x0 test.
__global__ void k_bi_init2(KState* ks, Dots d, double tol, int maxit, const KState* parent, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const double xx = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    const double bb = reduce_partials<DRD_TPB>(d.part + 3 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        ks->tol = parent != nullptr ? parent->itol : tol;  // an inner solve takes its parent's tolerance
        ks->maxit = maxit;
        ks->info = 0;
        ks->flags = 0u;
        ks->iter = maxit;   // ITER keeps MAXIT if the x0 test ends the solve (:248)
        ks->resid = ks->tol;  // RESID keeps TOL in that case
        ks->xnorm = sqrt(xx);
        ks->x_nonzero = (ks->xnorm != 0.0);
        ks->bnorm_raw = sqrt(bb);
        ks->bnrm2 = (ks->bnorm_raw == 0.0) ? 1.0 : ks->bnorm_raw;
        ks->rho = ks->rho1 = ks->alpha = ks->omega = ks->beta = 0.0;
        ks->first_next = 1;
        ks->mixed = 0;
        ks->do_update = 0;
        ks->restart = 0;
        ks->phase = (maxit <= 0) ? PH_DONE : PH_RUNNING;
        if (maxit <= 0) ks->info = -3;
        if (parent != nullptr && parent->phase != PH_RUNNING) ks->phase = PH_DONE;
    }
}

// The x0 test (:248) after r = b - A x0 (gated matvec wrote ||r||^2 into slot 0).
__global__ void k_bi_init3(KState* ks, Dots d, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const int run = (ks->phase == PH_RUNNING);
    const int xnz = ks->x_nonzero;
    double rr = 0.0;
    if (run && xnz) rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0 && run) {
        if (xnz && sqrt(rr) <= ks->tol) {
            ks->phase = PH_DONE;
            ks->info = 0;
            ks->flags |= DRD_FLAG_EARLY_X0;
        } else {
            ks->iter = 0;
        }
    }
}

// rtld = r and the first rho partials (rtld, r) into slot 1.
template <typename T>
__global__ void k_bi_init4(long n, const T* __restrict__ r, T* __restrict__ rtld, Dots d, const KState* ks,
                           ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, G_RUNNING)) return;
    double a = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const T rv = r[q];
        rtld[q] = rv;
        a += (double)rv * (double)rv;
    }
    __shared__ double sm[32];
    double s = block_sum<DRD_TPB>(a, sm);
    if (threadIdx.x == 0) d.part[1 * DRD_MAXB + blockIdx.x] = s;
}

// ITER = ITER + 1; RHO = (rtld, r); breakdown test; BETA (:261-269); then P = R (first
// iteration) or P = beta (P - omega V) + R (:268-275), fused with the preconditioner when it
// is diagonal (Jacobi) or the identity.
template <typename T>
__global__ void k_bi_p(long n, const T* __restrict__ r, const T* __restrict__ v, T* __restrict__ p,
                       T* __restrict__ phat, const T* __restrict__ diag, int ident, KState* ks, Dots d, ull* ctr) {
    count_launch(ctr);
    if (ks->phase != PH_RUNNING) return;
    __shared__ double sm[32];
    __shared__ double s_rho;
    const double rr = reduce_partials<DRD_TPB>(d.part + 1 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) s_rho = rr;
    __syncthreads();
    const double rho = s_rho;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (fabs(rho) < kBreakTol) {
        if (lead) {
            ks->iter = ks->iter + 1;
            ks->rho = rho;
            ks->info = -10;
            ks->phase = PH_DONE;
        }
        return;
    }
    const bool first = ks->first_next != 0;
    const double beta_d = first ? 0.0 : (rho / ks->rho1) * (ks->alpha / ks->omega);
    if (lead) {
        ks->iter = ks->iter + 1;
        ks->rho = rho;
        ks->beta = beta_d;
    }
    const T beta = (T)beta_d, nomega = (T)(-ks->omega);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        T pv;
        if (first) pv = r[q];
        else {
            pv = p[q] + nomega * v[q];
            pv = beta * pv;
            pv = pv + r[q];
        }
        p[q] = pv;
        if (diag) phat[q] = pv / diag[q];
        else if (ident) phat[q] = pv;
    }
}

// ALPHA = RHO / (rtld, v) (:307) from slot 4, then S = R - ALPHA V (:311-312, S aliases R)
// with ||S||^2 partials (slot 5).
template <typename T>
__global__ void k_bi_s(long n, const T* __restrict__ v, T* __restrict__ r, KState* ks, Dots d, ull* ctr) {
    count_launch(ctr);
    if (ks->phase != PH_RUNNING) return;
    __shared__ double sm[32];
    __shared__ double s_rv;
    const double rv0 = reduce_partials<DRD_TPB>(d.part + 4 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) s_rv = rv0;
    __syncthreads();
    const double rv = s_rv;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (ks->mixed && !(fabs(rv) > 0.0)) {  // mixed: fold and restart instead of dividing by zero
        if (lead) {
            ks->alpha = 0.0;
            ks->phase = PH_EARLY;
            ks->first_next = 0;
        }
        return;
    }
    const double alpha = ks->rho / rv;
    if (lead) {
        ks->alpha = alpha;
        ks->first_next = 0;  // every block of k_bi_p has read it
    }
    const T na = (T)(-alpha);
    double a = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const T sv = r[q] + na * v[q];
        r[q] = sv;
        a += (double)sv * (double)sv;
    }
    double t = block_sum<DRD_TPB>(a, sm);
    if (threadIdx.x == 0) d.part[5 * DRD_MAXB + blockIdx.x] = t;
}

// Early absolute test ||S|| <= TOL (:313-316).
// In mixed mode the test is relative (||s|| <= tol ||b|| / 10, or s == 0): the iteration then
// stops after the ALPHA half-step, and a reliable update decides on the FP64 residual.
__global__ void k_bi_snorm(KState* ks, Dots d, ull* ctr) {
    count_launch(ctr);
    if (ks->phase != PH_RUNNING) return;
    __shared__ double sm[32];
    const double ss = reduce_partials<DRD_TPB>(d.part + 5 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        ks->snorm = sqrt(ss);
        if (ks->mixed) {
            if (ks->snorm == 0.0 || ks->snorm <= 0.1 * ks->tol * ks->bnrm2 || !isfinite(ks->snorm)) {
                ks->phase = PH_EARLY;
                ks->flags |= DRD_FLAG_EARLY_S;
            }
        } else if (ks->snorm <= ks->tol) {
            ks->phase = PH_EARLY;
            ks->resid = ks->snorm / ks->bnrm2;
            ks->info = 0;
            ks->flags |= DRD_FLAG_EARLY_S;
        }
    }
}

template <typename T>
__global__ void k_bi_diag_apply(long n, const T* __restrict__ x, const T* __restrict__ diag, int ident,
                                T* __restrict__ y, const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        y[q] = ident ? x[q] : x[q] / diag[q];
}

// The solid-blended CH preconditioner's last step: y = q + w (x - q) with q = PSolve_CG(x)
// already in y (an extension of PhSolve.f90:296-313, w per packed cell).
template <typename T>
__global__ void k_pc_blend(long n, const T* __restrict__ x, const T* __restrict__ w, T* __restrict__ y,
                           const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const T v = y[q];
        y[q] = v + w[q] * (x[q] - v);
    }
}

// DRD_UV_ESOLP_SCALED's diagonal scaling s = sqrt(D0 / D): D the Jacobi diagonal of PSolve_uv_2_CG
// with rho and eta, D0 with rho = eta = 1.
template <typename T>
__global__ void k_uv_esolp_scale(OpScal<T> o, const T* __restrict__ rho, const T* __restrict__ eta, long n,
                                 T* __restrict__ s, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        s[q] = sqrt(uv_diag<T, true>(o, rho, eta, q) / uv_diag<T>(o, rho, eta, q));
}
// out = a s element-wise (out may be a), gated like the solve's other vector passes.
template <typename T>
__global__ void k_vmul(long n, const T* a, const T* __restrict__ s, T* out, const KState* ks, int gate, ull* ctr) {
    count_launch(ctr);
    if (gate_closed(ks, gate)) return;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        out[q] = a[q] * s[q];
}

// Entry q of Rademacher probe `probe`: the sign of the top bit of splitmix64(seed + (probe n +
// q + 1) G), G = 0x9E3779B97F4A7C15.
__device__ __forceinline__ double probe_sign(unsigned long long seed, long probe, long n, long q) {
    unsigned long long z = seed + (unsigned long long)(probe * n + q + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (z >> 63) ? -1.0 : 1.0;
}
__global__ void k_probe_fill(long n, unsigned long long seed, long probe, double* __restrict__ e, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        e[q] = probe_sign(seed, probe, n, q);
}
// With r = A e and qv = PSolve_CG(r): d = r - qv, t = e - qv; num += t d, den += d d.
__global__ void k_probe_acc(long n, unsigned long long seed, long probe, const double* __restrict__ r,
                            const double* __restrict__ qv, double* __restrict__ num, double* __restrict__ den,
                            int first, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double e = probe_sign(seed, probe, n, q), qq = qv[q];
        const double d = r[q] - qq, t = e - qq;
        num[q] = first ? t * d : fma(t, d, num[q]);
        den[q] = first ? d * d : fma(d, d, den[q]);
    }
}
// w = clamp(num / den, 0, 1), 0 where den = 0; FP64 and FP32 copies.
__global__ void k_probe_final(long n, const double* __restrict__ num, const double* __restrict__ den,
                              double* __restrict__ w, float* __restrict__ w32, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double dd = den[q];
        double v = dd > 0.0 ? num[q] / dd : 0.0;
        v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
        w[q] = v;
        w32[q] = (float)v;
    }
}

// OMEGA = (t, s) / (t, t) (:349-350) from slots 6/7, then X = X + ALPHA PHAT (+ OMEGA SHAT);
// R = R - OMEGA T (:314, :354-359) with ||R||^2 (slot 0) and (rtld, R) (slot 1) partials for
// STOPTEST2 and the next RHO.
template <typename T>
__global__ void k_bi_xr(long n, const T* __restrict__ phat, const T* __restrict__ shat, const T* __restrict__ t,
                        const T* __restrict__ rtld, T* __restrict__ x, T* __restrict__ r, KState* ks, Dots d,
                        ull* ctr) {
    count_launch(ctr);
    const int ph = ks->phase;
    if (ph == PH_DONE) return;
    const T al = (T)ks->alpha;
    if (ph == PH_EARLY) {
        for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
            x[q] = x[q] + al * phat[q];
        return;
    }
    __shared__ double sm[32];
    __shared__ double s_om;
    const double ts = reduce_partials<DRD_TPB>(d.part + 6 * DRD_MAXB, d.G, sm);
    const double tt = reduce_partials<DRD_TPB>(d.part + 7 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) s_om = (ks->mixed && !(tt > 0.0)) ? 0.0 : ts / tt;  // mixed: restart on omega = 0
    __syncthreads();
    const double omega = s_om;
    if (blockIdx.x == 0 && threadIdx.x == 0) ks->omega = omega;
    const T om = (T)omega, nom = (T)(-omega);
    double a0 = 0.0, a1 = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        T xv = x[q] + al * phat[q];
        xv = xv + om * shat[q];
        x[q] = xv;
        const T rv = r[q] + nom * t[q];
        r[q] = rv;
        a0 += (double)rv * (double)rv;
        a1 += (double)rtld[q] * (double)rv;
    }
    double s0 = block_sum<DRD_TPB>(a0, sm);
    if (threadIdx.x == 0) d.part[0 * DRD_MAXB + blockIdx.x] = s0;
    double s1 = block_sum<DRD_TPB>(a1, sm);
    if (threadIdx.x == 0) d.part[1 * DRD_MAXB + blockIdx.x] = s1;
}

// STOPTEST2 (:361-362 via lib/STOPTEST2.f:286-290), MAXIT test (:376-379), OMEGA breakdown
// (:383-388); sets the WHILE condition of the captured loop.  Iterations with a non-finite
// residual end the solve with DRD_ERR_NONFINITE instead of running on to MAXIT.
__global__ void k_bi_end(KState* ks, Dots d, cudaGraphConditionalHandle h, int use_graph, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const int ph = ks->phase;
    double rr = 0.0;
    if (ph == PH_RUNNING) rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        if (ph == PH_EARLY) {
            ks->phase = PH_DONE;
        } else if (ph == PH_RUNNING) {
            const double resid = sqrt(rr) / ks->bnrm2;
            ks->resid = resid;
            if (!isfinite(resid)) {
                ks->info = DRD_ERR_NONFINITE;
                ks->phase = PH_DONE;
            } else if (resid <= ks->tol) {
                ks->info = 0;
                ks->phase = PH_DONE;
            } else if (ks->iter >= ks->maxit) {
                ks->info = 1;
                ks->phase = PH_DONE;
            } else if (fabs(ks->omega) < kBreakTol) {
                ks->info = (fabs(ks->rho) < kBreakTol) ? -10 : -11;
                ks->phase = PH_DONE;
            } else {
                ks->rho1 = ks->rho;
            }
        }
        if (use_graph) cudaGraphSetConditional(h, ks->phase == PH_RUNNING ? 1u : 0u);
    }
}

// Sets a WHILE node's condition from the state it loops on.  Runs right before the node: a
// handle's default value is only applied when the top-level graph launches, so a loop nested
// in another loop's body must be re-armed each time the outer body runs.
__global__ void k_arm_while(const KState* ks, cudaGraphConditionalHandle h, ull* ctr) {
    count_launch(ctr);
    if (threadIdx.x == 0) cudaGraphSetConditional(h, ks->phase == PH_RUNNING ? 1u : 0u);
}

// ||b - A x|| / ||b|| from slot 0 (the residual's partials) and the stored ||b||.
__global__ void k_bi_true_resid(KState* ks, Dots d, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const double rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) ks->true_resid = sqrt(rr) / (ks->bnorm_raw == 0.0 ? 1.0 : ks->bnorm_raw);
}

template <typename T>
__global__ void k_copy(long n, const T* __restrict__ x, T* __restrict__ y, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) y[q] = x[q];
}

template <typename TO, typename TI>
__global__ void k_convert(long n, const TI* __restrict__ x, double scale, TO* __restrict__ y, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        y[q] = (TO)(scale * (double)x[q]);
}

template <typename T>
__global__ void k_norm2_partial(long n, const T* __restrict__ x, Dots d, int slot, ull* ctr) {
    count_launch(ctr);
    double a = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        a += (double)x[q] * (double)x[q];
    __shared__ double sm[32];
    double r = block_sum<DRD_TPB>(a, sm);
    if (threadIdx.x == 0) d.part[slot * DRD_MAXB + blockIdx.x] = r;
}

// ---- mixed precision: FP32 BiCGSTAB with FP64 reliable updates ---------------------------
// One FP32 BiCGSTAB runs on; whenever its recursive residual fell a decade below the last true
// residual (or claims convergence, or the iteration cap is hit), the FP32 increment is folded
// into the FP64 solution, b - A x is recomputed with the FP64 operator and replaces the
// recursive residual.  Convergence is decided on that FP64 residual only.

// After r64 = b - A x64 (slot 0) and ||b||^2 (slot 3).
__global__ void k_mr_init(KState* ks, Dots d, double tol, int maxit, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const double rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    const double bb = reduce_partials<DRD_TPB>(d.part + 3 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        ks->tol = tol;
        ks->maxit = maxit;
        ks->bnorm_raw = sqrt(bb);
        ks->bnrm2 = (ks->bnorm_raw == 0.0) ? 1.0 : ks->bnorm_raw;
        ks->rmax = sqrt(rr);
        ks->resid = ks->rmax / ks->bnrm2;
        ks->true_resid = ks->resid;
        ks->iter = 0;
        ks->inner_total = 0;
        ks->outer = 0;
        ks->info = 0;
        ks->flags = DRD_FLAG_REFINED;
        ks->rho = ks->rho1 = ks->alpha = ks->omega = ks->beta = 0.0;
        ks->first_next = 1;
        ks->mixed = 1;
        ks->do_update = 0;
        ks->restart = 0;
        ks->x_nonzero = 0;
        ks->phase = (ks->resid <= tol || ks->rmax == 0.0) ? PH_DONE : PH_RUNNING;
        if (!isfinite(ks->resid)) { ks->info = DRD_ERR_NONFINITE; ks->phase = PH_DONE; }
    }
}

// r32 = r64 (a fresh sequence also takes rtld = r32), and the (rtld, r) partials for the next RHO.
template <typename T>
__global__ void k_mr_reset(long n, const double* __restrict__ r64, T* __restrict__ r, T* __restrict__ rtld,
                           Dots d, const KState* ks, ull* ctr) {
    count_launch(ctr);
    if (ks->phase != PH_RUNNING) return;
    const bool fresh = ks->first_next != 0;
    double a = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const T rv = (T)r64[q];
        r[q] = rv;
        T tv;
        if (fresh) { rtld[q] = rv; tv = rv; }
        else tv = rtld[q];
        a += (double)tv * (double)rv;
    }
    __shared__ double sm[32];
    double s1 = block_sum<DRD_TPB>(a, sm);
    if (threadIdx.x == 0) d.part[1 * DRD_MAXB + blockIdx.x] = s1;
}

// End of an FP32 iteration: decides on a reliable update (IF node) and the loop condition.
__global__ void k_mr_end(KState* ks, Dots d, cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hif,
                         ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const int ph = ks->phase;
    double rr = 0.0;
    if (ph == PH_RUNNING) rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        int upd = 0;
        if (ph == PH_EARLY) {
            // the half-step ended the iteration: fold, recompute in FP64, restart the sequence
            upd = 1;
            ks->restart = 1;
            ks->phase = PH_RUNNING;
            ks->inner_total = ks->iter;
            ks->rho1 = ks->rho;
        } else if (ph == PH_RUNNING) {
            const double rn = sqrt(rr);
            ks->snorm = rn;
            ks->inner_total = ks->iter;
            if (!isfinite(rn)) upd = 1;
            else if (rn <= 0.1 * ks->rmax || rn / ks->bnrm2 <= ks->tol || ks->iter >= ks->maxit) upd = 1;
            else if (fabs(ks->omega) < kBreakTol) { upd = 1; ks->restart = 1; }
            ks->rho1 = ks->rho;
        } else if (ph == PH_DONE) {
            upd = 1;  // RHO breakdown this iteration: fold the FP32 increment in before stopping
        }
        ks->do_update = upd;
        cudaGraphSetConditional(hif, upd ? 1u : 0u);
        cudaGraphSetConditional(hw, (ks->phase == PH_RUNNING) ? 1u : 0u);
    }
}

// x64 += x32; x32 = 0
template <typename T>
__global__ void k_mr_fold(long n, T* __restrict__ x32, double* __restrict__ x64, ull* ctr) {
    count_launch(ctr);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        x64[q] = x64[q] + (double)x32[q];
        x32[q] = T(0);
    }
}

// After r64 = b - A x64 (slot 0): the FP64 convergence test and the loop condition.
__global__ void k_mr_check(KState* ks, Dots d, cudaGraphConditionalHandle hw, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const double rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        const double rn = sqrt(rr);
        const double tr = rn / ks->bnrm2;
        ks->outer += 1;
        ks->rmax = rn;
        ks->resid = tr;
        ks->true_resid = tr;
        if (!isfinite(tr)) { ks->info = DRD_ERR_NONFINITE; ks->phase = PH_DONE; }
        else if (tr <= ks->tol) { ks->info = 0; ks->phase = PH_DONE; }
        else if (ks->phase == PH_DONE) { /* breakdown: keep its INFO */ }
        else if (ks->iter >= ks->maxit) { ks->info = 1; ks->phase = PH_DONE; }
        else if (ks->restart) { ks->first_next = 1; ks->restart = 0; }
        ks->do_update = 0;
        cudaGraphSetConditional(hw, (ks->phase == PH_RUNNING) ? 1u : 0u);
    }
}

// ---- mixed-precision refinement ----------------------------------------------------------
// outer->snorm holds ||r64||; the FP32 system is solved for r64/||r64|| from a zero guess.
__global__ void k_mx_init(KState* o, Dots d, double tol, int max_refine, double itol, ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const double rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    const double bb = reduce_partials<DRD_TPB>(d.part + 3 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        o->tol = tol;
        o->itol = itol;
        o->maxit = max_refine;
        o->bnorm_raw = sqrt(bb);
        o->bnrm2 = (o->bnorm_raw == 0.0) ? 1.0 : o->bnorm_raw;
        o->snorm = sqrt(rr);
        o->resid = o->snorm / o->bnrm2;
        o->outer = 0;
        o->inner_total = 0;
        o->iter = 0;
        o->flags = DRD_FLAG_REFINED;
        o->info = 0;
        o->phase = (o->resid <= tol || o->snorm == 0.0) ? PH_DONE : PH_RUNNING;
        if (!isfinite(o->resid)) { o->info = DRD_ERR_NONFINITE; o->phase = PH_DONE; }
        o->true_resid = o->resid;
    }
}

template <typename TO>
__global__ void k_mx_scale_from_state(long n, const double* __restrict__ r, const KState* o, TO* __restrict__ y,
                                      TO* __restrict__ zero, ull* ctr) {
    count_launch(ctr);
    if (o->phase != PH_RUNNING) return;
    const double sc = 1.0 / o->snorm;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        y[q] = (TO)(r[q] * sc);
        zero[q] = TO(0);
    }
}

__global__ void k_mx_inner_setup(KState* in, const KState* o, double inner_tol, int inner_maxit, ull* ctr) {
    count_launch(ctr);
    if (threadIdx.x == 0) {
        const bool run = o->phase == PH_RUNNING;
        in->tol = inner_tol;
        in->maxit = inner_maxit;
        in->info = 0;
        in->flags = 0u;
        in->iter = 0;
        in->resid = 1.0;
        in->x_nonzero = 0;
        in->bnorm_raw = 1.0;
        in->bnrm2 = 1.0;
        in->rho = in->rho1 = in->alpha = in->omega = in->beta = 0.0;
        in->phase = run ? PH_RUNNING : PH_DONE;
    }
}

// x64 += ||r64|| d32
__global__ void k_axpy_f2d(long n, const KState* o, const float* __restrict__ d, double* __restrict__ x, ull* ctr) {
    count_launch(ctr);
    if (o->phase != PH_RUNNING) return;
    const double sc = o->snorm;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        x[q] = x[q] + sc * (double)d[q];
}

// True FP64 residual of the refined iterate (slot 0), refinement bookkeeping, WHILE condition.
__global__ void k_mx_check(KState* o, const KState* in, Dots d, cudaGraphConditionalHandle h, int use_graph,
                           ull* ctr) {
    count_launch(ctr);
    __shared__ double sm[32];
    const int run = o->phase == PH_RUNNING;
    double rr = 0.0;
    if (run) rr = reduce_partials<DRD_TPB>(d.part + 0 * DRD_MAXB, d.G, sm);
    if (threadIdx.x == 0) {
        if (run) {
            const double prev = o->resid;
            o->snorm = sqrt(rr);
            o->resid = o->snorm / o->bnrm2;
            o->true_resid = o->resid;
            o->outer += 1;
            o->inner_total += in->iter;
            o->iter = o->inner_total;
            if (in->info == DRD_ERR_TIMEOUT) { o->info = DRD_ERR_TIMEOUT; o->phase = PH_DONE; }
            else if (!isfinite(o->resid)) { o->info = DRD_ERR_NONFINITE; o->phase = PH_DONE; }
            else if (o->resid <= o->tol) { o->info = 0; o->phase = PH_DONE; }
            else if (o->outer >= o->maxit) { o->info = 1; o->phase = PH_DONE; }
            else if (o->resid > 0.9 * prev) {  // a sweep that gained < 10 %: tighten the inner solves
                if (o->itol > kMixedItolFloor) o->itol *= 0.1;
                else { o->info = 1; o->phase = PH_DONE; }  // stalled at the tightest inner tolerance
            }
        }
        if (use_graph) cudaGraphSetConditional(h, o->phase == PH_RUNNING ? 1u : 0u);
    }
}

// ======================================================================================
// Persistent cooperative BiCGSTAB for the FP32 inner solves of the mixed mode (CH and
// momentum systems).
//
// One cooperative launch (all blocks co-resident) runs the whole inner solve: setup and every
// iteration of lib/BiCGSTABREVCOM.f:229-388, with the same steps, tests and INFO codes as the
// k_bi_* kernels above, but with the phases of an iteration separated by grid-wide barriers
// instead of kernel boundaries.  Every block reduces the dot-product partials itself in a fixed
// order, so all blocks take the same decisions.  Data written in one phase by other blocks is
// read through L2 (ld.global.cg).  Each barrier's wait is bounded: a wait that runs out sets an
// error flag, the blocks leave the solve, and the state records DRD_ERR_TIMEOUT.
// ======================================================================================
namespace {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Optional phase timing: thread 0 of block 0 records %globaltimer at entry and exit of each
// barrier while `p` is set (one iteration of a solve), into p[2k], p[2k+1].
struct PbProf {
    unsigned long long* p;
    int k;
};
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Sub-phase mark: time at point `i` (0..3) of the first x pass of a timed iteration, p[124 + i].
__device__ __forceinline__ void pb_mark(const PbProf& pf, int i) {
    if (pf.p != nullptr && pf.k <= 1 && blockIdx.x == 0 && threadIdx.x == 0) pf.p[124 + i] = gtimer();
}
// Sub-phase mark of the first tridiagonal phase (ESOLP_x) of a timed iteration, p[106 + i].
__device__ __forceinline__ void pb_markt(const PbProf& pf, int i) {
    if (pf.p != nullptr && pf.k == 1 && blockIdx.x == 0 && threadIdx.x == 0) pf.p[106 + i] = gtimer();
}
// Sub-phase mark of the first z pass of a timed iteration, p[100 + i].
__device__ __forceinline__ void pb_markz(const PbProf* pf, int i) {
    if (pf != nullptr && pf->p != nullptr && pf->k == 1 && blockIdx.x == 0 && threadIdx.x == 0)
        pf->p[100 + i] = gtimer();
}

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier on one arrival counter, reset to zero before the launch: barrier k completes when
// the counter reaches k * gridDim.x.  Thread 0 publishes the block's writes with a release add
// (ordered after the block's writes by the preceding __syncthreads) and waits with acquire
// loads; `target` is its running count.
__device__ __noinline__ bool grid_sync(GridBar* gb, unsigned& target, PbProf& pf) {
    __shared__ int s_ok;
    __syncthreads();
    const bool rec = pf.p != nullptr && blockIdx.x == 0 && threadIdx.x == 0 && pf.k < 62;
    if (rec) pf.p[2 * pf.k] = gtimer();
    if (threadIdx.x == 0) {
        int ok = 1;
        target += gridDim.x;
        red_release_add(&gb->count, 1u);
        unsigned spins = 0;
        while ((int)(ld_acquire_u32(&gb->count) - target) < 0) {
            if (++spins > (1u << 22)) {  // seconds: a co-resident grid never gets here
                atomicExch(&gb->err, 1);
                ok = 0;
                break;
            }
        }
        if (*((volatile int*)&gb->err) != 0) ok = 0;
        s_ok = ok;
    }
    if (rec) pf.p[2 * pf.k++ + 1] = gtimer();
    __syncthreads();
    return s_ok != 0;
}

template <typename T>
struct PackedCG {  // packed vector written by other blocks in an earlier phase
    const T* p; int nr;
    __device__ __forceinline__ T operator()(int i, int k) const { return __ldcg(p + i + (long)nr * k); }
};

// Sum of a partials slot (gridDim.x values) in a fixed order, broadcast to the block.
template <int NT>
__device__ __forceinline__ double slot_sum(const double* part, int slot, double* sm) {
    double v = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += NT) v += __ldcg(part + slot * DRD_MAXB + q);
    const double r = block_sum<NT>(v, sm);
    __shared__ double s_b;
    if (threadIdx.x == 0) s_b = r;
    __syncthreads();
    const double out = s_b;
    __syncthreads();
    return out;
}

// Sums of two partials slots in one pass (one L2 round trip), broadcast to the block.
template <int NT>
__device__ __forceinline__ double2 slot_sum2(const double* part, int s1, int s2, double* sm) {
    double v1 = 0.0, v2 = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += NT) {
        v1 += __ldcg(part + s1 * DRD_MAXB + q);
        v2 += __ldcg(part + s2 * DRD_MAXB + q);
    }
    const double r1 = block_sum<NT>(v1, sm);
    __shared__ double s_b1;
    if (threadIdx.x == 0) s_b1 = r1;
    const double r2 = block_sum<NT>(v2, sm);  // its barriers also publish s_b1
    __shared__ double s_b2;
    if (threadIdx.x == 0) s_b2 = r2;
    __syncthreads();
    const double2 out = make_double2(s_b1, s_b2);
    __syncthreads();
    return out;
}

template <int NT>
__device__ __forceinline__ void slot_put(double* part, int slot, double v, double* sm) {
    const double r = block_sum<NT>(v, sm);
    if (threadIdx.x == 0) part[slot * DRD_MAXB + blockIdx.x] = r;
}

// GB300 issues FP64 at a small fraction of its FP32 rate, so the hot loop of the persistent
// solver does no FP64 work at all: its dot products, their block and grid sums and the scalar
// steps of an iteration are FP32, the precision of the inner solve itself (the FP64 work stays
// in the refinement around it).  A block partial is stored as an FP32 value in its slot of the
// partials buffer.  The scalar steps are evaluated by thread 0 and broadcast through shared
// memory.
__device__ __forceinline__ float* fslot(double* part, int slot, int b) {
    return reinterpret_cast<float*>(part + slot * DRD_MAXB + b);
}
// Grid sum of one FP32 partials slot by warp 0 (each lane its strided share in order, then an xor
// butterfly: every lane of every block gets the same bits).  Call from warp 0 only.
__device__ __forceinline__ float warp_slot_sum(double* part, int slot) {
    const int lane = threadIdx.x & 31;
    float v = 0.f;
    for (int q = lane; q < (int)gridDim.x; q += 32) v += __ldcg(fslot(part, slot, q));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block partials of up to three per-thread FP32 values into their slots (slot < 0: none).
template <int NT>
__device__ __forceinline__ void slots_put_f(double* part, int sl0, float v0, int sl1, float v1, int sl2, float v2,
                                            double* sm) {
    constexpr int NW = NT / 32;
    static_assert(3 * NW <= 128, "shared scratch");
    float* smf = reinterpret_cast<float*>(sm);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int sl[3] = {sl0, sl1, sl2};
    float v[3] = {v0, v1, v2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
        if (sl[i] >= 0)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    __syncthreads();  // an earlier sum may still read the scratch
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < 3; ++i) smf[i * NW + w] = v[i];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (sl[i] < 0) continue;
            float r = lane < NW ? smf[i * NW + lane] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
            if (lane == 0) *fslot(part, sl[i], blockIdx.x) = r;
        }
    }
}

constexpr int PB_NT = 512;  // threads per block of the persistent solver
// x-pass tile and K chunk (JA = 7 operand loads per thread).  A wide, short tile: every block
// whose tile covers a row reloads that row, so short tiles cut the operand traffic per SM, which
// bounds the load phase; 420x180 gives 12 x 8 = 96 tiles.
constexpr int PB_BM = 16, PB_BN = 64, PB_KC = 224;
constexpr int PB_AG = PB_BM / 4;  // float4 groups of an A row
constexpr int PB_CW = 4;                            // columns per z work item

// Shared-memory plan of the persistent CH solver (floats; see persist_ch_plan): the z-pass
// operands and the block's own x-pass B panel stay resident for the whole solve when they fit,
// so each transform phase only moves the vector data.
__device__ __forceinline__ int pb_xtiles(const PersistArgs& a, int& mt, int& nt0) {
    mt = (a.nz + PB_BM - 1) / PB_BM;
    nt0 = (a.Nxe + PB_BN - 1) / PB_BN;
    const int nt1 = (a.Nxo + PB_BN - 1) / PB_BN;
    return mt * (nt0 + nt1);
}

// Loads the resident operands at the start of the solve.
__device__ void pb_load_resident(const PersistArgs& a, float* smem) {
    if (a.z_res) {
        float* zA = smem + a.z_off;  // [2][Mze][Kz4], rows padded with zeros to a multiple of 4
        const int K = a.Kz, K4 = (K + 3) & ~3, tot = 2 * a.Mze * K4;
        for (int e = threadIdx.x; e < tot; e += PB_NT) {
            const int par = e / (a.Mze * K4), rest = e % (a.Mze * K4), m = rest / K4, jj = rest % K4;
            float v = 0.f;
            if (jj < K) {
                if (par == 0) v = __ldg(a.fze + (long)m * K + jj);
                else if (m < a.Mzo) v = __ldg(a.fzo + (long)m * K + jj);
            }
            zA[e] = v;
        }
    }
    if (a.b_res) {
        int mt, nt0;
        const int ntiles = pb_xtiles(a, mt, nt0);
        const int tile = blockIdx.x;
        if (tile < ntiles) {
            const int nrest = tile / mt, par = nrest >= nt0 ? 1 : 0, ntile = par ? nrest - nt0 : nrest;
            const int N = par ? a.Nxo : a.Nxe, n0 = ntile * PB_BN;
            const float* B = par ? a.fxo : a.fxe;
            float* Bs = smem + a.b_off;  // [Kx][PB_BN]
            for (int e = threadIdx.x; e < a.Kx * PB_BN; e += PB_NT) {
                const int kk = e / PB_BN, cc = e % PB_BN, n = n0 + cc;
                Bs[e] = n < N ? __ldg(B + (long)kk * a.Nxe + n) : 0.f;  // both stored Kx x Nxe
            }
        }
    }
    __syncthreads();
}

// x pass of the folded DCT-I: out[m][2n+p] = sum_k (X[m][k] +- X[m][L-k]) Bp[k][n], one
// PB_BM x PB_BN tile per block.  The block's 512 threads split K eight ways; each thread keeps
// a 4 x 4 register tile and reads its operands as float4 (two 16-byte shared loads per 16 FMA),
// and the eight partial tiles are summed through shared memory in a fixed order.
constexpr int PB_KG = 8;  // K groups of the x pass
__device__ __forceinline__ int pb_swz(int k, int m) {
    return k * PB_BM + ((((m >> 2) ^ (k & (PB_AG - 1))) << 2) | (m & 3));
}
static_assert((PB_BM / 4) * (PB_BN / 4) * PB_KG == PB_NT, "4 x 4 register tiles, PB_KG groups");
// bx, bw (optional): blend the result with bx as out = v + bw (bx - v) (the solid-blended CH
// preconditioner's last step; bx is the preconditioner's input, written inside this launch).
// One x-pass problem: the folded DCT-I of length L+1 along each of M rows (row stride ld) of X,
// out[m][2n+p] = sum_k (X[m][k] +- X[m][L-k]) Bp[k][n], with both Bp stored K x Ne; mt x (nt0 +
// nt1) tiles of PB_BM x PB_BN.
struct XProb {
    const float* X;
    float* out;
    int M, ld, L, K, Ne, No;
    const float *Be, *Bo;
    int mt, nt0, ntiles;
    const float* xs;  // optional: X is read as X xs (element-wise, same layout)
    const float* os;  // optional: out is written as the result times os
};
template <int BN = PB_BN>
__device__ __forceinline__ XProb xprob(const float* X, float* out, int M, int ld, int L, int K, int Ne, int No,
                                       const float* Be, const float* Bo) {
    XProb d{X, out, M, ld, L, K, Ne, No, Be, Bo, 0, 0, 0, nullptr, nullptr};
    d.mt = (M + PB_BM - 1) / PB_BM;
    d.nt0 = (Ne + BN - 1) / BN;
    d.ntiles = d.mt * (d.nt0 + (No + BN - 1) / BN);
    return d;
}

// One PB_BM x BN tile of problem d, K split KG ways.  Bres: the block's resident B panel of this
// tile ([K][BN]), or null (B chunks are then streamed from L2).  bx, bw (optional): blend the
// result with bx as out = v + bw (bx - v) (the solid-blended CH preconditioner's last step; bx is
// the preconditioner's input, written inside this launch).
template <int BN = PB_BN, int KG = PB_KG, int TM = 4>
__device__ __forceinline__ void pb_xtile(const XProb& d, int tile, const float* Bres, float* work, const PbProf& pf,
                                         const float* bx, const float* bw) {
    static_assert((PB_BM / TM) * (BN / 4) * KG == PB_NT, "TM x 4 register tiles, KG groups");
    static_assert(TM == 4 || TM == 8, "4 or 8 rows per thread");
    const int M = d.M, L = d.L, K = d.K;
    const float* X = d.X;
    float* out = d.out;
    float* At = work;                                     // [PB_KC][PB_BM], float4 groups swizzled by k
    float* Bw = At + PB_KC * PB_BM;                       // [PB_KC][BN] when B is not resident
    float* red = Bw + (Bres ? 0 : PB_KC * BN);         // [KG][PB_BM * BN]
    constexpr int TN = BN / 4;                         // threads of a K group along n
    constexpr int GT = (PB_BM / TM) * TN;                 // threads of a K group
    const int tid = threadIdx.x, g = tid / GT, t = tid % GT, mi = t / TN, ni = t % TN;
    {
        const int mtile = tile % d.mt, nrest = tile / d.mt;
        const int par = nrest >= d.nt0 ? 1 : 0;
        const int ntile = par ? nrest - d.nt0 : nrest;
        const int N = par ? d.No : d.Ne;
        const float* B = par ? d.Bo : d.Be;
        const int m0 = mtile * PB_BM, n0 = ntile * BN;
        float acc[TM][4];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
        for (int k0 = 0; k0 < K; k0 += PB_KC) {
            const int kc = min(PB_KC, K - k0);
            // all loads of the chunk first (one L2 round trip), then the folded stores
            constexpr int JA = PB_BM * PB_KC / PB_NT;
            float x0[JA], x1[JA];
            // element e = tid + j*PB_NT of the chunk is (row rr, column kk) = (e / kc, e % kc);
            // the quotient and remainder advance by those of PB_NT instead of dividing again
            const int dq = PB_NT / kc, dr = PB_NT % kc;
            int rr = tid / kc, kk = tid % kc;
#pragma unroll
            for (int j = 0; j < JA; ++j) {
                const int m = m0 + rr, k = k0 + kk;
                x0[j] = 0.f;
                x1[j] = 0.f;
                if (rr < PB_BM && m < M) {
                    const float* row = X + (long)m * d.ld;
                    x0[j] = __ldcg(row + k);
                    if (2 * k != L) x1[j] = __ldcg(row + L - k);
                    if (d.xs) {
                        const float* srow = d.xs + (long)m * d.ld;
                        x0[j] *= __ldg(srow + k);
                        if (2 * k != L) x1[j] *= __ldg(srow + L - k);
                    }
                }
                rr += dq;
                kk += dr;
                if (kk >= kc) { kk -= kc; rr += 1; }
            }
            __syncthreads();
            rr = tid / kc;
            kk = tid % kc;
#pragma unroll
            for (int j = 0; j < JA; ++j) {
                if (rr < PB_BM) {
                    // folded operand: x(k) + x(L-k) (even outputs) or x(k) - x(L-k) (odd); the
                    // middle column of an even L counts once and only for even outputs
                    const int k = k0 + kk;
                    float v = par ? x0[j] - x1[j] : x0[j] + x1[j];
                    if (2 * k == L) v = par ? 0.f : x0[j];
                    At[pb_swz(kk, rr)] = v;
                }
                rr += dq;
                kk += dr;
                if (kk >= kc) { kk -= kc; rr += 1; }
            }
            pb_mark(pf, 0);
            const float* Bk;
            if (Bres) {
                Bk = Bres + (long)k0 * BN;
            } else {
                for (int e = tid; e < kc * BN; e += PB_NT) {
                    const int kk = e / BN, cc = e % BN, n = n0 + cc;
                    Bw[e] = n < N ? __ldg(B + (long)(k0 + kk) * d.Ne + n) : 0.f;
                }
                Bk = Bw;
            }
            __syncthreads();
            const int kgn = (kc + KG - 1) / KG, kb = g * kgn, ke = min(kb + kgn, kc);
#pragma unroll 2
            for (int kk = kb; kk < ke; ++kk) {
                float ar[TM];
#pragma unroll
                for (int h = 0; h < TM / 4; ++h) {  // the thread's float4 row groups (TM / 4 of them)
                    const int grp = mi * (TM / 4) + h;
                    const float4 av = *reinterpret_cast<const float4*>(At + kk * PB_BM + ((grp ^ (kk & (PB_AG - 1))) << 2));
                    ar[4 * h] = av.x; ar[4 * h + 1] = av.y; ar[4 * h + 2] = av.z; ar[4 * h + 3] = av.w;
                }
                const float4 bv = *reinterpret_cast<const float4*>(Bk + kk * BN + (ni << 2));
                const float br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(ar[i], br[j], acc[i][j]);
            }
            pb_mark(pf, 1);
            __syncthreads();
        }
        // the eight K-group partial tiles, summed in group order
#pragma unroll
        for (int i = 0; i < TM; ++i)
            *reinterpret_cast<float4*>(red + g * (PB_BM * BN) + (TM * mi + i) * BN + 4 * ni) =
                make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
        __syncthreads();
        for (int o = tid; o < PB_BM * BN; o += PB_NT) {
            float v = 0.f;
#pragma unroll
            for (int gg = 0; gg < KG; ++gg) v += red[gg * (PB_BM * BN) + o];
            const int m = m0 + o / BN, n = n0 + o % BN;
            if (m < M && n < N) {
                const long q = (long)m * d.ld + 2 * n + par;
                float vo = bw ? v + __ldg(bw + q) * (__ldcg(bx + q) - v) : v;
                if (d.os) vo *= __ldg(d.os + q);
                out[q] = vo;
            }
        }
        pb_mark(pf, 2);
        __syncthreads();
    }
}


// x pass of the CH preconditioner over the packed nz x nr cells, one tile per block when the
// B panels are resident.
__device__ void pb_xpass(const PersistArgs& a, const float* X, float* out, float* smem, const PbProf& pf,
                         const float* bx = nullptr, const float* bw = nullptr) {
    const XProb d = xprob(X, out, a.nz, a.nr, a.nr - 1, a.Kx, a.Nxe, a.Nxo, a.fxe, a.fxo);
    const float* Bres = a.b_res ? smem + a.b_off : nullptr;
    for (int tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x)
        pb_xtile(d, tile, Bres, smem + a.work_off, pf, bx, bw);
}

// ---- ESOLP_x (Precipitation_dynamics/ESOLP.f90:1-54, VeloSolve_combined.f90:800-806) in the
// persistent momentum solver: per block of the packed vector (u: nz rows of nr+1, v: nz-1 rows of
// nr) VCOST along x, a tridiagonal solve along y per x mode, VCOST along x; three phases.

// Both blocks' row transforms as one tile space of PB_BM x PB_UBN tiles (8 x 4 register tiles, K
// split PB_UKG ways: the row operand is a warp broadcast, so each FMA costs half the shared-memory
// traffic of the 4 x 4 form),
// at most one tile per block at 420x180 and below; the block's own B panel stays in shared memory
// for the whole solve when the plan allows (a.b_res).
constexpr int PB_UBN = 128, PB_UKG = 8, PB_UTM = 8;
__device__ __forceinline__ void pb_uv_probs(const PersistArgs& a, const float* X, float* out, XProb& du, XProb& dv,
                                            const float* xs = nullptr, const float* os = nullptr) {
    const long mu = (long)(a.nr + 1) * a.nz;
    du = xprob<PB_UBN>(X, out, a.nz, a.nr + 1, a.nr, a.Ku, a.Nue, a.Nuo, a.fue, a.fuo);
    dv = xprob<PB_UBN>(X + mu, out + mu, a.nz - 1, a.nr, a.nr - 1, a.Kx, a.Nxe, a.Nxo, a.fxe, a.fxo);
    du.xs = xs; du.os = os;
    dv.xs = xs ? xs + mu : nullptr; dv.os = os ? os + mu : nullptr;
}
// xs, os (optional): scale the input / the output element-wise (DRD_UV_ESOLP_SCALED)
__device__ void pb_xpass_uv(const PersistArgs& a, const float* X, float* out, float* smem, const PbProf& pf,
                            const float* xs = nullptr, const float* os = nullptr) {
    XProb du, dv;
    pb_uv_probs(a, X, out, du, dv, xs, os);
    const int tot = du.ntiles + dv.ntiles;
    const float* Bres = a.b_res ? smem + a.b_off : nullptr;
    for (int tile = blockIdx.x; tile < tot; tile += gridDim.x) {
        if (tile < du.ntiles) pb_xtile<PB_UBN, PB_UKG, PB_UTM>(du, tile, Bres, smem, pf, nullptr, nullptr);
        else pb_xtile<PB_UBN, PB_UKG, PB_UTM>(dv, tile - du.ntiles, Bres, smem, pf, nullptr, nullptr);
    }
}
// The block's resident B panel ([K][PB_UBN]) of its tile, loaded once per launch.
__device__ void pb_load_resident_uv(const PersistArgs& a, float* smem) {
    XProb du, dv;
    pb_uv_probs(a, nullptr, nullptr, du, dv);
    const int tile = blockIdx.x;
    if (tile < du.ntiles + dv.ntiles) {
        const bool ub = tile < du.ntiles;
        const XProb& d = ub ? du : dv;
        const int tl = ub ? tile : tile - du.ntiles;
        const int nrest = tl / d.mt, par = nrest >= d.nt0 ? 1 : 0, ntile = par ? nrest - d.nt0 : nrest;
        const int N = par ? d.No : d.Ne, n0 = ntile * PB_UBN;
        const float* B = par ? d.Bo : d.Be;
        float* Bs = smem + a.b_off;
        for (int e = threadIdx.x; e < d.K * PB_UBN; e += PB_NT) {
            const int kk = e / PB_UBN, cc = e % PB_UBN, n = n0 + cc;
            Bs[e] = n < N ? __ldg(B + (long)kk * d.Ne + n) : 0.f;
        }
    }
    __syncthreads();
}

constexpr int PB_TRI_MB = 8;  // modes per batch of the tridiagonal phase (one warp each)

// The tridiagonal phase, in place on w: per x mode the forward elimination f_j = w_j + r_j f_{j-1}
// and the back substitution ff_j = (f_j - c_j ff_{j+1}) / b'_j (ff = 0 at the last row when
// |b'| <= 1e-12) with the factors of setup (rfords), held as r_j, 1/b'_j and c_j/b'_j.  A batch of PB_TRI_MB modes is staged in
// shared memory; each mode's warp splits its rows into 32 segments, composes each segment's
// affine map, scans the maps across the lanes, and then runs its segment from the scanned
// boundary value with the same recurrence.
__device__ void pb_tridiag_uv(const PersistArgs& a, float* w, float* smem, const PbProf& pf) {
    const int nr = a.nr, nz = a.nz;
    const long mu = (long)(nr + 1) * nz, mv = (long)nr * (nz - 1);
    const int nmu = nr + 1, total = 2 * nr + 1;
    // staged [PB_TRI_MB][nz]: a mode's rows are contiguous, so the lanes of its warp, which run
    // contiguous row segments, fall on distinct banks (2-way at most)
    float* sw = smem;                      // right-hand sides, then the solution
    float* sr = sw + nz * PB_TRI_MB;       // elimination factors r_j
    float* sb = sr + nz * PB_TRI_MB;       // 1 / b'_j
    float* sc = sb + nz * PB_TRI_MB;       // c_j / b'_j
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int g0 = blockIdx.x * PB_TRI_MB; g0 < total; g0 += gridDim.x * PB_TRI_MB) {
        __syncthreads();
        // staging: the loads of up to SU elements per thread are issued before any is stored
        constexpr int SU = 4;
        for (int e0 = 0; e0 < nz * PB_TRI_MB; e0 += SU * PB_NT) {
            float v[SU][4];
            int at[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                const int e = e0 + u * PB_NT + threadIdx.x;
                at[u] = -1;
                if (e >= nz * PB_TRI_MB) continue;
                const int sl = e % PB_TRI_MB, j = e / PB_TRI_MB, g = g0 + sl;
                if (g >= total) continue;
                const bool ub = g < nmu;
                const int k = ub ? g : g - nmu, len = ub ? nr + 1 : nr, rows = ub ? nz : nz - 1;
                if (j >= rows) continue;
                const float* f = ub ? a.esf : a.esf + 3 * mu;
                const long rb = ub ? mu : mv;
                const long q = k + (long)len * j;
                v[u][0] = __ldcg(w + (ub ? 0 : mu) + q);
                v[u][1] = __ldg(f + q);
                v[u][2] = __ldg(f + rb + q);
                v[u][3] = __ldg(f + 2 * rb + q);
                at[u] = sl * nz + j;
            }
#pragma unroll
            for (int u = 0; u < SU; ++u)
                if (at[u] >= 0) {
                    sw[at[u]] = v[u][0];
                    sr[at[u]] = v[u][1];
                    sb[at[u]] = v[u][2];
                    sc[at[u]] = v[u][3];
                }
        }
        __syncthreads();
        pb_markt(pf, 0);
        if (wp < PB_TRI_MB && g0 + wp < total) {
            const int sl = wp, g = g0 + sl;
            const int R = g < nmu ? nz : nz - 1;
            const int cl = (R + 31) / 32, j0 = lane * cl, j1 = min(j0 + cl, R);
            // forward: f_j = r_j f_{j-1} + w_j as maps (A, B) of f_{j-1}
            float A = 1.f, B = 0.f;
            for (int j = j0; j < j1; ++j) {
                const float r = sr[sl * nz + j];
                A = r * A;
                B = fmaf(r, B, sw[sl * nz + j]);
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {  // inclusive scan: lane l = segments 0..l
                const float Ap = __shfl_up_sync(0xffffffffu, A, o), Bp = __shfl_up_sync(0xffffffffu, B, o);
                if (lane >= o) { B = fmaf(A, Bp, B); A = A * Ap; }
            }
            float f = __shfl_up_sync(0xffffffffu, B, 1);  // f at the row before the segment (f_{-1} = 0)
            if (lane == 0) f = 0.f;
            for (int j = j0; j < j1; ++j) {
                const float wv = sw[sl * nz + j];
                f = (j == 0) ? wv : wv + sr[sl * nz + j] * f;
                sw[sl * nz + j] = f;
            }
            __syncwarp();
            // back substitution as maps of ff_{j+1}: ff_j = (-c_j / b'_j) ff_{j+1} + f_j / b'_j (the last
            // row's c / b' is 0, and so is its 1 / b' where rfords sets ff = 0)
            A = 1.f;
            B = 0.f;
            for (int j = j1 - 1; j >= j0; --j) {
                const float Aj = -sc[sl * nz + j], Bj = sw[sl * nz + j] * sb[sl * nz + j];
                B = fmaf(Aj, B, Bj);
                A = Aj * A;
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {  // inclusive suffix scan: lane l = segments l..31
                const float Ap = __shfl_down_sync(0xffffffffu, A, o), Bp = __shfl_down_sync(0xffffffffu, B, o);
                if (lane + o < 32) { B = fmaf(A, Bp, B); A = A * Ap; }
            }
            float nxt = __shfl_down_sync(0xffffffffu, B, 1);  // ff at the row after the segment
            if (lane == 31) nxt = 0.f;
            for (int j = j1 - 1; j >= j0; --j) {
                nxt = fmaf(-sc[sl * nz + j], nxt, sw[sl * nz + j] * sb[sl * nz + j]);
                sw[sl * nz + j] = nxt;
            }
        }
        __syncthreads();
        pb_markt(pf, 1);
        for (int e = threadIdx.x; e < nz * PB_TRI_MB; e += PB_NT) {
            const int sl = e % PB_TRI_MB, j = e / PB_TRI_MB, g = g0 + sl;
            if (g >= total) continue;
            const bool ub = g < nmu;
            const int k = ub ? g : g - nmu, len = ub ? nr + 1 : nr, rows = ub ? nz : nz - 1;
            if (j >= rows) continue;
            w[(ub ? 0 : mu) + k + (long)len * j] = sw[sl * nz + j];
        }
    }
}

// psolve of the momentum system with ESOLP_x: y = C_x T^-1 C_x x per block (three phases, two
// internal barriers); a.ff1 holds the intermediate.
__device__ bool pb_psolve_uv(const PersistArgs& a, const float* x, float* y, float* smem, unsigned& gen, PbProf& pf) {
    const float* sc = a.esolp == 2 ? a.diag : nullptr;  // DRD_UV_ESOLP_SCALED: y = s E(s x), s in a.diag
    pb_xpass_uv(a, x, a.ff1, smem, pf, sc, nullptr);
    if (!grid_sync(a.bar, gen, pf)) return false;
    pb_tridiag_uv(a, a.ff1, smem, pf);
    if (!grid_sync(a.bar, gen, pf)) return false;
    pb_xpass_uv(a, a.ff1, y, smem, pf, nullptr, sc);
    return true;
}

// One folded DCT-I along z of PB_CW columns held in xs[nz][PB_CW] -> ys[nz][PB_CW].  The folded
// columns are kept transposed, u[p][c][Kz4] (zero-padded), so both operands of the inner
// product are read as float4 when the z operands are resident in shared memory.
__device__ __forceinline__ void pb_zcols(const PersistArgs& a, const float* xs, float* u, float* ys,
                                         const float* zA) {
    const int nz = a.nz, L = nz - 1, K = a.Kz, K4 = (K + 3) & ~3;
    const int tid = threadIdx.x;
    for (int e = tid; e < K4 * PB_CW; e += PB_NT) {  // fold: u[p][c][j]
        const int c = e / K4, j = e % K4;
        float u0 = 0.f, u1 = 0.f;
        if (j < K) {
            const float x0 = xs[j * PB_CW + c];
            if (2 * j == L) {
                u0 = x0;
            } else {
                const float x1 = xs[(L - j) * PB_CW + c];
                u0 = x0 + x1;
                u1 = x0 - x1;
            }
        }
        u[c * K4 + j] = u0;
        u[(PB_CW + c) * K4 + j] = u1;
    }
    __syncthreads();
    if (zA) {
        // resident operands: a register-tiled product.  Work item = (parity, 4 output rows, one
        // of ZKS slices of K); each thread forms the 4 x PB_CW partial sums of its slice from
        // float4 reads (8 shared loads per 64 FMA), and the ZKS slices of a tile, consecutive
        // lanes of one warp, are summed by a reduce-scatter of shuffles in a fixed order.
        constexpr int ZKS = 8;
        static_assert(PB_CW == 4, "4 x 4 register tile");
        const int NJ4 = K4 / 4, JC = (NJ4 + ZKS - 1) / ZKS;
        const int G = (a.Mze + 3) / 4, W = 2 * G * ZKS;
        const int lane = tid & 31, ks = lane & (ZKS - 1);
        for (int base = 0; base < W; base += PB_NT) {  // uniform trip count: every lane shuffles
            const int w = base + tid;
            const bool valid = w < W;
            const int tile = w / ZKS, par = valid ? tile / G : 0, m0 = (valid ? tile % G : 0) * 4;
            float v[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
            if (valid) {
                const float4* U4 = reinterpret_cast<const float4*>(u + par * PB_CW * K4);
                const float4* A4 = reinterpret_cast<const float4*>(zA + (long)par * a.Mze * K4);
                const int jb = ks * JC, je = min(jb + JC, NJ4);
                for (int j4 = jb; j4 < je; ++j4) {
                    float4 av[4], uv[4];
#pragma unroll
                    for (int r = 0; r < 4; ++r)
                        av[r] = m0 + r < a.Mze ? A4[(long)(m0 + r) * (K4 / 4) + j4] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                    for (int c = 0; c < 4; ++c) uv[c] = U4[c * (K4 / 4) + j4];
#pragma unroll
                    for (int r = 0; r < 4; ++r)
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            float acc = v[r * 4 + c];
                            acc = fmaf(av[r].x, uv[c].x, acc);
                            acc = fmaf(av[r].y, uv[c].y, acc);
                            acc = fmaf(av[r].z, uv[c].z, acc);
                            acc = fmaf(av[r].w, uv[c].w, acc);
                            v[r * 4 + c] = acc;
                        }
                }
            }
            // reduce-scatter over the ZKS lanes: 16 -> 8 -> 4 -> 2 values per lane
            const bool b2 = ks & 4, b1 = ks & 2, b0 = ks & 1;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float snd = b2 ? v[i] : v[i + 8], keep = b2 ? v[i + 8] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, snd, 4);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float snd = b1 ? v[i] : v[i + 4], keep = b1 ? v[i + 4] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, snd, 2);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const float snd = b0 ? v[i] : v[i + 2], keep = b0 ? v[i + 2] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, snd, 1);
            }
            if (valid) {
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const int f = (b2 ? 8 : 0) + (b1 ? 4 : 0) + (b0 ? 2 : 0) + i, r = f >> 2, c = f & 3;
                    const int row = 2 * (m0 + r) + par;
                    if (row < nz) ys[row * PB_CW + c] = v[i];
                }
            }
        }
        __syncthreads();
        return;
    }
    for (int e = tid; e < nz * PB_CW; e += PB_NT) {
        const int row = e / PB_CW, c = e % PB_CW, par = row & 1, m = row >> 1;
        const float* up = u + (par * PB_CW + c) * K4;
        float acc0 = 0.f, acc1 = 0.f;
        if (zA) {
            const float4* A4 = reinterpret_cast<const float4*>(zA + ((long)par * a.Mze + m) * K4);
            const float4* U4 = reinterpret_cast<const float4*>(up);
#pragma unroll 4
            for (int j4 = 0; j4 < K4 / 4; ++j4) {
                const float4 av = A4[j4], uv = U4[j4];
                acc0 = fmaf(av.x, uv.x, acc0);
                acc1 = fmaf(av.y, uv.y, acc1);
                acc0 = fmaf(av.z, uv.z, acc0);
                acc1 = fmaf(av.w, uv.w, acc1);
            }
        } else {
            const float* A = (par ? a.fzo : a.fze) + (long)m * K;
            int j = 0;
#pragma unroll 4
            for (; j + 1 < K; j += 2) {
                acc0 = fmaf(__ldg(A + j), up[j], acc0);
                acc1 = fmaf(__ldg(A + j + 1), up[j + 1], acc1);
            }
            if (j < K) acc0 = fmaf(__ldg(A + j), up[j], acc0);
        }
        ys[row * PB_CW + c] = acc0 + acc1;
    }
    __syncthreads();
}

// Column pass along z (columns are independent along z): out = Cz ((Cz X) / Ph_Lcc).
__device__ void pb_zdz(const PersistArgs& a, const float* X, float* out, float* smem, const PbProf* pf = nullptr) {
    const int nz = a.nz, nr = a.nr, K = a.Kz;
    float* xs = smem + a.work_off;    // [nz][CW]
    float* u = xs + nz * PB_CW;       // [2][CW][Kz4]
    float* ys = u + 2 * PB_CW * ((K + 3) & ~3);  // [nz][CW]
    const float* zA = a.z_res ? smem + a.z_off : nullptr;
    const int nchunks = (nr + PB_CW - 1) / PB_CW;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int c0 = ch * PB_CW;
        __syncthreads();
        // the Ph_Lcc entries of the divide are fetched with the column data (one round trip)
        constexpr int LP = 4;
        float lv[LP];
#pragma unroll
        for (int i = 0; i < LP; ++i) {
            const int e = threadIdx.x + i * PB_NT, row = e / PB_CW, col = c0 + e % PB_CW;
            lv[i] = (e < nz * PB_CW && col < nr) ? __ldg(a.lcc + (long)row * nr + col) : 1.f;
        }
        for (int e = threadIdx.x; e < nz * PB_CW; e += PB_NT) {
            const int row = e / PB_CW, c = e % PB_CW, col = c0 + c;
            xs[e] = col < nr ? __ldcg(X + (long)row * nr + col) : 0.f;
        }
        __syncthreads();
        pb_markz(pf, 0);
        pb_zcols(a, xs, u, ys, zA);
        pb_markz(pf, 1);
#pragma unroll
        for (int i = 0; i < LP; ++i) {
            const int e = threadIdx.x + i * PB_NT, col = c0 + e % PB_CW;
            if (e < nz * PB_CW) xs[e] = col < nr ? ys[e] / lv[i] : 0.f;
        }
        for (int e = threadIdx.x + LP * PB_NT; e < nz * PB_CW; e += PB_NT) {
            const int row = e / PB_CW, c = e % PB_CW, col = c0 + c;
            xs[e] = col < nr ? ys[e] / __ldg(a.lcc + (long)row * nr + col) : 0.f;
        }
        __syncthreads();
        pb_markz(pf, 2);
        pb_zcols(a, xs, u, ys, zA);
        pb_markz(pf, 3);
        for (int e = threadIdx.x; e < nz * PB_CW; e += PB_NT) {
            const int row = e / PB_CW, c = e % PB_CW, col = c0 + c;
            if (col < nr) out[(long)row * nr + col] = ys[e];
        }
        pb_markz(pf, 4);
    }
}

// psolve: y = DCT-I preconditioner applied to x (three phases, two internal barriers), blended
// with x by the per-cell weights a.pcw when they are installed.
__device__ bool pb_psolve(const PersistArgs& a, const float* x, float* y, float* smem, unsigned& gen, PbProf& pf) {
    pb_xpass(a, x, a.w1, smem, pf);
    if (!grid_sync(a.bar, gen, pf)) return false;
    pb_zdz(a, a.w1, a.w2, smem, &pf);
    if (!grid_sync(a.bar, gen, pf)) return false;
    pb_xpass(a, a.w2, y, smem, pf, x, a.pcw);
    return true;
}

// ff1 = -(dt xld) L_M0(x) evaluated where it is needed (the first half of MATRIX_VECTOR_CG).
template <typename T, class XA>
struct ChFF1 {
    XA x; CellA<T> M0; int nr, nz; T dtxld, idr2, idz2;
    __device__ __forceinline__ T operator()(int i, int k) const {
        return -(dtxld * op_dgn<T>(i, k, nr, nz, idr2, idz2, x, M0));
    }
};

// y = A x (MATRIX_VECTOR_CG) in ONE phase: the outer operator reads ff1 at a cell and its four
// neighbours, and each of those five values is recomputed from x (a radius-2 stencil) instead
// of being stored and re-read after a grid barrier.  The arithmetic of every ff1 value is the
// same as the two-pass form, so the result is too.  Optional partial dots of y with d1 and with
// itself.
__device__ bool pb_matvec_ch(const PersistArgs& a, const float* x, float* y, float alpha, const float* yin,
                             const float* d1, int slot1, bool self2, int slot2, const float* d3, int slot3,
                             double* sm, unsigned& gen, PbProf& pf) {
    (void)gen;
    (void)pf;
    const int nr = a.nr, nz = a.nz;
    const long n = (long)nr * nz;
    const long stride = (long)gridDim.x * PB_NT;
    const ChFF1<float, PackedCG<float>> F{PackedCG<float>{x, nr}, CellA<float>{a.M0, nr}, nr, nz, a.o.dtxld,
                                          a.o.idr2, a.o.idz2};
    CellA<float> Mi{a.Mi, nr};
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (long q = blockIdx.x * (long)PB_NT + threadIdx.x; q < n; q += stride) {
        const int qi = (int)q, k = qi / nr, i = qi - k * nr;
        const float f = F(i, k);
        const float av = __ldcg(x + q) + (a.o.s * f / a.o.eps - a.o.eps * op_dgn<float>(i, k, nr, nz, a.o.idr2,
                                                                                        a.o.idz2, F, Mi));
        const float yn = yin ? alpha * av + __ldcg(yin + q) : alpha * av;
        y[q] = yn;
        if (d1) s1 = fmaf(__ldcg(d1 + q), yn, s1);
        if (self2) s2 = fmaf(yn, yn, s2);
        if (d3) s3 = fmaf(__ldcg(d3 + q), yn, s3);
    }
    if (d1 || self2 || d3)
        slots_put_f<PB_NT>(a.part, d1 ? slot1 : -1, s1, self2 ? slot2 : -1, s2, d3 ? slot3 : -1, s3, sm);
    return true;
}

// y = A x (MatrixVector_uv_2_CG / MatrixVector_uv_CG) in one phase, with the same options.
__device__ bool pb_matvec_uv(const PersistArgs& a, const float* x, float* y, float alpha, const float* yin,
                             const float* d1, int slot1, bool self2, int slot2, const float* d3, int slot3,
                             double* sm) {
    const long mn = (long)(a.nr + 1) * a.nz;
    const long stride = (long)gridDim.x * PB_NT;
    UVFetch<float, true> F{x, a.nr, a.nz, mn, a.o.lr_neumann};
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    // two rows per pass, both computed before either is stored, so their loads overlap
    for (long q = blockIdx.x * (long)PB_NT + threadIdx.x; q < a.n; q += 2 * stride) {
        const long q2 = q + stride;
        const bool two = q2 < a.n;
        const float av = uv_apply<float>(a.o, a.rho, a.eta, a.pen, F, q);
        const float av2 = two ? uv_apply<float>(a.o, a.rho, a.eta, a.pen, F, q2) : 0.f;
        const float y1 = yin ? alpha * av + __ldcg(yin + q) : alpha * av;
        const float y2 = two ? (yin ? alpha * av2 + __ldcg(yin + q2) : alpha * av2) : 0.f;
        const float e1 = d1 ? __ldcg(d1 + q) : 0.f, e2 = (d1 && two) ? __ldcg(d1 + q2) : 0.f;
        const float g1 = d3 ? __ldcg(d3 + q) : 0.f, g2 = (d3 && two) ? __ldcg(d3 + q2) : 0.f;
        y[q] = y1;
        if (two) y[q2] = y2;
        if (d1) s1 = fmaf(e2, y2, fmaf(e1, y1, s1));
        if (self2) s2 = fmaf(y2, y2, fmaf(y1, y1, s2));
        if (d3) s3 = fmaf(g2, y2, fmaf(g1, y1, s3));
    }
    if (d1 || self2 || d3)
        slots_put_f<PB_NT>(a.part, d1 ? slot1 : -1, s1, self2 ? slot2 : -1, s2, d3 ? slot3 : -1, s3, sm);
    return true;
}

template <int KIND>
__device__ __forceinline__ bool pb_matvec(const PersistArgs& a, const float* x, float* y, float alpha, const float* yin,
                                          const float* d1, int slot1, bool self2, int slot2, double* sm,
                                          unsigned& gen, PbProf& pf, const float* d3 = nullptr, int slot3 = 0) {
    if constexpr (KIND == PK_CH)
        return pb_matvec_ch(a, x, y, alpha, yin, d1, slot1, self2, slot2, d3, slot3, sm, gen, pf);
    (void)gen;
    (void)pf;
    return pb_matvec_uv(a, x, y, alpha, yin, d1, slot1, self2, slot2, d3, slot3, sm);
}

// Element-wise preconditioner of the momentum system: Jacobi (PSolve_uv_2_CG) or the identity.
__device__ __forceinline__ float pb_pre(const PersistArgs& a, long q, float v) {
    return a.ident ? v : v / __ldg(a.diag + q);
}

// The preconditioner as a phase sequence: the CH DCT-I solve, or ESOLP_x for the momentum system
// (the momentum system's Jacobi is element-wise and fused into the vector passes instead).
template <int KIND>
__device__ __forceinline__ bool pb_psolve_k(const PersistArgs& a, const float* x, float* y, float* smem, unsigned& gen,
                                            PbProf& pf) {
    if constexpr (KIND == PK_CH) return pb_psolve(a, x, y, smem, gen, pf);
    return pb_psolve_uv(a, x, y, smem, gen, pf);
}

// State of one inner BiCGSTAB run (the local scalars of BICGSTABREVCOM).
struct PbInner {  // FP32 like the inner iterations themselves
    int info, iter;
    unsigned flags;
    float resid, rho, rho1, alpha, omega, beta, snorm;
};

// The iterations (lib/BiCGSTABREVCOM.f:257-388) from R, RTLD, P = R (and, for the momentum
// system, PHAT = M^-1 P) and the first RHO = (rtld, r); X is updated in place.  Every block runs
// the same scalar steps; returns false when a barrier timed out.
//
// One change of schedule against the reference: the next RHO is formed as (rtld, s) -
// omega (rtld, t), from partials of the S pass and the T product, instead of (rtld, r) after R
// is updated.  BETA is then known when X and R are updated, and the next P = BETA (P - OMEGA V)
// + R is formed in the same pass: one phase and one grid barrier fewer per iteration.  The
// STOPTEST2 norm of the new R is read after the next barrier, so the transform of the next P is
// computed before a converged solve stops (its result is then unused).
template <int KIND>
__device__ bool pb_iterate(const PersistArgs& a, double bnrm2, double tol, int maxit, double rho_first, PbInner& st,
                           float* smem, double* sm, unsigned& gen, PbProf& pf) {
    const long n = a.n;
    const long stride = (long)gridDim.x * PB_NT;
    const long q0 = blockIdx.x * (long)PB_NT + threadIdx.x;
    bool ok = true;
    const float bn = (float)bnrm2, tl = (float)tol, kbt = (float)kBreakTol;
    float rho = (float)rho_first;
    __shared__ float s_sc[4];  // scalars evaluated by thread 0, read by the block
    st.iter = 0;
    while (true) {
        st.rho = rho;
        st.iter += 1;
        pf.p = (a.prof != nullptr && st.iter == 3 && pf.k == 0) ? a.prof : nullptr;  // time iteration 3 once
        if (pf.p != nullptr && blockIdx.x == 0 && threadIdx.x == 0) pf.p[123] = gtimer();
        if (fabsf(st.rho) < kbt) { st.info = -10; break; }  // (:261-263)
        if (KIND == PK_CH || a.esolp) {
            if (!(ok = pb_psolve_k<KIND>(a, a.p, a.phat, smem, gen, pf))) break;     // PHAT = M^-1 P
            if (!(ok = grid_sync(a.bar, gen, pf))) break;
        }
        if (!(ok = pb_matvec<KIND>(a, a.phat, a.v, 1.f, nullptr, a.rtld, 4, false, 0, sm, gen, pf))) break;  // V = A PHAT
        if (!(ok = grid_sync(a.bar, gen, pf))) break;
        // S = R - ALPHA V (:311-312), ||S||^2 and (rtld, S).  The loads of this thread's first two
        // elements do not depend on ALPHA: they are issued before thread 0 evaluates it.
        const long qa = q0, qb = q0 + stride;
        const bool ha = qa < n, hb = qb < n;
        float ra = 0.f, va = 0.f, ta = 0.f, rb = 0.f, vb = 0.f, tb = 0.f;
        if (ha) { ra = __ldcg(a.r + qa); va = __ldcg(a.v + qa); ta = __ldcg(a.rtld + qa); }
        if (hb) { rb = __ldcg(a.r + qb); vb = __ldcg(a.v + qb); tb = __ldcg(a.rtld + qb); }
        if (threadIdx.x < 32) {
            const float rv = warp_slot_sum(a.part, 4);
            if (threadIdx.x == 0) s_sc[0] = st.rho / rv;  // ALPHA (:307)
        }
        __syncthreads();
        st.alpha = s_sc[0];
        {
            const float na = -st.alpha;
            float s2 = 0.f, rs = 0.f;
            auto s_elem = [&](long q, float r, float v, float t) {
                const float sv = r + na * v;
                a.r[q] = sv;
                s2 = fmaf(sv, sv, s2);
                rs = fmaf(t, sv, rs);
                if (KIND == PK_UV && !a.esolp) a.shat[q] = pb_pre(a, q, sv);  // SHAT = M^-1 S, fused
            };
            if (ha) s_elem(qa, ra, va, ta);
            if (hb) s_elem(qb, rb, vb, tb);
            for (long q = q0 + 2 * stride; q < n; q += stride) s_elem(q, __ldcg(a.r + q), __ldcg(a.v + q), __ldcg(a.rtld + q));
            slots_put_f<PB_NT>(a.part, 5, s2, 2, rs, -1, 0.f, sm);
        }
        if (!(ok = grid_sync(a.bar, gen, pf))) break;
        if (threadIdx.x < 32) {
            const float ss = warp_slot_sum(a.part, 5);
            if (threadIdx.x == 0) s_sc[1] = sqrtf(ss);
        }
        __syncthreads();
        st.snorm = s_sc[1];
        if (st.snorm <= tl) {  // early absolute test (:313-316): X = X + ALPHA PHAT
            st.resid = st.snorm / bn;
            st.info = 0;
            st.flags |= DRD_FLAG_EARLY_S;
            const float al = st.alpha;
            for (long q = q0; q < n; q += stride) a.x[q] = __ldcg(a.x + q) + al * __ldcg(a.phat + q);
            break;
        }
        if (KIND == PK_CH || a.esolp) {
            if (!(ok = pb_psolve_k<KIND>(a, a.r, a.shat, smem, gen, pf))) break;     // SHAT = M^-1 S
            if (!(ok = grid_sync(a.bar, gen, pf))) break;
        }
        // T = A SHAT with (t, s), (t, t) and (rtld, t)
        if (!(ok = pb_matvec<KIND>(a, a.shat, a.t, 1.f, nullptr, a.r, 6, true, 7, sm, gen, pf, a.rtld, 1))) break;
        if (!(ok = grid_sync(a.bar, gen, pf))) break;
        // loads of this thread's first two elements of the X / R / P pass, issued before thread 0
        // evaluates OMEGA and BETA (they do not depend on them)
        float ea[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, eb[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        auto xrp_load = [&](long q, float (&e)[7]) {
            e[0] = __ldcg(a.x + q); e[1] = __ldcg(a.phat + q); e[2] = __ldcg(a.shat + q); e[3] = __ldcg(a.r + q);
            e[4] = __ldcg(a.t + q); e[5] = __ldcg(a.p + q); e[6] = __ldcg(a.v + q);
        };
        if (ha) xrp_load(qa, ea);
        if (hb) xrp_load(qb, eb);
        if (threadIdx.x < 32) {
            const float ts = warp_slot_sum(a.part, 6), tt = warp_slot_sum(a.part, 7);
            const float rs = warp_slot_sum(a.part, 2), rt = warp_slot_sum(a.part, 1);
            if (threadIdx.x == 0) {
                const float om = ts / tt;                      // (:349-350)
                const float rn = rs - om * rt;                 // (rtld, S - OMEGA T)
                s_sc[0] = om;
                s_sc[1] = rn;
                s_sc[2] = (rn / st.rho) * (st.alpha / om);     // (:269) for the next iteration
            }
        }
        __syncthreads();
        st.omega = s_sc[0];
        const float rho_new = s_sc[1];
        st.beta = s_sc[2];
        {
            // X = X + ALPHA PHAT + OMEGA SHAT, R = S - OMEGA T (:354-359), ||R||^2, and the next
            // P = BETA (P - OMEGA V) + R (:273-275); two elements per pass, loads before stores
            const float al = st.alpha, om = st.omega, nom = -st.omega;
            const float bt = st.beta;
            float r2 = 0.f;
            auto xrp = [&](long q, const float (&e)[7]) {
                float xv = e[0] + al * e[1];
                xv = xv + om * e[2];
                const float rv = e[3] + nom * e[4];
                float pv = e[5] + nom * e[6];
                pv = bt * pv;
                pv = pv + rv;
                a.x[q] = xv;
                a.r[q] = rv;
                a.p[q] = pv;
                if (KIND == PK_UV && !a.esolp) a.phat[q] = pb_pre(a, q, pv);  // PHAT = M^-1 P of the next iteration
                r2 = fmaf(rv, rv, r2);
            };
            if (ha) xrp(qa, ea);
            if (hb) xrp(qb, eb);
            for (long q = q0 + 2 * stride; q < n; q += stride) {
                float e[7];
                xrp_load(q, e);
                xrp(q, e);
            }
            slots_put_f<PB_NT>(a.part, 0, r2, -1, 0.f, -1, 0.f, sm);
        }
        if (!(ok = grid_sync(a.bar, gen, pf))) break;
        if (threadIdx.x < 32) {
            const float r2 = warp_slot_sum(a.part, 0);
            if (threadIdx.x == 0) s_sc[3] = sqrtf(r2) / bn;  // STOPTEST2 (:361-362)
        }
        __syncthreads();
        st.resid = s_sc[3];
        if (!isfinite(st.resid)) { st.info = DRD_ERR_NONFINITE; break; }
        if (st.resid <= tl) { st.info = 0; break; }
        if (st.iter >= maxit) { st.info = 1; break; }
        if (fabsf(st.omega) < kbt) {  // (:383-388)
            st.info = (fabsf(st.rho) < kbt) ? -10 : -11;
            break;
        }
        st.rho1 = st.rho;
        rho = rho_new;
    }
    pf.p = nullptr;
    return ok;
}

// FP64 residual of the refinement: r64 = b64 - A64 x64 (the reference-form FP64 operators),
// partials ||r64||^2 into slot 8 and, when `with_b`, ||b64||^2 into slot 9.
template <int KIND>
__device__ bool pb_residual64(const PersistArgs& a, bool with_b, double* sm, unsigned& gen, PbProf& pf) {
    const int nr = a.nr, nz = a.nz;
    const long n = a.n;
    const long stride = (long)gridDim.x * PB_NT;
    double r2 = 0.0, b2 = 0.0;
    if constexpr (KIND == PK_CH) {
        const ChFF1<double, PackedCG<double>> Fv{PackedCG<double>{a.x64, nr}, CellA<double>{a.M0d, nr}, nr, nz,
                                                 a.od.dtxld, a.od.idr2, a.od.idz2};
        CellA<double> Mi{a.Mid, nr};
        (void)gen;
        (void)pf;
        for (long q = blockIdx.x * (long)PB_NT + threadIdx.x; q < n; q += stride) {
            const int i = (int)(q % nr), k = (int)(q / nr);
            const double f = Fv(i, k), bq = __ldcg(a.b64 + q);
            const double av = __ldcg(a.x64 + q) + (a.od.s * f / a.od.eps -
                                                   a.od.eps * op_dgn<double>(i, k, nr, nz, a.od.idr2, a.od.idz2, Fv, Mi));
            const double rq = -1.0 * av + 1.0 * bq;
            a.r64[q] = rq;
            r2 += rq * rq;
            b2 += bq * bq;
        }
    } else {
        const long mn = (long)(nr + 1) * nz;
        UVFetch<double, true> F{a.x64, nr, nz, mn, a.od.lr_neumann};
        for (long q = blockIdx.x * (long)PB_NT + threadIdx.x; q < n; q += stride) {
            const double bq = __ldcg(a.b64 + q);
            const double av = uv_apply<double>(a.od, a.rhod, a.etad, a.pend, F, q);
            const double rq = -1.0 * av + 1.0 * bq;
            a.r64[q] = rq;
            r2 += rq * rq;
            b2 += bq * bq;
        }
    }
    // each thread's FP64 sums, then FP32 block and grid sums: the norms decide the sweep's tests
    // to about 1e-7 relative, far inside any tolerance, and ||r|| itself cancels in the update
    slots_put_f<PB_NT>(a.part, 8, (float)r2, with_b ? 9 : -1, (float)b2, -1, 0.f, sm);
    return true;
}

}  // namespace

template <int KIND>
__global__ void __launch_bounds__(PB_NT, 1) k_bicg_persist(PersistArgs a) {
    extern __shared__ __align__(16) float smem[];
    __shared__ double sm[64];
    count_launch(a.ctr);
    unsigned gen = 0u;  // arrivals counted so far (the counter is zeroed before the launch)
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    const long n = a.n;
    const long stride = (long)gridDim.x * PB_NT;
    const long q0 = blockIdx.x * (long)PB_NT + threadIdx.x;
    KState* ks = a.ks;
    PbProf pf{nullptr, 0};
    const unsigned long long t_begin = lead ? gtimer() : 0ull;
    // the parent (FP64 refinement) state decides whether this inner solve runs at all
    if (a.parent && *((volatile const int*)&a.parent->phase) != PH_RUNNING) {
        if (lead) { ks->phase = PH_DONE; ks->iter = 0; ks->info = 0; }
        return;
    }
    if constexpr (KIND == PK_CH) pb_load_resident(a, smem);
    else if (a.esolp && a.b_res) pb_load_resident_uv(a, smem);
    if (a.mode == PM_PSOLVE || a.mode == PM_MATVEC) {  // one application x = op(b), the solver's code
        bool done = true;
        if (a.mode == PM_PSOLVE) {
            if (KIND == PK_CH || a.esolp) done = pb_psolve_k<KIND>(a, a.b, a.x, smem, gen, pf);
            else
                for (long q = q0; q < n; q += stride) a.x[q] = pb_pre(a, q, __ldcg(a.b + q));
        } else {
            done = pb_matvec<KIND>(a, a.b, a.x, 1.f, nullptr, nullptr, 0, false, 0, sm, gen, pf);
        }
        if (lead) ks->info = done ? 0 : DRD_ERR_TIMEOUT;
        return;
    }
    if (a.mode == PM_REFINE) {
        // ---- the whole mixed solve: FP64 iterative refinement around the FP32 iterations.
        // Each sweep: r64 = b64 - A64 x64 and its tests, b32 = r64/||r64||, an inner solve of
        // A d = b32 from d = 0 to the inner tolerance, x64 += ||r64|| d.
        const double otol = a.outer_tol;
        double itol = a.tol;  // the inner tolerance, tightened tenfold when a sweep stalls
        int outer = 0, inner_total = 0, oinfo = 0;
        double bnorm64 = 0.0, bnrm64 = 1.0, rnorm = 0.0, oresid = 0.0, prev = 0.0;
        bool ok = true, run = true;
        PbInner in{};
        // the sweep's tests and scalars are evaluated by thread 0 (the other threads would only
        // repeat its FP64 operations) and broadcast: rnorm, oresid, 1/rnorm, stop, oinfo, itol
        __shared__ double s_rf[4];
        __shared__ int s_rs[2];
        while (run) {
            if (!(ok = pb_residual64<KIND>(a, outer == 0, sm, gen, pf) && grid_sync(a.bar, gen, pf))) break;
            if (threadIdx.x < 32) {
                const float r2 = warp_slot_sum(a.part, 8), b2 = outer == 0 ? warp_slot_sum(a.part, 9) : 0.f;
                if (threadIdx.x == 0) {
                    int stop = 0;
                    rnorm = sqrt((double)r2);
                    if (outer == 0) {  // k_mx_init
                        bnorm64 = sqrt((double)b2);
                        bnrm64 = bnorm64 == 0.0 ? 1.0 : bnorm64;
                        oresid = rnorm / bnrm64;
                        if (!isfinite(oresid)) { oinfo = DRD_ERR_NONFINITE; stop = 1; }
                        else if (oresid <= otol || rnorm == 0.0) stop = 1;
                    } else {  // k_mx_check
                        prev = oresid;
                        oresid = rnorm / bnrm64;
                        if (in.info == DRD_ERR_TIMEOUT) { oinfo = DRD_ERR_TIMEOUT; stop = 1; }
                        else if (!isfinite(oresid)) { oinfo = DRD_ERR_NONFINITE; stop = 1; }
                        else if (oresid <= otol) { oinfo = 0; stop = 1; }
                        else if (outer >= a.max_refine) { oinfo = 1; stop = 1; }
                        else if (oresid > 0.9 * prev) {  // a sweep that gained < 10 %: tighten the inner solves
                            if (itol > kMixedItolFloor) itol *= 0.1;
                            else { oinfo = 1; stop = 1; }  // stalled at the tightest inner tolerance
                        }
                    }
                    s_rf[0] = rnorm;
                    s_rf[1] = oresid;
                    s_rf[2] = rnorm > 0.0 ? 1.0 / rnorm : 0.0;
                    s_rf[3] = itol;
                    s_rs[0] = stop;
                    s_rs[1] = oinfo;
                }
            }
            __syncthreads();
            rnorm = s_rf[0];
            oresid = s_rf[1];
            itol = s_rf[3];
            oinfo = s_rs[1];
            if (outer > 0) inner_total += in.iter;
            if (s_rs[0]) break;
            // scale and inner setup in one pass: b32 = r = rtld = r64 / ||r64||, x32 = 0
            {
                const double sc = s_rf[2];
                float bb = 0.f;
                for (long q = q0; q < n; q += stride) {
                    const float bv = (float)(__ldcg(a.r64 + q) * sc);
                    a.b[q] = bv;
                    a.r[q] = bv;
                    a.rtld[q] = bv;
                    a.p[q] = bv;  // the first P = R (:268)
                    if constexpr (KIND == PK_UV) a.phat[q] = pb_pre(a, q, bv);
                    a.x[q] = 0.f;
                    bb = fmaf(bv, bv, bb);
                }
                slots_put_f<PB_NT>(a.part, 3, bb, -1, 0.f, -1, 0.f, sm);
            }
            if (!(ok = grid_sync(a.bar, gen, pf))) break;
            __shared__ double s_bb[2];
            if (threadIdx.x < 32) {
                const float bbs = warp_slot_sum(a.part, 3);
                if (threadIdx.x == 0) { s_bb[0] = bbs; s_bb[1] = sqrt((double)bbs); }
            }
            __syncthreads();
            const double bb = s_bb[0];
            const double bn = s_bb[1];
            in = PbInner{};
            if (a.maxit <= 0) { in.info = -3; in.iter = a.maxit; }
            else if (!(ok = pb_iterate<KIND>(a, bn == 0.0 ? 1.0 : bn, itol, a.maxit, bb, in, smem, sm, gen, pf)))
                break;
            // x64 += ||r64|| d32
            for (long q = q0; q < n; q += stride) a.x64[q] = __ldcg(a.x64 + q) + rnorm * (double)__ldcg(a.x + q);
            outer += 1;
            if (!(ok = grid_sync(a.bar, gen, pf))) break;
        }
        if (!ok) oinfo = DRD_ERR_TIMEOUT;
        if (lead) {
            ks->tol = otol;
            ks->maxit = a.max_refine;
            ks->bnorm_raw = bnorm64;
            ks->bnrm2 = bnrm64;
            ks->snorm = rnorm;
            ks->resid = oresid;
            ks->true_resid = oresid;  // the residual of the returned x64, recomputed in FP64
            ks->outer = outer;
            ks->inner_total = inner_total;
            ks->iter = inner_total;
            ks->info = oinfo;
            ks->flags = DRD_FLAG_REFINED;
            ks->mixed = 1;
            ks->t_begin = t_begin;
            ks->t_end = gtimer();
            ks->phase = PH_DONE;
        }
        return;
    }
    // ---- one inner solve (:229-255 setup, then the iterations)
    double xx = 0.0, bb = 0.0;
    for (long q = q0; q < n; q += stride) {
        const float bv = __ldcg(a.b + q), xv = __ldcg(a.x + q);
        a.r[q] = bv;
        xx += (double)xv * (double)xv;
        bb += (double)bv * (double)bv;
    }
    slot_put<PB_NT>(a.part, 0, xx, sm);
    slot_put<PB_NT>(a.part, 3, bb, sm);
    bool ok = grid_sync(a.bar, gen, pf);
    const double2 xb = slot_sum2<PB_NT>(a.part, 0, 3, sm);
    const double xnorm = sqrt(xb.x);
    const double bnorm_raw = sqrt(xb.y);
    const double bnrm2 = bnorm_raw == 0.0 ? 1.0 : bnorm_raw;
    const double tol = a.tol;
    const int maxit = a.maxit;
    PbInner st{};
    st.resid = tol;
    st.iter = maxit;
    bool run = maxit > 0;
    if (maxit <= 0) st.info = -3;
    if (ok && run && xnorm != 0.0) {  // r = b - A x0 and the absolute x0 test (:248)
        ok = pb_matvec<KIND>(a, a.x, a.r, -1.f, a.r, nullptr, 0, true, 0, sm, gen, pf) && grid_sync(a.bar, gen, pf);
        const double rr = sqrt(slot_sum<PB_NT>(a.part, 0, sm));
        if (rr <= tol) { run = false; st.info = 0; st.flags |= DRD_FLAG_EARLY_X0; }
    }
    if (ok && run) {
        double a1 = 0.0;
        for (long q = q0; q < n; q += stride) {
            const float rv = __ldcg(a.r + q);
            a.rtld[q] = rv;
            a.p[q] = rv;  // the first P = R (:268)
            if constexpr (KIND == PK_UV) a.phat[q] = pb_pre(a, q, rv);
            a1 += (double)rv * (double)rv;
        }
        slot_put<PB_NT>(a.part, 1, a1, sm);
        ok = grid_sync(a.bar, gen, pf);
        const double rho_first = slot_sum<PB_NT>(a.part, 1, sm);
        if (ok) ok = pb_iterate<KIND>(a, bnrm2, tol, maxit, rho_first, st, smem, sm, gen, pf);
    }
    if (!ok) st.info = DRD_ERR_TIMEOUT;
    if (lead) {
        ks->tol = tol;
        ks->maxit = maxit;
        ks->xnorm = xnorm;
        ks->x_nonzero = xnorm != 0.0;
        ks->bnorm_raw = bnorm_raw;
        ks->bnrm2 = bnrm2;
        ks->iter = st.iter;
        ks->info = st.info;
        ks->resid = st.resid;
        ks->snorm = st.snorm;
        ks->rho = st.rho;
        ks->rho1 = st.rho1;
        ks->alpha = st.alpha;
        ks->omega = st.omega;
        ks->beta = st.beta;
        ks->flags = st.flags;
        ks->mixed = 0;
        ks->t_begin = t_begin;
        ks->t_end = gtimer();
        ks->phase = PH_DONE;
    }
}

// ======================================================================================
// Host launchers
// ======================================================================================
#define GRID(n) grid_for(n), DRD_TPB, 0, s

__global__ void k_bar_reset(GridBar* b, ull* ctr) {
    count_launch(ctr);
    if (threadIdx.x == 0) {
        b->count = 0u;
        b->err = 0;
    }
}
void launch_bar_reset(GridBar* b, ull* ctr, cudaStream_t s) { k_bar_reset<<<1, 32, 0, s>>>(b, ctr); }
// %globaltimer at the start (end = 0) or end (end = 1) of a solve of the kernel-per-phase path
__global__ void k_stamp(KState* ks, int end, ull* ctr) {
    count_launch(ctr);
    if (threadIdx.x == 0) {
        if (end) ks->t_end = gtimer();
        else ks->t_begin = gtimer();
    }
}
void launch_stamp(KState* ks, int end, ull* ctr, cudaStream_t s) { k_stamp<<<1, 32, 0, s>>>(ks, end, ctr); }
// Two blocks run grid_sync; block `absent` (if any) returns without arriving, so the other's
// bounded wait runs out: out[b] = 0 or DRD_ERR_TIMEOUT per block that ran the barrier.
__global__ void k_bar_selftest(GridBar* bar, int absent, int* out, ull* ctr) {
    count_launch(ctr);
    if ((int)blockIdx.x == absent) {
        if (threadIdx.x == 0) out[blockIdx.x] = 1;  // did not take part
        return;
    }
    unsigned gen = 0u;
    PbProf pf{nullptr, 0};
    const bool ok = grid_sync(bar, gen, pf);
    if (threadIdx.x == 0) out[blockIdx.x] = ok ? 0 : DRD_ERR_TIMEOUT;
}
void launch_bar_selftest(GridBar* bar, int absent, int* out, ull* ctr, cudaStream_t s) {
    k_bar_reset<<<1, 32, 0, s>>>(bar, ctr);
    k_bar_selftest<<<2, 32, 0, s>>>(bar, absent, out, ctr);
}
// Shared-memory plan (offsets in floats) of the persistent CH solver for an nr x nz grid run by
// `grid` blocks within `budget` bytes: a work area (x-pass panels or z-pass columns), then the
// resident z-pass operands and the block's x-pass B panel where they fit.
PbPlan persist_ch_plan(int nr, int nz, int grid, size_t budget) {
    PbPlan p{};
    const int Kx = (nr - 1) / 2 + 1, Nxe = (nr + 1) / 2, Nxo = nr / 2;
    const int Kz = (nz - 1) / 2 + 1, Mze = (nz + 1) / 2;
    // x-pass work: A chunk and the K-group partial tiles, plus a B chunk when B is streamed
    const size_t xres = (size_t)PB_KC * PB_BM + (size_t)PB_KG * PB_BM * PB_BN;
    const size_t xstr = xres + (size_t)PB_KC * PB_BN;
    const int Kz4 = (Kz + 3) & ~3;
    const size_t zwork = (size_t)nz * PB_CW * 2 + (size_t)2 * Kz4 * PB_CW;
    auto up4 = [](size_t v) { return (v + 3) & ~(size_t)3; };  // float4-aligned offsets
    const size_t zres = (size_t)2 * Mze * Kz4;
    const int mt = (nz + PB_BM - 1) / PB_BM;
    const int ntiles = mt * ((Nxe + PB_BN - 1) / PB_BN + (Nxo + PB_BN - 1) / PB_BN);
    const size_t bres = (size_t)Kx * PB_BN;
    p.work_off = 0;
    // preferred: the z operands and the block's own B panel resident for the whole solve
    const size_t w = up4(xres > zwork ? xres : zwork);
    if (ntiles <= grid && (up4(w + zres) + bres) * sizeof(float) <= budget) {
        p.z_res = 1;
        p.z_off = (long)w;
        p.b_res = 1;
        p.b_off = (long)up4(w + zres);
        p.bytes = ((size_t)p.b_off + bres) * sizeof(float);
        return p;
    }
    size_t used = up4(xstr > zwork ? xstr : zwork);
    if ((used + zres) * sizeof(float) <= budget) {
        p.z_res = 1;
        p.z_off = (long)used;
        used = up4(used + zres);
    }
    p.bytes = used * sizeof(float);
    return p;
}
// Shared-memory plan of the persistent momentum solver with ESOLP_x (floats): a work area for
// the x pass (A chunk, K-group partial tiles, and a B chunk when B is streamed) that the
// tridiagonal phase's staged batch reuses, then the block's resident B panel when every tile
// has its own block and the panel fits.
PbPlan persist_esolp_plan(int nr, int nz, int grid, size_t budget) {
    PbPlan p{};
    auto up4 = [](size_t v) { return (v + 3) & ~(size_t)3; };
    const int Ku = nr / 2 + 1, Kx = (nr - 1) / 2 + 1, Kmax = Ku > Kx ? Ku : Kx;
    const int mtu = (nz + PB_BM - 1) / PB_BM, mtv = (nz - 1 + PB_BM - 1) / PB_BM;
    const int Nue = (nr + 2) / 2, Nuo = (nr + 1) / 2, Nxe = (nr + 1) / 2, Nxo = nr / 2;
    auto nt = [](int n) { return (n + PB_UBN - 1) / PB_UBN; };
    const int ntiles = mtu * (nt(Nue) + nt(Nuo)) + mtv * (nt(Nxe) + nt(Nxo));
    const size_t tri = (size_t)4 * nz * PB_TRI_MB;
    const size_t xres = (size_t)PB_KC * PB_BM + (size_t)PB_UKG * PB_BM * PB_UBN;
    const size_t xstr = xres + (size_t)PB_KC * PB_UBN;
    const size_t wres = up4(xres > tri ? xres : tri);
    p.work_off = 0;
    if (ntiles <= grid && (wres + (size_t)Kmax * PB_UBN) * sizeof(float) <= budget) {
        p.b_res = 1;
        p.b_off = (long)wres;
        p.bytes = (wres + (size_t)Kmax * PB_UBN) * sizeof(float);
        return p;
    }
    p.bytes = (xstr > tri ? xstr : tri) * sizeof(float);
    return p;
}
int persist_threads() { return PB_NT; }
const void* persist_kernel(int kind) {
    return kind == PK_CH ? (const void*)k_bicg_persist<PK_CH> : (const void*)k_bicg_persist<PK_UV>;
}
cudaError_t launch_bicg_persist(const PersistArgs& a, int grid, cudaStream_t s) {
    const size_t smem = a.smem_bytes;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(PB_NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (a.kind == PK_CH) return cudaLaunchKernelEx(&cfg, k_bicg_persist<PK_CH>, a);
    return cudaLaunchKernelEx(&cfg, k_bicg_persist<PK_UV>, a);
}

void launch_ch_f2(const DevParams& P, const double* u, const double* v, const double* ph, double* f2, ull* ctr,
                  cudaStream_t s) {
    k_ch_f2<<<GRID((long)(P.nr + 2) * (P.nz + 2))>>>(P, u, v, ph, f2, ctr);
}
void launch_ch_rhs(const DevParams& P, const double* ph, const double* rmu, const double* rmu_pre,
                   const double* rmu_pre2, const double* rmu_pre3, const double* bdr, const double* grad,
                   const double* Mi, const double* f2, double* b, double* x, ull* ctr, cudaStream_t s) {
    k_ch_rhs<<<GRID((long)P.nr * P.nz)>>>(P, ph, rmu, rmu_pre, rmu_pre2, rmu_pre3, bdr, grad, Mi, f2, b, x, ctr);
}
template <typename T>
void launch_ch_matvec(const OpScal<T>& o, const T* M0, const T* Mi, T alpha, const T* x, T beta, T* y, T* ff1,
                      const T* dot1, int self2, const Dots& d, int slot1, const KState* ks, int gate, ull* ctr,
                      cudaStream_t s) {
    const long n = (long)o.nr * o.nz;
    if constexpr (sizeof(T) == 4) {  // FP32: the fused tiled pass
        const int tiles = ((o.nr + kChTX - 1) / kChTX) * ((o.nz + kChTY - 1) / kChTY);
        const int g = (dot1 || self2) ? d.G : std::min(tiles, 152 * 8);
        k_ch_mv_tile<<<g, DRD_TPB, 0, s>>>(o, M0, Mi, x, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
        (void)ff1;
        return;
    }
    k_ch_mv1<T><<<GRID(n)>>>(o, M0, x, ff1, ks, gate, ctr);
    const int g = (dot1 || self2) ? d.G : grid_for(n);
    k_ch_mv2<T><<<g, DRD_TPB, 0, s>>>(o, Mi, x, ff1, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
}
void launch_ch_fin(const DevParams& P, const double* x, const double* f2, const double* M0, double* rmu_after,
                   double* ph_after, ull* ctr, cudaStream_t s) {
    k_ch_fin<<<GRID((long)P.nr * P.nz)>>>(P, x, f2, M0, rmu_after, ph_after, ctr);
    launch_fill_neumann(P.nr, P.nz, rmu_after, ph_after, ctr, s);
}
template <typename T>
void launch_tridiag(const TriBlock<T>& b0, const TriBlock<T>& b1, const KState* ks, int gate, ull* ctr, cudaStream_t s) {
    const int n = b0.len + b1.len;
    k_tridiag<T><<<(n + 63) / 64, 64, 0, s>>>(b0, b1, ks, gate, ctr);
}
template void launch_tridiag<double>(const TriBlock<double>&, const TriBlock<double>&, const KState*, int, ull*,
                                     cudaStream_t);
template void launch_tridiag<float>(const TriBlock<float>&, const TriBlock<float>&, const KState*, int, ull*,
                                    cudaStream_t);
void launch_fill_neumann(int nr, int nz, double* a, double* b, ull* ctr, cudaStream_t s) {
    k_fill_neumann<<<GRID(2L * (nr + 2) + 2L * nz)>>>(nr, nz, a, b, ctr);
}
void launch_ori_rhs(const DevParams& P, const double* ph, const double* f2, const double* cfb, const double* cft,
                    double alpha_s, double* b, double* x, double* pnb, double* pnt, ull* ctr, cudaStream_t s) {
    k_ori_rhs<<<GRID((long)P.nr * P.nz)>>>(P, ph, f2, cfb, cft, alpha_s, b, x, pnb, pnt, ctr);
}
template <typename T>
void launch_ori_matvec(const OpScal<T>& o, T alpha, const T* x, T beta, T* y, T* ff1, const T* dot1, int self2,
                       const Dots& d, int slot1, const KState* ks, int gate, ull* ctr, cudaStream_t s) {
    const long n = (long)o.nr * o.nz;
    k_ori_mv1<T><<<GRID(n)>>>(o, x, ff1, ks, gate, ctr);
    const int g = (dot1 || self2) ? d.G : grid_for(n);
    k_ori_mv2<T><<<g, DRD_TPB, 0, s>>>(o, x, ff1, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
}
void launch_ori_fin(const DevParams& P, const double* x, const double* pnb, const double* pnt, double cb, double ct,
                    double* ph_after, double* rmu_after, ull* ctr, cudaStream_t s) {
    k_ori_fin<<<GRID((long)(P.nr + 2) * (P.nz + 2))>>>(P, x, pnb, pnt, cb, ct, ph_after, rmu_after, ctr);
}
void launch_ori_rmu0(const DevParams& P, const double* ph, double* rmu, ull* ctr, cudaStream_t s) {
    k_ori_rmu0<<<GRID((long)P.nr * P.nz)>>>(P, ph, rmu, ctr);
}
void launch_ori_bdr(int nr, int nz, const double* ph, double* bdr, ull* ctr, cudaStream_t s) {
    k_ori_bdr<<<GRID((long)(nr + 2) * (nz + 2))>>>(nr, nz, ph, bdr, ctr);
}

void launch_phmu_prep(const DevParams& P, const double* u, const double* v, const double* ph, const double* bdr,
                      const double* used, double* M0, double* f2, ull* ctr, cudaStream_t s) {
    k_phmu_prep<<<GRID((long)(P.nr + 2) * (P.nz + 2))>>>(P, u, v, ph, bdr, used, M0, f2, ctr);
}
void launch_phmu_rhs(const DevParams& P, const double* ph, const double* rmu, const double* ph_pre,
                     const double* rmu_pre, const double* bdr, const double* grad, const double* f2, const double* cfB,
                     const double* cfT, double* b, double* x, double* pnb, double* pnt, ull* ctr, cudaStream_t s) {
    k_phmu_rhs<<<GRID((long)P.nr * P.nz)>>>(P, ph, rmu, ph_pre, rmu_pre, bdr, grad, f2, cfB, cfT, b, x, pnb, pnt, ctr);
}
template <typename T>
void launch_phmu_matvec(const OpScal<T>& o, const T* M0, const T* Mi, const T* used, T alpha, const T* x, T beta, T* y,
                        const T* dot1, int self2, const Dots& d, int slot1, const KState* ks, int gate, ull* ctr,
                        cudaStream_t s) {
    const long n = 2L * o.nr * o.nz;
    const int g = (dot1 || self2) ? d.G : grid_for(n);
    k_phmu_mv<T><<<g, DRD_TPB, 0, s>>>(o, M0, Mi, used, x, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
}
template <typename T>
void launch_phmu_diag(const OpScal<T>& o, T* diag, ull* ctr, cudaStream_t s) {
    k_phmu_diag<T><<<GRID((long)o.nr * o.nz)>>>(o, diag, ctr);
}
void launch_phmu_fin(const DevParams& P, const double* x, const double* pnb, const double* pnt, double cb, double ct,
                     double* ph_after, double* rmu_after, ull* ctr, cudaStream_t s) {
    k_phmu_fin<<<GRID((long)(P.nr + 2) * (P.nz + 2))>>>(P, x, pnb, pnt, cb, ct, ph_after, rmu_after, ctr);
}

void launch_uv_rhs(const DevParams& P, int bdf, const CallArgs* ca, const double* psi1, const double* psi2,
                   const double* u_pre, const double* u, const double* v_pre, const double* v, const double* p,
                   const double* rho, const double* eta, const double* bdr, const double* used, const double* ph_after,
                   const double* rmu_after, const double* pf1, const double* pf2, double* b, double* x, double* uL,
                   int extrap, const double* u_pre2, const double* v_pre2, const double* u_pre3,
                   const double* v_pre3, ull* ctr, cudaStream_t s) {
    const long N = (long)(P.nr + 1) * P.nz + (long)P.nr * (P.nz - 1);
    k_uv_rhs<<<GRID(N)>>>(P, bdf, ca, psi1, psi2, u_pre, u, v_pre, v, p, rho, eta, bdr, used, ph_after, rmu_after, pf1,
                          pf2, b, x, uL, extrap, u_pre2, v_pre2, u_pre3, v_pre3, ctr);
}
template <typename T>
void launch_uv_matvec(const OpScal<T>& o, const T* rho, const T* eta, const T* pen, T alpha, const T* x, T beta, T* y,
                      const T* dot1, int self2, const Dots& d, int slot1, const KState* ks, int gate, ull* ctr,
                      cudaStream_t s) {
    const long N = (long)(o.nr + 1) * o.nz + (long)o.nr * (o.nz - 1);
    if constexpr (sizeof(T) == 4) {
        // 16-deep tiles when they give every SM at least 4 tiles, else 8-deep ones
        const long nti = (o.nr + 1 + kUvTI - 1) / kUvTI;
        const bool deep = nti * ((o.nz + 15) / 16) >= 4L * 152;
        const long tiles = deep ? nti * ((o.nz + 15) / 16) : nti * ((o.nz + 7) / 8);
        const int g = (dot1 || self2) ? d.G : (int)std::min<long>(tiles, 152L * 8);
        if (deep)
            k_uv_mv_tile<16><<<g, DRD_TPB, 0, s>>>(o, rho, eta, pen, x, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
        else
            k_uv_mv_tile<8><<<g, DRD_TPB, 0, s>>>(o, rho, eta, pen, x, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
    } else {
        const int g = (dot1 || self2) ? d.G : grid_for(N);
        k_uv_mv<T><<<g, DRD_TPB, 0, s>>>(o, rho, eta, pen, x, alpha, beta, y, dot1, self2, d, slot1, ks, gate, ctr);
    }
}
template <typename T>
void launch_uv_diag(const OpScal<T>& o, const T* rho, const T* eta, T* diag, ull* ctr, cudaStream_t s) {
    const long N = (long)(o.nr + 1) * o.nz + (long)o.nr * (o.nz - 1);
    k_uv_diag<T><<<GRID(N)>>>(o, rho, eta, diag, ctr);
}
void launch_uv_fin(const DevParams& P, const double* x, const double* uL, double* u_after, double* v_after, ull* ctr,
                   cudaStream_t s) {
    const long n = (long)(P.nr + 3) * (P.nz + 2) + (long)(P.nr + 2) * (P.nz + 1);
    k_uv_fin<<<GRID(n)>>>(P, x, uL, u_after, v_after, ctr);
}

void launch_pre_div(const DevParams& P, const double* u, const double* v, double* w, ull* ctr, cudaStream_t s) {
    k_pre_div<<<GRID((long)P.nr * P.nz)>>>(P, u, v, w, ctr);
}
void launch_cell_add(long n, const double* x, double* y, ull* ctr, cudaStream_t s) {
    k_cell_add<<<GRID(n)>>>(n, x, y, ctr);
}
void launch_interp_coef(const DevParams& P, const double* dist, const double* bdr, double* fpd, double* rho, double* eta,
                        ull* ctr, cudaStream_t s) {
    k_interp_coef<<<GRID((long)(P.nr + 2) * (P.nz + 2))>>>(P, dist, bdr, fpd, rho, eta, ctr);
}
void launch_two_phase_coef(const DevParams& P, long cs, const double* fpd, const double* ph, double* rho, double* eta,
                           float* rho32, float* eta32, ull* ctr, cudaStream_t s) {
    k_two_phase_coef<<<GRID(cs)>>>(P, cs, fpd, ph, rho, eta, rho32, eta32, ctr);
}
void launch_dissipation(const DissipArgs& a, const double* u, const double* v, const double* ph, const double* rmu,
                        const double* angB, const double* angT, const Dots& d, double* out, ull* ctr, cudaStream_t s) {
    k_dissip_partial<<<d.G, DRD_TPB, 0, s>>>(a, u, v, ph, rmu, angB, angT, d, ctr);
    k_dissip_final<<<1, DRD_TPB, 0, s>>>(a, d, out, ctr);
}
void launch_threshold(long n, const double* x, double t, double* y, ull* ctr, cudaStream_t s) {
    k_threshold<<<GRID(n)>>>(n, x, t, y, ctr);
}
void launch_mass_partial(int nr, int nz, const double* ph, const Dots& d, int slot, ull* ctr, cudaStream_t s) {
    k_mass_partial<<<d.G, DRD_TPB, 0, s>>>(nr, nz, ph, d, slot, ctr);
}
void launch_mass_final(const Dots& d, int slot, double drdz, double* out, ull* ctr, cudaStream_t s) {
    k_mass_final<<<1, DRD_TPB, 0, s>>>(d, slot, drdz, out, ctr);
}

template <typename T>
void launch_bi_init1(long n, const T* b, const T* x, T* r, const Dots& d, ull* ctr, cudaStream_t s) {
    k_bi_init1<T><<<d.G, DRD_TPB, 0, s>>>(n, b, x, r, d, ctr);
}
void launch_bi_init2(KState* ks, const Dots& d, double tol, int maxit, const KState* parent, ull* ctr, cudaStream_t s) {
    k_bi_init2<<<1, DRD_TPB, 0, s>>>(ks, d, tol, maxit, parent, ctr);
}
void launch_bi_init3(KState* ks, const Dots& d, ull* ctr, cudaStream_t s) { k_bi_init3<<<1, DRD_TPB, 0, s>>>(ks, d, ctr); }
template <typename T>
void launch_bi_init4(long n, const T* r, T* rtld, const Dots& d, const KState* ks, ull* ctr, cudaStream_t s) {
    k_bi_init4<T><<<d.G, DRD_TPB, 0, s>>>(n, r, rtld, d, ks, ctr);
}
template <typename T>
void launch_bi_p(long n, const T* r, const T* v, T* p, T* phat, const T* diag, int ident, KState* ks, const Dots& d,
                 ull* ctr, cudaStream_t s) {
    k_bi_p<T><<<d.G, DRD_TPB, 0, s>>>(n, r, v, p, phat, diag, ident, ks, d, ctr);
}
template <typename T>
void launch_bi_s(long n, const T* v, T* r, KState* ks, const Dots& d, ull* ctr, cudaStream_t s) {
    k_bi_s<T><<<d.G, DRD_TPB, 0, s>>>(n, v, r, ks, d, ctr);
}
void launch_bi_snorm(KState* ks, const Dots& d, ull* ctr, cudaStream_t s) { k_bi_snorm<<<1, DRD_TPB, 0, s>>>(ks, d, ctr); }
template <typename T>
void launch_bi_diag_apply(long n, const T* x, const T* diag, int ident, T* y, const KState* ks, int gate, ull* ctr,
                          cudaStream_t s) {
    k_bi_diag_apply<T><<<GRID(n)>>>(n, x, diag, ident, y, ks, gate, ctr);
}
template <typename T>
void launch_uv_esolp_scale(const OpScal<T>& o, const T* rho, const T* eta, long n, T* sc, ull* ctr, cudaStream_t s) {
    k_uv_esolp_scale<T><<<GRID(n)>>>(o, rho, eta, n, sc, ctr);
}
template <typename T>
void launch_vmul(long n, const T* a, const T* sc, T* out, const KState* ks, int gate, ull* ctr, cudaStream_t s) {
    k_vmul<T><<<GRID(n)>>>(n, a, sc, out, ks, gate, ctr);
}
template <typename T>
void launch_pc_blend(long n, const T* x, const T* w, T* y, const KState* ks, int gate, ull* ctr, cudaStream_t s) {
    k_pc_blend<T><<<GRID(n)>>>(n, x, w, y, ks, gate, ctr);
}
void launch_probe_fill(long n, unsigned long long seed, long probe, double* e, ull* ctr, cudaStream_t s) {
    k_probe_fill<<<GRID(n)>>>(n, seed, probe, e, ctr);
}
void launch_probe_acc(long n, unsigned long long seed, long probe, const double* r, const double* qv, double* num,
                      double* den, int first, ull* ctr, cudaStream_t s) {
    k_probe_acc<<<GRID(n)>>>(n, seed, probe, r, qv, num, den, first, ctr);
}
void launch_probe_final(long n, const double* num, const double* den, double* w, float* w32, ull* ctr,
                        cudaStream_t s) {
    k_probe_final<<<GRID(n)>>>(n, num, den, w, w32, ctr);
}
template <typename T>
void launch_bi_xr(long n, const T* phat, const T* shat, const T* t, const T* rtld, T* x, T* r, KState* ks,
                  const Dots& d, ull* ctr, cudaStream_t s) {
    k_bi_xr<T><<<d.G, DRD_TPB, 0, s>>>(n, phat, shat, t, rtld, x, r, ks, d, ctr);
}
void launch_bi_end(KState* ks, const Dots& d, cudaGraphConditionalHandle h, int use_graph, ull* ctr, cudaStream_t s) {
    k_bi_end<<<1, DRD_TPB, 0, s>>>(ks, d, h, use_graph, ctr);
}
void launch_mr_init(KState* ks, const Dots& d, double tol, int maxit, ull* ctr, cudaStream_t s) {
    k_mr_init<<<1, DRD_TPB, 0, s>>>(ks, d, tol, maxit, ctr);
}
template <typename T>
void launch_mr_reset(long n, const double* r64, T* r, T* rtld, const Dots& d, const KState* ks, ull* ctr,
                     cudaStream_t s) {
    k_mr_reset<T><<<d.G, DRD_TPB, 0, s>>>(n, r64, r, rtld, d, ks, ctr);
}
template void launch_mr_reset<float>(long, const double*, float*, float*, const Dots&, const KState*, ull*, cudaStream_t);
void launch_mr_end(KState* ks, const Dots& d, cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hif, ull* ctr,
                   cudaStream_t s) {
    k_mr_end<<<1, DRD_TPB, 0, s>>>(ks, d, hw, hif, ctr);
}
template <typename T>
void launch_mr_fold(long n, T* x32, double* x64, ull* ctr, cudaStream_t s) {
    k_mr_fold<T><<<GRID(n)>>>(n, x32, x64, ctr);
}
template void launch_mr_fold<float>(long, float*, double*, ull*, cudaStream_t);
void launch_mr_check(KState* ks, const Dots& d, cudaGraphConditionalHandle hw, ull* ctr, cudaStream_t s) {
    k_mr_check<<<1, DRD_TPB, 0, s>>>(ks, d, hw, ctr);
}

void launch_arm_while(const KState* ks, cudaGraphConditionalHandle h, ull* ctr, cudaStream_t s) {
    k_arm_while<<<1, 32, 0, s>>>(ks, h, ctr);
}
void launch_bi_true_resid(KState* ks, const Dots& d, ull* ctr, cudaStream_t s) {
    k_bi_true_resid<<<1, DRD_TPB, 0, s>>>(ks, d, ctr);
}
template <typename T>
void launch_copy(long n, const T* x, T* y, ull* ctr, cudaStream_t s) { k_copy<T><<<GRID(n)>>>(n, x, y, ctr); }
template <typename T>
void launch_norm2_partial(long n, const T* x, const Dots& d, int slot, ull* ctr, cudaStream_t s) {
    k_norm2_partial<T><<<d.G, DRD_TPB, 0, s>>>(n, x, d, slot, ctr);
}
template <typename TO, typename TI>
void launch_convert_scale(long n, const TI* x, double scale, TO* y, ull* ctr, cudaStream_t s) {
    k_convert<TO, TI><<<GRID(n)>>>(n, x, scale, y, ctr);
}
template void launch_convert_scale<float, double>(long, const double*, double, float*, ull*, cudaStream_t);
template void launch_convert_scale<double, float>(long, const float*, double, double*, ull*, cudaStream_t);
template void launch_convert_scale<double, double>(long, const double*, double, double*, ull*, cudaStream_t);

void launch_axpy_f2d(long n, const KState* ks, const float* d, double* x, ull* ctr, cudaStream_t s) {
    k_axpy_f2d<<<GRID(n)>>>(n, ks, d, x, ctr);
}
void launch_mx_init(KState* outer, const Dots& d, double tol, int max_refine, double itol, ull* ctr,
                    cudaStream_t s) {
    k_mx_init<<<1, DRD_TPB, 0, s>>>(outer, d, tol, max_refine, itol, ctr);
}
void launch_mx_inner_setup(KState* inner, const KState* outer, double inner_tol, int inner_maxit, ull* ctr,
                           cudaStream_t s) {
    k_mx_inner_setup<<<1, 32, 0, s>>>(inner, outer, inner_tol, inner_maxit, ctr);
}
void launch_mx_check(KState* outer, const KState* inner, const Dots& d, cudaGraphConditionalHandle h, int use_graph,
                     ull* ctr, cudaStream_t s) {
    k_mx_check<<<1, DRD_TPB, 0, s>>>(outer, inner, d, h, use_graph, ctr);
}
template <typename TO>
void launch_mx_scale(long n, const double* r, const KState* o, TO* y, TO* zero, ull* ctr, cudaStream_t s) {
    k_mx_scale_from_state<TO><<<GRID(n)>>>(n, r, o, y, zero, ctr);
}
template void launch_mx_scale<float>(long, const double*, const KState*, float*, float*, ull*, cudaStream_t);

#define INST(T)                                                                                                        \
    template void launch_ch_matvec<T>(const OpScal<T>&, const T*, const T*, T, const T*, T, T*, T*, const T*, int,     \
                                      const Dots&, int, const KState*, int, ull*, cudaStream_t);                      \
    template void launch_ori_matvec<T>(const OpScal<T>&, T, const T*, T, T*, T*, const T*, int, const Dots&, int,      \
                                       const KState*, int, ull*, cudaStream_t);                                       \
    template void launch_phmu_matvec<T>(const OpScal<T>&, const T*, const T*, const T*, T, const T*, T, T*, const T*,  \
                                        int, const Dots&, int, const KState*, int, ull*, cudaStream_t);               \
    template void launch_phmu_diag<T>(const OpScal<T>&, T*, ull*, cudaStream_t);                                      \
    template void launch_uv_matvec<T>(const OpScal<T>&, const T*, const T*, const T*, T, const T*, T, T*, const T*,    \
                                      int, const Dots&, int, const KState*, int, ull*, cudaStream_t);                 \
    template void launch_uv_diag<T>(const OpScal<T>&, const T*, const T*, T*, ull*, cudaStream_t);                    \
    template void launch_bi_init1<T>(long, const T*, const T*, T*, const Dots&, ull*, cudaStream_t);                  \
    template void launch_bi_init4<T>(long, const T*, T*, const Dots&, const KState*, ull*, cudaStream_t);             \
    template void launch_bi_p<T>(long, const T*, const T*, T*, T*, const T*, int, KState*, const Dots&, ull*,          \
                                 cudaStream_t);                                                                       \
    template void launch_bi_s<T>(long, const T*, T*, KState*, const Dots&, ull*, cudaStream_t);                       \
    template void launch_bi_diag_apply<T>(long, const T*, const T*, int, T*, const KState*, int, ull*, cudaStream_t); \
    template void launch_pc_blend<T>(long, const T*, const T*, T*, const KState*, int, ull*, cudaStream_t);          \
    template void launch_uv_esolp_scale<T>(const OpScal<T>&, const T*, const T*, long, T*, ull*, cudaStream_t);     \
    template void launch_vmul<T>(long, const T*, const T*, T*, const KState*, int, ull*, cudaStream_t);              \
    template void launch_bi_xr<T>(long, const T*, const T*, const T*, const T*, T*, T*, KState*, const Dots&, ull*,   \
                                  cudaStream_t);                                                                      \
    template void launch_copy<T>(long, const T*, T*, ull*, cudaStream_t);                                            \
    template void launch_norm2_partial<T>(long, const T*, const Dots&, int, ull*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace drd
