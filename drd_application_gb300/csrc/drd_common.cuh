// drd_common.cuh — shared device definitions of the GB300 solver core.
//
// Layouts on the device are the Fortran ones of the C-ABI (include/drd_gb300.h):
//   CELL  (-1:nr, -1:nz)    ld = nr+2
//   UFACE (-1:nr+1, -1:nz)  ld = nr+3
//   VFACE (-1:nr, 0:nz)     ld = nr+2
// Krylov vectors use the reference's packed orders (microfluidics_complex_domain/
// matrix_tool.f90: Atob for CH, Atob_uv for momentum, Atob_ph_mu for the coupled CH).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/drd_gb300.h"

#define DRD_TPB 256        // threads per block of the element-wise / stencil kernels
#define DRD_MAXB 1024      // maximum blocks of a reduction grid (= partials per dot product)
#define DRD_NDOT 10        // dot-product slots in the partials buffer

namespace drd {

// Scalars of the deck and the grid, copied once per context (all FP64).
struct DevParams {
    int nr, nz, variant, phi_mode, lr_neumann, pad0;
    double dr, dz, dr2, dz2, idr2, idz2, dt, xld, re, ca, eps, s;
    double ggx, ggz, uwT, uwB, UU, twall, bdr_upp, bdr_low;
    double cang;    // cos(angle*pi/180), evaluated on the host like the reference's libm call
    double penalty_k, lambda_rho, lambda_eta, adjust;
};

// Per-call scalars read by the kernels from device memory, so that captured graphs stay valid
// while t and the pressure scale change between calls.
struct CallArgs {
    double t;       // solve time (t + dt in the mcl6 loop)
    double cf;      // 1 - exp(-t/twall) inlet ramp (VeloSolve_2_combined.f90:262)
    double coef;    // PreSolve_2 scale (re*gamma1/dt or 3*re*gamma1/(2dt))
    double pad;
};

// BiCGSTAB state of one solve (lib/BiCGSTABREVCOM.f local scalars) plus our bookkeeping.
enum : int { PH_RUNNING = 0, PH_EARLY = 1, PH_DONE = 2 };
struct KState {
    double rho, rho1, alpha, omega, beta;
    double bnrm2;      // STOPTEST2 denominator (||b||, 1 if zero)
    double bnorm_raw;  // ||b|| as computed
    double resid;      // RESID
    double tol;        // TOL
    double snorm;
    double true_resid;
    double xnorm;
    int iter, maxit, info, phase;
    unsigned flags;
    int x_nonzero;
    int outer;         // mixed mode: reliable updates (FP64 residual recomputes) so far
    int inner_total;   // mixed mode: FP32 iterations summed
    double rmax;       // mixed mode: ||r|| at the last reliable update
    double itol;       // mixed mode (outer state): the inner solves' tolerance, tightened on a stall
    int first_next;    // the next iteration starts a fresh Krylov sequence (P = R)
    int do_update;     // mixed mode: this iteration ends with a reliable update
    int mixed;         // mixed mode: no absolute ||s|| exit; convergence on the FP64 residual only
    int restart;       // mixed mode: the update also restarts the Krylov sequence (breakdown)
    unsigned long long t_begin, t_end;  // persistent solver: %globaltimer (ns) at its start and end
};

__host__ __device__ __forceinline__ long cidx(int nr, int i, int k) { return (long)(i + 1) + (long)(k + 1) * (nr + 2); }
__host__ __device__ __forceinline__ long uidx(int nr, int i, int k) { return (long)(i + 1) + (long)(k + 1) * (nr + 3); }
__host__ __device__ __forceinline__ long vidx(int nr, int i, int k) { return (long)(i + 1) + (long)k * (nr + 2); }

__device__ __forceinline__ void count_launch(unsigned long long* ctr) {
    if (ctr != nullptr && threadIdx.x == 0 && threadIdx.y == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0)
        atomicAdd(ctr, 1ull);
}

// Deterministic block sum: shuffle within warps, then warp 0 sums the warp totals in order.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sm) {
    static_assert(NT % 32 == 0 && NT <= 1024, "block size");
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sm[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (lane < NT / 32) ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// Sum of `n` partials in a fixed order by one block; result valid in thread 0.
template <int NT>
__device__ __forceinline__ double reduce_partials(const double* part, int n, double* sm) {
    double v = 0.0;
    for (int q = threadIdx.x; q < n; q += NT) v += part[q];
    return block_sum<NT>(v, sm);
}

}  // namespace drd
