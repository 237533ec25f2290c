// drd_pressure_fft.cu — PreSolve_2's direct pressure solve with FFT-based transforms.
//
// psi = REDFT01_2D(REDFT10_2D(div u) / Pre_Lcc) / (4 nr nz) * coef, the sequence of
// microfluidics_complex_domain/PreSolve_2.f90:16-47 and dct_fftw.f90:3-54, in three passes:
//   rows:    div u of two grid rows (the reference's expression), REDFT10 along x  -> T
//   columns: REDFT10 along z, / Pre_Lcc, REDFT01 along z, two columns at a time     -> T
//   rows:    REDFT01 along x, / (4 nr nz), * coef into psi's interior
// and the Neumann ghosts of dct_fftw.f90:41-51 by the existing ghost kernel.  Each pass moves a
// line pair through shared memory once; the intermediate T (nr*nz values) stays in L2 between
// passes.  The transforms follow FFTW's definitions (drd_fft.cuh): O(n log n) work and
// O(log n) rounding growth where the GEMM form has O(n^2) and O(sqrt n).
//
// The same passes in FP32 on plain arrays (a 2-D REDFT10 / divide / REDFT01 of an nr x nz
// field) are timed by drd_kernel_bench as the transform's HBM-roofline figure.
#include <cuda_runtime.h>

#include "drd_fft.cuh"
#include "drd_kernels.cuh"

namespace drd {
namespace {

constexpr int kPT = 256;  // most threads per block of the passes
// Threads per line pair: a stage has n/4 to n/2 butterflies.
__host__ __device__ __forceinline__ int pgroup(int n) { return n >= 1024 ? 256 : (n >= 256 ? 128 : 64); }
// Line pairs per block: FP64 takes one, so that the pairs spread over as many SMs as possible (the
// FP64 pipe of one SM is the limit); FP32 fills 256 threads.
template <typename R>
__host__ __device__ __forceinline__ int pgroups(int n) { return sizeof(R) == 8 ? 1 : kPT / pgroup(n); }

template <typename R>
struct PfftArgs {
    int nr, nz;
    FftPlan px, pz;
    const Cx<R>* twx;   // FFT_TABLE(nr): tw then tq
    const Cx<R>* twz;
    // pass 1 input: div of (u, v) (FP64 step) or a plain nr*nz array
    const double* u;
    const double* v;
    double dr, dz;
    const R* x;
    R* T;               // nr*nz, i fastest
    const double* lcc;  // Pre_Lcc, (nr+1) x (nz+1), i fastest (FP64 step); or
    const R* lccp;      // nr*nz plain table (bench)
    double* psi;        // CELL output (FP64 step) ...
    const CallArgs* ca; //   ... scaled by ca->coef
    R* out;             // or a plain nr*nz output
};

// Pass 1: rows la, lb -> REDFT10 along x into T.
template <typename R>
__global__ void __launch_bounds__(kPT) k_pfft_rows_fwd(PfftArgs<R> a, ull* ctr) {
    count_launch(ctr);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int n = a.nr, G = pgroup(n), groups = pgroups<R>(n);
    const int grp = threadIdx.x / G, lane = threadIdx.x - grp * G;
    Cx<R>* A = reinterpret_cast<Cx<R>*>(smraw) + (long)grp * 2 * n;
    Cx<R>* B = A + n;
    const Cx<R>* tq = a.twx + n;
    const int pairs = (a.nz + 1) / 2;
    const int pr = blockIdx.x * groups + grp;
    const bool act = pr < pairs;
    const int la = 2 * pr, lb = la + 1;
    const bool hb = lb < a.nz;
    auto val = [&](int k, int i) -> R {
        if (a.u) {
            return (R)((a.u[uidx(a.nr, i + 1, k)] - a.u[uidx(a.nr, i, k)]) / a.dr +
                       (a.v[vidx(a.nr, i, k + 1)] - a.v[vidx(a.nr, i, k)]) / a.dz);
        }
        return a.x[(long)k * a.nr + i];
    };
    if (act)
        for (int j = lane; j < n; j += G) {
            const int s = makhoul_src(j, n);
            A[j] = Cx<R>{val(la, s), hb ? val(lb, s) : R(0)};
        }
    __syncthreads();
    Cx<R>* Z = fft_line<R>(A, B, a.px, a.twx, false, lane, G, act);
    if (act)
        for (int k = lane; k < n; k += G) {
            R ya, yb;
            redft10_out<R>(Z, n, k, tq, ya, yb);
            a.T[(long)la * n + k] = ya;
            if (hb) a.T[(long)lb * n + k] = yb;
        }
}

// Pass 2: columns la, lb of T: REDFT10 along z, / Pre_Lcc, REDFT01 along z, back into T.
template <typename R>
__global__ void __launch_bounds__(kPT) k_pfft_cols(PfftArgs<R> a, ull* ctr) {
    count_launch(ctr);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int n = a.nz, G = pgroup(n), groups = pgroups<R>(n);
    const int grp = threadIdx.x / G, lane = threadIdx.x - grp * G;
    Cx<R>* A = reinterpret_cast<Cx<R>*>(smraw) + (long)grp * 2 * n;
    Cx<R>* B = A + n;
    const Cx<R>* tq = a.twz + n;
    const int nr = a.nr;
    const int pairs = (nr + 1) / 2;
    const int pr = blockIdx.x * groups + grp;
    const bool act = pr < pairs;
    const int la = 2 * pr, lb = la + 1;
    const bool hb = lb < nr;
    if (act)
        for (int j = lane; j < n; j += G) {
            const int s = makhoul_src(j, n);
            A[j] = Cx<R>{a.T[(long)s * nr + la], hb ? a.T[(long)s * nr + lb] : R(0)};
        }
    __syncthreads();
    Cx<R>* Z = fft_line<R>(A, B, a.pz, a.twz, false, lane, G, act);
    Cx<R>* Y = (Z == A) ? B : A;
    if (act)
        for (int k = lane; k < n; k += G) {
            R ya, yb;
            redft10_out<R>(Z, n, k, tq, ya, yb);
            if (a.lcc) {
                ya = ya / (R)a.lcc[la + (long)(nr + 1) * k];
                yb = hb ? yb / (R)a.lcc[lb + (long)(nr + 1) * k] : R(0);
            } else {
                ya = ya / a.lccp[la + (long)nr * k];
                yb = hb ? yb / a.lccp[lb + (long)nr * k] : R(0);
            }
            Y[k] = Cx<R>{ya, yb};
        }
    __syncthreads();
    if (act)
        for (int k = lane; k < n; k += G) {
            const Cx<R> yk = Y[k], ynk = k ? Y[n - k] : Cx<R>{R(0), R(0)};
            Z[k] = redft01_in<R>(yk.x, ynk.x, yk.y, ynk.y, tq[k]);
        }
    __syncthreads();
    Cx<R>* V = fft_line<R>(Z, Y, a.pz, a.twz, true, lane, G, act);
    if (act)
        for (int e = lane; e < n; e += G) {
            const Cx<R> v = V[makhoul_dst_src(e, n)];
            a.T[(long)e * nr + la] = v.x;
            if (hb) a.T[(long)e * nr + lb] = v.y;
        }
}

// Pass 3: rows la, lb of T -> REDFT01 along x, / (4 nr nz), * coef into psi (or the plain output).
template <typename R>
__global__ void __launch_bounds__(kPT) k_pfft_rows_inv(PfftArgs<R> a, ull* ctr) {
    count_launch(ctr);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int n = a.nr, G = pgroup(n), groups = pgroups<R>(n);
    const int grp = threadIdx.x / G, lane = threadIdx.x - grp * G;
    Cx<R>* A = reinterpret_cast<Cx<R>*>(smraw) + (long)grp * 2 * n;
    Cx<R>* B = A + n;
    const Cx<R>* tq = a.twx + n;
    const int pairs = (a.nz + 1) / 2;
    const int pr = blockIdx.x * groups + grp;
    const bool act = pr < pairs;
    const int la = 2 * pr, lb = la + 1;
    const bool hb = lb < a.nz;
    const R* ra = a.T + (long)la * n;
    const R* rb = a.T + (long)lb * n;
    if (act)
        for (int k = lane; k < n; k += G) {
            const R xa = ra[k], xan = k ? ra[n - k] : R(0);
            const R xb = hb ? rb[k] : R(0), xbn = (hb && k) ? rb[n - k] : R(0);
            A[k] = redft01_in<R>(xa, xan, xb, xbn, tq[k]);
        }
    __syncthreads();
    Cx<R>* V = fft_line<R>(A, B, a.px, a.twx, true, lane, G, act);
    if (act) {
        const double scale = 4.0 * a.nr * a.nz;
        const double coef = a.ca ? a.ca->coef : 1.0;
        for (int e = lane; e < n; e += G) {
            const Cx<R> v = V[makhoul_dst_src(e, n)];
            if (a.psi) {
                a.psi[cidx(a.nr, e, la)] = ((double)v.x / scale) * coef;  // dct_fftw.f90:33-35, PreSolve_2.f90:125
                if (hb) a.psi[cidx(a.nr, e, lb)] = ((double)v.y / scale) * coef;
            } else {
                a.out[(long)la * n + e] = v.x / (R)scale;
                if (hb) a.out[(long)lb * n + e] = v.y / (R)scale;
            }
        }
    }
}

template <typename R>
size_t pfft_smem(int n) {
    return (size_t)pgroups<R>(n) * 2 * n * sizeof(Cx<R>);
}

// The passes' shared memory above 48 KB needs an opt-in per kernel; set once per context, outside
// any stream capture.
template <typename R>
cudaError_t pfft_attrs(int nr, int nz) {
    const size_t sx = pfft_smem<R>(nr), sz = pfft_smem<R>(nz);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_pfft_rows_fwd<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx))) return e;
    if ((e = cudaFuncSetAttribute(k_pfft_cols<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz))) return e;
    return cudaFuncSetAttribute(k_pfft_rows_inv<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx);
}

template <typename R>
cudaError_t pfft_launch(const PfftArgs<R>& a, ull* ctr, cudaStream_t s) {
    const size_t sx = pfft_smem<R>(a.nr), sz = pfft_smem<R>(a.nz);
    const int gx = (a.nz + 1) / 2, gz = (a.nr + 1) / 2;
    const int px = pgroups<R>(a.nr), pz = pgroups<R>(a.nz);
    const int tx = px * pgroup(a.nr), tz = pz * pgroup(a.nz);
    k_pfft_rows_fwd<R><<<(gx + px - 1) / px, tx, sx, s>>>(a, ctr);
    k_pfft_cols<R><<<(gz + pz - 1) / pz, tz, sz, s>>>(a, ctr);
    k_pfft_rows_inv<R><<<(gx + px - 1) / px, tx, sx, s>>>(a, ctr);
    return cudaGetLastError();
}

}  // namespace

bool pfft_plan(int n, FftPlan& pl) {
    pl.n = n;
    pl.nst = 0;
    int m = n;
    for (int r : {4, 2, 3, 5, 7}) {
        while (m % r == 0) {
            if (pl.nst >= DRD_FFT_MAXST) return false;
            pl.radix[pl.nst++] = (unsigned char)r;
            m /= r;
        }
    }
    return m == 1 && n >= 2;
}

bool pfft_fits(int nr, int nz, int real_bytes) {
    FftPlan p;
    const size_t lim = 200 * 1024;
    const bool f64 = real_bytes == 8;
    auto bytes = [&](int n) {
        return f64 ? pfft_smem<double>(n) : pfft_smem<float>(n);
    };
    return pfft_plan(nr, p) && pfft_plan(nz, p) && bytes(nr) <= lim && bytes(nz) <= lim;
}

cudaError_t pfft_prepare(int nr, int nz) {
    cudaError_t e = pfft_attrs<double>(nr, nz);
    return e ? e : pfft_attrs<float>(nr, nz);
}

// The FP64 pressure step on the device (u, v -> psi interior; T scratch of nr*nz doubles).
cudaError_t launch_pressure_fft(int nr, int nz, double dr, double dz, const FftPlan& px, const FftPlan& pz,
                                const void* twx, const void* twz, const double* u, const double* v, double* T,
                                const double* pre_lcc, double* psi, const CallArgs* ca, ull* ctr, cudaStream_t s) {
    PfftArgs<double> a{};
    a.nr = nr; a.nz = nz; a.px = px; a.pz = pz;
    a.twx = reinterpret_cast<const Cx<double>*>(twx);
    a.twz = reinterpret_cast<const Cx<double>*>(twz);
    a.u = u; a.v = v; a.dr = dr; a.dz = dz; a.T = T; a.lcc = pre_lcc; a.psi = psi; a.ca = ca;
    return pfft_launch<double>(a, ctr, s);
}

// The FP32 2-D transform pair on plain arrays (kernel bench): out = REDFT01(REDFT10(x) / lcc)
// / (4 nr nz), lcc an nr*nz table.
cudaError_t launch_pressure_fft32(int nr, int nz, const FftPlan& px, const FftPlan& pz, const void* twx,
                                  const void* twz, const float* x, float* T, const float* lcc, float* out, ull* ctr,
                                  cudaStream_t s) {
    PfftArgs<float> a{};
    a.nr = nr; a.nz = nz; a.px = px; a.pz = pz;
    a.twx = reinterpret_cast<const Cx<float>*>(twx);
    a.twz = reinterpret_cast<const Cx<float>*>(twz);
    a.x = x; a.T = T; a.lccp = lcc; a.out = out;
    return pfft_launch<float>(a, ctr, s);
}

}  // namespace drd
