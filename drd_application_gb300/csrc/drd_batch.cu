// drd_batch.cu — batches of independent solves in one persistent launch.
//
// The batch is uploaded once: per system its coefficients (FP64 and FP32), right-hand side,
// guess, FP32 Krylov work vectors and, for the pressure systems, FFT plans and twiddle tables.
// One kernel launch (captured in a CUDA graph) then solves everything: each thread block pulls
// the next system from a device-side queue, ordered largest first, and runs that system's
// whole solve with block-level reductions only (no grid-wide synchronisation), so systems of
// every size run side by side and a block never waits for another.
//
// The solve is the library's mixed mode: FP64 iterative refinement (r = b - A x in FP64, stop on
// ||r|| / ||b|| <= tol) around a right-preconditioned FP32 BiCGSTAB for A d = r / ||r||
// (lib/BiCGSTABREVCOM.f:257-388 step for step, to the inner tolerance), x += ||r|| d.  The
// momentum operator and its Jacobi diagonal are the per-step kernels' device functions
// (drd_ops.cuh); the pressure preconditioner is PreSolve_2's DCT solve with FFT-based
// REDFT10 / REDFT01 (drd_fft.cuh) over the block's rows and columns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "drd_fft.cuh"
#include "drd_ops.cuh"

namespace drd {
namespace {

constexpr double kPiB = 3.14159265358979323846264338327950288;

struct BProb {
    int system, bdf, nr, nz;
    long n;                          // unknowns
    OpScal<float> o32;
    OpScal<double> o64;
    const double *rho, *eta, *pen;   // CELL, FP64 (UV); pressure: beta (nr*nz) in rho
    const float *rho32, *eta32, *pen32;
    const double* b;
    const double* x0;                // may be null
    double* x;
    double* r64;
    float* w;                        // 10 FP32 vectors of n: r rt p v s t ph sh d aux
    const FftPlan* plx;              // pressure: lengths nr, nz
    const FftPlan* plz;
    const Cx<float>* twx;            // FFT_TABLE(nr): tw then tq
    const Cx<float>* twz;
    const float* lcc;                // pressure: Pre_Lcc (nr*nz, i fastest)
    double tol, itol0;
    int maxit, max_refine;
    double cost;                     // host: scheduling weight
};

struct BStat {
    int info, iters, refinements, pad;
    double true_resid, resid;
    unsigned long long t0, t1;
};

template <int NT>
__device__ __forceinline__ void bsum3(float& a, float& b, float& c, float* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) { sm[3 * wid] = a; sm[3 * wid + 1] = b; sm[3 * wid + 2] = c; }
    __syncthreads();
    float x = 0.f, y = 0.f, z = 0.f;
    for (int q = 0; q < NT / 32; ++q) { x += sm[3 * q]; y += sm[3 * q + 1]; z += sm[3 * q + 2]; }
    a = x; b = y; c = z;
}

template <int NT>
__device__ __forceinline__ double bsum_d(double a, double* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = a;
    __syncthreads();
    double x = 0.0;
    for (int q = 0; q < NT / 32; ++q) x += sm[q];
    return x;
}

// ---- the pressure operator (FP64 or FP32) ------------------------------------------------
// (A psi)_(i,k) = [bx(i+1,k)(psi_(i+1) - psi_i) - bx(i,k)(psi_i - psi_(i-1))] / dr^2
//               + [bz(i,k+1)(psi_(k+1) - psi_k) - bz(i,k)(psi_k - psi_(k-1))] / dz^2,
// face coefficients the mean of the two cells' beta, zero on the domain faces.
template <typename T>
__device__ __forceinline__ T pres_apply(int nr, int nz, T idr2, T idz2, const T* __restrict__ beta,
                                        const T* __restrict__ x, long q) {
    const int k = (int)(q / nr), i = (int)(q - (long)k * nr);
    const T c = x[q], bc = beta[q];
    T fx = T(0), fz = T(0);
    if (i + 1 < nr) fx += (bc + beta[q + 1]) * T(0.5) * (x[q + 1] - c);
    if (i > 0) fx -= (bc + beta[q - 1]) * T(0.5) * (c - x[q - 1]);
    if (k + 1 < nz) fz += (bc + beta[q + nr]) * T(0.5) * (x[q + nr] - c);
    if (k > 0) fz -= (bc + beta[q - nr]) * T(0.5) * (c - x[q - nr]);
    return fx * idr2 + fz * idz2;
}

__host__ __device__ __forceinline__ int group_size_d(int n) { return n >= 512 ? 128 : (n >= 128 ? 64 : 32); }

// ---- the pressure preconditioner: out = REDFT01(REDFT10(in) / Pre_Lcc) / (4 nr nz) ---------
// Three block-wide phases over a scratch array T (nr*nz, i fastest): rows (REDFT10), columns
// (REDFT10, / Pre_Lcc, REDFT01), rows (REDFT01, scale).  Groups of G threads each take a pair of
// lines per round; `buf` holds two ping-pong lines of nmax complex values per group.
template <int NT>
__device__ void pres_precond(const BProb& P, const float* __restrict__ in, float* __restrict__ T_, float* __restrict__ out,
                             Cx<float>* buf, int nmax) {
    const int nr = P.nr, nz = P.nz;
    const float scale = 1.0f / (4.0f * (float)nr * (float)nz);
    for (int phase = 0; phase < 3; ++phase) {
        const bool rows = phase != 1;
        const int n = rows ? nr : nz;
        const int lines = rows ? nz : nr;
        const FftPlan& pl = rows ? *P.plx : *P.plz;
        const Cx<float>* tw = rows ? P.twx : P.twz;
        const Cx<float>* tq = tw + n;
        const int G = group_size_d(n);
        const int groups = NT / G;
        const int grp = threadIdx.x / G, lane = threadIdx.x - grp * G;
        Cx<float>* A = buf + (long)grp * 2 * n;
        Cx<float>* B = A + n;
        const int pairs = (lines + 1) / 2;
        const int rounds = (pairs + groups - 1) / groups;
        for (int rd = 0; rd < rounds; ++rd) {
            const int pr = rd * groups + grp;
            const bool act = pr < pairs;
            const int la = 2 * pr, lb = 2 * pr + 1;
            const bool hb = lb < lines;
            // element e of line l in the source array of this phase
            auto src = [&](const float* a, int l, int e) -> float {
                return rows ? a[(long)l * nr + e] : a[(long)e * nr + l];
            };
            const float* sin_ = (phase == 0) ? in : T_;
            if (act) {
                if (phase != 2) {  // REDFT10 input in Makhoul order
                    for (int j = lane; j < n; j += G) {
                        const int s = makhoul_src(j, n);
                        A[j] = Cx<float>{src(sin_, la, s), hb ? src(sin_, lb, s) : 0.f};
                    }
                } else {  // REDFT01 of the rows: W_k from X_k, X_(n-k)
                    for (int k = lane; k < n; k += G) {
                        const float xa = src(sin_, la, k), xan = k ? src(sin_, la, n - k) : 0.f;
                        const float xb = hb ? src(sin_, lb, k) : 0.f, xbn = (hb && k) ? src(sin_, lb, n - k) : 0.f;
                        A[k] = redft01_in<float>(xa, xan, xb, xbn, tq[k]);
                    }
                }
            }
            __syncthreads();
            Cx<float>* Z = fft_line<float>(A, B, pl, tw, phase == 2, lane, G, act);
            Cx<float>* Y = (Z == A) ? B : A;
            if (phase == 0) {
                if (act)
                    for (int k = lane; k < n; k += G) {
                        float ya, yb;
                        redft10_out<float>(Z, n, k, tq, ya, yb);
                        T_[(long)la * nr + k] = ya;
                        if (hb) T_[(long)lb * nr + k] = yb;
                    }
            } else if (phase == 1) {
                // columns la, lb: REDFT10 -> / Pre_Lcc -> REDFT01 (W built in Y from the values in Y's
                // second half... the coefficients are first stored as real pairs in Y)
                if (act)
                    for (int k = lane; k < n; k += G) {
                        float ya, yb;
                        redft10_out<float>(Z, n, k, tq, ya, yb);
                        ya = ya / P.lcc[(long)k * nr + la];
                        yb = hb ? yb / P.lcc[(long)k * nr + lb] : 0.f;
                        Y[k] = Cx<float>{ya, yb};
                    }
                __syncthreads();
                if (act)
                    for (int k = lane; k < n; k += G) {
                        const Cx<float> yk = Y[k], ynk = k ? Y[n - k] : Cx<float>{0.f, 0.f};
                        Z[k] = redft01_in<float>(yk.x, ynk.x, yk.y, ynk.y, tq[k]);
                    }
                __syncthreads();
                Cx<float>* V = fft_line<float>(Z, Y, *P.plz, tw, true, lane, G, act);
                if (act)
                    for (int e = lane; e < n; e += G) {
                        const Cx<float> v = V[makhoul_dst_src(e, n)];
                        T_[(long)e * nr + la] = v.x;
                        if (hb) T_[(long)e * nr + lb] = v.y;
                    }
            } else {
                if (act)
                    for (int e = lane; e < n; e += G) {
                        const Cx<float> v = Z[makhoul_dst_src(e, n)];
                        out[(long)la * nr + e] = v.x * scale;
                        if (hb) out[(long)lb * nr + e] = v.y * scale;
                    }
            }
            __syncthreads();
        }
    }
}

// y = A x for system P in FP32 (one row per q)
__device__ __forceinline__ float op32(const BProb& P, const float* __restrict__ x, long q) {
    if (P.system == DRD_SYS_UV) {
        const long mn = (long)(P.nr + 1) * P.nz;
        UVFetch<float> F{x, P.nr, P.nz, mn, 0};
        return uv_apply<float>(P.o32, P.rho32, P.eta32, P.pen32, F, q);
    }
    return pres_apply<float>(P.nr, P.nz, P.o32.idr2, P.o32.idz2, P.rho32, x, q);
}
__device__ __forceinline__ double op64(const BProb& P, const double* __restrict__ x, long q) {
    if (P.system == DRD_SYS_UV) {
        const long mn = (long)(P.nr + 1) * P.nz;
        UVFetch<double> F{x, P.nr, P.nz, mn, 0};
        return uv_apply<double>(P.o64, P.rho, P.eta, P.pen, F, q);
    }
    return pres_apply<double>(P.nr, P.nz, P.o64.idr2, P.o64.idz2, P.rho, x, q);
}

// One system's mixed-precision solve by the whole block.
template <int NT>
__device__ void solve_one(const BProb& P, BStat* st, Cx<float>* buf, int nmax, float* smf, double* smd) {
    const long n = P.n;
    const int tid = threadIdx.x;
    float* r = P.w;
    float* rt = r + n;
    float* p = rt + n;
    float* v = p + n;
    float* s = v + n;
    float* t = s + n;
    float* ph = t + n;
    float* sh = ph + n;
    float* d = sh + n;
    float* aux = d + n;  // UV: 1 / Jacobi diagonal; pressure: the transform scratch
    const bool uv = P.system == DRD_SYS_UV;
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    double bn = 0.0;
    for (long q = tid; q < n; q += NT) {
        const double bq = P.b[q];
        bn += bq * bq;
        P.x[q] = P.x0 ? P.x0[q] : 0.0;
        if (uv) aux[q] = 1.0f / uv_diag<float>(P.o32, P.rho32, P.eta32, q);
    }
    bn = sqrt(bsum_d<NT>(bn, smd));
    __syncthreads();
    int info = 1, iters = 0, sweeps = 0;
    double resid = 0.0, rn_prev = 0.0;
    float itol = (float)P.itol0;
    if (bn == 0.0) {
        for (long q = tid; q < n; q += NT) P.x[q] = 0.0;
        info = 0;
    }
    while (bn > 0.0) {
        // FP64 residual of the current x
        double rr = 0.0;
        for (long q = tid; q < n; q += NT) {
            const double rq = P.b[q] - op64(P, P.x, q);
            P.r64[q] = rq;
            rr += rq * rq;
        }
        const double rn = sqrt(bsum_d<NT>(rr, smd));
        resid = rn / bn;
        if (resid <= P.tol) { info = 0; break; }
        if (sweeps >= P.max_refine || !(resid == resid)) break;
        if (sweeps > 0 && rn > 0.9 * rn_prev) {
            itol *= 0.1f;
            if (itol < 1.5e-4f) break;  // the refinement has stalled
        }
        rn_prev = rn;
        ++sweeps;
        // FP32 BiCGSTAB for A d = r / ||r|| from d = 0
        const float inv = (float)(1.0 / rn);
        float a1 = 0.f, a2 = 0.f, a3 = 0.f;
        for (long q = tid; q < n; q += NT) {
            const float rq = (float)P.r64[q] * inv;
            r[q] = rq; rt[q] = rq; p[q] = 0.f; v[q] = 0.f; d[q] = 0.f;
            a1 += rq * rq;
        }
        bsum3<NT>(a1, a2, a3, smf);
        float rho = a1, rho1 = 1.f, alpha = 1.f, omega = 1.f;
        const float tiny = 1e-30f;
        for (int it = 0; it < P.maxit; ++it) {
            ++iters;
            const float beta = (rho / rho1) * (alpha / omega);
            // P = R + beta (P - omega V); PHAT = M^-1 P (Jacobi fused)
            for (long q = tid; q < n; q += NT) {
                const float pq = it == 0 ? r[q] : r[q] + beta * (p[q] - omega * v[q]);
                p[q] = pq;
                if (uv) ph[q] = pq * aux[q];
            }
            __syncthreads();
            if (!uv) pres_precond<NT>(P, p, aux, ph, buf, nmax);
            // V = A PHAT, (RT, V)
            a1 = 0.f; a2 = 0.f; a3 = 0.f;
            for (long q = tid; q < n; q += NT) {
                const float vq = op32(P, ph, q);
                v[q] = vq;
                a1 += rt[q] * vq;
            }
            bsum3<NT>(a1, a2, a3, smf);
            if (fabsf(a1) < tiny) break;  // breakdown: the refinement restarts
            alpha = rho / a1;
            // S = R - alpha V, ||S||; SHAT = M^-1 S (Jacobi fused)
            a1 = 0.f;
            for (long q = tid; q < n; q += NT) {
                const float sq = r[q] - alpha * v[q];
                s[q] = sq;
                if (uv) sh[q] = sq * aux[q];
                a1 += sq * sq;
            }
            bsum3<NT>(a1, a2, a3, smf);
            if (sqrtf(a1) <= itol) {  // early exit on ||s|| (:313-316)
                for (long q = tid; q < n; q += NT) d[q] += alpha * ph[q];
                __syncthreads();
                break;
            }
            if (!uv) pres_precond<NT>(P, s, aux, sh, buf, nmax);
            // T = A SHAT, (T, S), (T, T)
            a1 = 0.f; a2 = 0.f; a3 = 0.f;
            for (long q = tid; q < n; q += NT) {
                const float tq_ = op32(P, sh, q);
                t[q] = tq_;
                a1 += tq_ * s[q];
                a2 += tq_ * tq_;
            }
            bsum3<NT>(a1, a2, a3, smf);
            if (!(a2 > 0.f)) break;
            omega = a1 / a2;
            // D += alpha PHAT + omega SHAT; R = S - omega T; ||R||, (RT, R)
            a1 = 0.f; a2 = 0.f; a3 = 0.f;
            for (long q = tid; q < n; q += NT) {
                d[q] += alpha * ph[q] + omega * sh[q];
                const float rq = s[q] - omega * t[q];
                r[q] = rq;
                a1 += rq * rq;
                a2 += rt[q] * rq;
            }
            bsum3<NT>(a1, a2, a3, smf);
            rho1 = rho;
            rho = a2;
            if (sqrtf(a1) <= itol || fabsf(omega) < tiny || fabsf(rho) < tiny) break;
        }
        // x += ||r|| d in FP64
        for (long q = tid; q < n; q += NT) P.x[q] += rn * (double)d[q];
        __syncthreads();
    }
    unsigned long long t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    if (tid == 0) {
        st->info = info; st->iters = iters; st->refinements = sweeps;
        st->resid = resid; st->true_resid = resid; st->t0 = t0; st->t1 = t1;
    }
    __syncthreads();
}

// The persistent batch kernel: blocks pull systems from the queue (order[] is largest first).
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_batch(const BProb* __restrict__ probs, const int* __restrict__ order, int nprob,
                                              int* queue, BStat* stats, int nmax) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    Cx<float>* buf = reinterpret_cast<Cx<float>*>(sm_raw);
    __shared__ float smf[3 * 32];
    __shared__ double smd[32];
    __shared__ int next;
    __shared__ BProb P;
    for (;;) {
        if (threadIdx.x == 0) {
            next = atomicAdd(queue, 1);
            if (next < nprob) P = probs[order[next]];
        }
        __syncthreads();
        const int j = next;
        if (j >= nprob) break;
        solve_one<NT>(P, stats + order[j], buf, nmax, smf, smd);
        __syncthreads();
    }
}

// ---- host side ---------------------------------------------------------------------------
bool factor_plan(int n, FftPlan& pl) {
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
    return m == 1;
}

}  // namespace
}  // namespace drd

using namespace drd;

struct drd_batch {
    int nprob = 0;
    std::vector<BProb> hp;
    std::vector<long> n;
    std::vector<int> order;
    BProb* dp = nullptr;
    int* dorder = nullptr;
    int* dqueue = nullptr;
    BStat* dstat = nullptr;
    std::vector<BStat> hstat;
    std::vector<void*> allocs;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraphExec_t gx = nullptr;
    int threads = 512, bps = 2, nmax = 0, sms = 0;
    std::vector<int> lens;  // distinct transform lengths
    double last_bytes = 0.0;
    std::string err;
};

namespace {

#define BCK(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            b->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            return DRD_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

template <typename T>
int dalloc(drd_batch* b, T** p, size_t count) {
    void* q = nullptr;
    BCK(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    b->allocs.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return DRD_OK;
}
template <typename T>
int dup(drd_batch* b, T** p, const T* src, size_t count) {
    int rc = dalloc(b, p, count);
    if (rc) return rc;
    BCK(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, b->s));
    return DRD_OK;
}

// Shared memory of the transforms: per line length n, NT / G(n) groups of two lines of n complex
// values (G = 32, 64 or 128 threads by length, as pres_precond picks it).
size_t smem_bytes(const drd_batch* b, int threads);

size_t smem_bytes(const drd_batch* b, int threads) {
    size_t m = 16;
    for (int n : b->lens) m = std::max(m, (size_t)(threads / group_size_d(n)) * 2 * n * sizeof(Cx<float>));
    return m;
}

int launch(drd_batch* b, cudaStream_t s) {
    BCK(cudaMemsetAsync(b->dqueue, 0, sizeof(int), s));
    const int grid = b->sms * b->bps;
    const size_t sm = smem_bytes(b, b->threads);
    if (b->threads == 256)
        k_batch<256><<<grid, 256, sm, s>>>(b->dp, b->dorder, b->nprob, b->dqueue, b->dstat, b->nmax);
    else if (b->threads == 512)
        k_batch<512><<<grid, 512, sm, s>>>(b->dp, b->dorder, b->nprob, b->dqueue, b->dstat, b->nmax);
    else
        k_batch<1024><<<grid, 1024, sm, s>>>(b->dp, b->dorder, b->nprob, b->dqueue, b->dstat, b->nmax);
    BCK(cudaGetLastError());
    return DRD_OK;
}

int set_shape(drd_batch* b, int threads, int bps) {
    const size_t sm = smem_bytes(b, threads);
    cudaError_t e;
    if (threads == 256) e = cudaFuncSetAttribute(k_batch<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    else if (threads == 512) e = cudaFuncSetAttribute(k_batch<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    else e = cudaFuncSetAttribute(k_batch<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return DRD_ERR_CUDA; }
    int occ = 0;
    if (threads == 256) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch<256>, threads, sm);
    else if (threads == 512) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch<512>, threads, sm);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch<1024>, threads, sm);
    if (e != cudaSuccess || occ < 1) { b->err = "batch kernel does not fit on an SM"; return DRD_ERR_CUDA; }
    b->threads = threads;
    b->bps = std::min(bps, occ);
    if (b->gx) { cudaGraphExecDestroy(b->gx); b->gx = nullptr; }
    return DRD_OK;
}

int build_graph(drd_batch* b) {
    if (b->gx) return DRD_OK;
    BCK(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
    int rc = launch(b, b->s);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->s, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return DRD_ERR_CUDA; }
    e = cudaGraphInstantiate(&b->gx, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return DRD_ERR_CUDA; }
    return DRD_OK;
}

int run(drd_batch* b, double* seconds) {
    int rc = build_graph(b);
    if (rc) return rc;
    BCK(cudaEventRecord(b->e0, b->s));
    BCK(cudaGraphLaunch(b->gx, b->s));
    BCK(cudaEventRecord(b->e1, b->s));
    BCK(cudaMemcpyAsync(b->hstat.data(), b->dstat, sizeof(BStat) * b->nprob, cudaMemcpyDeviceToHost, b->s));
    BCK(cudaStreamSynchronize(b->s));
    float ms = 0.f;
    BCK(cudaEventElapsedTime(&ms, b->e0, b->e1));
    if (seconds) *seconds = ms * 1e-3;
    // algorithmic bytes: per FP32 iteration the fused minimum (the survey formula 23-25 vector
    // passes plus the coefficient reads), per FP64 sweep the residual (x, b, r, coefficients)
    double by = 0.0;
    for (int i = 0; i < b->nprob; ++i) {
        const BProb& P = b->hp[i];
        const double cs = (double)(P.nr + 2) * (P.nz + 2);
        const double it = b->hstat[i].iters, sw = b->hstat[i].refinements + 1;
        if (P.system == DRD_SYS_UV) by += it * 4.0 * (25.0 * P.n + 6.0 * cs) + sw * 8.0 * (3.0 * P.n + 3.0 * cs);
        else by += it * 4.0 * (23.0 * P.n + 4.0 * P.n) + sw * 8.0 * (4.0 * P.n);
    }
    b->last_bytes = by;
    return DRD_OK;
}

}  // namespace

extern "C" {

long drd_batch_length(int system, int nr, int nz) {
    if (system == DRD_SYS_UV) return (long)(nr + 1) * nz + (long)nr * (nz - 1);
    if (system == DRD_SYS_PRESSURE) return (long)nr * nz;
    return -1;
}

const char* drd_batch_last_error(drd_batch* b) { return b ? b->err.c_str() : "null batch"; }

int drd_batch_destroy(drd_batch* b) {
    if (!b) return DRD_ERR_BADARG;
    if (b->s) cudaStreamSynchronize(b->s);
    if (b->gx) cudaGraphExecDestroy(b->gx);
    for (void* p : b->allocs) cudaFree(p);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
    return DRD_OK;
}

int drd_batch_create(int nprob, const drd_batch_problem* probs, int autotune, drd_batch** out) {
    if (!out || nprob <= 0 || !probs) return DRD_ERR_BADARG;
    *out = nullptr;
    drd_batch* b = new drd_batch();
    auto fail = [&](int rc, const std::string& why) {
        if (!why.empty()) std::fprintf(stderr, "drd_batch_create: %s\n", why.c_str());
        drd_batch_destroy(b);
        return rc;
    };
    // validate everything before touching the device
    for (int i = 0; i < nprob; ++i) {
        const drd_batch_problem& q = probs[i];
        const drd_params& P = q.params;
        const bool uv = q.system == DRD_SYS_UV, pr = q.system == DRD_SYS_PRESSURE;
        FftPlan tmp;
        if ((!uv && !pr) || P.nr < 3 || P.nz < 3 || P.nr > DRD_BATCH_MAX_LINE || P.nz > DRD_BATCH_MAX_LINE ||
            !q.bdr_ph || !q.b || (uv && (!q.rho || !q.eta || (q.bdf != 1 && q.bdf != 2))) ||
            (pr && (!factor_plan(P.nr, tmp) || !factor_plan(P.nz, tmp))) || !(P.dr > 0) || !(P.dz > 0) ||
            !(P.dt > 0) || !(P.tol > 0) || !(P.mixed_inner_tol > 0) || P.mixed_max_refine <= 0 || P.uv_maxit <= 0 ||
            P.variant != DRD_VARIANT_MF)
            return fail(DRD_ERR_BADARG, "problem " + std::to_string(i) + " has invalid arguments");
    }
    b->nprob = nprob;
    if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess)
        return fail(DRD_ERR_CUDA, "stream or event creation failed");
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    // FFT plans and tables, one per distinct length
    std::map<int, std::pair<FftPlan*, Cx<float>*>> fft;
    auto fft_of = [&](int n) -> std::pair<FftPlan*, Cx<float>*> {
        auto it = fft.find(n);
        if (it != fft.end()) return it->second;
        FftPlan pl;
        factor_plan(n, pl);
        std::vector<Cx<float>> tab(FFT_TABLE(n));
        for (int m = 0; m < n; ++m) {
            const double a = -2.0 * kPiB * m / n;
            tab[m] = {(float)std::cos(a), (float)std::sin(a)};
            const double c = -kPiB * m / (2.0 * n);
            tab[n + m] = {(float)std::cos(c), (float)std::sin(c)};
        }
        FftPlan* dpl = nullptr;
        Cx<float>* dtab = nullptr;
        if (dup(b, &dpl, &pl, 1) || dup(b, &dtab, tab.data(), tab.size())) return {nullptr, nullptr};
        fft[n] = {dpl, dtab};
        b->lens.push_back(n);
        return fft[n];
    };
    b->hp.resize(nprob);
    for (int i = 0; i < nprob; ++i) {
        const drd_batch_problem& q = probs[i];
        const drd_params& Pp = q.params;
        BProb P{};
        P.system = q.system; P.bdf = q.bdf; P.nr = Pp.nr; P.nz = Pp.nz;
        P.n = drd_batch_length(q.system, P.nr, P.nz);
        const long n = P.n, cs = (long)(P.nr + 2) * (P.nz + 2);
        OpScal<double> o{};
        o.dt = Pp.dt; o.re = Pp.re; o.pk = Pp.penalty_k; o.dr = Pp.dr; o.dz = Pp.dz;
        o.dr2 = Pp.dr * Pp.dr; o.dz2 = Pp.dz * Pp.dz; o.idr2 = 1.0 / o.dr2; o.idz2 = 1.0 / o.dz2;
        o.idrdz = 1.0 / (Pp.dr * Pp.dz);
        o.nr = P.nr; o.nz = P.nz; o.variant = DRD_VARIANT_MF; o.lr_neumann = 0; o.bdf = q.bdf; o.phi_mode = 1;
        P.o64 = o;
        OpScal<float> f{};
        f.dt = (float)o.dt; f.re = (float)o.re; f.pk = (float)o.pk; f.dr = (float)o.dr; f.dz = (float)o.dz;
        f.dr2 = (float)o.dr2; f.dz2 = (float)o.dz2; f.idr2 = (float)o.idr2; f.idz2 = (float)o.idz2;
        f.idrdz = (float)o.idrdz; f.nr = o.nr; f.nz = o.nz; f.variant = o.variant; f.lr_neumann = 0; f.bdf = o.bdf;
        f.phi_mode = 1;
        P.o32 = f;
        P.tol = Pp.tol; P.itol0 = Pp.mixed_inner_tol; P.maxit = Pp.uv_maxit; P.max_refine = Pp.mixed_max_refine;
        int rc = 0;
        double *x, *r64;
        float* w;
        rc |= dalloc(b, &x, n) | dalloc(b, &r64, n) | dalloc(b, &w, 10 * (size_t)n);
        P.x = x; P.r64 = r64; P.w = w;
        double* db = nullptr;
        rc |= dup(b, &db, q.b, n);
        P.b = db;
        if (q.x0) {
            double* dx0 = nullptr;
            rc |= dup(b, &dx0, q.x0, n);
            P.x0 = dx0;
        }
        if (q.system == DRD_SYS_UV) {
            std::vector<float> f32(cs);
            double *r_, *e_, *p_;
            float *r32, *e32, *p32;
            rc |= dup(b, &r_, q.rho, cs) | dup(b, &e_, q.eta, cs) | dup(b, &p_, q.bdr_ph, cs);
            for (long k = 0; k < cs; ++k) f32[k] = (float)q.rho[k];
            rc |= dup(b, &r32, f32.data(), cs);
            for (long k = 0; k < cs; ++k) f32[k] = (float)q.eta[k];
            rc |= dup(b, &e32, f32.data(), cs);
            for (long k = 0; k < cs; ++k) f32[k] = (float)q.bdr_ph[k];
            rc |= dup(b, &p32, f32.data(), cs);
            P.rho = r_; P.eta = e_; P.pen = p_; P.rho32 = r32; P.eta32 = e32; P.pen32 = p32;
            P.cost = (double)n * 1.0;
        } else {
            // beta = 1 / (1 + penalty_k dt bdr_ph) on the interior cells, and Pre_Lcc (setup.f90:106-131)
            std::vector<double> beta(n);
            std::vector<float> b32(n), lcc(n);
            for (int k = 0; k < P.nz; ++k)
                for (int ii = 0; ii < P.nr; ++ii) {
                    const double bd = q.bdr_ph[(ii + 1) + (long)(k + 1) * (P.nr + 2)];
                    beta[ii + (long)k * P.nr] = 1.0 / (1.0 + Pp.penalty_k * Pp.dt * bd);
                    b32[ii + (long)k * P.nr] = (float)beta[ii + (long)k * P.nr];
                    const double tx = kPiB * ii / 2.0 / P.nr, tz = kPiB * k / 2.0 / P.nz;
                    double l = -(4.0 * std::sin(tx) * std::sin(tx) / o.dr2 + 4.0 * std::sin(tz) * std::sin(tz) / o.dz2);
                    if (ii == 0 && k == 0) l = -1.0;
                    lcc[ii + (long)k * P.nr] = (float)l;
                }
            double* db_;
            float *b32d, *lccd;
            rc |= dup(b, &db_, beta.data(), n) | dup(b, &b32d, b32.data(), n) | dup(b, &lccd, lcc.data(), n);
            P.rho = db_; P.rho32 = b32d; P.lcc = lccd;
            auto fx = fft_of(P.nr);
            auto fz = fft_of(P.nz);
            if (!fx.first || !fz.first) rc |= DRD_ERR_CUDA;
            P.plx = fx.first; P.twx = fx.second; P.plz = fz.first; P.twz = fz.second;
            b->nmax = std::max(b->nmax, std::max(P.nr, P.nz));
            P.cost = (double)n * 2.5;  // the transforms roughly double an iteration
        }
        if (rc) return fail(DRD_ERR_CUDA, b->err);
        b->hp[i] = P;
    }
    if (b->nmax == 0) b->nmax = 32;
    b->order.resize(nprob);
    for (int i = 0; i < nprob; ++i) b->order[i] = i;
    std::stable_sort(b->order.begin(), b->order.end(),
                     [&](int a, int c) { return b->hp[a].cost > b->hp[c].cost; });
    if (dup(b, &b->dp, b->hp.data(), nprob) || dup(b, &b->dorder, b->order.data(), nprob) ||
        dalloc(b, &b->dqueue, 1) || dalloc(b, &b->dstat, nprob))
        return fail(DRD_ERR_CUDA, b->err);
    b->hstat.assign(nprob, BStat{});
    if (cudaStreamSynchronize(b->s) != cudaSuccess) return fail(DRD_ERR_CUDA, "upload failed");
    int rc = set_shape(b, 512, 2);
    if (rc) return fail(rc, b->err);
    if (autotune) {
        // the launch shape: time the whole batch once per candidate, keep the fastest
        double best = 1e30;
        int bt = b->threads, bb = b->bps;
        const int cand[][2] = {{256, 4}, {512, 2}, {512, 1}, {1024, 1}};
        for (auto& c : cand) {
            if (set_shape(b, c[0], c[1])) continue;
            double sec = 0.0;
            if (run(b, &sec)) return fail(DRD_ERR_CUDA, b->err);
            if (sec < best) { best = sec; bt = b->threads; bb = b->bps; }
        }
        rc = set_shape(b, bt, bb);
        if (rc) return fail(rc, b->err);
    }
    *out = b;
    return DRD_OK;
}

int drd_batch_run(drd_batch* b, double* seconds) {
    if (!b) return DRD_ERR_BADARG;
    return run(b, seconds);
}

int drd_batch_result(drd_batch* b, int i, double* x, drd_status* st) {
    if (!b || i < 0 || i >= b->nprob) return DRD_ERR_BADARG;
    const BProb& P = b->hp[i];
    if (x) BCK(cudaMemcpy(x, P.x, sizeof(double) * P.n, cudaMemcpyDeviceToHost));
    const BStat& s = b->hstat[i];
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->info = s.info;
        st->iter = s.iters;
        st->resid = s.resid;
        st->true_resid = s.true_resid;
        st->refinements = s.refinements;
        st->flags = DRD_FLAG_REFINED;
        st->seconds = (double)(s.t1 - s.t0) * 1e-9;
    }
    return s.info;
}

int drd_batch_info(drd_batch* b, int* threads, int* blocks_per_sm, double* bytes_last_run) {
    if (!b) return DRD_ERR_BADARG;
    if (threads) *threads = b->threads;
    if (blocks_per_sm) *blocks_per_sm = b->bps;
    if (bytes_last_run) *bytes_last_run = b->last_bytes;
    return DRD_OK;
}

}  // extern "C"
