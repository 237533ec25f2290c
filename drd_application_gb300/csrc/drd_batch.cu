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
    int team, pad_;                  // blocks that share the system
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

// ---- teams: several blocks on one system --------------------------------------------------
// A large system is split over a team of T blocks (T = 1 for most): member m owns a contiguous
// chunk of the unknowns and of the transform lines.  Members meet at a counter barrier in global
// memory; the launch is cooperative, so every block of the grid is resident and a member that
// waits only waits for blocks that are running.  Values other members wrote are read with
// ld.global.cg (L2), never from a stale L1 line.  Reductions: each member stores its block sum
// in a double-buffered slot, all members then add the T slots in member order, so every member
// holds the same value.
#define DRD_BATCH_SPIN (1u << 23)  // polls of a barrier wait (256 ns apart: about 2 s)
struct Team {
    int m, T;
    int* bar;        // arrivals, zero before the launch
    float* redf;     // [2][T][4]
    double* redd;    // [2][T]
    int* err;        // set when a wait gave up
    int ep, rep;     // barrier and reduction episodes so far
};

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ void team_sync(Team& tm, int* sbad) {
    __syncthreads();
    if (tm.T > 1) {
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(tm.bar, 1);
            const int target = (tm.ep + 1) * tm.T;
            if (!*sbad) {
                unsigned polls = 0;
                while (ld_acquire(tm.bar) < target) {
                    if (++polls > DRD_BATCH_SPIN) { *sbad = 1; atomicExch(tm.err, 1); break; }
                    __nanosleep(256);
                }
            }
            __threadfence();
        }
        ++tm.ep;
        __syncthreads();
    }
}

template <int NT>
__device__ __forceinline__ void team_sum3(Team& tm, float& a, float& b, float& c, float* smf, int* sbad) {
    bsum3<NT>(a, b, c, smf);
    if (tm.T > 1) {
        float* slot = tm.redf + (tm.rep & 1) * tm.T * 4;
        if (threadIdx.x == 0) { slot[4 * tm.m] = a; slot[4 * tm.m + 1] = b; slot[4 * tm.m + 2] = c; }
        team_sync(tm, sbad);
        a = 0.f; b = 0.f; c = 0.f;
        for (int j = 0; j < tm.T; ++j) {
            a += __ldcg(slot + 4 * j); b += __ldcg(slot + 4 * j + 1); c += __ldcg(slot + 4 * j + 2);
        }
        ++tm.rep;
    }
}

template <int NT>
__device__ __forceinline__ double team_sumd(Team& tm, double a, double* smd, int* sbad) {
    a = bsum_d<NT>(a, smd);
    if (tm.T > 1) {
        double* slot = tm.redd + (tm.rep & 1) * tm.T;
        if (threadIdx.x == 0) slot[tm.m] = a;
        team_sync(tm, sbad);
        a = 0.0;
        for (int j = 0; j < tm.T; ++j) a += __ldcg(slot + j);
        ++tm.rep;
    }
    return a;
}

// ---- the pressure operator (FP64 or FP32) ------------------------------------------------
// (A psi)_(i,k) = [bx(i+1,k)(psi_(i+1) - psi_i) - bx(i,k)(psi_i - psi_(i-1))] / dr^2
//               + [bz(i,k+1)(psi_(k+1) - psi_k) - bz(i,k)(psi_k - psi_(k-1))] / dz^2,
// face coefficients the mean of the two cells' beta, zero on the domain faces.
template <typename T>
__device__ __forceinline__ T ldv(const T* p) { return __ldcg(p); }

template <typename T>
__device__ __forceinline__ T pres_apply(int nr, int nz, T idr2, T idz2, const T* __restrict__ beta,
                                        const T* __restrict__ x, long q) {
    const int k = (int)(q / nr), i = (int)(q - (long)k * nr);
    const T c = ldv(x + q), bc = beta[q];
    T fx = T(0), fz = T(0);
    if (i + 1 < nr) fx += (bc + beta[q + 1]) * T(0.5) * (ldv(x + q + 1) - c);
    if (i > 0) fx -= (bc + beta[q - 1]) * T(0.5) * (c - ldv(x + q - 1));
    if (k + 1 < nz) fz += (bc + beta[q + nr]) * T(0.5) * (ldv(x + q + nr) - c);
    if (k > 0) fz -= (bc + beta[q - nr]) * T(0.5) * (c - ldv(x + q - nr));
    return fx * idr2 + fz * idz2;
}

__host__ __device__ __forceinline__ int group_size_d(int n) { return n >= 512 ? 128 : (n >= 128 ? 64 : 32); }

// ---- the pressure preconditioner: out = REDFT01(REDFT10(in) / Pre_Lcc) / (4 nr nz) ---------
// Three phases over a scratch array T (nr*nz, i fastest): rows (REDFT10), columns (REDFT10,
// / Pre_Lcc, REDFT01), rows (REDFT01, scale), with a team barrier after each.  Groups of G
// threads take a pair of lines per round (the team's groups share the lines); `buf` holds two
// ping-pong lines of n complex values per group.
template <int NT>
__device__ void pres_precond(const BProb& P, const float* __restrict__ in, float* __restrict__ T_, float* __restrict__ out,
                             Cx<float>* buf, Team& tm, int* sbad) {
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
        const int tg = groups * tm.T;                 // the team's groups
        const int rounds = (pairs + tg - 1) / tg;
        for (int rd = 0; rd < rounds; ++rd) {
            const int pr = rd * tg + tm.m * groups + grp;
            const bool act = pr < pairs;
            const int la = 2 * pr, lb = 2 * pr + 1;
            const bool hb = lb < lines;
            auto src = [&](const float* a, int l, int e) -> float {
                return ldv(rows ? a + (long)l * nr + e : a + (long)e * nr + l);
            };
            const float* sin_ = (phase == 0) ? in : T_;
            if (act) {
                if (phase != 2) {  // REDFT10 input in Makhoul order
                    for (int j = lane; j < n; j += G) {
                        const int sj = makhoul_src(j, n);
                        A[j] = Cx<float>{src(sin_, la, sj), hb ? src(sin_, lb, sj) : 0.f};
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
                // columns la, lb: REDFT10, / Pre_Lcc into Y as (a, b) pairs, then REDFT01's W in Z
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
        team_sync(tm, sbad);
    }
}

// y = A x for system P in FP32 (one row per q); x is read through L2
__device__ __forceinline__ float op32(const BProb& P, const float* __restrict__ x, long q) {
    if (P.system == DRD_SYS_UV) {
        const long mn = (long)(P.nr + 1) * P.nz;
        UVFetch<float, true> F{x, P.nr, P.nz, mn, 0};
        return uv_apply<float>(P.o32, P.rho32, P.eta32, P.pen32, F, q);
    }
    return pres_apply<float>(P.nr, P.nz, P.o32.idr2, P.o32.idz2, P.rho32, x, q);
}

// One system's mixed-precision solve by a team of blocks (a single block when T = 1).  The
// member's unknowns are [lo, hi).  Every pass handles U rows per thread per step, with all of
// their loads issued before any use, so that a thread keeps U memory requests in flight (the
// passes are bound by memory latency, not bandwidth, at one or a few blocks per system).
#define BU 4
#define FOR_U(q0) for (long q0 = lo + tid; q0 < hi; q0 += BU * NT)
#define LANES(u) _Pragma("unroll") for (int u = 0; u < BU; ++u)
template <int NT>
__device__ void solve_one(const BProb& P, BStat* st, Cx<float>* buf, float* smf, double* smd, Team& tm, int* sbad) {
    const long n = P.n;
    const long lo = n * tm.m / tm.T, hi = n * (tm.m + 1) / tm.T;
    const int tid = threadIdx.x;
    float* __restrict__ r = P.w;
    float* __restrict__ rt = r + n;
    float* __restrict__ p = rt + n;
    float* __restrict__ v = p + n;
    float* __restrict__ s = v + n;
    float* __restrict__ t = s + n;
    float* __restrict__ ph = t + n;
    float* __restrict__ sh = ph + n;
    float* __restrict__ d = sh + n;
    float* __restrict__ aux = d + n;  // UV: 1 / Jacobi diagonal; pressure: the transform scratch
    const bool uv = P.system == DRD_SYS_UV;
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    double bn = 0.0;
    for (long q = lo + tid; q < hi; q += NT) {
        const double bq = P.b[q];
        bn += bq * bq;
        P.x[q] = P.x0 ? P.x0[q] : 0.0;
        if (uv) aux[q] = 1.0f / uv_diag<float>(P.o32, P.rho32, P.eta32, q);
    }
    bn = sqrt(team_sumd<NT>(tm, bn, smd, sbad));
    int info = 1, iters = 0, sweeps = 0;
    double resid = 0.0, rn_prev = 0.0;
    float itol = (float)P.itol0;
    if (bn == 0.0) info = 0;
    while (bn > 0.0 && !*sbad) {
        // FP64 residual of the current x (every member's x chunk is complete: barrier above);
        // the operator in the difference form with reciprocals, off GB300's slow FP64 divide
        double rr = 0.0;
        FOR_U(q0) {
            double ax[BU];
            LANES(u) {
                const long q = q0 + (long)u * NT;
                if (q < hi) {
                    if (P.system == DRD_SYS_UV) {
                        UVFetch<double, true> F{P.x, P.nr, P.nz, (long)(P.nr + 1) * P.nz, 0};
                        ax[u] = uv_apply<double, UVFetch<double, true>, true>(P.o64, P.rho, P.eta, P.pen, F, q);
                    } else {
                        ax[u] = pres_apply<double>(P.nr, P.nz, P.o64.idr2, P.o64.idz2, P.rho, P.x, q);
                    }
                }
            }
            LANES(u) {
                const long q = q0 + (long)u * NT;
                if (q < hi) {
                    const double rq = P.b[q] - ax[u];
                    P.r64[q] = rq;
                    rr += rq * rq;
                }
            }
        }
        const double rn = sqrt(team_sumd<NT>(tm, rr, smd, sbad));
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
        FOR_U(q0) {
            float rq[BU];
            LANES(u) { const long q = q0 + (long)u * NT; rq[u] = q < hi ? (float)__ldcg(P.r64 + q) * inv : 0.f; }
            LANES(u) {
                const long q = q0 + (long)u * NT;
                if (q < hi) { r[q] = rq[u]; rt[q] = rq[u]; p[q] = 0.f; v[q] = 0.f; d[q] = 0.f; a1 += rq[u] * rq[u]; }
            }
        }
        team_sum3<NT>(tm, a1, a2, a3, smf, sbad);
        float rho = a1, rho1 = 1.f, alpha = 1.f, omega = 1.f;
        const float tiny = 1e-30f;
        for (int it = 0; it < P.maxit && !*sbad; ++it) {
            ++iters;
            const float beta = (rho / rho1) * (alpha / omega);
            // P = R + beta (P - omega V); PHAT = M^-1 P (Jacobi fused)
            FOR_U(q0) {
                float rq[BU], pq[BU], vq[BU], dq[BU];
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) {
                        rq[u] = __ldcg(r + q); pq[u] = __ldcg(p + q); vq[u] = __ldcg(v + q);
                        dq[u] = uv ? __ldcg(aux + q) : 0.f;
                    }
                }
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) {
                        const float pn = it == 0 ? rq[u] : rq[u] + beta * (pq[u] - omega * vq[u]);
                        p[q] = pn;
                        if (uv) ph[q] = pn * dq[u];
                    }
                }
            }
            team_sync(tm, sbad);
            if (!uv) pres_precond<NT>(P, p, aux, ph, buf, tm, sbad);
            // V = A PHAT, (RT, V)
            a1 = 0.f; a2 = 0.f; a3 = 0.f;
            FOR_U(q0) {
                float vq[BU], tq[BU];
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) { vq[u] = op32(P, ph, q); tq[u] = __ldcg(rt + q); }
                }
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) { v[q] = vq[u]; a1 += tq[u] * vq[u]; }
                }
            }
            team_sum3<NT>(tm, a1, a2, a3, smf, sbad);
            if (fabsf(a1) < tiny) break;  // breakdown: the refinement restarts
            alpha = rho / a1;
            // S = R - alpha V, ||S||; SHAT = M^-1 S (Jacobi fused)
            a1 = 0.f;
            FOR_U(q0) {
                float rq[BU], vq[BU], dq[BU];
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) { rq[u] = __ldcg(r + q); vq[u] = __ldcg(v + q); dq[u] = uv ? __ldcg(aux + q) : 0.f; }
                }
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) {
                        const float sq = rq[u] - alpha * vq[u];
                        s[q] = sq;
                        if (uv) sh[q] = sq * dq[u];
                        a1 += sq * sq;
                    }
                }
            }
            team_sum3<NT>(tm, a1, a2, a3, smf, sbad);
            if (sqrtf(a1) <= itol) {  // early exit on ||s|| (:313-316)
                for (long q = lo + tid; q < hi; q += NT) d[q] = __ldcg(d + q) + alpha * __ldcg(ph + q);
                break;
            }
            if (!uv) pres_precond<NT>(P, s, aux, sh, buf, tm, sbad);
            // T = A SHAT, (T, S), (T, T)
            a1 = 0.f; a2 = 0.f; a3 = 0.f;
            FOR_U(q0) {
                float wq[BU], sq[BU];
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) { wq[u] = op32(P, sh, q); sq[u] = __ldcg(s + q); }
                }
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) { t[q] = wq[u]; a1 += wq[u] * sq[u]; a2 += wq[u] * wq[u]; }
                }
            }
            team_sum3<NT>(tm, a1, a2, a3, smf, sbad);
            if (!(a2 > 0.f)) break;
            omega = a1 / a2;
            // D += alpha PHAT + omega SHAT; R = S - omega T; ||R||, (RT, R)
            a1 = 0.f; a2 = 0.f; a3 = 0.f;
            FOR_U(q0) {
                float dq[BU], pq[BU], hq[BU], sq[BU], wq[BU], tq[BU];
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) {
                        dq[u] = __ldcg(d + q); pq[u] = __ldcg(ph + q); hq[u] = __ldcg(sh + q);
                        sq[u] = __ldcg(s + q); wq[u] = __ldcg(t + q); tq[u] = __ldcg(rt + q);
                    }
                }
                LANES(u) {
                    const long q = q0 + (long)u * NT;
                    if (q < hi) {
                        d[q] = dq[u] + alpha * pq[u] + omega * hq[u];
                        const float rq = sq[u] - omega * wq[u];
                        r[q] = rq;
                        a1 += rq * rq;
                        a2 += tq[u] * rq;
                    }
                }
            }
            team_sum3<NT>(tm, a1, a2, a3, smf, sbad);
            rho1 = rho;
            rho = a2;
            if (sqrtf(a1) <= itol || fabsf(omega) < tiny || fabsf(rho) < tiny) break;
        }
        // x += ||r|| d in FP64, then every member's chunk is complete before the next residual
        for (long q = lo + tid; q < hi; q += NT) P.x[q] = __ldcg(P.x + q) + rn * (double)__ldcg(d + q);
        team_sync(tm, sbad);
    }
    unsigned long long t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    if (tid == 0 && tm.m == 0) {
        st->info = *sbad ? DRD_ERR_TIMEOUT : info; st->iters = iters; st->refinements = sweeps;
        st->resid = resid; st->true_resid = resid; st->t0 = t0; st->t1 = t1;
    }
    __syncthreads();
}
#undef FOR_U
#undef LANES
#undef BU

// The persistent batch kernel (cooperative launch: every block resident).  Blocks pull slots
// from the queue: slot j names a system and a member index; a system of team size T has T
// consecutive slots (systems largest first).
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_batch(const BProb* __restrict__ probs, const int2* __restrict__ slots,
                                                         int nslots, int* queue, BStat* stats, int* bars, float* redf,
                                                         double* redd, const int* tbase, int* err) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    Cx<float>* buf = reinterpret_cast<Cx<float>*>(sm_raw);
    __shared__ float smf[3 * 32];
    __shared__ double smd[32];
    __shared__ int next;
    __shared__ int sbad;
    __shared__ BProb P;
    for (;;) {
        if (threadIdx.x == 0) {
            next = atomicAdd(queue, 1);
            if (next < nslots) P = probs[slots[next].x];
            sbad = 0;
        }
        __syncthreads();
        const int j = next;
        if (j >= nslots) break;
        const int id = slots[j].x;
        Team tm;
        tm.m = slots[j].y;
        tm.T = P.team;
        tm.bar = bars + id;
        tm.redf = redf + 8L * tbase[id];
        tm.redd = redd + 2L * tbase[id];
        tm.err = err;
        tm.ep = 0;
        tm.rep = 0;
        solve_one<NT>(P, stats + id, buf, smf, smd, tm, &sbad);
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
    std::vector<int> order;          // systems, largest first
    BProb* dp = nullptr;
    int2* dslots = nullptr;          // (system, member) per slot
    int nslots = 0;
    int* dqueue = nullptr;           // [0] next slot, [1] error flag
    int* dbars = nullptr;            // team barrier counters, one per system
    float* dredf = nullptr;          // team reduction slots
    double* dredd = nullptr;
    int* dtbase = nullptr;           // per system: first team slot (prefix sum of team sizes)
    BStat* dstat = nullptr;
    double team_scale = 2.0;         // teams sized so that the work splits into ~scale x grid parts
    std::vector<BStat> hstat;
    std::vector<void*> allocs;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraphExec_t gx = nullptr;
    int threads = 512, bps = 2, regs = 64, nmax = 0, sms = 0;
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

typedef void (*BatchKernel)(const BProb*, const int2*, int, int*, BStat*, int*, float*, double*, const int*, int*);
// Instantiations: threads per block x register budget (64 or 128 registers per thread).
BatchKernel kernel_of(int threads, int regs) {
    if (threads == 256) return regs > 64 ? k_batch<256, 2> : k_batch<256, 4>;
    if (threads == 512) return regs > 64 ? k_batch<512, 1> : k_batch<512, 2>;
    return k_batch<1024, 1>;
}

int launch(drd_batch* b, cudaStream_t s) {
    BCK(cudaMemsetAsync(b->dqueue, 0, 2 * sizeof(int), s));
    BCK(cudaMemsetAsync(b->dbars, 0, sizeof(int) * b->nprob, s));
    const int grid = b->sms * b->bps;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(b->threads);
    cfg.dynamicSmemBytes = smem_bytes(b, b->threads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every block resident: team waits end
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kernel_of(b->threads, b->regs), (const BProb*)b->dp,
                                       (const int2*)b->dslots, b->nslots, b->dqueue, b->dstat, b->dbars, b->dredf,
                                       b->dredd, (const int*)b->dtbase, b->dqueue + 1);
    if (e != cudaSuccess) { b->err = std::string("batch launch: ") + cudaGetErrorString(e); return DRD_ERR_CUDA; }
    return DRD_OK;
}

// Team sizes and the slot queue: with `scale` > 0 a system of cost c gets
// T = clamp(ceil(c / (total / (scale * grid))), 1, 8) blocks; scale 0 gives every system one.
int plan_teams(drd_batch* b, double scale) {
    const int grid = b->sms * b->bps;
    double total = 0.0;
    for (const BProb& P : b->hp) total += P.cost;
    const double part = scale > 0 ? total / (scale * grid) : 1e300;
    std::vector<int2> slots;
    std::vector<int> tbase(b->nprob);
    int base = 0;
    for (int i = 0; i < b->nprob; ++i) {
        BProb& P = b->hp[i];
        P.team = std::max(1, std::min(8, (int)std::ceil(P.cost / part)));
        P.team = std::min(P.team, grid);
        tbase[i] = base;
        base += P.team;
    }
    for (int id : b->order)
        for (int m = 0; m < b->hp[id].team; ++m) slots.push_back(make_int2(id, m));
    b->nslots = (int)slots.size();
    if (b->dslots) { cudaFree(b->dslots); b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void*)b->dslots)); }
    if (b->dredf) { cudaFree(b->dredf); b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void*)b->dredf)); }
    if (b->dredd) { cudaFree(b->dredd); b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void*)b->dredd)); }
    b->dslots = nullptr; b->dredf = nullptr; b->dredd = nullptr;
    if (dup(b, &b->dslots, slots.data(), slots.size()) || dalloc(b, &b->dredf, 8 * (size_t)base) ||
        dalloc(b, &b->dredd, 2 * (size_t)base))
        return DRD_ERR_CUDA;
    BCK(cudaMemcpyAsync(b->dtbase, tbase.data(), sizeof(int) * b->nprob, cudaMemcpyHostToDevice, b->s));
    BCK(cudaMemcpyAsync(b->dp, b->hp.data(), sizeof(BProb) * b->nprob, cudaMemcpyHostToDevice, b->s));
    BCK(cudaStreamSynchronize(b->s));
    b->team_scale = scale;
    if (b->gx) { cudaGraphExecDestroy(b->gx); b->gx = nullptr; }
    return DRD_OK;
}

int set_shape(drd_batch* b, int threads, int regs) {
    const size_t sm = smem_bytes(b, threads);
    BatchKernel k = kernel_of(threads, regs);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return DRD_ERR_CUDA; }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, sm);
    if (e != cudaSuccess || occ < 1) { b->err = "batch kernel does not fit on an SM"; return DRD_ERR_CUDA; }
    b->threads = threads;
    b->regs = (threads == 1024) ? 64 : regs;
    b->bps = occ;  // registers and shared memory per block decide how many fit
    if (b->gx) { cudaGraphExecDestroy(b->gx); b->gx = nullptr; }
    return plan_teams(b, b->team_scale);
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
    int flags[2] = {0, 0};
    BCK(cudaMemcpyAsync(flags, b->dqueue, sizeof(flags), cudaMemcpyDeviceToHost, b->s));
    BCK(cudaStreamSynchronize(b->s));
    if (flags[1]) { b->err = "a team barrier wait gave up"; return DRD_ERR_TIMEOUT; }
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
            P.cost = (double)n * std::sqrt((double)n);  // Jacobi: iterations grow like the grid's side
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
            P.cost = (double)n * 40.0;  // about 20 iterations, each about twice a momentum one
        }
        if (rc) return fail(DRD_ERR_CUDA, b->err);
        b->hp[i] = P;
    }
    if (b->nmax == 0) b->nmax = 32;
    b->order.resize(nprob);
    for (int i = 0; i < nprob; ++i) b->order[i] = i;
    std::stable_sort(b->order.begin(), b->order.end(),
                     [&](int a, int c) { return b->hp[a].cost > b->hp[c].cost; });
    if (dup(b, &b->dp, b->hp.data(), nprob) || dalloc(b, &b->dqueue, 2) || dalloc(b, &b->dstat, nprob) ||
        dalloc(b, &b->dbars, nprob) || dalloc(b, &b->dtbase, nprob))
        return fail(DRD_ERR_CUDA, b->err);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return fail(DRD_ERR_UNSUPPORTED, "the device has no cooperative launch");
    b->hstat.assign(nprob, BStat{});
    if (cudaStreamSynchronize(b->s) != cudaSuccess) return fail(DRD_ERR_CUDA, "upload failed");
    int rc = set_shape(b, 512, 64);
    if (rc) return fail(rc, b->err);
    if (autotune) {
        // the launch shape, then the team sizes: time the whole batch once per candidate and
        // keep the fastest
        double best = 1e30;
        int bt = b->threads, bb = b->regs;
        const int cand[][2] = {{256, 64}, {512, 64}, {1024, 64}, {256, 128}, {512, 128}};
        for (auto& c : cand) {
            if (set_shape(b, c[0], c[1])) continue;
            double sec = 0.0;
            if (run(b, &sec)) return fail(DRD_ERR_CUDA, b->err);
            if (sec < best) { best = sec; bt = b->threads; bb = b->regs; }
        }
        rc = set_shape(b, bt, bb);
        if (rc) return fail(rc, b->err);
        double bs = b->team_scale;
        for (double sc : {0.0, 1.0, 4.0}) {
            if (plan_teams(b, sc)) return fail(DRD_ERR_CUDA, b->err);
            double sec = 0.0;
            if (run(b, &sec)) return fail(DRD_ERR_CUDA, b->err);
            if (sec < best) { best = sec; bs = sc; }
        }
        if (plan_teams(b, bs)) return fail(DRD_ERR_CUDA, b->err);
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
