// drd_noalloc.cu — the pressure step without any device allocation.
//
// drd_presolve_2_noalloc computes what drd_presolve_2 computes (PreSolve_2 + dct_fftw:
// div u -> DCT-II -> / Pre_Lcc -> DCT-III -> / (4 nr nz) -> Neumann ghosts -> * coef) for
// callers that must not have the library allocate GPU memory: a host application whose
// device memory is entirely owned by its own pool allocator, or a driver that issues this
// step from code where cudaMalloc is not allowed.  The caller passes device pointers for the
// inputs and the output; every intermediate (divergence, transform passes, cosine and
// eigenvalue tables) lives in one file-scope __device__ array of fixed size, which every GPU
// that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "drd_common.cuh"

namespace {

constexpr int kMaxCells = DRD_NOALLOC_MAX_CELLS;  // nr * nz
constexpr int kMaxLine = DRD_NOALLOC_MAX_LINE;    // nr, nz
// layout: w | t1 | t2 (kMaxCells each) | cos_x (4 kMaxLine) | cos_z (4 kMaxLine) | eig_x | eig_z
constexpr long kScratchDoubles = 3L * kMaxCells + 8L * kMaxLine + 2L * (kMaxLine + 1);

// The scratch of every call.  Calls share it: each call overwrites every element it reads
// before reading it, so nothing has to start at zero, but two calls that overlap on the GPU
// (different streams, no ordering between them) race on it.
static __device__ __align__(256) double g_presolve_scratch[kScratchDoubles];

constexpr double kPi = 3.14159265358979323846264338327950288;

struct Scratch {
    double *w, *t1, *t2, *cx, *cz, *ex, *ez;
};

__host__ __device__ inline Scratch carve(double* base) {
    Scratch s;
    s.w = base;
    s.t1 = s.w + kMaxCells;
    s.t2 = s.t1 + kMaxCells;
    s.cx = s.t2 + kMaxCells;
    s.cz = s.cx + 4L * kMaxLine;
    s.ex = s.cz + 4L * kMaxLine;
    s.ez = s.ex + (kMaxLine + 1);
    return s;
}

// cos(pi q / (2n)) tables and the eigenvalues 4 sin^2(pi i / (2n)) / h^2 of setup()
// (microfluidics_complex_domain/setup.f90:108-131).
__global__ void k_na_tables(int nr, int nz, double dr2, double dz2, double* base) {
    Scratch s = carve(base);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (int q = tid; q < 4 * nr; q += nt) s.cx[q] = cos(kPi * (double)q / (2.0 * nr));
    for (int q = tid; q < 4 * nz; q += nt) s.cz[q] = cos(kPi * (double)q / (2.0 * nz));
    for (int i = tid; i <= nr; i += nt) {
        const double t = kPi * i / 2.0 / nr;
        s.ex[i] = 4.0 * (sin(t) * sin(t)) / dr2;
    }
    for (int j = tid; j <= nz; j += nt) {
        const double t = kPi * j / 2.0 / nz;
        s.ez[j] = 4.0 * (sin(t) * sin(t)) / dz2;
    }
}

// div u (PreSolve_2.f90:16-21)
__global__ void k_na_div(int nr, int nz, double dr, double dz, const double* __restrict__ u,
                         const double* __restrict__ v, double* base) {
    Scratch s = carve(base);
    const long n = (long)nr * nz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        s.w[q] = (u[drd::uidx(nr, i + 1, k)] - u[drd::uidx(nr, i, k)]) / dr +
                 (v[drd::vidx(nr, i, k + 1)] - v[drd::vidx(nr, i, k)]) / dz;
    }
}

// Transform along x of every row k: REDFT10 (kind 0, Y_o = 2 sum_j X_j cos(pi(2j+1)o/(2n)))
// or REDFT01 (kind 1, Y_o = X_0 + 2 sum_{j>=1} X_j cos(pi j(2o+1)/(2n))).  One block per row.
__global__ void k_na_xpass(int nr, int nz, int kind, const double* in, double* out, const double* cx) {
    const int k = blockIdx.x;
    if (k >= nz) return;
    const double* row = in + (long)k * nr;
    const long per = 4L * nr;
    for (int o = threadIdx.x; o < nr; o += blockDim.x) {
        double acc = 0.0;
        if (kind == 0) {
            for (int j = 0; j < nr; ++j) acc += row[j] * cx[((long)(2 * j + 1) * o) % per];
            out[(long)k * nr + o] = 2.0 * acc;
        } else {
            for (int j = 1; j < nr; ++j) acc += row[j] * cx[((long)j * (2 * o + 1)) % per];
            out[(long)k * nr + o] = row[0] + 2.0 * acc;
        }
    }
}

// Transform along z of every column i, threads over (i, k).  kind 0 (REDFT10) divides by
// Pre_Lcc(i,k) = -(ex(i) + ez(k)), -1 at (0,0); kind 1 (REDFT01) scales by coef / (4 nr nz) and
// writes psi's interior.
__global__ void k_na_zpass(int nr, int nz, int kind, const double* in, double* out, const double* cz,
                           const double* ex, const double* ez, double coef, double* psi) {
    const long n = (long)nr * nz;
    const long per = 4L * nz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        double acc = 0.0;
        if (kind == 0) {
            for (int j = 0; j < nz; ++j) acc += in[(long)j * nr + i] * cz[((long)(2 * j + 1) * k) % per];
            const double lcc = (i == 0 && k == 0) ? -1.0 : -(ex[i] + ez[k]);
            out[q] = (2.0 * acc) / lcc;
        } else {
            for (int j = 1; j < nz; ++j) acc += in[(long)j * nr + i] * cz[((long)j * (2 * k + 1)) % per];
            const double val = in[i] + 2.0 * acc;
            psi[drd::cidx(nr, i, k)] = (val / (4.0 * nr * nz)) * coef;
        }
    }
}

// Neumann ghosts of psi (dct_fftw.f90:41-51).  The interior was already scaled by coef, the
// reference's psi = psi*coef (PreSolve_2.f90:125), so the copies carry the scaled values.
__global__ void k_na_ghosts(int nr, int nz, double* psi) {
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
        psi[drd::cidx(nr, i, k)] = psi[drd::cidx(nr, si, sk)];
    }
}

// Device address of g_presolve_scratch in the current context, looked up on every call (a cheap
// host query): no address is cached, so a cudaDeviceReset, which unloads the module that holds
// the array, leaves nothing stale behind.
int scratch_address(double** out) {
    double* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_presolve_scratch);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "drd_presolve_2_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
        return DRD_ERR_CUDA;
    }
    *out = p;
    return DRD_OK;
}

}  // namespace

extern "C" int drd_presolve_2_noalloc(int nr, int nz, double dr, double dz, const double* d_u, const double* d_v,
                                      double coef, double* d_psi, void* stream) {
    if (!d_u || !d_v || !d_psi || nr < 3 || nz < 3 || !(dr > 0) || !(dz > 0)) return DRD_ERR_BADARG;
    if (nr > kMaxLine || nz > kMaxLine || (long)nr * nz > kMaxCells) {
        std::fprintf(stderr,
                     "drd_presolve_2_noalloc: grid %d x %d exceeds the fixed scratch (nr, nz <= %d, nr*nz <= %d)\n",
                     nr, nz, kMaxLine, kMaxCells);
        return DRD_ERR_TOO_LARGE;
    }
    double* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    Scratch sc = carve(base);
    const long n = (long)nr * nz;
    const int tpb = 256;
    const int gb = (int)std::min<long>((n + tpb - 1) / tpb, 2048);
    k_na_tables<<<8, tpb, 0, s>>>(nr, nz, dr * dr, dz * dz, base);
    k_na_div<<<gb, tpb, 0, s>>>(nr, nz, dr, dz, d_u, d_v, base);
    k_na_xpass<<<nz, 128, 0, s>>>(nr, nz, 0, sc.w, sc.t1, sc.cx);
    k_na_zpass<<<gb, tpb, 0, s>>>(nr, nz, 0, sc.t1, sc.t2, sc.cz, sc.ex, sc.ez, coef, d_psi);
    k_na_xpass<<<nz, 128, 0, s>>>(nr, nz, 1, sc.t2, sc.t1, sc.cx);
    k_na_zpass<<<gb, tpb, 0, s>>>(nr, nz, 1, sc.t1, sc.t2, sc.cz, sc.ex, sc.ez, coef, d_psi);
    k_na_ghosts<<<4, tpb, 0, s>>>(nr, nz, d_psi);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "drd_presolve_2_noalloc: launch failed: %s\n", cudaGetErrorString(e));
        return DRD_ERR_CUDA;
    }
    return DRD_OK;
}
