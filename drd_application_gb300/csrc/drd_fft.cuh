// drd_fft.cuh — mixed-radix FFTs in shared memory and the DCT-II / DCT-III (FFTW's REDFT10 /
// REDFT01, the transforms of microfluidics_complex_domain/dct_fftw.f90) built on them.
//
// A line of length n = 2^a 3^b 5^c 7^d is transformed by a group of G threads with a Stockham
// autosort FFT (one radix-R stage per pass, ping-pong between two shared-memory buffers, no
// bit reversal).  Two real lines travel as one complex line (re = line a, im = line b).
//
// DCT-II by one complex FFT of the same length (J. Makhoul, "A fast cosine transform in one
// and two dimensions", IEEE Trans. ASSP 28(1), 1980): v_j = x_2j, v_(n-1-j) = x_(2j+1),
// V = FFT(v), REDFT10(x)_k = 2 Re(e^(-i pi k / 2n) V_k).  DCT-III inverts that map:
// W_k = e^(i pi k / 2n) (X_k - i X_(n-k)) (X_n = 0) is Hermitian, v = sum_k W_k e^(2 pi i jk/n)
// is real, and REDFT01(X)_(2j) = v_j, REDFT01(X)_(2j+1) = v_(n-1-j).
//
// Tables per length n (host-built, FFT_TABLE(n) complex entries): tw[m] = e^(-2 pi i m / n),
// m < n; then tq[k] = e^(-i pi k / 2n), k < n.
#pragma once

#include <cuda_runtime.h>

namespace drd {

#define DRD_FFT_MAXST 24
struct FftPlan {
    int n;                              // transform length
    int nst;                            // radix stages
    unsigned char radix[DRD_FFT_MAXST]; // radices in stage order (4 first, then 2, 3, 5, 7)
};
#define FFT_TABLE(n) (2 * (n))

template <typename R>
struct Cx {
    R x, y;
};
template <typename R>
__device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename R>
__device__ __forceinline__ Cx<R> cadd(Cx<R> a, Cx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <typename R>
__device__ __forceinline__ Cx<R> csub(Cx<R> a, Cx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <typename R>
__device__ __forceinline__ Cx<R> conjx(Cx<R> a) { return {a.x, -a.y}; }

// cos and sin of 2 pi j / R for j = 0..R-1 (R = 3, 5, 7), to 21 digits; j and R - j mirror.
__host__ __device__ constexpr double root_c(int r, int j) {
    const int q = (j <= r / 2) ? j : r - j;
    return q == 0 ? 1.0
         : r == 3 ? -0.5
         : r == 5 ? (q == 1 ? 0.309016994374947424102 : -0.809016994374947424102)
                  : (q == 1 ? 0.623489801858733530525 : q == 2 ? -0.222520933956314404289 : -0.900968867902419126236);
}
__host__ __device__ constexpr double root_s(int r, int j) {
    const int q = (j <= r / 2) ? j : r - j;
    const double v = q == 0 ? 0.0
                   : r == 3 ? 0.866025403784438646764
                   : r == 5 ? (q == 1 ? 0.951056516295153572116 : 0.587785252292473129169)
                            : (q == 1 ? 0.781831482468029808708 : q == 2 ? 0.974927912181823607018 : 0.433883739117558120476);
    return (j <= r / 2) ? v : -v;
}

// In-place DFT of R points: X_m = sum_t v_t e^(-+2 pi i t m / R) (inverse: +).  Radix 2 and 4 by
// sums and differences; 3, 5 and 7 by the direct sum with constant roots (the loops unroll, so
// every root is an immediate).
template <int RAD, typename R>
__device__ __forceinline__ void dft_small(Cx<R> (&v)[RAD], bool inverse) {
    if constexpr (RAD == 2) {
        const Cx<R> a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (RAD == 4) {
        const Cx<R> a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        const Cx<R> b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
        // forward: X1 = a1 - i b1, X3 = a1 + i b1; inverse swaps them
        const Cx<R> jb1 = inverse ? Cx<R>{-b1.y, b1.x} : Cx<R>{b1.y, -b1.x};
        v[0] = cadd(a0, b0);
        v[2] = csub(a0, b0);
        v[1] = cadd(a1, jb1);
        v[3] = csub(a1, jb1);
    } else {
        Cx<R> o[RAD];
        const R sg = inverse ? R(1) : R(-1);
#pragma unroll
        for (int m = 0; m < RAD; ++m) {
            Cx<R> acc = v[0];
#pragma unroll
            for (int t = 1; t < RAD; ++t) {
                const int j = (t * m) % RAD;
                const Cx<R> e = {(R)root_c(RAD, j), sg * (R)root_s(RAD, j)};
                acc = cadd(acc, cmul(v[t], e));
            }
            o[m] = acc;
        }
#pragma unroll
        for (int m = 0; m < RAD; ++m) v[m] = o[m];
    }
}

// One Stockham stage of radix RAD over a group's line: a -> b.  Ns = product of the radices
// of the stages before it.
template <int RAD, typename R>
__device__ __forceinline__ void fft_stage(const Cx<R>* a, Cx<R>* b, int n, int Ns, const Cx<R>* __restrict__ w,
                                          bool inverse, int lane, int G) {
    const int m = n / RAD;
    const int twstep = n / (Ns * RAD);
    for (int j = lane; j < m; j += G) {
        const int k = j % Ns;
        Cx<R> v[RAD];
#pragma unroll
        for (int t = 0; t < RAD; ++t) {
            Cx<R> x = a[j + t * m];
            if (t > 0 && k > 0) {
                Cx<R> e = w[k * t * twstep];  // k t twstep < n
                if (inverse) e.y = -e.y;
                x = cmul(x, e);
            }
            v[t] = x;
        }
        dft_small<RAD, R>(v, inverse);
        const int o = (j / Ns) * Ns * RAD + k;
#pragma unroll
        for (int t = 0; t < RAD; ++t) b[o + t * Ns] = v[t];
    }
}

// The FFT of the line in `a` (length pl.n) by `G` threads with lanes 0..G-1; returns the buffer
// (a or b) that holds the result.  Every thread of the block must call it with the same plan
// (it synchronises the block between stages).
template <typename R>
__device__ Cx<R>* fft_line(Cx<R>* a, Cx<R>* b, const FftPlan& pl, const Cx<R>* __restrict__ w, bool inverse, int lane,
                           int G, bool active) {
    int Ns = 1;
    for (int s = 0; s < pl.nst; ++s) {
        const int rad = pl.radix[s];
        if (active) {
            switch (rad) {
                case 4: fft_stage<4, R>(a, b, pl.n, Ns, w, inverse, lane, G); break;
                case 2: fft_stage<2, R>(a, b, pl.n, Ns, w, inverse, lane, G); break;
                case 3: fft_stage<3, R>(a, b, pl.n, Ns, w, inverse, lane, G); break;
                case 5: fft_stage<5, R>(a, b, pl.n, Ns, w, inverse, lane, G); break;
                default: fft_stage<7, R>(a, b, pl.n, Ns, w, inverse, lane, G); break;
            }
        }
        __syncthreads();
        Cx<R>* t = a;
        a = b;
        b = t;
        Ns *= rad;
    }
    return a;
}

// Makhoul's input order: position j of the FFT line holds element src(j) of the real line.
__device__ __forceinline__ int makhoul_src(int j, int n) { return j < (n + 1) / 2 ? 2 * j : 2 * (n - 1 - j) + 1; }

// REDFT10 output k of lines a (re) and b (im) from their packed FFT Z (length n).
template <typename R>
__device__ __forceinline__ void redft10_out(const Cx<R>* Z, int n, int k, const Cx<R>* __restrict__ tq, R& ya, R& yb) {
    const Cx<R> zk = Z[k], zc = conjx(Z[k == 0 ? 0 : n - k]);
    const Cx<R> A = {(zk.x + zc.x) * R(0.5), (zk.y + zc.y) * R(0.5)};
    const Cx<R> D = csub(zk, zc);                      // 2 i B
    const Cx<R> B = {D.y * R(0.5), -D.x * R(0.5)};     // (zk - zc) / (2 i)
    const Cx<R> e = tq[k];
    ya = R(2) * (e.x * A.x - e.y * A.y);
    yb = R(2) * (e.x * B.x - e.y * B.y);
}

// REDFT01 input position k of the packed line from the coefficients Xa, Xb (X_n = 0):
// W_a + i W_b with W = conj(tq_k) (X_k - i X_(n-k)).
template <typename R>
__device__ __forceinline__ Cx<R> redft01_in(R xak, R xank, R xbk, R xbnk, const Cx<R> e) {
    const Cx<R> ec = conjx(e);
    const Cx<R> wa = cmul(ec, Cx<R>{xak, -xank});
    const Cx<R> wb = cmul(ec, Cx<R>{xbk, -xbnk});
    return {wa.x - wb.y, wa.y + wb.x};
}

// Output position of REDFT01 element y: even y = 2j comes from v_j, odd y = 2j+1 from v_(n-1-j).
__device__ __forceinline__ int makhoul_dst_src(int y, int n) { return (y & 1) ? n - 1 - (y >> 1) : (y >> 1); }

}  // namespace drd
