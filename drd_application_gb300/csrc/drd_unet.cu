// drd_unet.cu — the learned initial guess of the Krylov solves: a 4-level U-Net (32 base
// channels, 3x3 convolutions, BF16 weights and activations, FP32 accumulation) with its
// forward pass, backward pass and Adam update, all as hand-written kernels.  The convolutions
// and weight gradients run on the BF16 tensor cores (mma.sync m16n8k16 with FP32 accumulators)
// from ldmatrix fragments of pixel tiles staged in shared memory with their halo.
//
// The network maps (normalised residual, resistance, phase field) on the solver's grid to a
// normalised correction of the solve's initial guess; the caller scales it back and the
// solver's FP64 true residual judges the corrected guess against the plain one.
//
// Layout on the device:
//   activations  NHWC BF16, grid padded to Hp x Wp (multiples of 8, zero input outside the
//                caller's H x W); level l has (Hp >> l) x (Wp >> l) pixels and 32 << l channels.
//   skip joins   the encoder output of level l is written straight into channels [C_l, 2C_l)
//                of the decoder's concatenation buffer cat_l; the upsampling convolution
//                writes channels [0, C_l).  No copy joins them.
//   parameters   one flat FP32 array (master copy, Adam state alongside); conv weights are
//                [tap][Cout][Cin], then the bias [Cout].  Two BF16 copies are kept: the same
//                layout for the forward pass, and [8 - tap][Cin][Cout] (the flipped transpose)
//                for the data gradient, which then runs through the forward kernel.
//   caller I/O   FP32 NCHW (batch, channels, H, W) on the caller's H x W grid, host or device.
//
// Architecture (conv = 3x3 same-padding + bias + ReLU):
//   enc l (l = 0..3): conv(C_in_l -> C_l), conv(C_l -> C_l) = e_l;  2x2 average pool between levels
//   dec l (l = 2..0): conv(up2(d_{l+1}) -> C_l) || e_l  ->  conv(2C_l -> C_l), conv(C_l -> C_l) = d_l
//   out: 1x1 conv(C_0 -> out_ch), no activation.  d_3 = e_3 (the bottleneck).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "../../include/drd_gb300.h"

typedef __nv_bfloat16 bf16;

namespace {

constexpr int kLevels = 4;
constexpr int kBase = 32;
constexpr int kCinPad = 16;   // the input's channels, zero-padded to one MMA K step
constexpr int kMaxOut = 4;
constexpr int kConvTPB = 128; // 4 warps per block of the convolution, one tile row each

// ------------------------------------------------------------------------------------------
// tensor-core primitive: D(16x8, f32) += A(16x16, bf16, row) * B(16x8, bf16, col)
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}


// ------------------------------------------------------------------------------------------
// 3x3 convolution as an implicit GEMM: M = pixels, N = output channels, K = 9 taps x Cin.
// A block computes a tile of kTH x kTW pixels (one image row of kTW pixels per warp, two MMA
// row tiles) for 32 output channels.  Per chunk of kc input channels it stages the tile's
// input with its one-pixel halo and the 9 taps' weights in shared memory (rows padded by 8
// elements, so that the 8 rows an ldmatrix phase reads fall in distinct banks); the MMA
// fragments then come from shared memory through ldmatrix.  With `up`, the input is at half
// resolution and is read through nearest upsampling.  The same kernel computes data
// gradients (weights = the flipped transpose, no bias/ReLU); `mask` then applies the ReLU
// derivative of the layer below (zero where mask <= 0).
constexpr int kTH = 4, kTW = 32, kKC = 32;
constexpr int kHaloPix = (kTH + 2) * (kTW + 2);

struct ConvArgs {
    const bf16* x; long xbs; int ldx;
    const bf16* w; const float* bias;
    bf16* y; float* yf; long ybs; int ldy;
    const bf16* mask; long mbs; int ldm;
    int H, W, Cin, Cout, up, relu;
};

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const bf16* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__global__ void __launch_bounds__(kConvTPB) k_conv3(ConvArgs a) {
    __shared__ __align__(16) bf16 s_in[kHaloPix * (kKC + 8)];
    __shared__ __align__(16) bf16 s_w[9 * 32 * (kKC + 8)];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int nco = a.Cout / 32;
    const int b = blockIdx.z / nco, co0 = (blockIdx.z % nco) * 32;
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    const int kc = (a.Cin % kKC == 0) ? kKC : 16;  // channels per staged chunk
    const int ps = kc + 8;                          // padded row of one pixel / one weight row
    const int parts = kc / 8;                       // 16-byte pieces per row
    const bf16* xb = a.x + (long)b * a.xbs;
    const int Wl = a.W >> 1;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
    // ldmatrix row addresses: A rows are pixels (lane&7) + 8*((lane>>3)&1), k offset 8*(lane>>4);
    // B rows are output channels 8*(lane>>4) + (lane&7), k offset 8*((lane>>3)&1)
    const int a_row = (lane & 7) + ((lane >> 3) & 1) * 8, a_k = (lane >> 4) * 8;
    const int b_row = (lane >> 4) * 8 + (lane & 7), b_k = ((lane >> 3) & 1) * 8;

    for (int c0 = 0; c0 < a.Cin; c0 += kc) {
        for (int i = threadIdx.x; i < kHaloPix * parts; i += kConvTPB) {
            const int pix = i / parts, part = i - pix * parts;
            const int ty = pix / (kTW + 2), tx = pix - ty * (kTW + 2);
            const int gy = y0 + ty - 1, gx = x0 + tx - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) {
                const long sp = a.up ? (long)(gy >> 1) * Wl + (gx >> 1) : (long)gy * a.W + gx;
                v = __ldg(reinterpret_cast<const uint4*>(xb + sp * a.ldx + c0 + part * 8));
            }
            *reinterpret_cast<uint4*>(s_in + pix * ps + part * 8) = v;
        }
        for (int i = threadIdx.x; i < 9 * 32 * parts; i += kConvTPB) {
            const int row = i / parts, part = i - row * parts;  // row = tap * 32 + co
            const int tap = row >> 5, co = row & 31;
            *reinterpret_cast<uint4*>(s_w + row * ps + part * 8) =
                __ldg(reinterpret_cast<const uint4*>(a.w + ((long)tap * a.Cout + co0 + co) * a.Cin + c0 + part * 8));
        }
        __syncthreads();
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3, dx = tap % 3;  // halo-tile offsets (0..2)
            for (int ks = 0; ks < kc; ks += 16) {
                uint32_t af[2][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
                    ldsm_x4(af[mt], s_in + ((warp + dy) * (kTW + 2) + mt * 16 + a_row + dx) * ps + ks + a_k);
#pragma unroll
                for (int np = 0; np < 2; ++np) {
                    uint32_t bfr[4];
                    ldsm_x4(bfr, s_w + (tap * 32 + np * 16 + b_row) * ps + ks + b_k);
                    mma_bf16(acc[0][2 * np], af[0], bfr[0], bfr[1]);
                    mma_bf16(acc[1][2 * np], af[1], bfr[0], bfr[1]);
                    mma_bf16(acc[0][2 * np + 1], af[0], bfr[2], bfr[3]);
                    mma_bf16(acc[1][2 * np + 1], af[1], bfr[2], bfr[3]);
                }
            }
        }
        __syncthreads();
    }
    const int py = y0 + warp;
    if (py >= a.H) return;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int px = x0 + mt * 16 + g + 8 * h;
            if (px >= a.W) continue;
            const long p = (long)py * a.W + px;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int co = co0 + nt * 8 + 2 * t;
                float v0 = acc[mt][nt][2 * h], v1 = acc[mt][nt][2 * h + 1];
                if (a.bias) { v0 += a.bias[co]; v1 += a.bias[co + 1]; }
                if (a.relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                if (a.mask) {
                    const bf16* m = a.mask + (long)b * a.mbs + p * a.ldm + co;
                    if (!(__bfloat162float(m[0]) > 0.f)) v0 = 0.f;
                    if (!(__bfloat162float(m[1]) > 0.f)) v1 = 0.f;
                }
                if (a.y) {
                    *reinterpret_cast<__nv_bfloat162*>(a.y + (long)b * a.ybs + p * a.ldy + co) = __floats2bfloat162_rn(v0, v1);
                } else {
                    *reinterpret_cast<float2*>(a.yf + (long)b * a.ybs + p * a.ldy + co) = make_float2(v0, v1);
                }
            }
        }
}

// ------------------------------------------------------------------------------------------
// The same 3x3 convolution on the fifth-generation tensor cores: tcgen05.mma (M = 128 pixels of
// a 4 x 32 tile, N = up to 256 output channels, K = 16) issued by one thread, operands in shared
// memory in the K-major, unswizzled core-matrix layout (8 rows x 16 bytes per core matrix), the
// FP32 accumulator in tensor memory (TMEM), read back by tcgen05.ld for the epilogue.
//
// Per chunk of kc input channels a stage holds
//   A: the tile's input with its halo, three times, shifted by dx = 0, 1, 2 pixels, each
//      [k-core][6 halo rows][32 columns][8 channels]: the operand of tap (dy, dx) is then copy dx
//      from halo row dy on, with a uniform 128-byte stride between 8-pixel groups;
//   B: the 9 taps' weights [tap][k-core][n][8 channels].
// Two stages alternate: the block fills one while the MMAs of the other run; an mbarrier that
// tcgen05.commit arrives on tells the block when a stage's MMAs are done.  Waits are bounded:
// a wait that runs out sets the network's error flag and the block skips the rest.
constexpr int kTcThreads = 256;   // 8 warps: all load; warps w and w+4 share TMEM lanes 32 (w%4)
constexpr int kTcSpin = 1 << 22;  // mbarrier polls before a wait gives up

__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    // shared-memory matrix descriptor: start >> 4 (bits 0-13), leading-dimension byte offset >> 4
    // (K-direction core-matrix stride, 16-29), stride byte offset >> 4 (8-row-group stride,
    // 32-45), descriptor version 1 (46-47), no swizzle (61-63 = 0)
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < kTcSpin; ++it) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

struct TcArgs {
    ConvArgs c;
    int nt, kc;   // output channels per block (16..256, multiple of 16), input channels per chunk
    int* err;     // set when a wait gave up
};

__global__ void __launch_bounds__(kTcThreads) k_conv3_tc(TcArgs t) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int bad;
    const ConvArgs& a = t.c;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nt = t.nt, kc = t.kc, kcores = kc / 8;
    const int ncot = (a.Cout + nt - 1) / nt;
    const int b = blockIdx.z / ncot, co0 = (blockIdx.z % ncot) * nt;
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    const uint32_t a_bytes = 3u * kcores * 3072u, b_bytes = 9u * kcores * nt * 16u;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tsm);
    const uint32_t tcols = nt <= 32 ? 32u : (nt <= 64 ? 64u : (nt <= 128 ? 128u : 256u));
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tmem_base);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(tcols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[i]);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        bad = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tbase = tmem_base;
    const bf16* xb = a.x + (long)b * a.xbs;
    const int Wl = a.W >> 1;
    const int nchunks = a.Cin / kc;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nt >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    for (int c = 0; c < nchunks; ++c) {
        const int st = c & 1;
        const int c0 = c * kc;
        unsigned char* sA = tsm + st * stage_bytes;
        unsigned char* sB = sA + a_bytes;
        if (c >= 2) {  // the MMAs of chunk c - 2 read this stage
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[st]);
            if (!bad && !tc_wait(mb, (uint32_t)(((c - 2) >> 1) & 1))) { bad = 1; atomicExch(t.err, 1); }
            __syncthreads();
        }
        if (bad) break;
        // A: the halo tile (6 x 34 pixels) into the three shifted copies
        for (int i = tid; i < (kTH + 2) * (kTW + 2) * kcores; i += kTcThreads) {
            const int ki = i % kcores, pix = i / kcores;
            const int hr = pix / (kTW + 2), hc = pix - hr * (kTW + 2);
            const int gy = y0 + hr - 1, gx = x0 + hc - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) {
                const long sp = a.up ? (long)(gy >> 1) * Wl + (gx >> 1) : (long)gy * a.W + gx;
                v = __ldg(reinterpret_cast<const uint4*>(xb + sp * a.ldx + c0 + ki * 8));
            }
#pragma unroll
            for (int dx = 0; dx < 3; ++dx) {
                const int col = hc - dx;
                if (col >= 0 && col < kTW)
                    *reinterpret_cast<uint4*>(sA + dx * kcores * 3072 + ki * 3072 + hr * 512 + col * 16) = v;
            }
        }
        // B: the 9 taps' weights of output channels co0 .. co0 + nt - 1
        for (int i = tid; i < 9 * kcores * nt; i += kTcThreads) {
            const int n = i % nt, r = i / nt, ki = r % kcores, tap = r / kcores;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (co0 + n < a.Cout)
                v = __ldg(reinterpret_cast<const uint4*>(a.w + ((long)tap * a.Cout + co0 + n) * a.Cin + c0 + ki * 8));
            *reinterpret_cast<uint4*>(sB + tap * kcores * nt * 16 + ki * nt * 16 + n * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t aS = sbase + st * stage_bytes, bS = aS + a_bytes;
            for (int tap = 0; tap < 9; ++tap) {
                const int dy = tap / 3, dx = tap % 3;
                for (int j = 0; j < kc / 16; ++j) {
                    const uint64_t ad = tc_desc(aS + dx * kcores * 3072 + 2 * j * 3072 + dy * 512, 3072, 128);
                    const uint64_t bd = tc_desc(bS + tap * kcores * nt * 16 + 2 * j * nt * 16, nt * 16, 128);
                    const uint32_t acc = (c > 0 || tap > 0 || j > 0) ? 1u : 0u;
                    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                                 ::"r"(tbase), "l"(ad), "l"(bd), "r"(idesc), "r"(acc) : "memory");
                }
            }
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[st]);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb) : "memory");
        }
    }
    // the last chunk's commit covers every MMA of the block
    if (!bad && nchunks > 0) {
        const int lc = nchunks - 1;
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[lc & 1]);
        if (!tc_wait(mb, (uint32_t)((lc >> 1) & 1))) { bad = 1; atomicExch(t.err, 1); }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. (pixels of tile row w % 4) and half of the
    // columns (all of them when nt < 32, by warps 0-3)
    const int q = warp & 3, half = warp >> 2;
    const int ncol = nt >= 32 ? nt / 2 : nt;
    const bool ep = !bad && (nt >= 32 || half == 0);
    const int py = y0 + q, px = x0 + lane;
    if (ep) {
        for (int cc = 0; cc < ncol; cc += 16) {
            const int col = half * ncol + cc;
            uint32_t r[16];
            const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)col;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                         : "r"(ta));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (py < a.H && px < a.W) {
                const long p = (long)py * a.W + px;
#pragma unroll
                for (int e = 0; e < 16; e += 2) {
                    const int co = co0 + col + e;
                    if (co >= a.Cout) break;
                    float v0 = __uint_as_float(r[e]), v1 = __uint_as_float(r[e + 1]);
                    if (a.bias) { v0 += a.bias[co]; v1 += a.bias[co + 1]; }
                    if (a.relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                    if (a.mask) {
                        const bf16* m = a.mask + (long)b * a.mbs + p * a.ldm + co;
                        if (!(__bfloat162float(m[0]) > 0.f)) v0 = 0.f;
                        if (!(__bfloat162float(m[1]) > 0.f)) v1 = 0.f;
                    }
                    if (a.y)
                        *reinterpret_cast<__nv_bfloat162*>(a.y + (long)b * a.ybs + p * a.ldy + co) = __floats2bfloat162_rn(v0, v1);
                    else
                        *reinterpret_cast<float2*>(a.yf + (long)b * a.ybs + p * a.ldy + co) = make_float2(v0, v1);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(tcols) : "memory");
}

// Output channels per block and input channels per chunk of the tensor-core convolution, and
// its shared memory (two stages).
void tc_shape(int Cin, int Cout, int* nt, int* kc) {
    *nt = Cout >= 256 ? 256 : Cout;
    *kc = (*nt >= 128 || Cin % 32 != 0) ? 16 : 32;
}
size_t tc_smem(int nt, int kc) { return 2 * (3 * (size_t)(kc / 8) * 3072 + 9 * (size_t)(kc / 8) * nt * 16); }

// ------------------------------------------------------------------------------------------
// Weight gradient: dW[tap][co][ci] += sum over pixels of G[p][co] * X[p + off(tap)][ci], an MMA
// with M = output channels, N = input channels, K = pixels.  A block owns one 32 x ci_tile
// weight tile for all 9 taps (warp w = tap w) and walks kWgTiles pixel tiles of kTH x kTW:
// per tile it stages G (the tile) and X (the tile with its halo) in shared memory, and every
// warp reads its fragments with ldmatrix.trans (both operands are pixel-major there).  The
// block's sums go to dW with one atomic per weight and tap.
constexpr int kWgTiles = 8;
constexpr int kWgThreads = 9 * 32;

struct WgArgs {
    const bf16* x; long xbs; int ldx;
    const bf16* g; long gbs; int ldg;
    float* dw;
    int H, W, Cin, Cout, up, ci_tile, batch;
};

__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const bf16* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__global__ void __launch_bounds__(kWgThreads) k_wgrad(WgArgs a) {
    constexpr int PS = 32 + 8;  // padded pixel row (32 channels max per tile)
    __shared__ __align__(16) bf16 s_g[kTH * kTW * PS];
    __shared__ __align__(16) bf16 s_x[kHaloPix * PS];
    const int tap = threadIdx.x >> 5, lane = threadIdx.x & 31, t = lane & 3, g = lane >> 2;
    const int nco = a.Cout / 32;
    const int co0 = (blockIdx.y % nco) * 32, ci0 = (blockIdx.y / nco) * a.ci_tile;
    const int nnt = a.ci_tile / 8;       // 2 or 4 n-tiles
    const int xparts = a.ci_tile / 8;    // 16-byte pieces of an X row
    const int dy = tap / 3, dx = tap % 3;
    const int tx_n = (a.W + kTW - 1) / kTW, ty_n = (a.H + kTH - 1) / kTH;
    const long ntiles = (long)a.batch * tx_n * ty_n;
    const int Wl = a.W >> 1;
    // ldmatrix.trans row addresses: rows are pixels.  A (G^T): matrices (k 0-7, m 0-7),
    // (k 0-7, m 8-15), (k 8-15, m 0-7), (k 8-15, m 8-15); B (X): (k 0-7, n 0-7), (k 8-15, n 0-7),
    // (k 0-7, n 8-15), (k 8-15, n 8-15)
    const int ar = (lane & 7) + (lane >> 4) * 8, am = ((lane >> 3) & 1) * 8;
    const int br = (lane & 7) + ((lane >> 3) & 1) * 8, bn = (lane >> 4) * 8;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;

    for (int it = 0; it < kWgTiles; ++it) {
        const long tile = (long)blockIdx.x * kWgTiles + it;
        if (tile >= ntiles) break;  // uniform over the block
        const int b = (int)(tile / ((long)tx_n * ty_n));
        const int rem = (int)(tile - (long)b * tx_n * ty_n);
        const int y0 = (rem / tx_n) * kTH, x0 = (rem % tx_n) * kTW;
        for (int i = threadIdx.x; i < kTH * kTW * 4; i += kWgThreads) {
            const int pix = i >> 2, part = i & 3;
            const int gy = y0 + pix / kTW, gx = x0 + pix % kTW;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy < a.H && gx < a.W)
                v = __ldg(reinterpret_cast<const uint4*>(a.g + (long)b * a.gbs + ((long)gy * a.W + gx) * a.ldg + co0 +
                                                         part * 8));
            *reinterpret_cast<uint4*>(s_g + pix * PS + part * 8) = v;
        }
        for (int i = threadIdx.x; i < kHaloPix * xparts; i += kWgThreads) {
            const int pix = i / xparts, part = i - pix * xparts;
            const int gy = y0 + pix / (kTW + 2) - 1, gx = x0 + pix % (kTW + 2) - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) {
                const long sp = a.up ? (long)(gy >> 1) * Wl + (gx >> 1) : (long)gy * a.W + gx;
                v = __ldg(reinterpret_cast<const uint4*>(a.x + (long)b * a.xbs + sp * a.ldx + ci0 + part * 8));
            }
            *reinterpret_cast<uint4*>(s_x + pix * PS + part * 8) = v;
        }
        __syncthreads();
#pragma unroll 1
        for (int ks = 0; ks < kTH * 2; ++ks) {  // 16 pixels: half a tile row
            const int ry = ks >> 1, cx = (ks & 1) * 16;
            uint32_t af[2][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) ldsm_x4_t(af[mt], s_g + (ry * kTW + cx + ar) * PS + mt * 16 + am);
            const bf16* xrow = s_x + ((ry + dy) * (kTW + 2) + cx + dx + br) * PS + bn;
#pragma unroll
            for (int np = 0; np < 2; ++np) {
                if (2 * np >= nnt) break;
                uint32_t bfr[4];
                ldsm_x4_t(bfr, xrow + np * 16);
                mma_bf16(acc[0][2 * np], af[0], bfr[0], bfr[1]);
                mma_bf16(acc[1][2 * np], af[1], bfr[0], bfr[1]);
                mma_bf16(acc[0][2 * np + 1], af[0], bfr[2], bfr[3]);
                mma_bf16(acc[1][2 * np + 1], af[1], bfr[2], bfr[3]);
            }
        }
        __syncthreads();
    }
    float* dwt = a.dw + (long)tap * a.Cout * a.Cin;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            if (nt >= nnt) break;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int co = co0 + mt * 16 + g + (k >> 1) * 8, ci = ci0 + nt * 8 + 2 * t + (k & 1);
                atomicAdd(dwt + (long)co * a.Cin + ci, acc[mt][nt][k]);
            }
        }
}

// bias gradient: db[c] += sum over pixels of G[p][c].  A block sums 256 pixels; its threads
// are (pixel row, channel pair), the rows reduced through shared memory.
__global__ void __launch_bounds__(256) k_colsum(const bf16* g, long gbs, int ldg, int HW, int batch, int C, float* db) {
    __shared__ float2 part[256];
    const int np = C >> 1;        // channel pairs: 16..128, divides 256
    const int rows = 256 / np;
    const int cp = threadIdx.x % np, r = threadIdx.x / np;
    const long total = (long)batch * HW;
    const long q0 = (long)blockIdx.x * 256;
    float2 s = make_float2(0.f, 0.f);
    for (long q = q0 + r; q < q0 + 256 && q < total; q += rows) {
        const int b = (int)(q / HW);
        const long p = q - (long)b * HW;
        const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(g + (long)b * gbs + p * ldg + 2 * cp));
        s.x += v.x;
        s.y += v.y;
    }
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < np) {
        float2 t = make_float2(0.f, 0.f);
        for (int k = 0; k < rows; ++k) {
            t.x += part[k * np + threadIdx.x].x;
            t.y += part[k * np + threadIdx.x].y;
        }
        atomicAdd(db + 2 * threadIdx.x, t.x);
        atomicAdd(db + 2 * threadIdx.x + 1, t.y);
    }
}

// 2x2 average pool: y (H/2 x W/2) from x (H x W)
__global__ void k_pool(const bf16* x, long xbs, int ldx, bf16* y, long ybs, int ldy, int H, int W, int C, int batch) {
    const int Hl = H >> 1, Wl = W >> 1;
    const long n = (long)batch * Hl * Wl * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long q = i / C;
        const int xl = (int)(q % Wl);
        q /= Wl;
        const int yl = (int)(q % Hl);
        const int b = (int)(q / Hl);
        const bf16* s = x + (long)b * xbs + ((long)(2 * yl) * W + 2 * xl) * ldx + c;
        const float v = __bfloat162float(s[0]) + __bfloat162float(s[ldx]) + __bfloat162float(s[(long)W * ldx]) +
                        __bfloat162float(s[(long)W * ldx + ldx]);
        y[(long)b * ybs + ((long)yl * Wl + xl) * ldy + c] = __float2bfloat16_rn(0.25f * v);
    }
}

// gradient through nearest upsampling: dl[q] = sum of the 4 children dh[p]
__global__ void k_up_bwd(const float* dh, long hbs, int ldh, float* dl, long lbs, int ldl, int H, int W, int C, int batch) {
    const int Hl = H >> 1, Wl = W >> 1;
    const long n = (long)batch * Hl * Wl * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long q = i / C;
        const int xl = (int)(q % Wl);
        q /= Wl;
        const int yl = (int)(q % Hl);
        const int b = (int)(q / Hl);
        const float* s = dh + (long)b * hbs + ((long)(2 * yl) * W + 2 * xl) * ldh + c;
        dl[(long)b * lbs + ((long)yl * Wl + xl) * ldl + c] = s[0] + s[ldh] + s[(long)W * ldh] + s[(long)W * ldh + ldh];
    }
}

// pre-activation gradient of a ReLU layer: G = (mask > 0) * (a + 0.25 * b[parent]) in BF16,
// with b (optional) the gradient of the 2x2 average pool that also reads this layer.
__global__ void k_mask_grad(const float* a, long abs_, int lda, const float* bsrc, long bbs, int ldb, const bf16* mask,
                            long mbs, int ldm, bf16* G, long gbs, int ldg, int H, int W, int C, int batch) {
    const long n = (long)batch * H * W * C;
    const int Wl = W >> 1;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long q = i / C;
        const int x = (int)(q % W);
        q /= W;
        const int y = (int)(q % H);
        const int b = (int)(q / H);
        const long p = (long)y * W + x;
        float v = 0.f;
        if (__bfloat162float(mask[(long)b * mbs + p * ldm + c]) > 0.f) {
            v = a[(long)b * abs_ + p * lda + c];
            if (bsrc) v += 0.25f * bsrc[(long)b * bbs + ((long)(y >> 1) * Wl + (x >> 1)) * ldb + c];
        }
        G[(long)b * gbs + p * ldg + c] = __float2bfloat16_rn(v);
    }
}

// caller's FP32 NCHW input on H0 x W0 -> NHWC BF16 on Hp x Wp with kCinPad channels
__global__ void k_pack_in(const float* x, int cin, int H0, int W0, bf16* xin, int Hp, int Wp, int batch) {
    const long n = (long)batch * Hp * Wp;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int w = (int)(i % Wp);
        const int h = (int)((i / Wp) % Hp);
        const int b = (int)(i / ((long)Wp * Hp));
        alignas(16) bf16 v[kCinPad];
#pragma unroll
        for (int c = 0; c < kCinPad; ++c) {
            float f = 0.f;
            if (c < cin && h < H0 && w < W0) f = x[(((long)b * cin + c) * H0 + h) * W0 + w];
            v[c] = __float2bfloat16_rn(f);
        }
        uint4* dst = reinterpret_cast<uint4*>(xin + i * kCinPad);
        dst[0] = *reinterpret_cast<uint4*>(&v[0]);
        dst[1] = *reinterpret_cast<uint4*>(&v[8]);
    }
}

// 1x1 output convolution on the caller's grid: y[b][o][h][w] = bo[o] + sum_c d0[p][c] Wo[o][c]
__global__ void k_out_fwd(const bf16* d0, const float* wo, const float* bo, int cout, float* y, int H0, int W0, int Hp,
                          int Wp, int batch) {
    const long n = (long)batch * H0 * W0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int w = (int)(i % W0);
        const int h = (int)((i / W0) % H0);
        const int b = (int)(i / ((long)W0 * H0));
        const bf16* s = d0 + ((long)b * Hp * Wp + (long)h * Wp + w) * kBase;
        float acc[kMaxOut];
        for (int o = 0; o < cout; ++o) acc[o] = bo[o];
        for (int c = 0; c < kBase; ++c) {
            const float v = __bfloat162float(s[c]);
            for (int o = 0; o < cout; ++o) acc[o] += v * wo[o * kBase + c];
        }
        for (int o = 0; o < cout; ++o) y[(((long)b * cout + o) * H0 + h) * W0 + w] = acc[o];
    }
}

// mean squared error over the caller's grid; dy = d(loss)/dy
__global__ void k_loss(const float* y, const float* tg, float* dy, long n, float inv_n, float* loss) {
    __shared__ float sm[32];
    float s = 0.f;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float d = y[i] - tg[i];
        dy[i] = 2.f * d * inv_n;
        s += d * d;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.f;
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(loss, s * inv_n);
    }
}

// output layer backward, data part: G0[p][c] = (d0 > 0) * sum_o dy[o][p] Wo[o][c] (dy = 0 off the caller's grid)
__global__ void k_out_bwd_x(const float* dy, const float* wo, int cout, const bf16* d0, bf16* G, int H0, int W0, int Hp,
                            int Wp, int batch) {
    const long n = (long)batch * Hp * Wp;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int w = (int)(i % Wp);
        const int h = (int)((i / Wp) % Hp);
        const int b = (int)(i / ((long)Wp * Hp));
        float dv[kMaxOut];
        const bool in = h < H0 && w < W0;
        for (int o = 0; o < cout; ++o) dv[o] = in ? dy[(((long)b * cout + o) * H0 + h) * W0 + w] : 0.f;
        const bf16* m = d0 + i * kBase;
        bf16* gp = G + i * kBase;
        for (int c = 0; c < kBase; ++c) {
            float v = 0.f;
            if (__bfloat162float(m[c]) > 0.f)
                for (int o = 0; o < cout; ++o) v += dv[o] * wo[o * kBase + c];
            gp[c] = __float2bfloat16_rn(v);
        }
    }
}

// output layer backward, weight part: dWo[o][c] += sum_p dy[o][p] d0[p][c]; dbo[o] += sum_p dy[o][p]
__global__ void k_out_bwd_w(const float* dy, int cout, const bf16* d0, float* dwo, float* dbo, int H0, int W0, int Hp,
                            int Wp, int batch) {
    const int o = threadIdx.x / kBase, c = threadIdx.x % kBase;
    if (o >= cout) return;
    const long n = (long)batch * H0 * W0;
    const long i0 = (long)blockIdx.x * 256;
    float s = 0.f, sb = 0.f;
    for (long i = i0; i < i0 + 256 && i < n; ++i) {
        const int w = (int)(i % W0);
        const int h = (int)((i / W0) % H0);
        const int b = (int)(i / ((long)W0 * H0));
        const float d = dy[(((long)b * cout + o) * H0 + h) * W0 + w];
        s += d * __bfloat162float(d0[((long)b * Hp * Wp + (long)h * Wp + w) * kBase + c]);
        sb += d;
    }
    atomicAdd(dwo + o * kBase + c, s);
    if (c == 0) atomicAdd(dbo + o, sb);
}

// Adam step on the FP32 master weights, then the two BF16 copies
__global__ void k_adam(float* w, const float* gr, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2, bf16* wb, bf16* wt, const int* tmap, int update) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float x = w[i];
        if (update) {
            const float gi = gr[i];
            const float mi = b1 * m[i] + (1.f - b1) * gi;
            const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            x -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
            w[i] = x;
        }
        const bf16 xb = __float2bfloat16_rn(x);
        wb[i] = xb;
        const int j = tmap[i];
        if (j >= 0) wt[j] = xb;
    }
}

inline int grid_for(long n, int tpb = 256) {
    long b = (n + tpb - 1) / tpb;
    if (b > 152 * 32) b = 152 * 32;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

// ------------------------------------------------------------------------------------------
struct drd_unet {
    struct Layer {
        int cin, cout, level, up;
        long w_off, b_off;
    };
    int H0, W0, Hp, Wp, cin, cout, maxb;
    cudaStream_t s = nullptr;
    std::vector<Layer> L;
    long nparam = 0, wo_off = 0, bo_off = 0, adam_t = 0;
    float *W32 = nullptr, *G32 = nullptr, *M = nullptr, *V = nullptr;
    bf16 *Wb = nullptr, *Wt = nullptr;
    int* tmap = nullptr;
    // activations (see the header comment)
    bf16 *xin = nullptr, *ea[kLevels] = {}, *cat[kLevels - 1] = {}, *pool[kLevels] = {}, *b3 = nullptr;
    bf16 *db[kLevels - 1] = {}, *dd[kLevels - 1] = {};
    // gradients
    bf16* Gl[17] = {};
    float *dcat[kLevels - 1] = {}, *dU = nullptr, *dlow = nullptr, *dpool = nullptr;
    float *y = nullptr, *dy = nullptr, *tg = nullptr, *xstage = nullptr, *ystage = nullptr, *loss = nullptr;
    std::vector<void*> allocs;
    std::string err;
    int tc = 0;            // 3x3 convolutions on tcgen05 (DRD_UNET_TC=1) instead of mma.sync
    int* dflag = nullptr;  // device: set by a tensor-core wait that gave up

    int HWl(int l) const { return (Hp >> l) * (Wp >> l); }
    int Hl(int l) const { return Hp >> l; }
    int Wl(int l) const { return Wp >> l; }
    static int C(int l) { return kBase << l; }
};

namespace {

template <class T>
int dalloc(drd_unet* n, T** p, size_t count) {
    if (cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)) != cudaSuccess) return DRD_ERR_CUDA;
    n->allocs.push_back((void*)*p);
    return cudaMemsetAsync(*p, 0, sizeof(T) * (count ? count : 1), n->s) == cudaSuccess ? DRD_OK : DRD_ERR_CUDA;
}

// One 3x3 convolution: the tensor-core kernel (tcgen05) unless it is switched off, else the
// mma.sync kernel (which needs Cout % 32 == 0).
void launch_conv3(drd_unet* n, const ConvArgs& a, int batch) {
    if (n->tc) {
        TcArgs t{};
        t.c = a;
        tc_shape(a.Cin, a.Cout, &t.nt, &t.kc);
        t.err = n->dflag;
        const int ncot = (a.Cout + t.nt - 1) / t.nt;
        dim3 grid((a.W + kTW - 1) / kTW, (a.H + kTH - 1) / kTH, batch * ncot);
        k_conv3_tc<<<grid, kTcThreads, tc_smem(t.nt, t.kc), n->s>>>(t);
        return;
    }
    dim3 grid((a.W + kTW - 1) / kTW, (a.H + kTH - 1) / kTH, batch * (a.Cout / 32));
    k_conv3<<<grid, kConvTPB, 0, n->s>>>(a);
}

void conv(drd_unet* n, int li, const bf16* x, int ldx, long xbs, bf16* y, int ldy, long ybs, int batch) {
    const auto& Ly = n->L[li];
    ConvArgs a{};
    a.x = x; a.xbs = xbs; a.ldx = ldx;
    a.w = n->Wb + Ly.w_off; a.bias = n->W32 + Ly.b_off;
    a.y = y; a.yf = nullptr; a.ybs = ybs; a.ldy = ldy;
    a.mask = nullptr; a.mbs = 0; a.ldm = 0;
    a.H = n->Hl(Ly.level); a.W = n->Wl(Ly.level); a.Cin = Ly.cin; a.Cout = Ly.cout; a.up = Ly.up; a.relu = 1;
    launch_conv3(n, a, batch);
}

// data gradient of layer li: out (bf16 with mask, or fp32) = conv(G, flipped transpose)
void dgrad(drd_unet* n, int li, const bf16* G, int batch, bf16* out_b, float* out_f, int ldo, long obs,
           const bf16* mask, int ldm, long mbs) {
    const auto& Ly = n->L[li];
    const int H = n->Hl(Ly.level), W = n->Wl(Ly.level);
    ConvArgs a{};
    a.x = G; a.xbs = (long)H * W * Ly.cout; a.ldx = Ly.cout;
    a.w = n->Wt + Ly.w_off; a.bias = nullptr;
    a.y = out_b; a.yf = out_f; a.ybs = obs; a.ldy = ldo;
    a.mask = mask; a.mbs = mbs; a.ldm = ldm;
    a.H = H; a.W = W; a.Cin = Ly.cout; a.Cout = Ly.cin; a.up = 0; a.relu = 0;
    launch_conv3(n, a, batch);
}

void wgrad(drd_unet* n, int li, const bf16* x, int ldx, long xbs, const bf16* G, int batch) {
    const auto& Ly = n->L[li];
    const int H = n->Hl(Ly.level), W = n->Wl(Ly.level);
    WgArgs a{};
    a.x = x; a.xbs = xbs; a.ldx = ldx;
    a.g = G; a.gbs = (long)H * W * Ly.cout; a.ldg = Ly.cout;
    a.dw = n->G32 + Ly.w_off;
    a.H = H; a.W = W; a.Cin = Ly.cin; a.Cout = Ly.cout; a.up = Ly.up; a.batch = batch;
    a.ci_tile = Ly.cin < 32 ? Ly.cin : 32;
    const long total = (long)batch * H * W;
    const long ntiles = (long)batch * ((H + kTH - 1) / kTH) * ((W + kTW - 1) / kTW);
    dim3 grid((unsigned)((ntiles + kWgTiles - 1) / kWgTiles), (Ly.cout / 32) * (Ly.cin / a.ci_tile));
    k_wgrad<<<grid, kWgThreads, 0, n->s>>>(a);
    k_colsum<<<(unsigned)((total + 255) / 256), 256, 0, n->s>>>(G, a.gbs, Ly.cout, H * W, batch, Ly.cout,
                                                                 n->G32 + Ly.b_off);
}

void mask_grad(drd_unet* n, int l, const float* a, int lda, const float* b, int ldb, const bf16* mask, int ldm, bf16* G,
               int C, int batch) {
    const long hw = n->HWl(l);
    const long hwl = l + 1 < kLevels ? n->HWl(l + 1) : 0;
    k_mask_grad<<<grid_for((long)batch * hw * C), 256, 0, n->s>>>(a, hw * lda, lda, b, hwl * ldb, ldb, mask, hw * ldm, ldm,
                                                                  G, hw * C, C, n->Hl(l), n->Wl(l), C, batch);
}

void up_bwd(drd_unet* n, int l, const float* dh, int C, float* dl, int batch) {
    // dh at level l (C channels), dl at level l+1
    k_up_bwd<<<grid_for((long)batch * n->HWl(l + 1) * C), 256, 0, n->s>>>(dh, (long)n->HWl(l) * C, C, dl,
                                                                          (long)n->HWl(l + 1) * C, C, n->Hl(l),
                                                                          n->Wl(l), C, batch);
}

void forward(drd_unet* n, const float* x, int batch) {
    const long n0 = (long)batch * n->Hp * n->Wp;
    k_pack_in<<<grid_for(n0), 256, 0, n->s>>>(x, n->cin, n->H0, n->W0, n->xin, n->Hp, n->Wp, batch);
    // encoder
    for (int l = 0; l < kLevels; ++l) {
        const int C = drd_unet::C(l);
        const long hw = n->HWl(l);
        const bf16* in = l == 0 ? n->xin : n->pool[l];
        const int ldin = l == 0 ? kCinPad : drd_unet::C(l - 1);
        conv(n, 2 * l, in, ldin, hw * ldin, n->ea[l], C, hw * C, batch);
        if (l < kLevels - 1) {
            conv(n, 2 * l + 1, n->ea[l], C, hw * C, n->cat[l] + C, 2 * C, hw * 2 * C, batch);
            const long hwl = n->HWl(l + 1);
            k_pool<<<grid_for((long)batch * hwl * C), 256, 0, n->s>>>(n->cat[l] + C, hw * 2 * C, 2 * C, n->pool[l + 1],
                                                                      hwl * C, C, n->Hl(l), n->Wl(l), C, batch);
        } else {
            conv(n, 2 * l + 1, n->ea[l], C, hw * C, n->b3, C, hw * C, batch);
        }
    }
    // decoder
    for (int l = kLevels - 2; l >= 0; --l) {
        const int C = drd_unet::C(l);
        const long hw = n->HWl(l), hwl = n->HWl(l + 1);
        const bf16* below = l == kLevels - 2 ? n->b3 : n->dd[l + 1];
        const int li = 8 + 3 * (kLevels - 2 - l);
        conv(n, li, below, 2 * C, hwl * 2 * C, n->cat[l], 2 * C, hw * 2 * C, batch);
        conv(n, li + 1, n->cat[l], 2 * C, hw * 2 * C, n->db[l], C, hw * C, batch);
        conv(n, li + 2, n->db[l], C, hw * C, n->dd[l], C, hw * C, batch);
    }
    k_out_fwd<<<grid_for((long)batch * n->H0 * n->W0), 256, 0, n->s>>>(n->dd[0], n->W32 + n->wo_off, n->W32 + n->bo_off,
                                                                       n->cout, n->y, n->H0, n->W0, n->Hp, n->Wp, batch);
}

void backward(drd_unet* n, int batch) {
    const long hw0 = n->HWl(0);
    k_out_bwd_w<<<(unsigned)(((long)batch * n->H0 * n->W0 + 255) / 256), kMaxOut * kBase, 0, n->s>>>(
        n->dy, n->cout, n->dd[0], n->G32 + n->wo_off, n->G32 + n->bo_off, n->H0, n->W0, n->Hp, n->Wp, batch);
    k_out_bwd_x<<<grid_for((long)batch * hw0), 256, 0, n->s>>>(n->dy, n->W32 + n->wo_off, n->cout, n->dd[0], n->Gl[16],
                                                                n->H0, n->W0, n->Hp, n->Wp, batch);
    // decoder, top level first
    for (int l = 0; l <= kLevels - 2; ++l) {
        const int C = drd_unet::C(l);
        const long hw = n->HWl(l);
        const int li = 8 + 3 * (kLevels - 2 - l);  // the level's upsampling conv; li+1, li+2 follow
        // conv li+2: db[l] -> dd[l]
        wgrad(n, li + 2, n->db[l], C, hw * C, n->Gl[li + 2], batch);
        dgrad(n, li + 2, n->Gl[li + 2], batch, n->Gl[li + 1], nullptr, C, hw * C, n->db[l], C, hw * C);
        // conv li+1: cat[l] -> db[l]; gradient of the concatenation in FP32
        wgrad(n, li + 1, n->cat[l], 2 * C, hw * 2 * C, n->Gl[li + 1], batch);
        dgrad(n, li + 1, n->Gl[li + 1], batch, nullptr, n->dcat[l], 2 * C, hw * 2 * C, nullptr, 0, 0);
        // conv li (upsampling): input up2(d_{l+1}), output channels [0, C) of cat[l]
        mask_grad(n, l, n->dcat[l], 2 * C, nullptr, 0, n->cat[l], 2 * C, n->Gl[li], C, batch);
        const bf16* below = l == kLevels - 2 ? n->b3 : n->dd[l + 1];
        wgrad(n, li, below, 2 * C, n->HWl(l + 1) * 2 * C, n->Gl[li], batch);
        dgrad(n, li, n->Gl[li], batch, nullptr, n->dU, 2 * C, hw * 2 * C, nullptr, 0, 0);
        up_bwd(n, l, n->dU, 2 * C, n->dlow, batch);
        // pre-activation gradient of the layer producing d_{l+1} (or the bottleneck)
        const int lo = l + 1;
        const int prod = lo == kLevels - 1 ? 7 : 8 + 3 * (kLevels - 2 - lo) + 2;
        mask_grad(n, lo, n->dlow, 2 * C, nullptr, 0, below, 2 * C, n->Gl[prod], 2 * C, batch);
    }
    // encoder, bottom level first (the bottleneck's G7 is set above)
    for (int l = kLevels - 1; l >= 0; --l) {
        const int C = drd_unet::C(l);
        const long hw = n->HWl(l);
        // conv 2l+1: ea[l] -> e_l
        const bf16* ein = n->ea[l];
        wgrad(n, 2 * l + 1, ein, C, hw * C, n->Gl[2 * l + 1], batch);
        dgrad(n, 2 * l + 1, n->Gl[2 * l + 1], batch, n->Gl[2 * l], nullptr, C, hw * C, n->ea[l], C, hw * C);
        // conv 2l: input pool[l] (or the packed input)
        const bf16* in = l == 0 ? n->xin : n->pool[l];
        const int ldin = l == 0 ? kCinPad : drd_unet::C(l - 1);
        wgrad(n, 2 * l, in, ldin, hw * ldin, n->Gl[2 * l], batch);
        if (l == 0) break;
        const int Cp = drd_unet::C(l - 1);
        dgrad(n, 2 * l, n->Gl[2 * l], batch, nullptr, n->dpool, Cp, hw * Cp, nullptr, 0, 0);
        // e_{l-1}: the decoder's concatenation half plus the pool's share
        mask_grad(n, l - 1, n->dcat[l - 1] + Cp, 2 * Cp, n->dpool, Cp, n->cat[l - 1] + Cp, 2 * Cp,
                  n->Gl[2 * (l - 1) + 1], Cp, batch);
    }
}

int set_err(drd_unet* n, const char* m) {
    n->err = m;
    return DRD_ERR_BADARG;
}

bool is_device_ptr(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// the caller's FP32 NCHW array (host or device) as a device pointer
const float* stage_in(drd_unet* n, const float* p, long count, float* stage) {
    if (is_device_ptr(p)) return p;
    cudaMemcpyAsync(stage, p, sizeof(float) * count, cudaMemcpyHostToDevice, n->s);
    return stage;
}

int finish(drd_unet* n) {
    cudaError_t e = cudaStreamSynchronize(n->s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        n->err = cudaGetErrorString(e);
        return DRD_ERR_CUDA;
    }
    if (n->dflag) {
        int f = 0;
        if (cudaMemcpy(&f, n->dflag, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && f) {
            cudaMemset(n->dflag, 0, sizeof(int));
            n->err = "a tensor-core convolution gave up waiting for its MMAs";
            return DRD_ERR_TIMEOUT;
        }
    }
    return DRD_OK;
}

int refresh_bf16(drd_unet* n, int update, float lr) {
    float bc1 = 1.f, bc2 = 1.f;
    if (update) {
        ++n->adam_t;
        bc1 = 1.f - std::pow(0.9f, (float)n->adam_t);
        bc2 = 1.f - std::pow(0.999f, (float)n->adam_t);
    }
    k_adam<<<grid_for(n->nparam), 256, 0, n->s>>>(n->W32, n->G32, n->M, n->V, n->nparam, lr, 0.9f, 0.999f, 1e-8f, bc1,
                                                  bc2, n->Wb, n->Wt, n->tmap, update);
    return DRD_OK;
}

int loss_and_grads(drd_unet* n, int batch, const float* x, const float* target) {
    const long nin = (long)batch * n->cin * n->H0 * n->W0, nout = (long)batch * n->cout * n->H0 * n->W0;
    const float* xd = stage_in(n, x, nin, n->xstage);
    const float* td = stage_in(n, target, nout, n->ystage);
    forward(n, xd, batch);
    cudaMemsetAsync(n->loss, 0, sizeof(float), n->s);
    k_loss<<<grid_for(nout), 256, 0, n->s>>>(n->y, td, n->dy, nout, 1.f / (float)nout, n->loss);
    cudaMemsetAsync(n->G32, 0, sizeof(float) * n->nparam, n->s);
    backward(n, batch);
    return DRD_OK;
}

}  // namespace

extern "C" {

int drd_unet_create(int H, int W, int in_ch, int out_ch, int max_batch, uint64_t seed, drd_unet** out) {
    if (!out || H < 8 || W < 8 || in_ch < 1 || in_ch > kCinPad || out_ch < 1 || out_ch > kMaxOut || max_batch < 1)
        return DRD_ERR_BADARG;
    *out = nullptr;
    auto* n = new drd_unet();
    n->H0 = H; n->W0 = W; n->cin = in_ch; n->cout = out_ch; n->maxb = max_batch;
    n->Hp = (H + 7) / 8 * 8;
    n->Wp = (W + 7) / 8 * 8;
    if (cudaStreamCreateWithFlags(&n->s, cudaStreamNonBlocking) != cudaSuccess) {
        delete n;
        return DRD_ERR_CUDA;
    }
    // layer table: encoder (2 per level), then 3 per decoder level from the bottom
    long off = 0;
    auto add = [&](int ci, int co, int lev, int up) {
        drd_unet::Layer Ly{ci, co, lev, up, off, 0};
        off += 9L * ci * co;
        Ly.b_off = off;
        off += co;
        n->L.push_back(Ly);
    };
    for (int l = 0; l < kLevels; ++l) {
        add(l == 0 ? kCinPad : drd_unet::C(l - 1), drd_unet::C(l), l, 0);
        add(drd_unet::C(l), drd_unet::C(l), l, 0);
    }
    for (int l = kLevels - 2; l >= 0; --l) {
        add(drd_unet::C(l + 1), drd_unet::C(l), l, 1);
        add(2 * drd_unet::C(l), drd_unet::C(l), l, 0);
        add(drd_unet::C(l), drd_unet::C(l), l, 0);
    }
    n->wo_off = off;
    off += (long)out_ch * kBase;
    n->bo_off = off;
    off += out_ch;
    n->nparam = off;

    // initial weights: He-normal (std sqrt(2 / fan_in)) from mt19937_64(seed); zero biases and
    // zero weights on the padded input channels; the output layer at a tenth of the He scale
    std::vector<float> w(n->nparam, 0.f);
    std::vector<int> tm(n->nparam, -1);
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (const auto& Ly : n->L) {
        const int real_cin = Ly.w_off == 0 ? in_ch : Ly.cin;
        const double sd = std::sqrt(2.0 / (9.0 * real_cin));
        for (int tap = 0; tap < 9; ++tap)
            for (int co = 0; co < Ly.cout; ++co)
                for (int ci = 0; ci < Ly.cin; ++ci) {
                    const long i = Ly.w_off + ((long)tap * Ly.cout + co) * Ly.cin + ci;
                    const double r = nd(rng);
                    w[i] = ci < real_cin ? (float)(sd * r) : 0.f;
                    tm[i] = (int)(Ly.w_off + ((long)(8 - tap) * Ly.cin + ci) * Ly.cout + co);
                }
    }
    for (long i = 0; i < (long)out_ch * kBase; ++i) w[n->wo_off + i] = (float)(0.1 * std::sqrt(2.0 / kBase) * nd(rng));

    int rc = dalloc(n, &n->W32, n->nparam) | dalloc(n, &n->G32, n->nparam) | dalloc(n, &n->M, n->nparam) |
             dalloc(n, &n->V, n->nparam) | dalloc(n, &n->Wb, n->nparam) | dalloc(n, &n->Wt, n->nparam) |
             dalloc(n, &n->tmap, n->nparam);
    const int B = max_batch;
    rc |= dalloc(n, &n->xin, (size_t)B * n->HWl(0) * kCinPad);
    for (int l = 0; l < kLevels; ++l) {
        const size_t hw = (size_t)B * n->HWl(l), C = drd_unet::C(l);
        rc |= dalloc(n, &n->ea[l], hw * C);
        if (l > 0) rc |= dalloc(n, &n->pool[l], hw * drd_unet::C(l - 1));
        if (l < kLevels - 1) {
            rc |= dalloc(n, &n->cat[l], hw * 2 * C) | dalloc(n, &n->db[l], hw * C) | dalloc(n, &n->dd[l], hw * C) |
                  dalloc(n, &n->dcat[l], hw * 2 * C);
        } else {
            rc |= dalloc(n, &n->b3, hw * C);
        }
    }
    for (int li = 0; li < 17; ++li) rc |= dalloc(n, &n->Gl[li], (size_t)B * n->HWl(n->L[li].level) * n->L[li].cout);
    // the largest temporaries: up-conv input gradient (2C_l at level l) and its low-res sum;
    // the pool gradient (C_{l-1} at level l)
    size_t du = 0, dl = 0, dp = 0;
    for (int l = 0; l < kLevels - 1; ++l) {
        du = std::max(du, (size_t)n->HWl(l) * 2 * drd_unet::C(l));
        dl = std::max(dl, (size_t)n->HWl(l + 1) * 2 * drd_unet::C(l));
        dp = std::max(dp, (size_t)n->HWl(l + 1) * drd_unet::C(l));
    }
    rc |= dalloc(n, &n->dU, du * B) | dalloc(n, &n->dlow, dl * B) | dalloc(n, &n->dpool, dp * B);
    const size_t nio = (size_t)B * n->H0 * n->W0;
    rc |= dalloc(n, &n->y, nio * out_ch) | dalloc(n, &n->dy, nio * out_ch) | dalloc(n, &n->xstage, nio * in_ch) |
          dalloc(n, &n->ystage, nio * out_ch) | dalloc(n, &n->loss, 1) | dalloc(n, &n->dflag, 1);
    // the tcgen05 convolutions on request (DRD_UNET_TC=1): correct, but their operand staging
    // (plain loads into shared memory, the weights reloaded for every 128-pixel tile) leaves the
    // tensor pipe idle most of the time, and the mma.sync kernels are faster on this network
    const char* tce = std::getenv("DRD_UNET_TC");
    n->tc = (tce && tce[0] == '1');
    if (n->tc && cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)tc_smem(256, 16)) != cudaSuccess)
        n->tc = 0;
    if (rc) {
        drd_unet_destroy(n);
        return DRD_ERR_CUDA;
    }
    cudaMemcpyAsync(n->W32, w.data(), sizeof(float) * n->nparam, cudaMemcpyHostToDevice, n->s);
    cudaMemcpyAsync(n->tmap, tm.data(), sizeof(int) * n->nparam, cudaMemcpyHostToDevice, n->s);
    refresh_bf16(n, 0, 0.f);
    rc = finish(n);
    if (rc) {
        drd_unet_destroy(n);
        return rc;
    }
    *out = n;
    return DRD_OK;
}

int drd_unet_destroy(drd_unet* n) {
    if (!n) return DRD_OK;
    if (n->s) cudaStreamSynchronize(n->s);
    for (void* p : n->allocs) cudaFree(p);
    if (n->s) cudaStreamDestroy(n->s);
    delete n;
    return DRD_OK;
}

int64_t drd_unet_param_count(drd_unet* n) { return n ? n->nparam : -1; }

const char* drd_unet_last_error(drd_unet* n) { return n ? n->err.c_str() : "null network"; }

int drd_unet_get_params(drd_unet* n, float* host) {
    if (!n || !host) return DRD_ERR_BADARG;
    cudaMemcpyAsync(host, n->W32, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost, n->s);
    return finish(n);
}

int drd_unet_set_params(drd_unet* n, const float* host) {
    if (!n || !host) return DRD_ERR_BADARG;
    cudaMemcpyAsync(n->W32, host, sizeof(float) * n->nparam, cudaMemcpyHostToDevice, n->s);
    refresh_bf16(n, 0, 0.f);
    n->adam_t = 0;
    cudaMemsetAsync(n->M, 0, sizeof(float) * n->nparam, n->s);
    cudaMemsetAsync(n->V, 0, sizeof(float) * n->nparam, n->s);
    return finish(n);
}

int drd_unet_forward(drd_unet* n, int batch, const float* x, float* y) {
    if (!n || !x || !y || batch < 1 || batch > n->maxb) return n ? set_err(n, "bad forward arguments") : DRD_ERR_BADARG;
    const long nin = (long)batch * n->cin * n->H0 * n->W0, nout = (long)batch * n->cout * n->H0 * n->W0;
    forward(n, stage_in(n, x, nin, n->xstage), batch);
    cudaMemcpyAsync(y, n->y, sizeof(float) * nout, cudaMemcpyDefault, n->s);
    return finish(n);
}

int drd_unet_gradients(drd_unet* n, int batch, const float* x, const float* target, float* loss, float* grads) {
    if (!n || !x || !target || batch < 1 || batch > n->maxb) return n ? set_err(n, "bad gradient arguments") : DRD_ERR_BADARG;
    loss_and_grads(n, batch, x, target);
    if (loss) cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDefault, n->s);
    if (grads) cudaMemcpyAsync(grads, n->G32, sizeof(float) * n->nparam, cudaMemcpyDefault, n->s);
    return finish(n);
}

int drd_unet_train_step(drd_unet* n, int batch, const float* x, const float* target, float lr, float* loss) {
    if (!n || !x || !target || batch < 1 || batch > n->maxb || !(lr >= 0.f))
        return n ? set_err(n, "bad train-step arguments") : DRD_ERR_BADARG;
    loss_and_grads(n, batch, x, target);
    refresh_bf16(n, 1, lr);
    if (loss) cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDefault, n->s);
    return finish(n);
}

int drd_unet_stream(drd_unet* n, void** stream) {
    if (!n || !stream) return DRD_ERR_BADARG;
    *stream = (void*)n->s;
    return DRD_OK;
}

}  // extern "C"
