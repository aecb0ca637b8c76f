// The learned shooting guess of the Bragg solve: a 4-level U-Net (32 base
// channels, BF16 storage, FP32 accumulation) trained and run by this
// library's own kernels.  No DYFOX counterpart: the network only proposes
// the GMRES starting vector D_g(0) of each plane; the solve itself (and its
// true-residual test) is unchanged, so a poor guess costs iterations, never
// accuracy.
//
// Layout: activations NHWC in bfloat16; 3x3 weights W[co][tap][ci] (and
// the transposed copy Wt[ci][tap][co] for the data gradient); the FP32
// master parameters, their gradients and the Adam moments are flat arrays
// in the order of the network's layer list (oracle/unet_oracle.py's
// param_layout, the checker of these kernels).
//
// The forward and data-gradient products run on the tcgen05 tensor cores
// with TMEM accumulators and TMA-staged operands (unet_tc.cu) whenever the
// image rows fit its 128-pixel tiles.  The weight gradient, and the other
// two where the rows do not fit, are implicit GEMMs on the tensor cores
// with mma.sync (m16n8k16 bf16 -> f32): 64 x BN x 32 tiles, 4 warps, cp.async
// double-buffered gathers with zero fill at the image border, ldmatrix
// (transposed where the operand is stored M- or N-contiguous):
//   forward      C[p][co]      = sum_(t,ci) X[p+t][ci] W[co][t][ci]
//   data grad    C[p][ci]      = sum_(t,co) G[p-t][co] Wt[ci][t][co]
//   weight grad  C[(t,ci)][co] = sum_p X[p+t][ci] G[p][co]  (split over p)
// with bias + ReLU + bf16 rounding fused into the forward epilogue.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>

#include "common.cuh"
#include "unet_tc.cuh"

namespace dyfox {

using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------------------
// Network definition (must match oracle/unet_oracle.py).
constexpr int kUnetCin = 32;
constexpr int kNumConv = 14;
struct ConvDef {
    int cin, cout, level;      // level: spatial size H >> level
};
constexpr ConvDef kConvs[kNumConv] = {
    {32, 32, 0},   {32, 32, 0},                    // e0a e0b
    {32, 64, 1},   {64, 64, 1},                    // e1a e1b
    {64, 128, 2},  {128, 128, 2},                  // e2a e2b
    {128, 256, 3}, {256, 256, 3},                  // ba bb
    {384, 128, 2}, {128, 128, 2},                  // d2a d2b
    {192, 64, 1},  {64, 64, 1},                    // d1a d1b
    {96, 32, 0},   {32, 32, 0}};                   // d0a d0b

static size_t conv_wsize(int i) { return (size_t)9 * kConvs[i].cin * kConvs[i].cout; }

static size_t unet_param_count_host() {
    size_t n = 0;
    for (int i = 0; i < kNumConv; ++i) n += conv_wsize(i) + kConvs[i].cout;
    return n + 2 * 32 + 2;
}

// ---------------------------------------------------------------------------
// Implicit-GEMM convolution on the tensor cores.
enum ConvMode { CM_FWD = 0, CM_DGRAD = 1, CM_WGRAD = 2 };

constexpr int kBM = 64, kBK = 32, kThreads = 128;
constexpr int kKStride = kBK + 8;     // K-contiguous tile row (bf16)
constexpr int kMNStride = 64 + 8;     // M/N-contiguous tile row (bf16)

struct ConvArgs {
    const bf16 *X;        // FWD / WGRAD: input (N, H, W, Cin)
    const bf16 *G;        // DGRAD / WGRAD: masked output gradient (N,H,W,Cout)
    const bf16 *Wk;       // FWD: W[co][t][ci]; DGRAD: Wt[ci][t][co]
    const float *bias;    // FWD
    bf16 *Y;              // FWD: relu(conv + bias) as bf16
    float *dX;            // DGRAD: (N, H, W, Cin)
    float *part;          // WGRAD: (splits, 9 Cin, Cout)
    int N, H, W, Cin, Cout;
    int M, Ncols, K;      // GEMM sizes
    int ktiles_per_split;
};

__device__ __forceinline__ void cp_async16_zfill(void *dst, const void *src,
                                                 bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d),
                 "l"(src), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ldsm_x4(unsigned &r0, unsigned &r1,
                                        unsigned &r2, unsigned &r3,
                                        const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned &r0, unsigned &r1,
                                          unsigned &r2, unsigned &r3,
                                          const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile(
        "ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
        : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
        : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float *c, const unsigned *a,
                                         unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Pixel p of the (N, H, W) grid displaced by (dy, dx): its linear index, or
// -1 outside the image.
__device__ __forceinline__ int shifted_pixel(int p, int H, int W, int dy,
                                             int dx) {
    const int hw = H * W;
    const int n = p / hw, r = p - n * hw;
    const int y = r / W + dy, x = r - (r / W) * W + dx;
    if (y < 0 || y >= H || x < 0 || x >= W) return -1;
    return (n * H + y) * W + x;
}

template <int MODE, int BN>
__global__ void __launch_bounds__(kThreads)
conv_gemm_kernel(const ConvArgs a) {
    // A: FWD / DGRAD K-contiguous [64][kKStride]; WGRAD M-contiguous
    //    [kBK][kMNStride].  B: FWD / DGRAD K-contiguous [BN][kKStride];
    //    WGRAD N-contiguous [kBK][kMNStride].
    constexpr bool kA_K = MODE != CM_WGRAD, kB_K = MODE != CM_WGRAD;
    constexpr int kASize = kA_K ? kBM * kKStride : kBK * kMNStride;
    constexpr int kBSize = kB_K ? BN * kKStride : kBK * kMNStride;
    __shared__ __align__(16) bf16 sA[2][kASize];
    __shared__ __align__(16) bf16 sB[2][kBSize];
    constexpr int NI = BN / 16;          // n8 tiles per warp (warp: 32 x BN/2)

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    // FWD / DGRAD: the tile's 64 output pixels stay fixed over the whole K
    // loop; their (y, x) are decoded once (y = -2^20 marks a pixel past M).
    __shared__ int sRowY[kBM], sRowX[kBM];
    if (MODE != CM_WGRAD) {
        for (int r = tid; r < kBM; r += kThreads) {
            const int p = m0 + r;
            int y = -(1 << 20), x = 0;
            if (p < a.M) {
                const int rem = p % (a.H * a.W);
                y = rem / a.W;
                x = rem - y * a.W;
            }
            sRowY[r] = y;
            sRowX[r] = x;
        }
        __syncthreads();
    }
    const int kt0 = blockIdx.z * a.ktiles_per_split;
    const int ktiles_total = (a.K + kBK - 1) / kBK;
    int kt1 = kt0 + a.ktiles_per_split;
    if (kt1 > ktiles_total) kt1 = ktiles_total;
    const int H = a.H, W = a.W;

    auto load = [&](int kt, int stage) {
        const int k0 = kt * kBK;
        if (MODE == CM_FWD || MODE == CM_DGRAD) {
            const int C = MODE == CM_FWD ? a.Cin : a.Cout;   // K channels
            const int t = k0 / C, c0 = k0 - t * C;
            const int dy = t / 3 - 1, dx = t % 3 - 1;
            const bf16 *src = MODE == CM_FWD ? a.X : a.G;
            // A: 64 pixels x 4 chunks; the source pixel is p + (dy, dx)
            // (forward) or p - (dy, dx) (data gradient).
            const int sy = MODE == CM_FWD ? dy : -dy;
            const int sx = MODE == CM_FWD ? dx : -dx;
            const int sq = sy * W + sx;
            for (int c = tid; c < kBM * 4; c += kThreads) {
                const int row = c >> 2, kc = c & 3;
                const int y = sRowY[row] + sy, x = sRowX[row] + sx;
                const bool ok = (unsigned)y < (unsigned)H &&
                                (unsigned)x < (unsigned)W;
                const bf16 *g = ok ? src + (size_t)(m0 + row + sq) * C + c0 + 8 * kc
                                   : src;
                cp_async16_zfill(&sA[stage][row * kKStride + 8 * kc], g, ok);
            }
            // B: BN output channels x 4 chunks, rows of Wk[n][t][c]
            for (int c = tid; c < BN * 4; c += kThreads) {
                const int row = c >> 2, kc = c & 3;
                const int n = n0 + row;
                const bool ok = n < a.Ncols;
                const bf16 *g = ok ? a.Wk + ((size_t)n * 9 + t) * C + c0 + 8 * kc
                                   : a.Wk;
                cp_async16_zfill(&sB[stage][row * kKStride + 8 * kc], g, ok);
            }
        } else {
            // A: rows k = pixel, cols m = (t, ci); B: rows k = pixel, cols co.
            for (int c = tid; c < kBK * 8; c += kThreads) {
                const int row = c >> 3, mc = c & 7;
                const int p = k0 + row;
                const int m = m0 + 8 * mc;
                int q = -1, ci = 0;
                if (m < a.M && p < a.K) {
                    const int t = m / a.Cin;
                    ci = m - t * a.Cin;
                    q = shifted_pixel(p, H, W, t / 3 - 1, t % 3 - 1);
                }
                const bf16 *g = q >= 0 ? a.X + (size_t)q * a.Cin + ci : a.X;
                cp_async16_zfill(&sA[stage][row * kMNStride + 8 * mc], g, q >= 0);
            }
            for (int c = tid; c < kBK * (BN / 8); c += kThreads) {
                const int row = c / (BN / 8), nc = c - row * (BN / 8);
                const int p = k0 + row;
                const int n = n0 + 8 * nc;
                const bool ok = n < a.Ncols && p < a.K;
                const bf16 *g = ok ? a.G + (size_t)p * a.Cout + n : a.G;
                cp_async16_zfill(&sB[stage][row * kMNStride + 8 * nc], g, ok);
            }
        }
        cp_commit();
    };

    float acc[2][NI][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

    if (kt0 < kt1) load(kt0, 0);
    for (int kt = kt0; kt < kt1; ++kt) {
        const int st = (kt - kt0) & 1;
        if (kt + 1 < kt1) {
            load(kt + 1, st ^ 1);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        __syncthreads();
        const bf16 *A = sA[st], *B = sB[st];
#pragma unroll
        for (int ks = 0; ks < kBK / 16; ++ks) {
            unsigned af[2][4], bfr[NI][2];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi) {
                const int mrow = wm * 32 + mi * 16;
                if (kA_K) {
                    const bf16 *p = A + (mrow + (lane & 15)) * kKStride +
                                    ks * 16 + (lane >> 4) * 8;
                    ldsm_x4(af[mi][0], af[mi][1], af[mi][2], af[mi][3], p);
                } else {
                    const int j = lane >> 3;
                    const bf16 *p = A + (ks * 16 + (j >> 1) * 8 + (lane & 7)) *
                                            kMNStride + mrow + (j & 1) * 8;
                    ldsm_x4_t(af[mi][0], af[mi][1], af[mi][2], af[mi][3], p);
                }
            }
#pragma unroll
            for (int np = 0; np < NI / 2; ++np) {
                const int ncol = wn * (BN / 2) + np * 16;
                const int j = lane >> 3;
                unsigned r0, r1, r2, r3;
                if (kB_K) {
                    const bf16 *p = B + (ncol + (j >> 1) * 8 + (lane & 7)) *
                                            kKStride + ks * 16 + (j & 1) * 8;
                    ldsm_x4(r0, r1, r2, r3, p);
                } else {
                    const bf16 *p = B + (ks * 16 + (j & 1) * 8 + (lane & 7)) *
                                            kMNStride + ncol + (j >> 1) * 8;
                    ldsm_x4_t(r0, r1, r2, r3, p);
                }
                bfr[2 * np][0] = r0;
                bfr[2 * np][1] = r1;
                bfr[2 * np + 1][0] = r2;
                bfr[2 * np + 1][1] = r3;
            }
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < NI; ++ni)
                    mma_bf16(acc[mi][ni], af[mi], bfr[ni][0], bfr[ni][1]);
        }
        __syncthreads();
    }

    // ---- epilogue
    const int g = lane >> 2, c2 = (lane & 3) * 2;
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < NI; ++ni)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int m = m0 + wm * 32 + mi * 16 + g + 8 * h;
                const int n = n0 + wn * (BN / 2) + ni * 8 + c2;
                if (m >= a.M || n >= a.Ncols) continue;
                const float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
                if (MODE == CM_FWD) {
                    const float y0 = fmaxf(v0 + a.bias[n], 0.f);
                    const float y1 = fmaxf(v1 + a.bias[n + 1], 0.f);
                    *reinterpret_cast<__nv_bfloat162 *>(a.Y + (size_t)m * a.Ncols + n) =
                        __floats2bfloat162_rn(y0, y1);
                } else if (MODE == CM_DGRAD) {
                    *reinterpret_cast<float2 *>(a.dX + (size_t)m * a.Ncols + n) =
                        make_float2(v0, v1);
                } else {
                    *reinterpret_cast<float2 *>(
                        a.part + ((size_t)blockIdx.z * a.M + m) * a.Ncols + n) =
                        make_float2(v0, v1);
                }
            }
}

// ---------------------------------------------------------------------------
// Elementwise and reduction kernels (grid-stride, deterministic).

// Average pool 2 x 2 (bf16 in / out).
__global__ void pool_fwd_kernel(const bf16 *in, bf16 *out, int N, int H,
                                int W, int C) {
    const int Ho = H / 2, Wo = W / 2;
    const long total = (long)N * Ho * Wo * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long t = i / C;
        const int x = (int)(t % Wo);
        t /= Wo;
        const int y = (int)(t % Ho);
        const int n = (int)(t / Ho);
        const bf16 *b = in + (((size_t)n * H + 2 * y) * W + 2 * x) * C + c;
        const float s = __bfloat162float(b[0]) + __bfloat162float(b[C]) +
                        __bfloat162float(b[(size_t)W * C]) +
                        __bfloat162float(b[(size_t)W * C + C]);
        out[i] = __float2bfloat16_rn(0.25f * s);
    }
}

// out = concat(up2(lo), skip) along channels; lo (N, H/2, W/2, Cl).
__global__ void upcat_fwd_kernel(const bf16 *lo, const bf16 *skip, bf16 *out,
                                 int N, int H, int W, int Cl, int Cs) {
    const int C = Cl + Cs;
    const long total = (long)N * H * W * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long p = i / C;
        const int x = (int)(p % W);
        const long t = p / W;
        const int y = (int)(t % H);
        const int n = (int)(t / H);
        out[i] = c < Cl
            ? lo[(((size_t)n * (H / 2) + y / 2) * (W / 2) + x / 2) * Cl + c]
            : skip[(size_t)p * Cs + (c - Cl)];
    }
}

// G = bf16(dOut * (Y > 0)).
__global__ void mask_round_kernel(const float *dout, const bf16 *Y, bf16 *G,
                                  long n) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        G[i] = __float2bfloat16_rn(__bfloat162float(Y[i]) > 0.f ? dout[i] : 0.f);
}

// From the gradient of a concatenated input: d_lo = sum over each 2 x 2
// block of the first Cl channels, d_skip = the last Cs channels (written).
__global__ void upcat_bwd_kernel(const float *dc, float *dlo, float *dskip,
                                 int N, int H, int W, int Cl, int Cs) {
    const int C = Cl + Cs;
    const long total_lo = (long)N * (H / 2) * (W / 2) * Cl;
    const long total_sk = (long)N * H * W * Cs;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
         i < total_lo + total_sk; i += (long)gridDim.x * blockDim.x) {
        if (i < total_lo) {
            const int c = (int)(i % Cl);
            long t = i / Cl;
            const int x = (int)(t % (W / 2));
            t /= (W / 2);
            const int y = (int)(t % (H / 2));
            const int n = (int)(t / (H / 2));
            const float *b = dc + (((size_t)n * H + 2 * y) * W + 2 * x) * C + c;
            dlo[i] = (b[0] + b[C]) + (b[(size_t)W * C] + b[(size_t)W * C + C]);
        } else {
            const long j = i - total_lo;
            const int c = (int)(j % Cs);
            const long p = j / Cs;
            dskip[j] = dc[(size_t)p * C + Cl + c];
        }
    }
}

// dOut(e) += pool_backward(d_pooled): each of the 2 x 2 sources gets 1/4.
__global__ void pool_bwd_add_kernel(const float *dp, float *de, int N, int H,
                                    int W, int C) {
    const long total = (long)N * H * W * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long t = i / C;
        const int x = (int)(t % W);
        t /= W;
        const int y = (int)(t % H);
        const int n = (int)(t / H);
        de[i] += 0.25f * dp[(((size_t)n * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
    }
}

// Split-K partials (splits, 9 Cin, Cout) -> dW[co][t][ci].
__global__ void wgrad_reduce_kernel(const float *part, float *dW, int splits,
                                    int Cin, int Cout) {
    const long total = (long)9 * Cin * Cout;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % Cin);
        const long t2 = i / Cin;
        const int t = (int)(t2 % 9);
        const int co = (int)(t2 / 9);
        const size_t m = (size_t)t * Cin + ci;
        float s = 0.f;
        for (int z = 0; z < splits; ++z)
            s += part[((size_t)z * 9 * Cin + m) * Cout + co];
        dW[i] = s;
    }
}

// Column sums of G (P, C) in two passes: partial[b][c] over pixel blocks,
// then db[c] = sum_b partial[b][c].
constexpr int kColBlocks = 256;
__global__ void colsum_partial_kernel(const bf16 *G, float *partial, long P,
                                      int C) {
    const long per = (P + kColBlocks - 1) / kColBlocks;
    const long p0 = blockIdx.x * per;
    long p1 = p0 + per;
    if (p1 > P) p1 = P;
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        float s = 0.f;
        for (long p = p0; p < p1; ++p) s += __bfloat162float(G[(size_t)p * C + c]);
        partial[(size_t)blockIdx.x * C + c] = s;
    }
}
__global__ void colsum_final_kernel(const float *partial, float *out, int C,
                                    int nb) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C;
         c += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nb; ++b) s += partial[(size_t)b * C + c];
        out[c] = s;
    }
}

// Head: y = W d0 + b (2 outputs of 32 channels).  With a target: dy =
// (y - t) / count, the loss's per-block partial sums, dd0 = dy W (FP32),
// and per-block partials of dW (2 x 32) and db (2).
constexpr int kHeadThreads = 256;
__global__ void __launch_bounds__(kHeadThreads)
head_kernel(const bf16 *d0, const float *Wh, const float *bh, float *y,
            const float *target, float inv_count, float *dd0, float *part,
            long P) {
    __shared__ float w[64], red[kHeadThreads / 32][67];
    if (threadIdx.x < 64) w[threadIdx.x] = Wh[threadIdx.x];
    __syncthreads();
    float acc[67];
#pragma unroll
    for (int j = 0; j < 67; ++j) acc[j] = 0.f;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P;
         p += (long)gridDim.x * blockDim.x) {
        float x[32];
        const __nv_bfloat162 *src =
            reinterpret_cast<const __nv_bfloat162 *>(d0 + (size_t)p * 32);
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            const float2 f = __bfloat1622float2(src[c]);
            x[2 * c] = f.x;
            x[2 * c + 1] = f.y;
        }
        float y0 = bh[0], y1 = bh[1];
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            y0 = fmaf(w[c], x[c], y0);
            y1 = fmaf(w[32 + c], x[c], y1);
        }
        y[2 * p] = y0;
        y[2 * p + 1] = y1;
        if (target) {
            const float e0 = y0 - target[2 * p], e1 = y1 - target[2 * p + 1];
            acc[66] += e0 * e0 + e1 * e1;
            const float g0 = e0 * inv_count, g1 = e1 * inv_count;
            acc[64] += g0;
            acc[65] += g1;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                dd0[(size_t)p * 32 + c] = g0 * w[c] + g1 * w[32 + c];
                acc[c] = fmaf(g0, x[c], acc[c]);
                acc[32 + c] = fmaf(g1, x[c], acc[32 + c]);
            }
        }
    }
    if (!target) return;
    // block reduction of the 67 partials (fixed order)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 67; ++j) {
        float v = acc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 67) {
        float s = 0.f;
        for (int k = 0; k < kHeadThreads / 32; ++k) s += red[k][threadIdx.x];
        part[(size_t)blockIdx.x * 67 + threadIdx.x] = s;
    }
}

// Sum of the head's per-block partials: dW (64), db (2) into the gradient
// vector, and the loss sse * loss_scale.
__global__ void head_reduce_kernel(const float *part, int nb, float *g_w,
                                   float *g_b, float *loss, float loss_scale) {
    const int j = threadIdx.x;
    if (j >= 67) return;
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * 67 + j];
    if (j < 64) g_w[j] = s;
    else if (j < 66) g_b[j - 64] = s;
    else if (loss) *loss = s * loss_scale;
}

// Adam on the flat parameters (FP32 master copy).
__global__ void adam_kernel(float *p, const float *g, float *m, float *v,
                            long n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// bf16 copies of one 3x3 weight: Wb[co][t][ci] and Wt[ci][t][co].
__global__ void cast_weights_kernel(const float *Wf, bf16 *Wb, bf16 *Wt,
                                    int Cin, int Cout) {
    const long total = (long)9 * Cin * Cout;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % Cin);
        const long t2 = i / Cin;
        const int t = (int)(t2 % 9);
        const int co = (int)(t2 / 9);
        const bf16 b = __float2bfloat16_rn(Wf[i]);
        Wb[i] = b;
        Wt[((size_t)ci * 9 + t) * Cout + co] = b;
    }
}

// He-normal initialisation from a counter-based generator (splitmix64 of
// (seed, index) -> two uniforms -> Box-Muller); biases zero.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__global__ void he_init_kernel(float *p, long n, float stdev,
                               unsigned long long seed,
                               unsigned long long base) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const unsigned long long r = splitmix64(seed ^ splitmix64(base + i));
        const double u1 = ((r >> 11) + 1.0) * (1.0 / 9007199254740993.0);
        const double u2 = (splitmix64(r) >> 11) * (1.0 / 9007199254740992.0);
        p[i] = (float)(stdev * sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2));
    }
}

// Network input from the top depth slices of H: x[n][y][x][2k, 2k+1] =
// cos, sin H(plane y, slice k, column (col0 + x) mod Nx) for k < 8 (the
// lateral grid is periodic); x[..][16] = s_n; channels 17..31 zero.
// h: (n_y, 8, Nx) doubles.
__global__ void features_kernel(const double *h, int n_y, int Nx, int col0,
                                int W, const double *s, int n_s, bf16 *out) {
    const long total = (long)n_s * n_y * W;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % W);
        const long t = i / W;
        const int y = (int)(t % n_y);
        const int n = (int)(t / n_y);
        bf16 *o = out + (size_t)i * kUnetCin;
        for (int k = 0; k < 8; ++k) {
            const double hv = h[((size_t)y * 8 + k) * Nx + (col0 + x) % Nx];
            double sn, c;
            sincos(hv, &sn, &c);
            o[2 * k] = __float2bfloat16_rn((float)c);
            o[2 * k + 1] = __float2bfloat16_rn((float)sn);
        }
        o[16] = __float2bfloat16_rn((float)s[n]);
        for (int c = 17; c < kUnetCin; ++c) o[c] = __float2bfloat16_rn(0.f);
    }
}

static int grid_for(long n, int threads = 256) {
    long b = (n + threads - 1) / threads;
    if (b > 152L * 32) b = 152L * 32;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace dyfox

// ---------------------------------------------------------------------------
// The network object: every buffer is a slice of one caller workspace.
using namespace dyfox;

struct dyfox_unet {
    int batch, H, W;
    char *ws;
    size_t bytes;
    // parameters (FP32, flat), gradients, Adam moments
    float *params, *grads, *m, *v;
    size_t n_params;
    size_t off_w[kNumConv], off_b[kNumConv], off_hw, off_hb;   // in floats
    bf16 *Wb[kNumConv], *Wt[kNumConv];
    // activations (bf16) and gradients (fp32 dOut, bf16 G)
    bf16 *act[kNumConv];             // conv outputs
    bf16 *pool[3];                   // pooled e0, e1, e2
    bf16 *cat[3];                    // concat inputs of d2a, d1a, d0a
    float *dout[kNumConv];           // dL/d act
    float *dtmp;                     // data gradient of a pooled / concat input
    bf16 *G;                         // masked gradient (largest activation)
    float *wpart;                    // weight-gradient split partials
    size_t wpart_floats;
    float *colpart;                  // bias-gradient partials
    float *headpart;                 // head partials
    float *y;                        // head output (batch, H, W, 2)
    const bf16 *x;                   // current input
    int n;                           // current batch
    int steps;                       // Adam steps taken
    int head_blocks;
};

namespace dyfox {

static size_t a256u(size_t v) { return (v + 255) & ~(size_t)255; }

// Lay the network out in a workspace (ws NULL: sizes only).
static size_t unet_layout(dyfox_unet *u, int batch, int H, int W, char *ws) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char *p = ws ? ws + o : nullptr;
        o = a256u(o + bytes);
        return p;
    };
    const size_t np = unet_param_count_host();
    u->n_params = np;
    u->params = (float *)take(np * 4);
    u->grads = (float *)take(np * 4);
    u->m = (float *)take(np * 4);
    u->v = (float *)take(np * 4);
    size_t f = 0;
    for (int i = 0; i < kNumConv; ++i) {
        u->off_w[i] = f; f += conv_wsize(i);
        u->off_b[i] = f; f += kConvs[i].cout;
    }
    u->off_hw = f; f += 64;
    u->off_hb = f; f += 2;
    for (int i = 0; i < kNumConv; ++i) {
        u->Wb[i] = (bf16 *)take(conv_wsize(i) * 2);
        u->Wt[i] = (bf16 *)take(conv_wsize(i) * 2);
    }
    const size_t P0 = (size_t)batch * H * W;
    auto pix = [&](int level) { return P0 >> (2 * level); };
    size_t max_act = 0;
    for (int i = 0; i < kNumConv; ++i) {
        const size_t n = pix(kConvs[i].level) * kConvs[i].cout;
        u->act[i] = (bf16 *)take(n * 2);
        u->dout[i] = (float *)take(n * 4);
        if (n > max_act) max_act = n;
    }
    for (int l = 0; l < 3; ++l) {
        const int c = kConvs[2 * l + 1].cout;               // e0b e1b e2b
        u->pool[l] = (bf16 *)take(pix(l + 1) * c * 2);
    }
    // concat inputs: d2a (level 2, 384), d1a (level 1, 192), d0a (level 0, 96)
    u->cat[0] = (bf16 *)take(pix(2) * 384 * 2);
    u->cat[1] = (bf16 *)take(pix(1) * 192 * 2);
    u->cat[2] = (bf16 *)take(pix(0) * 96 * 2);
    size_t max_in = 0;
    for (int i = 0; i < kNumConv; ++i)
        max_in = std::max(max_in, pix(kConvs[i].level) * kConvs[i].cin);
    u->dtmp = (float *)take(max_in * 4);
    u->G = (bf16 *)take(max_act * 2);
    // split-K partials: up to 8 splits of the largest 9 Cin x Cout
    size_t wmax = 0;
    for (int i = 0; i < kNumConv; ++i) wmax = std::max(wmax, conv_wsize(i));
    u->wpart_floats = wmax * 64;
    u->wpart = (float *)take(u->wpart_floats * 4);
    u->colpart = (float *)take((size_t)kColBlocks * 384 * 4);
    u->head_blocks = 152 * 4;
    u->headpart = (float *)take((size_t)u->head_blocks * 67 * 4);
    u->y = (float *)take(P0 * 2 * 4);
    return o;
}

static int unet_check_shape(int batch, int H, int W) {
    if (batch < 1 || H < 8 || W < 8 || H % 8 || W % 8) {
        set_error("U-Net needs batch >= 1 and H, W multiples of 8 (got %d, "
                  "%d, %d)", batch, H, W);
        return DYFOX_EINVAL;
    }
    if ((long)batch * H * W > (1L << 26)) {
        set_error("U-Net batch x H x W above 2^26");
        return DYFOX_ENOSYS;
    }
    return DYFOX_OK;
}

// One forward or data-gradient product (no split of K): on the tcgen05
// tensor cores when the shapes allow (unet_tc.cu), else (or with `legacy`)
// the mma.sync implicit GEMM above.
template <int MODE>
static cudaError_t run_conv(const ConvArgs &a0, cudaStream_t s,
                            bool legacy = false) {
    if (!legacy) {
        TcConv c;
        c.mode = MODE == CM_FWD ? 0 : 1;
        c.act = MODE == CM_FWD ? (const void *)a0.X : (const void *)a0.G;
        c.wk = a0.Wk;
        c.bias = a0.bias;
        c.out = MODE == CM_FWD ? (void *)a0.Y : (void *)a0.dX;
        c.N = a0.N; c.H = a0.H; c.W = a0.W;
        c.Ck = MODE == CM_FWD ? a0.Cin : a0.Cout;
        c.Ncols = a0.Ncols;
        if (conv_tc_supported(c)) return conv_tc_launch(c, s);
    }
    ConvArgs a = a0;
    const int BN = a.Ncols >= 64 && a.Ncols % 64 == 0 ? 64 : 32;
    dim3 grid((a.M + kBM - 1) / kBM, (a.Ncols + BN - 1) / BN, 1);
    a.ktiles_per_split = a.K / kBK;
    if (BN == 64) conv_gemm_kernel<MODE, 64><<<grid, kThreads, 0, s>>>(a);
    else conv_gemm_kernel<MODE, 32><<<grid, kThreads, 0, s>>>(a);
    count_launch(1);
    return cudaGetLastError();
}

static cudaError_t unet_cast(dyfox_unet *u, cudaStream_t s) {
    for (int i = 0; i < kNumConv; ++i) {
        cast_weights_kernel<<<grid_for((long)conv_wsize(i)), 256, 0, s>>>(
            u->params + u->off_w[i], u->Wb[i], u->Wt[i], kConvs[i].cin,
            kConvs[i].cout);
        count_launch(1);
    }
    return cudaGetLastError();
}

// Input of conv i in the forward pass.
static const bf16 *conv_input(const dyfox_unet *u, int i) {
    switch (i) {
    case 0: return u->x;
    case 2: return u->pool[0];
    case 4: return u->pool[1];
    case 6: return u->pool[2];
    case 8: return u->cat[0];
    case 10: return u->cat[1];
    case 12: return u->cat[2];
    default: return u->act[i - 1];
    }
}

static int unet_forward_impl(dyfox_unet *u, cudaStream_t s) {
    const int n = u->n, H = u->H, W = u->W;
    cudaError_t e;
    for (int i = 0; i < kNumConv; ++i) {
        const int lv = kConvs[i].level, h = H >> lv, w = W >> lv;
        // producers of this conv's input
        if (i == 2 || i == 4 || i == 6) {
            const int l = i / 2 - 1;                    // pool of e0/e1/e2
            const int src = 2 * l + 1;
            const int hs = H >> l, wsz = W >> l;
            const long tot = (long)n * h * w * kConvs[src].cout;
            pool_fwd_kernel<<<grid_for(tot), 256, 0, s>>>(
                u->act[src], u->pool[l], n, hs, wsz, kConvs[src].cout);
            count_launch(1);
        } else if (i == 8 || i == 10 || i == 12) {
            const int c = (i - 8) / 2;                  // cat 0, 1, 2
            const int lo = i - 1;                       // bb, d2b, d1b
            const int sk = 5 - 2 * c;                   // e2b, e1b, e0b
            const long tot = (long)n * h * w * kConvs[i].cin;
            upcat_fwd_kernel<<<grid_for(tot), 256, 0, s>>>(
                u->act[lo], u->act[sk], u->cat[c], n, h, w, kConvs[lo].cout,
                kConvs[sk].cout);
            count_launch(1);
        }
        ConvArgs a;
        memset(&a, 0, sizeof a);
        a.X = conv_input(u, i);
        a.Wk = u->Wb[i];
        a.bias = u->params + u->off_b[i];
        a.Y = u->act[i];
        a.N = n; a.H = h; a.W = w;
        a.Cin = kConvs[i].cin; a.Cout = kConvs[i].cout;
        a.M = n * h * w; a.Ncols = a.Cout; a.K = 9 * a.Cin;
        if ((e = run_conv<CM_FWD>(a, s))) return cuda_status(e, "unet conv");
    }
    head_kernel<<<u->head_blocks, kHeadThreads, 0, s>>>(
        u->act[13], u->params + u->off_hw, u->params + u->off_hb, u->y,
        nullptr, 0.f, nullptr, nullptr, (long)n * H * W);
    count_launch(1);
    return cuda_status(cudaGetLastError(), "unet head");
}

static int unet_backward_impl(dyfox_unet *u, const float *target, float *loss,
                              cudaStream_t s) {
    const int n = u->n, H = u->H, W = u->W;
    const long P = (long)n * H * W;
    cudaError_t e;
    // head: y, dy, dd0 -> dout[13]; partial sums of dW_head, db_head, loss
    head_kernel<<<u->head_blocks, kHeadThreads, 0, s>>>(
        u->act[13], u->params + u->off_hw, u->params + u->off_hb, u->y, target,
        1.0f / (float)(2 * P), u->dout[13], u->headpart, P);
    // L = sum (y - t)^2 / (2 * 2P)
    head_reduce_kernel<<<1, 96, 0, s>>>(u->headpart, u->head_blocks,
                                        u->grads + u->off_hw,
                                        u->grads + u->off_hb, loss,
                                        1.0f / (float)(4 * P));
    count_launch(2);
    for (int i = kNumConv - 1; i >= 0; --i) {
        const int lv = kConvs[i].level, h = H >> lv, w = W >> lv;
        const long Pi = (long)n * h * w;
        const int ci = kConvs[i].cin, co = kConvs[i].cout;
        // G = bf16(dOut * (Y > 0))
        mask_round_kernel<<<grid_for(Pi * co), 256, 0, s>>>(
            u->dout[i], u->act[i], u->G, Pi * co);
        count_launch(1);
        // bias gradient
        colsum_partial_kernel<<<kColBlocks, 128, 0, s>>>(u->G, u->colpart, Pi,
                                                         co);
        colsum_final_kernel<<<(co + 127) / 128, 128, 0, s>>>(
            u->colpart, u->grads + u->off_b[i], co, kColBlocks);
        count_launch(2);
        // weight gradient
        ConvArgs a;
        memset(&a, 0, sizeof a);
        a.X = conv_input(u, i);
        a.G = u->G;
        a.part = u->wpart;
        a.N = n; a.H = h; a.W = w; a.Cin = ci; a.Cout = co;
        a.M = 9 * ci; a.Ncols = co; a.K = (int)Pi;
        TcWgrad tw;
        tw.X = a.X; tw.G = a.G; tw.part = u->wpart;
        tw.part_floats = u->wpart_floats;
        tw.N = n; tw.H = h; tw.W = w; tw.Cin = ci; tw.Cout = co;
        int tsplits = 0;
        if (conv_tc_wgrad_supported(tw) &&
            conv_tc_wgrad_launch(tw, &tsplits, s) == cudaSuccess) {
            wgrad_reduce_kernel<<<grid_for((long)conv_wsize(i)), 256, 0, s>>>(
                u->wpart, u->grads + u->off_w[i], tsplits, ci, co);
            count_launch(1);
            if ((e = cudaGetLastError())) return cuda_status(e, "unet wgrad");
        } else {
            // splits are bounded by the partial buffer
            ConvArgs b = a;
            const int BN = co >= 64 && co % 64 == 0 ? 64 : 32;
            const int tiles = ((a.M + kBM - 1) / kBM) * ((co + BN - 1) / BN);
            int kt = (a.K + kBK - 1) / kBK;
            int splits = (2 * 152 + tiles - 1) / tiles;
            const int cap = (int)(u->wpart_floats / ((size_t)a.M * co));
            if (splits > cap) splits = cap;
            if (splits > kt) splits = kt;
            if (splits < 1) splits = 1;
            b.ktiles_per_split = (kt + splits - 1) / splits;
            const int z = (kt + b.ktiles_per_split - 1) / b.ktiles_per_split;
            dim3 grid((a.M + kBM - 1) / kBM, (co + BN - 1) / BN, z);
            if (BN == 64) conv_gemm_kernel<CM_WGRAD, 64><<<grid, kThreads, 0, s>>>(b);
            else conv_gemm_kernel<CM_WGRAD, 32><<<grid, kThreads, 0, s>>>(b);
            count_launch(1);
            wgrad_reduce_kernel<<<grid_for((long)conv_wsize(i)), 256, 0, s>>>(
                u->wpart, u->grads + u->off_w[i], z, ci, co);
            count_launch(1);
            if ((e = cudaGetLastError())) return cuda_status(e, "unet wgrad");
        }
        if (i == 0) break;                          // no input gradient
        // data gradient into the producer's dOut (or a temporary)
        const bool direct = !(i == 2 || i == 4 || i == 6 || i == 8 ||
                              i == 10 || i == 12);
        ConvArgs d;
        memset(&d, 0, sizeof d);
        d.G = u->G;
        d.Wk = u->Wt[i];
        d.dX = direct ? u->dout[i - 1] : u->dtmp;
        d.N = n; d.H = h; d.W = w; d.Cin = ci; d.Cout = co;
        d.M = (int)Pi; d.Ncols = ci; d.K = 9 * co;
        if ((e = run_conv<CM_DGRAD>(d, s))) return cuda_status(e, "unet dgrad");
        if (i == 8 || i == 10 || i == 12) {
            const int c = (i - 8) / 2, lo = i - 1, sk = 5 - 2 * c;
            const long tot = Pi / 4 * kConvs[lo].cout + Pi * kConvs[sk].cout;
            upcat_bwd_kernel<<<grid_for(tot), 256, 0, s>>>(
                u->dtmp, u->dout[lo], u->dout[sk], n, h, w, kConvs[lo].cout,
                kConvs[sk].cout);
            count_launch(1);
        } else if (i == 2 || i == 4 || i == 6) {
            const int l = i / 2 - 1, src = 2 * l + 1;
            const int hs = H >> l, wsz = W >> l;
            const long tot = (long)n * hs * wsz * kConvs[src].cout;
            pool_bwd_add_kernel<<<grid_for(tot), 256, 0, s>>>(
                u->dtmp, u->dout[src], n, hs, wsz, kConvs[src].cout);
            count_launch(1);
        }
        if ((e = cudaGetLastError())) return cuda_status(e, "unet backward");
    }
    return DYFOX_OK;
}

}  // namespace dyfox

extern "C" size_t dyfox_unet_param_count(void) {
    return unet_param_count_host();
}

extern "C" int dyfox_unet_workspace_bytes(int batch, int H, int W,
                                          size_t *bytes) {
    set_error("");
    if (!bytes) {
        set_error("NULL bytes");
        return DYFOX_EINVAL;
    }
    int st = unet_check_shape(batch, H, W);
    if (st) return st;
    dyfox_unet u;
    *bytes = unet_layout(&u, batch, H, W, nullptr);
    return DYFOX_OK;
}

extern "C" int dyfox_unet_create(int batch, int H, int W, void *workspace,
                                 size_t bytes, dyfox_unet **out) {
    set_error("");
    if (!out) {
        set_error("NULL handle");
        return DYFOX_EINVAL;
    }
    *out = nullptr;
    int st = unet_check_shape(batch, H, W);
    if (st) return st;
    dyfox_unet probe;
    const size_t need = unet_layout(&probe, batch, H, W, nullptr);
    if (!workspace || bytes < need) {
        set_error("workspace of %zu bytes, %zu needed", bytes, need);
        return DYFOX_ENOMEM;
    }
    if ((uintptr_t)workspace & 255) {
        set_error("workspace must be 256-byte aligned");
        return DYFOX_EINVAL;
    }
    dyfox_unet *u = new (std::nothrow) dyfox_unet;
    if (!u) {
        set_error("out of host memory");
        return DYFOX_ENOMEM;
    }
    memset(u, 0, sizeof *u);
    u->batch = batch; u->H = H; u->W = W;
    u->ws = (char *)workspace;
    u->bytes = bytes;
    unet_layout(u, batch, H, W, (char *)workspace);
    *out = u;
    return DYFOX_OK;
}

extern "C" int dyfox_unet_destroy(dyfox_unet *u) {
    delete u;
    return DYFOX_OK;
}

extern "C" int dyfox_unet_params(dyfox_unet *u, float **params,
                                 float **grads) {
    if (!u) {
        set_error("NULL network");
        return DYFOX_EINVAL;
    }
    if (params) *params = u->params;
    if (grads) *grads = u->grads;
    return DYFOX_OK;
}

extern "C" int dyfox_unet_init(dyfox_unet *u, unsigned long long seed,
                               void *stream) {
    set_error("");
    if (!u) {
        set_error("NULL network");
        return DYFOX_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(u->params, 0, u->n_params * 4, s)) ||
        (e = cudaMemsetAsync(u->m, 0, u->n_params * 4, s)) ||
        (e = cudaMemsetAsync(u->v, 0, u->n_params * 4, s)) ||
        (e = cudaMemsetAsync(u->grads, 0, u->n_params * 4, s)))
        return cuda_status(e, "unet init");
    for (int i = 0; i < kNumConv; ++i) {
        const long nw = (long)conv_wsize(i);
        he_init_kernel<<<grid_for(nw), 256, 0, s>>>(
            u->params + u->off_w[i], nw, sqrtf(2.0f / (9.0f * kConvs[i].cin)),
            seed, (unsigned long long)u->off_w[i]);
        count_launch(1);
    }
    he_init_kernel<<<1, 64, 0, s>>>(u->params + u->off_hw, 64,
                                    sqrtf(2.0f / 32.0f), seed,
                                    (unsigned long long)u->off_hw);
    count_launch(1);
    u->steps = 0;
    if ((e = unet_cast(u, s))) return cuda_status(e, "unet cast");
    return DYFOX_OK;
}

extern "C" int dyfox_unet_refresh(dyfox_unet *u, void *stream) {
    set_error("");
    if (!u) {
        set_error("NULL network");
        return DYFOX_EINVAL;
    }
    cudaError_t e = unet_cast(u, (cudaStream_t)stream);
    return e ? cuda_status(e, "unet cast") : DYFOX_OK;
}

extern "C" int dyfox_unet_forward(dyfox_unet *u, const void *x, int n,
                                  float *y, void *stream) {
    set_error("");
    if (!u || !x) {
        set_error("NULL network or input");
        return DYFOX_EINVAL;
    }
    if (n < 1 || n > u->batch) {
        set_error("batch %d outside [1, %d]", n, u->batch);
        return DYFOX_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    u->x = (const bf16 *)x;
    u->n = n;
    int st = unet_forward_impl(u, s);
    if (st) return st;
    if (y) {
        cudaError_t e = cudaMemcpyAsync(y, u->y, (size_t)n * u->H * u->W * 2 * 4,
                                        cudaMemcpyDeviceToDevice, s);
        if (e) return cuda_status(e, "unet output");
    }
    return DYFOX_OK;
}

extern "C" int dyfox_unet_backward(dyfox_unet *u, const float *target,
                                   float *loss, void *stream) {
    set_error("");
    if (!u || !target || !u->x) {
        set_error("NULL network or target, or no forward pass");
        return DYFOX_EINVAL;
    }
    return unet_backward_impl(u, target, loss, (cudaStream_t)stream);
}

extern "C" int dyfox_unet_adam(dyfox_unet *u, float lr, float beta1,
                               float beta2, float eps, void *stream) {
    set_error("");
    if (!u) {
        set_error("NULL network");
        return DYFOX_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    ++u->steps;
    const float c1 = 1.0f / (1.0f - powf(beta1, (float)u->steps));
    const float c2 = 1.0f / (1.0f - powf(beta2, (float)u->steps));
    adam_kernel<<<grid_for((long)u->n_params), 256, 0, s>>>(
        u->params, u->grads, u->m, u->v, (long)u->n_params, lr, beta1, beta2,
        eps, c1, c2);
    count_launch(1);
    cudaError_t e = unet_cast(u, s);
    return e ? cuda_status(e, "unet adam") : DYFOX_OK;
}

extern "C" int dyfox_unet_features(const double *h_top, int n_y, int Nx,
                                   int col0, int W, const double *s_values,
                                   int n_s, void *x_out, void *stream) {
    set_error("");
    if (!h_top || !s_values || !x_out || n_y < 1 || n_s < 1 || W < 1 ||
        Nx < 1 || col0 < 0 || col0 >= Nx) {
        set_error("bad feature arguments (n_y=%d Nx=%d col0=%d W=%d n_s=%d)",
                  n_y, Nx, col0, W, n_s);
        return DYFOX_EINVAL;
    }
    const long tot = (long)n_s * n_y * W;
    features_kernel<<<grid_for(tot), 256, 0, (cudaStream_t)stream>>>(
        h_top, n_y, Nx, col0, W, s_values, n_s, (bf16 *)x_out);
    count_launch(1);
    return cuda_status(cudaGetLastError(), "unet features");
}

extern "C" int dyfox_unet_conv(int mode, const void *X, const void *G,
                               const void *Wk, const float *bias, void *out,
                               int N, int H, int W, int Cin, int Cout,
                               void *workspace, size_t workspace_bytes,
                               void *stream) {
    set_error("");
    if (N < 1 || H < 1 || W < 1 || Cin < 32 || Cout < 32 || Cin % 32 ||
        Cout % 32 || (long)N * H * W > (1L << 26)) {
        set_error("bad conv sizes N=%d H=%d W=%d Cin=%d Cout=%d (channels "
                  "multiples of 32)", N, H, W, Cin, Cout);
        return DYFOX_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const bool legacy = (mode & DYFOX_CONV_MMA_SYNC) != 0;
    mode &= ~DYFOX_CONV_MMA_SYNC;
    ConvArgs a;
    memset(&a, 0, sizeof a);
    a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout;
    cudaError_t e;
    if (mode == CM_FWD) {
        if (!X || !Wk || !bias || !out) {
            set_error("NULL argument");
            return DYFOX_EINVAL;
        }
        a.X = (const bf16 *)X; a.Wk = (const bf16 *)Wk; a.bias = bias;
        a.Y = (bf16 *)out;
        a.M = N * H * W; a.Ncols = Cout; a.K = 9 * Cin;
        e = run_conv<CM_FWD>(a, s, legacy);
    } else if (mode == CM_DGRAD) {
        if (!G || !Wk || !out) {
            set_error("NULL argument");
            return DYFOX_EINVAL;
        }
        a.G = (const bf16 *)G; a.Wk = (const bf16 *)Wk; a.dX = (float *)out;
        a.M = N * H * W; a.Ncols = Cin; a.K = 9 * Cout;
        e = run_conv<CM_DGRAD>(a, s, legacy);
    } else if (mode == CM_WGRAD) {
        if (!X || !G || !out) {
            set_error("NULL argument");
            return DYFOX_EINVAL;
        }
        if (!legacy && workspace) {
            TcWgrad tw;
            tw.X = X; tw.G = G; tw.part = (float *)workspace;
            tw.part_floats = workspace_bytes / sizeof(float);
            tw.N = N; tw.H = H; tw.W = W; tw.Cin = Cin; tw.Cout = Cout;
            int tsplits = 0;
            if (tw.part_floats >= (size_t)9 * Cin * Cout &&
                conv_tc_wgrad_supported(tw)) {
                if ((e = conv_tc_wgrad_launch(tw, &tsplits, s)))
                    return cuda_status(e, "unet conv");
                wgrad_reduce_kernel<<<grid_for((long)9 * Cin * Cout), 256, 0,
                                      s>>>(tw.part, (float *)out, tsplits, Cin,
                                           Cout);
                count_launch(1);
                return cuda_status(cudaGetLastError(), "unet conv");
            }
        }
        a.X = (const bf16 *)X; a.G = (const bf16 *)G;
        a.M = 9 * Cin; a.Ncols = Cout; a.K = N * H * W;
        const int BN = Cout % 64 == 0 ? 64 : 32;
        const int tiles = ((a.M + kBM - 1) / kBM) * ((Cout + BN - 1) / BN);
        const int kt = (a.K + kBK - 1) / kBK;
        int splits = (2 * 152 + tiles - 1) / tiles;
        const size_t per = (size_t)a.M * Cout * sizeof(float);
        const int cap = (int)(workspace_bytes / per);
        if (splits > cap) splits = cap;
        if (splits > kt) splits = kt;
        if (splits < 1 || !workspace) {
            set_error("workspace of %zu bytes, %zu needed", workspace_bytes,
                      per);
            return DYFOX_ENOMEM;
        }
        a.part = (float *)workspace;
        a.ktiles_per_split = (kt + splits - 1) / splits;
        const int z = (kt + a.ktiles_per_split - 1) / a.ktiles_per_split;
        dim3 grid((a.M + kBM - 1) / kBM, (Cout + BN - 1) / BN, z);
        if (BN == 64) conv_gemm_kernel<CM_WGRAD, 64><<<grid, kThreads, 0, s>>>(a);
        else conv_gemm_kernel<CM_WGRAD, 32><<<grid, kThreads, 0, s>>>(a);
        count_launch(1);
        if ((e = cudaGetLastError())) return cuda_status(e, "unet conv");
        wgrad_reduce_kernel<<<grid_for((long)9 * Cin * Cout), 256, 0, s>>>(
            a.part, (float *)out, z, Cin, Cout);
        count_launch(1);
        e = cudaGetLastError();
    } else {
        set_error("mode is 0 (forward), 1 (data gradient) or 2 (weight "
                  "gradient)");
        return DYFOX_EINVAL;
    }
    return cuda_status(e, "unet conv");
}

extern "C" int dyfox_unet_buffer(dyfox_unet *u, int which, int index,
                                 void **ptr, size_t *bytes) {
    set_error("");
    if (!u || !ptr) {
        set_error("NULL argument");
        return DYFOX_EINVAL;
    }
    const size_t P0 = (size_t)u->batch * u->H * u->W;
    auto pix = [&](int level) { return P0 >> (2 * level); };
    size_t n = 0;
    void *p = nullptr;
    switch (which) {
    case 0:                                   // conv output, bf16
    case 3:                                   // its gradient dL/dY, float
        if (index < 0 || index >= kNumConv) break;
        n = pix(kConvs[index].level) * kConvs[index].cout;
        p = which == 0 ? (void *)u->act[index] : (void *)u->dout[index];
        n *= which == 0 ? 2 : 4;
        break;
    case 1:                                   // pooled e0 / e1 / e2, bf16
        if (index < 0 || index >= 3) break;
        n = pix(index + 1) * kConvs[2 * index + 1].cout * 2;
        p = u->pool[index];
        break;
    case 2:                                   // concat inputs, bf16
        if (index < 0 || index >= 3) break;
        n = pix(2 - index) * kConvs[8 + 2 * index].cin * 2;
        p = u->cat[index];
        break;
    default:
        break;
    }
    if (!p) {
        set_error("no buffer (%d, %d)", which, index);
        return DYFOX_EINVAL;
    }
    *ptr = p;
    if (bytes) *bytes = n;
    return DYFOX_OK;
}
