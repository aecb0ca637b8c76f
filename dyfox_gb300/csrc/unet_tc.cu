// The forward and data-gradient 3x3 convolution products of the U-Net on
// the fifth-generation tensor cores (sm_100 family: tcgen05 + TMEM + TMA).
//
// Both products are implicit GEMMs D[M=pixels][N] = A[M][K] B[N][K]^T with
// K = (tap, channel):
//   forward      A[p][(t,c)] = X[p + t][c],  B[co][(t,c)] = W[co][t][c]
//   data grad    A[p][(t,c)] = G[p - t][c],  B[ci][(t,c)] = Wt[ci][t][c]
// One CTA computes a 128-pixel x BN tile (BN <= 128 output channels) with
// the FP32 accumulator in tensor memory (TMEM, BN columns x 128 lanes).
// A K-step is one tap and 32 channels: its A tile (128 pixels x 32
// channels, 8 KB) is one TMA load of a 4-D box (channels, x, y, image) of
// the NHWC activations, started at the tap's displaced pixel; coordinates
// past an image border read as zero, which is the convolution's zero
// padding.  Its B tile (BN x 32 channels) is one 2-D TMA load of the weight
// rows.  Both land 64-byte swizzled (rows of 64 bytes) and feed
// tcgen05.mma kind::f16 (bf16 x bf16 -> f32) directly, two K = 16 slices
// per step.  A four-stage ring of full / empty mbarriers overlaps the loads
// with the MMAs; one thread issues both.  The epilogue reads the
// accumulator back with tcgen05.ld (each warp its 32 TMEM lanes = rows),
// adds the bias and applies ReLU with bf16 rounding (forward), or stores
// FP32 (data gradient).
//
// Every wait is bounded (about 2 s of the global timer): on expiry the CTA
// records an error code in g_tc_error, waits (bounded) for its own loads in
// flight, frees its TMEM and returns; dyfox_unet_tc_error reads the code.
#include <cuda.h>
#include <cuda_bf16.h>
#include <string.h>

#include "common.cuh"
#include "unet_tc.cuh"

namespace dyfox {

__device__ int g_tc_error;

namespace {

constexpr int kTcStages = 4;
constexpr int kTcM = 128;              // pixels per tile (TMEM lanes)
constexpr int kTcK = 32;               // channels per K-step (64-byte rows)
constexpr int kTcThreads = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;

enum TcError { TC_OK = 0, TC_FULL_TIMEOUT = 1, TC_EMPTY_TIMEOUT = 2,
               TC_DONE_TIMEOUT = 3 };

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar,
                                               unsigned bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned long long *bar,
                                         unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of `parity` to complete, at most kWaitNs; false (and
// the error code recorded) when it did not.
__device__ bool mbar_wait(unsigned long long *bar, unsigned parity, int code) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 255u) == 255u && global_ns() - t0 > kWaitNs) {
            atomicCAS(&g_tc_error, 0, code);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map,
                                            int c0, int c1, int c2, int c3,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::"
        "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map,
                                            int c0, int c1,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::"
        "complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major operand in the canonical
// 64-byte-swizzled layout: 8-row groups of 64-byte rows (512 bytes) one
// after another (stride 512 bytes); the K offset inside the 64-byte row is
// part of the start address; version 1 (bit 46), swizzle mode 4 (64 B).
__device__ __forceinline__ unsigned long long sw64_desc(const void *p) {
    const unsigned long long a = smem_u32(p);
    return ((a & 0x3FFFFull) >> 4)          // start address
           | (1ull << 16)                     // leading offset (unused)
           | ((512ull >> 4) << 32)            // stride between 8-row groups
           | (1ull << 46)                     // descriptor version
           | (4ull << 61);                    // 64-byte swizzle
}

// Instruction descriptor of kind::f16: bf16 A and B, both K-major, FP32
// accumulator, M = 128, N = n.
__host__ __device__ constexpr unsigned idesc_bf16(int n) {
    return (1u << 4)                 // D format F32
           | (1u << 7)               // A format BF16
           | (1u << 10)              // B format BF16
           | ((unsigned)(n >> 3) << 17)
           | ((unsigned)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned tmem_d, unsigned long long a,
                                       unsigned long long b, unsigned idesc,
                                       unsigned accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64"
        " [%0];" ::"r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float *v) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, "
        "%7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
          "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcParams {
    int mode;               // 0 forward (bf16 ReLU out), 1 data gradient
    int N, H, W, Ck, Ncols, BN;
    int bw, bh;             // the A box: bw x bh pixels = 128
    int ktiles;             // 9 Ck / 32
    const float *bias;
    void *out;
};

// Dynamic shared memory: the stage ring (1024-byte aligned), then the
// barriers and the TMEM address.
__host__ __device__ inline size_t tc_stage_bytes(int BN) {
    return (size_t)kTcM * kTcK * 2 + (size_t)BN * kTcK * 2;
}
__host__ __device__ inline size_t tc_smem_bytes(int BN) {
    return 1024 + kTcStages * tc_stage_bytes(BN) + 256;
}

__global__ void __launch_bounds__(kTcThreads, 1)
conv_tc_kernel(const __grid_constant__ CUtensorMap mapA,
               const __grid_constant__ CUtensorMap mapB, const TcParams p) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const size_t stage_bytes = tc_stage_bytes(p.BN);
    unsigned char *ring = smem;
    unsigned long long *full =
        reinterpret_cast<unsigned long long *>(ring + kTcStages * stage_bytes);
    unsigned long long *empty = full + kTcStages;
    unsigned long long *done = empty + kTcStages;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(done + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tile_m = blockIdx.x, n0 = blockIdx.y * p.BN;
    // Tile origin: image, first row and first column of its 128 pixels.
    const int per_img = p.H * p.W / kTcM;
    const int img = tile_m / per_img;
    const int q0 = (tile_m - img * per_img) * kTcM;
    const int y0 = q0 / p.W, x0 = q0 - y0 * p.W;
    const int ncols_tmem = p.BN <= 32 ? 32 : p.BN <= 64 ? 64 : 128;

    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile(
            "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
            ::"r"(smem_u32(tmem_slot)), "r"(ncols_tmem)
            : "memory");
        asm volatile(
            "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
                : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    const unsigned a_bytes = kTcM * kTcK * 2, b_bytes = p.BN * kTcK * 2;
    const int cblocks = p.Ck / kTcK;
    const int sgn = p.mode == 0 ? 1 : -1;          // X[p + t] or G[p - t]

    if (tid == 0) {
        const unsigned idesc = idesc_bf16(p.BN);
        bool ok = true;
        int issued = 0, consumed = 0;
        for (int it = 0; it < p.ktiles + kTcStages - 1 && ok; ++it) {
            if (it < p.ktiles) {
                const int s = it % kTcStages;
                if (it >= kTcStages)
                    ok = mbar_wait(&empty[s], ((it / kTcStages) - 1) & 1,
                                   TC_EMPTY_TIMEOUT);
                if (!ok) break;
                const int t = it / cblocks, c0 = (it - t * cblocks) * kTcK;
                const int dy = t / 3 - 1, dx = t % 3 - 1;
                unsigned char *sa = ring + s * stage_bytes;
                unsigned char *sb = sa + a_bytes;
                mbar_expect_tx(&full[s], a_bytes + b_bytes);
                tma_load_4d(sa, &mapA, c0, x0 + sgn * dx, y0 + sgn * dy, img,
                            &full[s]);
                tma_load_2d(sb, &mapB, t * p.Ck + c0, n0, &full[s]);
                ++issued;
            }
            const int j = it - (kTcStages - 1);
            if (j >= 0) {
                const int s = j % kTcStages;
                ok = mbar_wait(&full[s], (j / kTcStages) & 1, TC_FULL_TIMEOUT);
                if (!ok) break;
                ++consumed;
                tc_fence_after();
                const unsigned char *sa = ring + s * stage_bytes;
                const unsigned char *sb = sa + a_bytes;
#pragma unroll
                for (int kk = 0; kk < kTcK / 16; ++kk)
                    tc_mma(tmem, sw64_desc(sa + 32 * kk), sw64_desc(sb + 32 * kk),
                           idesc, (j > 0 || kk > 0) ? 1u : 0u);
                tc_commit(&empty[s]);
            }
        }
        if (!ok) {
            *abort_flag = 1;
            // Loads issued but never consumed: let them land before the
            // CTA leaves (bounded).
            for (int j = consumed; j < issued; ++j)
                mbar_wait(&full[j % kTcStages], (j / kTcStages) & 1,
                          TC_FULL_TIMEOUT);
        }
        // Arrives once every MMA issued above has completed.
        tc_commit(done);
    }
    __syncwarp();
    const bool done_ok = mbar_wait(done, 0, TC_DONE_TIMEOUT);
    tc_fence_after();
    __syncthreads();
    if (done_ok && !*abort_flag) {
        // Row m of the tile is TMEM lane m: warp w reads lanes 32w..32w+31.
        const int row = warp * 32 + lane;
        const long m = (long)tile_m * kTcM + row;
        const unsigned lane_base = tmem + ((unsigned)(warp * 32) << 16);
        for (int c = 0; c < p.BN; c += 16) {
            float v[16];
            tmem_ld16(lane_base + (unsigned)c, v);
            if (p.mode == 0) {
                __nv_bfloat162 h[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float a0 = fmaxf(v[2 * i] + p.bias[n0 + c + 2 * i], 0.f);
                    const float a1 =
                        fmaxf(v[2 * i + 1] + p.bias[n0 + c + 2 * i + 1], 0.f);
                    h[i] = __floats2bfloat162_rn(a0, a1);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(
                    reinterpret_cast<__nv_bfloat16 *>(p.out) + m * p.Ncols + n0 + c);
                const uint4 *src = reinterpret_cast<const uint4 *>(h);
                dst[0] = src[0];
                dst[1] = src[1];
            } else {
                float4 *dst = reinterpret_cast<float4 *>(
                    reinterpret_cast<float *>(p.out) + m * p.Ncols + n0 + c);
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2],
                                         v[4 * i + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile(
            "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
            "r"(ncols_tmem)
            : "memory");
    }
}

// ---------------------------------------------------------------------------
// Weight gradient C[(t,ci)][co] = sum_p X[p + t][ci] G[p][co]: M = 9 Cin
// rows (tap, input channel), N = Cout, K = pixels, split over pixel tiles.
// A CTA computes 128 rows x BN channels for its share of the pixel tiles
// into TMEM and writes the FP32 partial (split, 9 Cin, Cout) that
// wgrad_reduce_kernel sums in split order.  Both operands are pixel-major
// in memory, so both are MN-major for the tensor core: a K-step is one
// tile of 128 pixels, its A operand four TMA boxes of (32 channels x 128
// pixels) of X, each displaced by its tap (zero padding from the tensor
// map's bounds), its B operand BN / 32 boxes of G; every box lands as 128
// rows of 64 bytes, 64-byte swizzled (8-row atoms of 512 bytes).  In the
// shared-memory descriptor of such an MN-major operand the leading offset
// is the distance between 32-element atoms along M (or N), 8 KB here, and
// the stride offset the distance between 8-row groups along K, 512 bytes;
// an MMA of K = 16 takes two groups, so the start advances by 1 KB.
constexpr int kTwStages = 3;
constexpr unsigned kTwBox = kTcM * kTcK * 2;     // 8 KB: 128 pixels x 32 ch

struct TwParams {
    int H, W, Cin, Cout, BN, M9;
    int bw, bh;
    int ptiles, tps;        // pixel tiles in all, per split
    float *part;
};

__host__ __device__ inline size_t tw_stage_bytes(int BN) {
    return (size_t)4 * kTwBox + (size_t)(BN / kTcK) * kTwBox;
}
__host__ __device__ inline size_t tw_smem_bytes(int BN) {
    return 1024 + kTwStages * tw_stage_bytes(BN) + 256;
}

// Descriptor of an MN-major operand: atoms of 32 elements (64 bytes) along
// M or N `lbo` bytes apart, 8-row groups along K 512 bytes apart.
__device__ __forceinline__ unsigned long long sw64_desc_mn(const void *p,
                                                           unsigned lbo) {
    const unsigned long long a = smem_u32(p);
    return ((a & 0x3FFFFull) >> 4)
           | ((unsigned long long)(lbo >> 4) << 16)
           | ((512ull >> 4) << 32)
           | (1ull << 46)
           | (4ull << 61);
}

__global__ void __launch_bounds__(kTcThreads, 1)
conv_tc_wgrad_kernel(const __grid_constant__ CUtensorMap mapX,
                     const __grid_constant__ CUtensorMap mapG,
                     const TwParams p) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const size_t stage_bytes = tw_stage_bytes(p.BN);
    unsigned char *ring = smem;
    unsigned long long *full =
        reinterpret_cast<unsigned long long *>(ring + kTwStages * stage_bytes);
    unsigned long long *empty = full + kTwStages;
    unsigned long long *done = empty + kTwStages;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(done + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTcM, n0 = blockIdx.y * p.BN, z = blockIdx.z;
    const int pt0 = z * p.tps;
    const int npt = p.ptiles - pt0 < p.tps ? p.ptiles - pt0 : p.tps;
    const int per_img = p.H * p.W / kTcM;
    const int ncols_tmem = p.BN <= 32 ? 32 : p.BN <= 64 ? 64 : 128;
    const int nb = p.BN / kTcK;
    // A atoms of this tile inside the 9 Cin rows
    int na = 0;
    while (na < 4 && m0 + na * kTcK < p.M9) ++na;

    if (tid == 0) {
        for (int s = 0; s < kTwStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile(
            "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
            ::"r"(smem_u32(tmem_slot)), "r"(ncols_tmem)
            : "memory");
        asm volatile(
            "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
                : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    if (tid == 0) {
        // both operands MN-major (bits 15, 16)
        const unsigned idesc = idesc_bf16(p.BN) | (1u << 15) | (1u << 16);
        const unsigned bytes = (unsigned)(na + nb) * kTwBox;
        bool ok = true;
        int issued = 0, consumed = 0;
        for (int it = 0; it < npt + kTwStages - 1 && ok; ++it) {
            if (it < npt) {
                const int s = it % kTwStages;
                if (it >= kTwStages)
                    ok = mbar_wait(&empty[s], ((it / kTwStages) - 1) & 1,
                                   TC_EMPTY_TIMEOUT);
                if (!ok) break;
                const int tile = pt0 + it;
                const int img = tile / per_img;
                const int q0 = (tile - img * per_img) * kTcM;
                const int y0 = q0 / p.W, x0 = q0 - y0 * p.W;
                unsigned char *sa = ring + s * stage_bytes;
                unsigned char *sb = sa + 4 * kTwBox;
                mbar_expect_tx(&full[s], bytes);
                for (int a = 0; a < na; ++a) {
                    const int m = m0 + a * kTcK;
                    const int t = m / p.Cin, c0 = m - t * p.Cin;
                    tma_load_4d(sa + a * kTwBox, &mapX, c0, x0 + t % 3 - 1,
                                y0 + t / 3 - 1, img, &full[s]);
                }
                for (int b = 0; b < nb; ++b)
                    tma_load_4d(sb + b * kTwBox, &mapG, n0 + b * kTcK, x0, y0,
                                img, &full[s]);
                ++issued;
            }
            const int j = it - (kTwStages - 1);
            if (j >= 0) {
                const int s = j % kTwStages;
                ok = mbar_wait(&full[s], (j / kTwStages) & 1, TC_FULL_TIMEOUT);
                if (!ok) break;
                ++consumed;
                tc_fence_after();
                const unsigned char *sa = ring + s * stage_bytes;
                const unsigned char *sb = sa + 4 * kTwBox;
#pragma unroll
                for (int kk = 0; kk < kTcM / 16; ++kk)
                    tc_mma(tmem, sw64_desc_mn(sa + 1024 * kk, kTwBox),
                           sw64_desc_mn(sb + 1024 * kk, kTwBox), idesc,
                           (j > 0 || kk > 0) ? 1u : 0u);
                tc_commit(&empty[s]);
            }
        }
        if (!ok) {
            *abort_flag = 1;
            for (int j = consumed; j < issued; ++j)
                mbar_wait(&full[j % kTwStages], (j / kTwStages) & 1,
                          TC_FULL_TIMEOUT);
        }
        tc_commit(done);
    }
    __syncwarp();
    const bool done_ok = mbar_wait(done, 0, TC_DONE_TIMEOUT);
    tc_fence_after();
    __syncthreads();
    const int row = warp * 32 + lane;
    const int m = m0 + row;
    if (done_ok && !*abort_flag && m < p.M9) {
        const unsigned lane_base = tmem + ((unsigned)(warp * 32) << 16);
        float *dst = p.part + ((size_t)z * p.M9 + m) * p.Cout + n0;
        for (int c = 0; c < p.BN; c += 16) {
            float v[16];
            tmem_ld16(lane_base + (unsigned)c, v);
            float4 *d4 = reinterpret_cast<float4 *>(dst + c);
#pragma unroll
            for (int i = 0; i < 4; ++i)
                d4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2],
                                    v[4 * i + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile(
            "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
            "r"(ncols_tmem)
            : "memory");
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t,
                                 void *, const cuuint64_t *, const cuuint64_t *,
                                 const cuuint32_t *, const cuuint32_t *,
                                 CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion,
                                 CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p,
                                             12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

}  // namespace

bool conv_tc_supported(const TcConv &c) {
    if (c.mode != 0 && c.mode != 1) return false;
    if (c.Ck % kTcK || c.Ncols % 16 || c.Ncols < 16) return false;
    if (c.W >= kTcM ? c.W % kTcM != 0 : (kTcM % c.W != 0 || c.H % (kTcM / c.W)))
        return false;
    if (((long)c.H * c.W) % kTcM) return false;
    if ((uintptr_t)c.act % 16 || (uintptr_t)c.wk % 16 || (uintptr_t)c.out % 16)
        return false;
    return encode_fn() != nullptr;
}

cudaError_t conv_tc_launch(const TcConv &c, cudaStream_t stream) {
    EncodeTiled enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    TcParams p;
    memset(&p, 0, sizeof p);
    p.mode = c.mode;
    p.N = c.N; p.H = c.H; p.W = c.W; p.Ck = c.Ck; p.Ncols = c.Ncols;
    p.BN = c.Ncols <= 128 ? c.Ncols : (c.Ncols % 128 == 0 ? 128 : 0);
    if (!p.BN) {
        // N above 128 split into equal tiles of at most 128, multiples of 16
        for (int t = 2; t <= c.Ncols / 16 && !p.BN; ++t)
            if (c.Ncols % t == 0 && (c.Ncols / t) % 16 == 0 &&
                c.Ncols / t <= 128)
                p.BN = c.Ncols / t;
        if (!p.BN) return cudaErrorNotSupported;
    }
    p.bw = c.W >= kTcM ? kTcM : c.W;
    p.bh = kTcM / p.bw;
    p.ktiles = 9 * c.Ck / kTcK;
    p.bias = c.bias;
    p.out = c.out;

    CUtensorMap mapA, mapB;
    {
        const cuuint64_t dims[4] = {(cuuint64_t)c.Ck, (cuuint64_t)c.W,
                                    (cuuint64_t)c.H, (cuuint64_t)c.N};
        const cuuint64_t strides[3] = {(cuuint64_t)c.Ck * 2,
                                       (cuuint64_t)c.W * c.Ck * 2,
                                       (cuuint64_t)c.H * c.W * c.Ck * 2};
        const cuuint32_t box[4] = {kTcK, (cuuint32_t)p.bw, (cuuint32_t)p.bh, 1};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        if (enc(&mapA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                const_cast<void *>(c.act), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    {
        const cuuint64_t dims[2] = {(cuuint64_t)9 * c.Ck, (cuuint64_t)c.Ncols};
        const cuuint64_t strides[1] = {(cuuint64_t)9 * c.Ck * 2};
        const cuuint32_t box[2] = {kTcK, (cuuint32_t)p.BN};
        const cuuint32_t estr[2] = {1, 1};
        if (enc(&mapB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                const_cast<void *>(c.wk), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    const size_t smem = tc_smem_bytes(p.BN);
    cudaError_t e = cudaFuncSetAttribute(
        conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long tiles = (long)c.N * c.H * c.W / kTcM;
    dim3 grid((unsigned)tiles, (unsigned)(c.Ncols / p.BN), 1);
    conv_tc_kernel<<<grid, kTcThreads, smem, stream>>>(mapA, mapB, p);
    count_launch(1);
    return cudaGetLastError();
}

bool conv_tc_wgrad_supported(const TcWgrad &w) {
    if (w.Cin % kTcK || w.Cout % kTcK) return false;
    if (w.W >= kTcM ? w.W % kTcM != 0 : (kTcM % w.W != 0 || w.H % (kTcM / w.W)))
        return false;
    if (((long)w.H * w.W) % kTcM) return false;
    if ((uintptr_t)w.X % 16 || (uintptr_t)w.G % 16 || (uintptr_t)w.part % 16)
        return false;
    return encode_fn() != nullptr;
}

cudaError_t conv_tc_wgrad_launch(const TcWgrad &w, int *splits,
                                 cudaStream_t stream) {
    EncodeTiled enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    TwParams p;
    memset(&p, 0, sizeof p);
    p.H = w.H; p.W = w.W; p.Cin = w.Cin; p.Cout = w.Cout;
    p.M9 = 9 * w.Cin;
    p.BN = w.Cout <= 128 ? w.Cout : (w.Cout % 128 == 0 ? 128 : 64);
    if (w.Cout % p.BN) p.BN = 32;
    p.bw = w.W >= kTcM ? kTcM : w.W;
    p.bh = kTcM / p.bw;
    p.part = w.part;
    p.ptiles = (int)((long)w.N * w.H * w.W / kTcM);
    const int mt = (p.M9 + kTcM - 1) / kTcM, nt = w.Cout / p.BN;
    // about two CTAs per SM, bounded by the partial buffer and the tiles
    int sp = (2 * 152 + mt * nt - 1) / (mt * nt);
    const long cap = (long)(w.part_floats / ((size_t)p.M9 * w.Cout));
    if (sp > cap) sp = (int)cap;
    if (sp > p.ptiles) sp = p.ptiles;
    if (sp < 1) return cudaErrorInvalidValue;
    p.tps = (p.ptiles + sp - 1) / sp;
    const int z = (p.ptiles + p.tps - 1) / p.tps;

    CUtensorMap mapX, mapG;
    auto act_map = [&](CUtensorMap *map, const void *ptr, int C) {
        const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)w.W,
                                    (cuuint64_t)w.H, (cuuint64_t)w.N};
        const cuuint64_t strides[3] = {(cuuint64_t)C * 2,
                                       (cuuint64_t)w.W * C * 2,
                                       (cuuint64_t)w.H * w.W * C * 2};
        const cuuint32_t box[4] = {kTcK, (cuuint32_t)p.bw, (cuuint32_t)p.bh, 1};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                   const_cast<void *>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    if (!act_map(&mapX, w.X, w.Cin) || !act_map(&mapG, w.G, w.Cout))
        return cudaErrorInvalidValue;
    const size_t smem = tw_smem_bytes(p.BN);
    cudaError_t e = cudaFuncSetAttribute(
        conv_tc_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)mt, (unsigned)nt, (unsigned)z);
    conv_tc_wgrad_kernel<<<grid, kTcThreads, smem, stream>>>(mapX, mapG, p);
    count_launch(1);
    *splits = z;
    return cudaGetLastError();
}

}  // namespace dyfox

extern "C" int dyfox_unet_tc_error(int *code, int clear) {
    dyfox::set_error("");
    if (!code) {
        dyfox::set_error("NULL argument");
        return DYFOX_EINVAL;
    }
    cudaError_t e = cudaMemcpyFromSymbol(code, dyfox::g_tc_error, sizeof(int));
    if (e == cudaSuccess && clear) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(dyfox::g_tc_error, &zero, sizeof(int));
    }
    return dyfox::cuda_status(e, "dyfox_unet_tc_error");
}
