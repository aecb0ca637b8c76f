// The compensated single-precision Laue march of laue_march.cuh with two
// deviation parameters per thread, in packed f32x2 arithmetic (sm_100 and
// later: one FFMA2 / FADD2 / FMUL2 issues two single-precision operations).
//
// The march is issue-bound: an FP32 update costs ~28 floating-point
// operations per voxel-step and as many again in shuffles, shared-memory
// traffic, moves and loop control.  Both deviation parameters of a pair see
// the same e^{iH(k, x)}, so every operation of the update pairs up
// elementwise (x: first angle, y: second) with no swizzle: the coupling
// products take the pair's kappa constants against the broadcast (cos, cos)
// and (sin, sin) of the column.  The per-step overhead is paid once per two
// angles.  Operation order and rounding are those of the scalar kernel
// (explicit FMAs, Fast2Sum with the subtractions as FMAs by -1), so both
// produce the same bits.
//
// Layout: one CTA per (grid row, group of P angle pairs); each pair owns WA
// warps, lane L holds columns [L*CPL, (L+1)*CPL) of both angles.  Sources:
// the fused Volterra phase (HT_SEG / HT_SEG64: e^{iH} produced once per CTA
// per step into a double-buffered row of (c, c, s, s) float4s) or the
// staged e^{iH} rows (HT_GENERIC with a float2 HS_CS32 source copied by
// cp.async into three stages).
#pragma once
#include "laue_march.cuh"

namespace dyfox {

// Coupling constants of one step for an angle pair (x: first angle, y:
// second), with the negations the products need: 64 bytes, 4 float4.
struct KPair {
    float2 k12r, k12i, nk12i, nk12r, k21r, k21i, nk21r, nk21i;
};
static_assert(sizeof(KPair) == 64, "KPair is four float4");

__device__ __forceinline__ KPair ldg_kpair(const float4 *p) {
    KPair k;
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2),
                 d = __ldg(p + 3);
    k.k12r = make_float2(a.x, a.y); k.k12i = make_float2(a.z, a.w);
    k.nk12i = make_float2(b.x, b.y); k.nk12r = make_float2(b.z, b.w);
    k.k21r = make_float2(c.x, c.y); k.k21i = make_float2(c.z, c.w);
    k.nk21r = make_float2(d.x, d.y); k.nk21i = make_float2(d.z, d.w);
    return k;
}

__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
    return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
    return __fmul2_rn(a, b);
}

// Fast2Sum on pairs: s = a + b, err = b - (s - a), each subtraction an FMA
// by -1 (one rounding, as the scalar subtraction).
__device__ __forceinline__ float2 fast_two_sum2(float2 a, float2 b,
                                                float2 &err) {
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 s = __fadd2_rn(a, b);
    const float2 z = f2fma(a, m1, s);
    err = f2fma(z, m1, b);
    return s;
}

__device__ __forceinline__ float2 shfl_down2(float2 v) {
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, 1),
                       __shfl_down_sync(0xffffffffu, v.y, 1));
}
__device__ __forceinline__ float2 shfl_up2(float2 v) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, 1),
                       __shfl_up_sync(0xffffffffu, v.y, 1));
}

// Shared-memory plan of the pair kernel (bytes), shared with the host.
struct PairSmem {
    size_t cs, raw, raw_stage, bnd, segf, hc, total;
};

__host__ __device__ inline PairSmem pair_smem(int CPL, int WA, int P,
                                              int n_seg, bool fused) {
    PairSmem m;
    const size_t ncols = (size_t)32 * WA * CPL;
    const int nwarps = WA * P;
    size_t off = 0;
    m.cs = off;
    if (fused) off += 2 * ncols * sizeof(float4);
    m.raw = off;
    m.raw_stage = fused ? 0 : ((ncols * sizeof(float2) + 15) & ~(size_t)15);
    off += 3 * m.raw_stage;
    m.bnd = off;
    off += (size_t)2 * nwarps * 4 * sizeof(float4);
    m.segf = off;
    if (fused) off += (size_t)n_seg * sizeof(SegF);
    off = (off + 15) & ~(size_t)15;
    m.hc = off;
    off += sizeof(double);
    m.total = off;
    return m;
}

// The march of one (row, pair group): row a.row0 + row_blk, angle pairs
// [grp * P, grp * P + P) with P = a.A; pair q holds angles 2q and 2q + 1
// (the last pair of an odd count repeats its angle and writes it once).
template <int CPL, int HT>
__device__ __forceinline__ void march_pair_block(const MarchArgs &a,
                                                 int row_blk, int grp,
                                                 unsigned char *smem) {
    constexpr bool kFused = HT != HT_GENERIC;
    const int WA = a.WA;
    const int nthreads = blockDim.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nwarps = nthreads >> 5;
    const int g = warp / WA, wa = warp - g * WA;
    const int L = wa * 32 + lane;
    const int iy = a.row0 + row_blk;
    const int n_pairs = (a.n_e + 1) >> 1;
    const int pr_raw = grp * a.A + g;
    const int pr = pr_raw < n_pairs ? pr_raw : n_pairs - 1;
    const int Nx = a.Nx, nsteps = a.Nz - 1, ncols = a.ncols;
    const PairSmem plan = pair_smem(CPL, WA, a.A, a.n_seg, kFused);
    float4 *cs = reinterpret_cast<float4 *>(smem + plan.cs);
    unsigned char *raw = smem + plan.raw;
    float4 *bnd = reinterpret_cast<float4 *>(smem + plan.bnd);
    SegF *segf = reinterpret_cast<SegF *>(smem + plan.segf);
    double *hc_sm = reinterpret_cast<double *>(smem + plan.hc);
    const float4 zero4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);

    // ---------------------------------------------------------- prologue
    if constexpr (kFused) {
        if (tid == 0) *hc_sm = sum_hconst(a.segs, a.n_seg);
        for (int s = tid; s < a.n_seg; s += nthreads)
            segf[s] = seg_f32(a.segs + (size_t)s * DYFOX_SEG_STRIDE);
        for (int x = Nx + tid; x < ncols; x += nthreads) {
            cs[x] = zero4;
            cs[ncols + x] = zero4;
        }
    } else {
        // Columns beyond Nx of every stage read as zero coupling.
        for (int st = 0; st < 3; ++st) {
            float2 *row = reinterpret_cast<float2 *>(raw + (size_t)st * plan.raw_stage);
            for (int x = Nx + tid; x < ncols; x += nthreads)
                row[x] = make_float2(0.0f, 0.0f);
        }
    }
    __syncthreads();
    double hconst = 0.0;
    float hcr = 0.0f;
    int nmine = 0;
    if constexpr (kFused) {
        hconst = *hc_sm;
        hcr = reduce_2pi(hconst);
        nmine = tid < Nx ? (Nx - 1 - tid) / nthreads + 1 : 0;
        nmine = nmine < CPL ? nmine : CPL;
    }

    // Staged source: the e^{iH} row of step kk into stage kk % 3, two steps
    // ahead; every thread commits one group per call, copy or not.
    const unsigned char *raw_src =
        static_cast<const unsigned char *>(a.csgrid);
    const size_t raw_row = (size_t)row_blk * nsteps;
    const int chunks = (Nx * (int)sizeof(float2)) >> 4;
    auto stage_issue = [&](int kk) {
        if (kk < nsteps) {
            const unsigned char *src =
                raw_src + (raw_row + kk) * (size_t)Nx * sizeof(float2);
            unsigned char *dst = raw + (size_t)(kk % 3) * plan.raw_stage;
            for (int c = tid; c < chunks; c += nthreads)
                cp_async16(dst + 16 * c, src + 16 * c);
        }
        cp_async_commit();
    };

    // Fused source: (c, c, s, s) of this thread's columns into buffer buf.
    auto produce = [&](int kk, int buf) {
        float4 *dst = cs + (size_t)buf * ncols;
        const float4 *pv = a.piv + ((size_t)row_blk * nsteps + kk) * a.n_seg;
        if (a.n_seg == 1) {
            const SegF f = segf[0];
            const float4 p0 = __ldg(pv);
#pragma unroll
            for (int i = 0; i < CPL; ++i) {
                if (i < nmine) {
                    const int x = tid + i * nthreads;
                    const float2 v = seg_phase_one<HT>(f, p0, x, hcr, hconst);
                    dst[x] = make_float4(v.x, v.x, v.y, v.y);
                }
            }
            return;
        }
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            if (i < nmine) {
                const int x = tid + i * nthreads;
                const float2 v = seg_phase<HT>(segf, pv, a.n_seg, x, hcr, hconst);
                dst[x] = make_float4(v.x, v.x, v.y, v.y);
            }
        }
    };

    // Initial state: A = input beam (both angles), B = 0.
    float2 Ar[CPL], Ai[CPL], Br[CPL], Bi[CPL];
    float2 Alr[CPL], Ali[CPL], Blr[CPL], Bli[CPL];
    const float2 z2 = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int x = L * CPL + j;
        const float b = x < Nx ? (float)beam_profile(x, Nx, a.dx, a.sheet_hw) : 0.0f;
        Ar[j] = make_float2(b, b);
        Ai[j] = z2; Br[j] = z2; Bi[j] = z2;
        Alr[j] = z2; Ali[j] = z2; Blr[j] = z2; Bli[j] = z2;
    }
    if constexpr (kFused) {
        produce(0, 0);
    } else {
        stage_issue(0);
        stage_issue(1);
        cp_async_wait<1>();
    }
    // Boundary slots per warp and parity: 0 = A[0], 1 = A_err[0] (left
    // edge, read by the warp to the left), 2 = B[CPL-1], 3 = B_err[CPL-1]
    // (right edge, read by the warp to the right); (re.x, re.y, im.x, im.y).
    auto put_bnd = [&](int par) {
        float4 *b = bnd + (size_t)(par * nwarps + warp) * 4;
        if (lane == 0) {
            b[0] = make_float4(Ar[0].x, Ar[0].y, Ai[0].x, Ai[0].y);
            b[1] = make_float4(Alr[0].x, Alr[0].y, Ali[0].x, Ali[0].y);
        }
        if (lane == 31) {
            b[2] = make_float4(Br[CPL - 1].x, Br[CPL - 1].y, Bi[CPL - 1].x,
                               Bi[CPL - 1].y);
            b[3] = make_float4(Blr[CPL - 1].x, Blr[CPL - 1].y,
                               Bli[CPL - 1].x, Bli[CPL - 1].y);
        }
    };
    put_bnd(0);
    __syncthreads();

    const float4 *kp = a.kpair + (size_t)pr * nsteps * 4;
    // ------------------------------------------------------------ march
    for (int k = 0; k < nsteps; ++k) {
        const int p = k & 1;
        const KPair kc = ldg_kpair(kp + (size_t)k * 4);
        if constexpr (kFused) {
            if (k + 1 < nsteps) produce(k + 1, p ^ 1);
        } else {
            stage_issue(k + 2);
        }

        // Neighbour values of the previous state.
        float2 ainr = shfl_down2(Ar[0]), aini = shfl_down2(Ai[0]);
        float2 ainlr = shfl_down2(Alr[0]), ainli = shfl_down2(Ali[0]);
        float2 binr = shfl_up2(Br[CPL - 1]), bini = shfl_up2(Bi[CPL - 1]);
        float2 binlr = shfl_up2(Blr[CPL - 1]), binli = shfl_up2(Bli[CPL - 1]);
        if (lane == 31) {
            if (wa + 1 < WA) {
                const float4 *b = bnd + (size_t)(p * nwarps + warp + 1) * 4;
                const float4 t = b[0], u = b[1];
                ainr = make_float2(t.x, t.y); aini = make_float2(t.z, t.w);
                ainlr = make_float2(u.x, u.y); ainli = make_float2(u.z, u.w);
            } else {
                ainr = z2; aini = z2; ainlr = z2; ainli = z2;
            }
        }
        if (lane == 0) {
            if (wa > 0) {
                const float4 *b = bnd + (size_t)(p * nwarps + warp - 1) * 4;
                const float4 t = b[2], u = b[3];
                binr = make_float2(t.x, t.y); bini = make_float2(t.z, t.w);
                binlr = make_float2(u.x, u.y); binli = make_float2(u.z, u.w);
            } else {
                binr = z2; bini = z2; binlr = z2; binli = z2;
            }
        }
        const float4 *src4 = cs + (size_t)p * ncols + L * CPL;
        const float2 *src2 = reinterpret_cast<const float2 *>(
                                 raw + (size_t)(k % 3) * plan.raw_stage) + L * CPL;
        float2 pbr = binr, pbi = bini, pblr = binlr, pbli = binli;
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            float2 ER, EI;
            if constexpr (kFused) {
                const float4 e = src4[j];
                ER = make_float2(e.x, e.y);
                EI = make_float2(e.z, e.w);
            } else {
                const float2 e = src2[j];
                ER = make_float2(e.x, e.x);
                EI = make_float2(e.y, e.y);
            }
            const float2 ar = j + 1 < CPL ? Ar[j + 1] : ainr;
            const float2 ai = j + 1 < CPL ? Ai[j + 1] : aini;
            const float2 alr = j + 1 < CPL ? Alr[j + 1] : ainlr;
            const float2 ali = j + 1 < CPL ? Ali[j + 1] : ainli;
            const float2 br = pbr, bi = pbi, blr = pblr, bli = pbli;
            pbr = Br[j]; pbi = Bi[j]; pblr = Blr[j]; pbli = Bli[j];
            const float2 m12r = f2fma(kc.k12r, ER, f2mul(kc.nk12i, EI));
            const float2 m12i = f2fma(kc.k12r, EI, f2mul(kc.k12i, ER));
            const float2 nm12i = f2fma(kc.nk12r, EI, f2mul(kc.nk12i, ER));
            const float2 m21r = f2fma(kc.k21r, ER, f2mul(kc.k21i, EI));
            const float2 m21i = f2fma(kc.k21i, ER, f2mul(kc.nk21r, EI));
            const float2 nm21i = f2fma(kc.nk21i, ER, f2mul(kc.k21r, EI));
            const float2 tr = f2fma(m12r, br, f2fma(nm12i, bi, alr));
            const float2 ti = f2fma(m12r, bi, f2fma(m12i, br, ali));
            const float2 ur = f2fma(m21r, ar, f2fma(nm21i, ai, blr));
            const float2 ui = f2fma(m21r, ai, f2fma(m21i, ar, bli));
            Ar[j] = fast_two_sum2(ar, tr, Alr[j]);
            Ai[j] = fast_two_sum2(ai, ti, Ali[j]);
            Br[j] = fast_two_sum2(br, ur, Blr[j]);
            Bi[j] = fast_two_sum2(bi, ui, Bli[j]);
        }
        put_bnd(p ^ 1);
        // The stage of step k + 1 is complete and, after the barrier,
        // visible to every thread.
        if constexpr (!kFused) cp_async_wait<1>();
        __syncthreads();
    }
    if constexpr (!kFused) cp_async_wait<0>();

    // ---------------------------------------------------------- output
    if (pr_raw >= n_pairs) return;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int ie = 2 * pr + t;
        if (ie >= a.n_e) break;
        const double2 S = __ldg(a.scale + ie);
        float2 *out = reinterpret_cast<float2 *>(a.out) + ((size_t)ie * a.Ny + iy) * Nx;
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const int x = L * CPL + j;
            if (x < Nx) {
                const double br = (double)(t ? Br[j].y : Br[j].x) +
                                  (double)(t ? Blr[j].y : Blr[j].x);
                const double bi = (double)(t ? Bi[j].y : Bi[j].x) +
                                  (double)(t ? Bli[j].y : Bli[j].x);
                out[x] = make_float2((float)(S.x * br - S.y * bi),
                                     (float)(S.x * bi + S.y * br));
            }
        }
    }
}

template <int CPL, int HT>
__global__ void laue_pair_kernel(const MarchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int row_blk = blockIdx.x / a.n_groups;
    march_pair_block<CPL, HT>(a, row_blk, blockIdx.x - row_blk * a.n_groups,
                              smem);
}

template <int CPL, int HT>
cudaError_t launch_pair(const MarchArgs &a, int grid, int block, size_t smem,
                        cudaStream_t stream) {
    auto *k = laue_pair_kernel<CPL, HT>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k<<<grid, block, smem, stream>>>(a);
    count_launch(1);
    return cudaGetLastError();
}

template <int CPL, int HT>
cudaError_t attr_pair(cudaFuncAttributes *attr) {
    return cudaFuncGetAttributes(attr, laue_pair_kernel<CPL, HT>);
}

// Defined in laue_f32p.cu; {nullptr, nullptr} for a missing instantiation.
MarchEntry march_entry_f32_pair(int cpl, int ht);
constexpr int kCplPair[] = {3, 5, 7};
constexpr int kNumCplPair = 3;

}  // namespace dyfox
