// Takagi-Taupin depth march of the Laue geometry (DYFOX laue/kernels.py
// 48-352), register-resident, for exact advection (shift_px == 1).
//
// The reference update per depth step k (kernels.py:95-141) is
//   D0'(x) = M11 D0(x+1) + M12(x) Dg(x-1)
//   Dg'(x) = M21(x) D0(x+1) + M22 Dg(x-1)
// with M = e_p P, P11 = cg - i(a/2)sg, P22 = cg + i(a/2)sg = rho e^{i th},
// M12 = e_p sg sigma_hbar e^{+iH(k,x)}, M21 = e_p sg sigma_h e^{-iH(k,x)},
// zero fill beyond both edges.  The march here runs in the interaction
// picture D0_k = (e_p rho)^k e^{-ik th} A_k, Dg_k = (e_p rho)^k e^{ik th} B_k:
//   A'(x) = A(x+1) + kappa12_k e^{+iH} B(x-1)
//   B'(x) = B(x-1) + kappa21_k e^{-iH} A(x+1)
// kappa12_k = (sg/rho) sigma_hbar e^{i(2k+1)th},
// kappa21_k = (sg/rho) sigma_h e^{-i(2k+1)th},
// and D_g(t) = M22^(Nz-1) B_(Nz-1).  Mathematically identical; the diagonal
// becomes an exact shift (no rounding drift in single precision) and a step
// costs 16 real FMA-class operations per column instead of 24.
//
// Work layout: one CTA per (grid row, group of `A` deviation parameters).
// Each angle owns WA warps; lane L of an angle holds the CPL contiguous
// columns [L*CPL, (L+1)*CPL) of A and B in registers.  The one-column shift
// moves in registers, across lanes by warp shuffle and across warps through
// a shared-memory boundary slot rotated over three buffers; one
// __syncthreads per step.
// e^{iH(k,.)} for the row is produced once per CTA per step into a
// double-buffered shared-memory row (all angles of the CTA share it) while
// the previous step is consumed.
#pragma once
#include "common.cuh"
#include "volterra.cuh"

namespace dyfox {

enum HSrc { HS_NONE = 0, HS_GRID64 = 1, HS_GRID32 = 2, HS_CS32 = 3,
            HS_SEG = 4, HS_ANALYTIC = 5, HS_CS64 = 6 };
// H source compiled into a march: cheap sources chosen at run time, or the
// Volterra field of the segments evaluated per voxel.  In single precision
// HT_SEG sums the segment terms in float-float (two-sum) and reduces mod
// 2 pi in single precision; HT_SEG64 sums and reduces in double.  In double
// precision HT_SEG is the reference-order double evaluation.
// HT_STAGED is the march over e^{iH} staged in the march's own precision
// (HS_CS32 single, HS_CS64 double), copied two steps ahead into a shared
// ring: the staging mode is fixed at compile time, so the step carries no
// branch on the source.
enum HTemplate { HT_GENERIC = 0, HT_SEG = 1, HT_SEG64 = 2, HT_STAGED = 3 };

// A ring index known at compile time (the unrolled staged march).
template <int N>
struct RingIdx {
    __host__ __device__ constexpr operator int() const { return N; }
};

// Interaction-picture coupling constants of one (angle, step).
struct Kappa {
    double2 k12, k21;
};

__device__ __forceinline__ Kappa ldg_kappa(const Kappa *p) {
    Kappa k;
    k.k12 = __ldg(&p->k12);
    k.k21 = __ldg(&p->k21);
    return k;
}

struct MarchArgs {
    int Nx, Ny, Nz, n_e;
    int WA, A, ncols, n_groups;
    int row0, n_rows;
    double dx, dz, sheet_hw;
    int hsrc;
    const void *hgrid;          // GRID64 / GRID32: (Ny, Nz, Nx)
    const void *csgrid;         // CS32 / CS64: staged e^{iH} as float2 /
                                // double2, (n_rows, Nz - 1, Nx), row-relative
    const double *segs;         // SEG: segment table
    const float4 *piv;          // SEG single: pivots (n_rows, Nz - 1, n_seg)
    int n_seg;
    VolterraConsts vc;
    double an[12];              // ANALYTIC
    const Kappa *kappa;         // (n_e, Nz - 1): kappa12, kappa21
    const float4 *kappa32;      // the same, rounded to float (FP32 march)
    const float4 *kpair;        // pair march: (n_e + 1) / 2 x (Nz - 1) KPair
    const double2 *scale;       // (n_e): M22^(Nz-1)
    void *out;                  // (n_e, Ny, Nx) complex (R2)
    int stage;                  // StageMode of a GENERIC source
    int raw_elem;               // bytes per column of a staged raw row
    int *err;                   // set to 1 when a bounded wait ran out
                                // (NULL: not recorded)
};

// Input beam D0(z=0) at column x (kernels.py:77-88), in double.
__device__ __forceinline__ double beam_profile(int x, int Nx, double dx,
                                               double sheet_hw) {
    double x_pos = (x - Nx / 2) * dx;
    return sheet_hw > 0.0 ? (fabs(x_pos) < sheet_hw ? 1.0 : 0.0)
                          : exp(-x_pos * x_pos / (2.0 * sheet_hw * sheet_hw));
}

// Closed-form H(y, z_k) of a single line along x (kernels.py:216-228).
__device__ __forceinline__ double analytic_h(const double *an, double y_pix,
                                             int k, double dz) {
    double dy = y_pix - an[0];
    double onu = 1.0 - an[10];
    double c1 = an[9] / (2.0 * kPi);
    double dzv = k * dz - an[1];
    double d1 = dy * an[2] + dzv * an[3];
    double d2 = dy * an[4] + dzv * an[5];
    double r2 = d1 * d1 + d2 * d2;
    double r2c = (r2 > an[11]) ? r2 : an[11];
    double H = an[6] * atan2(d2, d1);
    if (an[9] > 0.0) {
        double nu = an[10];
        double ux = c1 * d1 * d2 / (2.0 * onu * r2c);
        double uy = -c1 * ((1.0 - 2.0 * nu) / (4.0 * onu) * log(r2c)
                           + (d1 * d1 - d2 * d2) / (4.0 * onu * r2c));
        H += 2.0 * kPi * (an[7] * ux + an[8] * uy);
    }
    return H;
}

template <typename R> struct CS;
template <> struct CS<double> {
    static __device__ __forceinline__ double2 of_f64(double h) {
        double s, c;
        sincos(h, &s, &c);
        return make_double2(c, s);
    }
    static __device__ __forceinline__ double2 of_f32(float h) {
        return of_f64((double)h);
    }
    static __device__ __forceinline__ double2 of_cs(float2 v) {
        return make_double2(v.x, v.y);
    }
    static __device__ __forceinline__ double2 of_cs(double2 v) { return v; }
};
template <> struct CS<float> {
    static __device__ __forceinline__ float2 of_f64(double h) {
        float s, c;
        __sincosf(reduce_2pi(h), &s, &c);     // argument within [-pi, pi]
        return make_float2(c, s);
    }
    static __device__ __forceinline__ float2 of_f32(float h) {
        float s, c;
        sincosf(h, &s, &c);
        return make_float2(c, s);
    }
    static __device__ __forceinline__ float2 of_cs(float2 v) { return v; }
    static __device__ __forceinline__ float2 of_cs(double2 v) {
        return make_float2((float)v.x, (float)v.y);
    }
};

// Knuth's error-free sum: s + err == a + b exactly (round to nearest).
template <typename R>
__device__ __forceinline__ R two_sum(R a, R b, R &err) {
    R s = a + b;
    R bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}

// Dekker's Fast2Sum: s + err == a + b exactly when |a| >= |b| (round to
// nearest).  In the march a is an amplitude and b its increment, at most
// |kappa| ~ 0.02 of the other amplitude, so the sum is exact except near a
// zero of the amplitude, where err is still b - (s - a) rounded: a
// compensation no worse than none, at 3 operations instead of 6.
template <typename R>
__device__ __forceinline__ R fast_two_sum(R a, R b, R &err) {
    R s = a + b;
    err = b - (s - a);
    return s;
}
constexpr bool kFastCompensation = true;

__device__ __forceinline__ double fmaR(double a, double b, double c) {
    return fma(a, b, c);
}
__device__ __forceinline__ float fmaR(float a, float b, float c) {
    return fmaf(a, b, c);
}

// How the e^{iH} row of each depth step reaches shared memory.
//   ST_COMPUTE  the producer evaluates every column (Volterra field,
//               closed form, perfect crystal, or a grid that cannot be
//               staged asynchronously);
//   ST_DIRECT   staged e^{iH} rows of the march's own precision are copied
//               two steps ahead into three stages and read in place by the
//               update (the staged march: one thread's bulk copy a row;
//               the generic march: every thread's cp.async);
//   ST_CONVERT  raw rows (H grids, or e^{iH} of the other precision) are
//               copied with cp.async and turned into e^{iH} by the
//               producer.
enum StageMode { ST_COMPUTE = 0, ST_DIRECT = 1, ST_CONVERT = 2 };

// Shared-memory plan of the march kernel (bytes), shared with the host.
// Rows use the natural column layout: element x of a row is column x; lane
// L reads x = L * CPL + j (odd CPL keeps 8-byte reads conflict-free).
struct MarchSmem {
    size_t cs, raw, raw_stage, bnd, an, segf, hc, bars, total;
};

template <typename R>
__host__ __device__ inline MarchSmem march_smem(int CPL, int WA, int A,
                                                int Nz, int hsrc, int n_seg,
                                                bool comp, int stage,
                                                int raw_elem) {
    using R2 = typename RT<R>::R2;
    MarchSmem m;
    const size_t ncols = (size_t)32 * WA * CPL;
    const int nwarps = WA * A;
    size_t off = 0;
    m.cs = off;
    if (stage != ST_DIRECT) off += 2 * ncols * sizeof(R2);
    off = (off + 15) & ~(size_t)15;
    m.raw = off;
    m.raw_stage = stage != ST_COMPUTE
        ? ((ncols * raw_elem + 15) & ~(size_t)15) : 0;
    off += 3 * m.raw_stage;
    m.bnd = off;
    // three ring stages of slots a warp, and one slot of zeros (the
    // missing neighbour of a row's first and last warp)
    off += (size_t)(3 * nwarps + 1) * (comp ? 4 : 2) * sizeof(R2);
    off = (off + 15) & ~(size_t)15;
    m.an = off;
    if (hsrc == HS_ANALYTIC) off += (size_t)Nz * sizeof(R2);
    off = (off + 15) & ~(size_t)15;
    m.segf = off;
    if (hsrc == HS_SEG && sizeof(R) == 4) off += (size_t)n_seg * sizeof(SegF);
    off = (off + 15) & ~(size_t)15;
    m.hc = off;
    off += sizeof(double);
    // three mbarriers of the bulk row copies (direct staging)
    off = (off + 7) & ~(size_t)7;
    m.bars = off;
    if (stage == ST_DIRECT) off += 3 * sizeof(unsigned long long);
    m.total = off;
    return m;
}

// One thread's bulk copy of a staged row (cp.async.bulk, completion counted
// in bytes on an mbarrier) and the waits on it.  Both addresses 16-byte
// aligned, bytes a multiple of 16 (the direct staging guarantees both).
__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void row_bar_init(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void row_bar_inval(unsigned long long *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_row(void *dst, const void *src,
                                         unsigned bytes,
                                         unsigned long long *bar) {
    // the generic-proxy reads of this stage (ordered by the barrier that
    // preceded) before the async-proxy write
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool row_bar_try(unsigned long long *bar,
                                            unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase `parity` of bar, at most about 2 s of the global
// timer; false when it gave up.
static __device__ __noinline__ bool row_bar_wait_slow(unsigned long long *bar,
                                               unsigned parity) {
    unsigned long long t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (unsigned it = 0;; ++it) {
        if (row_bar_try(bar, parity)) return true;
        if ((it & 255u) == 255u) {
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t - t0 > 2000000000ull) return false;
        }
    }
}
__device__ __forceinline__ bool row_bar_wait(unsigned long long *bar,
                                             unsigned parity) {
    return row_bar_try(bar, parity) || row_bar_wait_slow(bar, parity);
}

// Predicated shared-memory accesses of a boundary slot: only the lanes with
// p load (keeping their registers otherwise) or store, with no branch.
__device__ __forceinline__ void ld_shared_if(bool p, const float2 *a,
                                             float &x, float &y) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n"
        " @q ld.shared.v2.f32 {%0, %1}, [%3];\n}\n"
        : "+f"(x), "+f"(y)
        : "r"((unsigned)p), "r"(smem_addr(a))
        : "memory");
}
__device__ __forceinline__ void ld_shared_if(bool p, const double2 *a,
                                             double &x, double &y) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n"
        " @q ld.shared.v2.f64 {%0, %1}, [%3];\n}\n"
        : "+d"(x), "+d"(y)
        : "r"((unsigned)p), "r"(smem_addr(a))
        : "memory");
}
__device__ __forceinline__ void st_shared_if(bool p, float2 *a, float x,
                                             float y) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n"
        " @q st.shared.v2.f32 [%1], {%2, %3};\n}\n" ::"r"((unsigned)p),
        "r"(smem_addr(a)), "f"(x), "f"(y)
        : "memory");
}
__device__ __forceinline__ void st_shared_if(bool p, double2 *a, double x,
                                             double y) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n"
        " @q st.shared.v2.f64 [%1], {%2, %3};\n}\n" ::"r"((unsigned)p),
        "r"(smem_addr(a)), "d"(x), "d"(y)
        : "memory");
}

__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// e^{iH} (cos, sin) of column x in single precision from the segment
// constants and the row's pivots.  HT_SEG: float-float sum started at the
// reduced constant hcr, reduced mod 2 pi in float-float; HT_SEG64: the
// segment terms summed exactly (seg_sum64), added to the constant hconst
// and reduced in double.
template <int HT>
__device__ __forceinline__ float2 seg_phase_one(const SegF &f, float4 p0,
                                                int x, float hcr,
                                                double hconst) {
    const float h = h_seg_f32(f, p0, x);
    if constexpr (HT == HT_SEG) {
        float e;
        const float hi = two_sum(hcr, h, e);
        float sn, c;
        __sincosf(reduce_2pi_ff(hi, e), &sn, &c);
        return make_float2(c, sn);
    } else {
        return CS<float>::of_f64(seg_sum64(1, hconst, [&](int) { return h; }));
    }
}

template <int HT>
__device__ __forceinline__ float2 seg_phase(const SegF *segf,
                                            const float4 *pv, int n_seg,
                                            int x, float hcr, double hconst) {
    if constexpr (HT == HT_SEG) {
        float hi = hcr, lo = 0.0f;
        for (int s = 0; s < n_seg; ++s) {
            float e;
            hi = two_sum(hi, h_seg_f32(load_segf(segf + s), __ldg(pv + s), x),
                         e);
            lo += e;
        }
        float sn, c;
        __sincosf(reduce_2pi_ff(hi, lo), &sn, &c);
        return make_float2(c, sn);
    } else {
        return CS<float>::of_f64(seg_sum64(n_seg, hconst, [&](int s) {
            return h_seg_f32(load_segf(segf + s), __ldg(pv + s), x);
        }));
    }
}

// The march of one (row, angle group): row a.row0 + row_blk, deviation
// parameters [grp * A, grp * A + A).  Every thread of the CTA calls it; the
// CTA has 32 * WA * A threads or more (warps beyond WA * A idle).  smem: the
// dynamic shared memory of march_smem's plan.
template <typename R, int CPL, int HT, bool COMP>
__device__ __forceinline__ void march_block(const MarchArgs &a, int row_blk,
                                            int grp, unsigned char *smem) {
    using R2 = typename RT<R>::R2;
    const int WA = a.WA;
    const int nthreads = blockDim.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nwarps = nthreads >> 5;
    const int g = warp / WA, wa = warp - g * WA;
    const int L = wa * 32 + lane;
    const int iy = a.row0 + row_blk;
    const int ie_raw = grp * a.A + g;
    const int ie = ie_raw < a.n_e ? ie_raw : a.n_e - 1;
    const int Nx = a.Nx, Nz = a.Nz, nsteps = Nz - 1, ncols = a.ncols;
    constexpr bool kSingle = sizeof(R) == 4;
    constexpr bool kSeg = HT == HT_SEG || HT == HT_SEG64;
    constexpr bool kStaged = HT == HT_STAGED;
    const int hsrc = kSeg ? (int)HS_SEG
                     : kStaged ? (kSingle ? (int)HS_CS32 : (int)HS_CS64)
                               : a.hsrc;
    const int stage = kSeg ? (int)ST_COMPUTE
                      : kStaged ? (int)ST_DIRECT : a.stage;
    const int raw_elem = kStaged ? (int)sizeof(R2) : a.raw_elem;
    const MarchSmem plan = march_smem<R>(CPL, WA, a.A, Nz, hsrc, a.n_seg,
                                         COMP, stage, raw_elem);
    R2 *cs = reinterpret_cast<R2 *>(smem + plan.cs);
    unsigned char *raw = smem + plan.raw;
    R2 *bnd = reinterpret_cast<R2 *>(smem + plan.bnd);
    R2 *an_cs = reinterpret_cast<R2 *>(smem + plan.an);
    SegF *segf = reinterpret_cast<SegF *>(smem + plan.segf);
    double *hc_sm = reinterpret_cast<double *>(smem + plan.hc);
    unsigned long long *bars =
        reinterpret_cast<unsigned long long *>(smem + plan.bars);
    // staged rows arrive by one thread's bulk copy per step (an mbarrier a
    // ring stage) instead of every thread's cp.async
    constexpr bool kBulk = kStaged;
    bool bulk_ok = true;
    const int NB = COMP ? 4 : 2;
    const double y_pix = (iy - a.Ny / 2) * a.dx;

    // ---------------------------------------------------------- prologue
    if (kSeg && kSingle) {
        if (tid == 0) *hc_sm = sum_hconst(a.segs, a.n_seg);
        for (int s = tid; s < a.n_seg; s += nthreads)
            segf[s] = seg_f32(a.segs + (size_t)s * DYFOX_SEG_STRIDE);
    }
    if (HT == HT_GENERIC && hsrc == HS_ANALYTIC) {
        for (int k = tid; k < nsteps; k += nthreads)
            an_cs[k] = CS<R>::of_f64(analytic_h(a.an, y_pix, k, a.dz));
    }
    if (kBulk && tid == 0) {
        for (int st = 0; st < 3; ++st) row_bar_init(&bars[st]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < NB)                // the zero slot of the missing neighbours
        bnd[3 * nwarps * NB + tid] = R2{R(0), R(0)};
    if (stage == ST_DIRECT) {
        // Columns beyond Nx of every stage read as zero coupling.
        for (int st = 0; st < 3; ++st) {
            R2 *row = reinterpret_cast<R2 *>(raw + (size_t)st * plan.raw_stage);
            for (int x = Nx + tid; x < ncols; x += nthreads)
                row[x] = R2{R(0), R(0)};
        }
    }
    // Columns this thread evaluates the fused single-precision phase of:
    // x = tid + i nthreads, i < nmine, all below Nx (CPL nthreads >= ncols
    // bounds nmine by CPL).  The padding columns of both buffers are zeroed
    // once here.
    constexpr bool kFusedF32 = kSeg && kSingle;
    int nmine = 0;
    if constexpr (kFusedF32) {
        nmine = tid < Nx ? (Nx - 1 - tid) / nthreads + 1 : 0;
        nmine = nmine < CPL ? nmine : CPL;
        for (int x = Nx + tid; x < ncols; x += nthreads) {
            cs[x] = R2{R(0), R(0)};
            cs[ncols + x] = R2{R(0), R(0)};
        }
    }
    __syncthreads();
    // Sum over segments of the constant the single evaluator drops (double),
    // and that sum reduced mod 2 pi (start of the float-float sum).
    double hconst = 0.0;
    float hcr = 0.0f;
    if (kSeg && kSingle) {
        hconst = *hc_sm;
        hcr = reduce_2pi(hconst);
    }

    // Asynchronous copy of the raw row of step kk into stage kk % 3: the
    // staged march's thread 0 issues one bulk copy; otherwise every thread
    // copies its 16-byte chunks and commits one group per call, copy or
    // not.
    const unsigned char *raw_src = nullptr;
    size_t raw_row = 0;
    if (stage != ST_COMPUTE) {
        const bool grid = hsrc == HS_GRID64 || hsrc == HS_GRID32;
        raw_src = static_cast<const unsigned char *>(grid ? a.hgrid : a.csgrid);
        raw_row = grid ? (size_t)iy * Nz : (size_t)row_blk * nsteps;
    }
    const int chunks = (Nx * raw_elem) >> 4;
    // ring: the stage (kk % 3) of step kk, tracked by the caller.
    auto stage_issue = [&](int kk, int ring) {
        if constexpr (kBulk) {
            if (tid == 0 && kk < nsteps)
                bulk_row(raw + (size_t)ring * plan.raw_stage,
                         raw_src + (raw_row + kk) * (size_t)Nx * raw_elem,
                         (unsigned)(Nx * raw_elem), &bars[ring]);
            return;
        }
        if (kk < nsteps) {
            const unsigned char *src =
                raw_src + (raw_row + kk) * (size_t)Nx * raw_elem;
            unsigned char *dst = raw + (size_t)ring * plan.raw_stage;
            for (int c = tid; c < chunks; c += nthreads)
                cp_async16(dst + 16 * c, src + 16 * c);
        }
        cp_async_commit();
    };

    // Fused single precision: e^{iH(kk, x)} of this thread's columns into
    // cs buffer `buf`.  One segment keeps its constants and pivot in
    // registers across the columns; more segments sum in table order per
    // column.  Both give the same bits for one segment.
    auto produce_f32 = [&](int kk, int buf) {
        R2 *dst = cs + (size_t)buf * ncols;
        const float4 *pv = a.piv + ((size_t)row_blk * nsteps + kk) * a.n_seg;
        if (a.n_seg == 1) {
            const SegF f = segf[0];
            const float4 p0 = __ldg(pv);
#pragma unroll
            for (int i = 0; i < CPL; ++i) {
                if (i < nmine) {
                    const int x = tid + i * nthreads;
                    dst[x] = CS<R>::of_cs(seg_phase_one<HT>(f, p0, x, hcr, hconst));
                }
            }
            return;
        }
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            if (i < nmine) {
                const int x = tid + i * nthreads;
                dst[x] = CS<R>::of_cs(
                    seg_phase<HT>(segf, pv, a.n_seg, x, hcr, hconst));
            }
        }
    };

    // e^{iH(kk, x)} of every padded column into cs buffer `buf`.
    auto produce = [&](int kk, int buf) {
        if constexpr (kFusedF32) {
            produce_f32(kk, buf);
        } else {
        R2 *dst = cs + (size_t)buf * ncols;
        const unsigned char *st = raw + (size_t)(kk % 3) * plan.raw_stage;
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            const int x = tid + i * nthreads;
            if (x >= ncols) continue;
            R2 v;
            if (x >= Nx) {
                v.x = R(0); v.y = R(0);
            } else if (kSeg) {
                if constexpr (!kSingle) {
                    const double X0 = __dmul_rn((double)x - 0.5 * Nx, a.dx);
                    const double yv = __dmul_rn((double)iy - 0.5 * a.Ny, a.dx);
                    const double zv = __dmul_rn((double)kk, a.dz);
                    double acc = 0.0;
                    for (int s = 0; s < a.n_seg; ++s) {
                        const double *sg = a.segs + (size_t)s * DYFOX_SEG_STRIDE;
                        acc = __dadd_rn(acc, h_seg_f64(
                            sg, __dsub_rn(X0, __ldg(sg + SEG_CX)),
                            __dsub_rn(yv, __ldg(sg + SEG_CY)),
                            __dsub_rn(zv, __ldg(sg + SEG_CZ)), a.vc));
                    }
                    v = CS<R>::of_f64(acc);
                }
            } else if (stage == ST_CONVERT) {
                switch (hsrc) {
                case HS_GRID64:
                    v = CS<R>::of_f64(reinterpret_cast<const double *>(st)[x]);
                    break;
                case HS_GRID32:
                    v = CS<R>::of_f32(reinterpret_cast<const float *>(st)[x]);
                    break;
                case HS_CS32:
                    v = CS<R>::of_cs(reinterpret_cast<const float2 *>(st)[x]);
                    break;
                default:
                    v = CS<R>::of_cs(reinterpret_cast<const double2 *>(st)[x]);
                }
            } else {
                switch (hsrc) {
                case HS_GRID64:
                    v = CS<R>::of_f64(__ldg(
                        (const double *)a.hgrid +
                        ((size_t)iy * Nz + kk) * Nx + x));
                    break;
                case HS_GRID32:
                    v = CS<R>::of_f32(__ldg(
                        (const float *)a.hgrid +
                        ((size_t)iy * Nz + kk) * Nx + x));
                    break;
                case HS_CS32:
                    v = CS<R>::of_cs(__ldg(
                        (const float2 *)a.csgrid +
                        ((size_t)row_blk * nsteps + kk) * Nx + x));
                    break;
                case HS_CS64:
                    v = CS<R>::of_cs(__ldg(
                        (const double2 *)a.csgrid +
                        ((size_t)row_blk * nsteps + kk) * Nx + x));
                    break;
                case HS_ANALYTIC:
                    v = an_cs[kk];
                    break;
                default:
                    v.x = R(1); v.y = R(0);
                }
            }
            dst[x] = v;
        }
        }
    };

    // Initial state: A = input beam, B = 0.
    R Ar[CPL], Ai[CPL], Br[CPL], Bi[CPL];
    R Alr[COMP ? CPL : 1], Ali[COMP ? CPL : 1], Blr[COMP ? CPL : 1],
        Bli[COMP ? CPL : 1];
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int x = L * CPL + j;
        Ar[j] = x < Nx ? (R)beam_profile(x, Nx, a.dx, a.sheet_hw) : R(0);
        Ai[j] = R(0); Br[j] = R(0); Bi[j] = R(0);
        if constexpr (COMP) { Alr[j] = 0; Ali[j] = 0; Blr[j] = 0; Bli[j] = 0; }
    }
    if (stage == ST_DIRECT) {
        stage_issue(0, 0);
        stage_issue(1, 1);
        cp_async_wait<1>();
    } else if (stage == ST_CONVERT) {
        stage_issue(0, 0);
        stage_issue(1, 1);
        cp_async_wait<0>();
        __syncthreads();
        produce(0, 0);
    } else {
        produce(0, 0);
    }
    if (lane == 0) {
        bnd[(0 * nwarps + warp) * NB + 0] = R2{Ar[0], Ai[0]};
        if constexpr (COMP) bnd[(0 * nwarps + warp) * NB + 2] = R2{Alr[0], Ali[0]};
    }
    if (lane == 31) {
        bnd[(0 * nwarps + warp) * NB + 1] = R2{Br[CPL - 1], Bi[CPL - 1]};
        if constexpr (COMP) bnd[(0 * nwarps + warp) * NB + 3] = R2{Blr[CPL - 1], Bli[CPL - 1]};
    }
    __syncthreads();

    const Kappa *kap = a.kappa + (size_t)ie * nsteps;
    const float4 *kap32 = a.kappa32 + (size_t)ie * nsteps;
    Kappa kn;
    float4 kn32;
    if constexpr (kSingle) kn32 = __ldg(kap32);
    else kn = ldg_kappa(kap);
    // ------------------------------------------------------------ march
    // Lane 31 takes A(0) of the next warp of its angle (zero past the last),
    // lane 0 B(CPL - 1) of the previous one (zero before the first).
    const bool is_last = lane == 31, is_first = lane == 0;
    const bool has_next = wa + 1 < WA, has_prev = wa > 0;
    const int nb_next = has_next ? warp + 1 : warp;
    const int nb_prev = has_prev ? warp - 1 : warp;
    // One depth step.  rc is the step's ring index k % 3 (the stage of the
    // staged row and the boundary slot it reads): a compile-time constant
    // in the staged march, which runs the steps unrolled by three, so that
    // every shared-memory address of the step is a constant offset; a
    // run-time value in the other marches.
    // Staged march: every ring stage's row and boundary-slot addresses,
    // fixed for the whole march (the unrolled steps index them by their
    // compile-time stage).
    const R2 *st_src[3], *st_next[3], *st_prev[3];
    R2 *st_own[3];
    if constexpr (kStaged) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            st_src[r] = reinterpret_cast<const R2 *>(
                            raw + (size_t)r * plan.raw_stage) + L * CPL;
            st_next[r] = has_next ? bnd + (r * nwarps + nb_next) * NB
                                  : bnd + 3 * nwarps * NB;   // zeros
            st_prev[r] = has_prev ? bnd + (r * nwarps + nb_prev) * NB
                                  : bnd + 3 * nwarps * NB;
            st_own[r] = bnd + (r * nwarps + warp) * NB + (is_first ? 0 : 1);
        }
    }
    // phase: the parity of the ring stage's barrier for step k (k / 3 mod
    // 2; the staged loop passes its unrolled round's parity).
    auto step = [&](const int k, auto rc, unsigned phase) {
        const int ring = rc;
        const int ring2 = ring == 0 ? 2 : ring - 1;      // (k + 2) % 3
        const int nslot = ring == 2 ? 0 : ring + 1;      // (k + 1) % 3
        const int p = k & 1;
        R k12r, k12i, k21r, k21i;
        if constexpr (kSingle) {
            k12r = kn32.x; k12i = kn32.y; k21r = kn32.z; k21i = kn32.w;
            // the next step's couplings (the last step reloads its own)
            kn32 = __ldg(kap32 + (k + 1 < nsteps ? k + 1 : k));
        } else {
            k12r = (R)kn.k12.x; k12i = (R)kn.k12.y;
            k21r = (R)kn.k21.x; k21i = (R)kn.k21.y;
            if (k + 1 < nsteps) kn = ldg_kappa(kap + k + 1);
        }
        if (stage != ST_COMPUTE) stage_issue(k + 2, ring2);
        if (stage != ST_DIRECT && k + 1 < nsteps) produce(k + 1, p ^ 1);

        // Neighbour values of the previous state.
        R ainr = __shfl_down_sync(0xffffffffu, Ar[0], 1);
        R aini = __shfl_down_sync(0xffffffffu, Ai[0], 1);
        R binr = __shfl_up_sync(0xffffffffu, Br[CPL - 1], 1);
        R bini = __shfl_up_sync(0xffffffffu, Bi[CPL - 1], 1);
        R ainlr = 0, ainli = 0, binlr = 0, binli = 0;
        (void)ainlr; (void)ainli; (void)binlr; (void)binli;
        if constexpr (COMP) {
            ainlr = __shfl_down_sync(0xffffffffu, Alr[0], 1);
            ainli = __shfl_down_sync(0xffffffffu, Ali[0], 1);
            binlr = __shfl_up_sync(0xffffffffu, Blr[CPL - 1], 1);
            binli = __shfl_up_sync(0xffffffffu, Bli[CPL - 1], 1);
        }
        // lane 31 loads the next warp's A(0), lane 0 the previous warp's
        // B(CPL - 1) (zeros at the row's ends): predicated loads, or (the
        // fused marches with FP64 sum or few columns per lane, where those
        // cost registers and occupancy) broadcast loads that the two lanes
        // keep by selection
        constexpr bool kPredBnd =
            HT != HT_SEG64 && !(HT == HT_SEG && CPL < 7);
        {
            const R2 *nxt, *prv;
            if constexpr (kStaged) {
                nxt = st_next[ring];
                prv = st_prev[ring];
            } else {
                nxt = has_next ? bnd + (ring * nwarps + nb_next) * NB
                               : bnd + 3 * nwarps * NB;
                prv = has_prev ? bnd + (ring * nwarps + nb_prev) * NB
                               : bnd + 3 * nwarps * NB;
            }
            if constexpr (kPredBnd) {
                ld_shared_if(is_last, nxt + 0, ainr, aini);
                ld_shared_if(is_first, prv + 1, binr, bini);
                if constexpr (COMP) {
                    ld_shared_if(is_last, nxt + 2, ainlr, ainli);
                    ld_shared_if(is_first, prv + 3, binlr, binli);
                }
            } else {
                const R2 t = nxt[0], v = prv[1];
                ainr = is_last ? t.x : ainr;
                aini = is_last ? t.y : aini;
                binr = is_first ? v.x : binr;
                bini = is_first ? v.y : bini;
                if constexpr (COMP) {
                    const R2 u = nxt[2], w = prv[3];
                    ainlr = is_last ? u.x : ainlr;
                    ainli = is_last ? u.y : ainli;
                    binlr = is_first ? w.x : binlr;
                    binli = is_first ? w.y : binli;
                }
            }
        }
        const R2 *src;
        if constexpr (kStaged) {
            src = st_src[ring];
        } else {
            src = (stage == ST_DIRECT
                       ? reinterpret_cast<const R2 *>(
                             raw + (size_t)ring * plan.raw_stage)
                       : cs + (size_t)p * ncols) + L * CPL;
        }
        // the row of step k: the (k / 3)-th phase of its stage's barrier
        if constexpr (kBulk) bulk_ok &= row_bar_wait(&bars[ring], phase);
        R pbr = binr, pbi = bini, pblr = binlr, pbli = binli;
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const R ar = j + 1 < CPL ? Ar[j + 1] : ainr;
            const R ai = j + 1 < CPL ? Ai[j + 1] : aini;
            const R br = pbr, bi = pbi;
            pbr = Br[j]; pbi = Bi[j];
            const R2 e = src[j];
            // Fixed rounding order (the packed pair march repeats it).
            const R m12r = fmaR(k12r, e.x, -k12i * e.y);
            const R m12i = fmaR(k12r, e.y, k12i * e.x);
            const R m21r = fmaR(k21r, e.x, k21i * e.y);
            const R m21i = fmaR(k21i, e.x, -k21r * e.y);
            if constexpr (!COMP) {
                Ar[j] = fmaR(m12r, br, fmaR(-m12i, bi, ar));
                Ai[j] = fmaR(m12r, bi, fmaR(m12i, br, ai));
                Br[j] = fmaR(m21r, ar, fmaR(-m21i, ai, br));
                Bi[j] = fmaR(m21r, ai, fmaR(m21i, ar, bi));
            } else {
                const R alr = j + 1 < CPL ? Alr[j + 1] : ainlr;
                const R ali = j + 1 < CPL ? Ali[j + 1] : ainli;
                const R blr = pblr, bli = pbli;
                pblr = Blr[j]; pbli = Bli[j];
                const R tr = fmaR(m12r, br, fmaR(-m12i, bi, alr));
                const R ti = fmaR(m12r, bi, fmaR(m12i, br, ali));
                const R ur = fmaR(m21r, ar, fmaR(-m21i, ai, blr));
                const R ui = fmaR(m21r, ai, fmaR(m21i, ar, bli));
                R e0, e1, e2, e3;
                if constexpr (kFastCompensation) {
                    Ar[j] = fast_two_sum(ar, tr, e0);
                    Ai[j] = fast_two_sum(ai, ti, e1);
                    Br[j] = fast_two_sum(br, ur, e2);
                    Bi[j] = fast_two_sum(bi, ui, e3);
                } else {
                    Ar[j] = two_sum(ar, tr, e0);
                    Ai[j] = two_sum(ai, ti, e1);
                    Br[j] = two_sum(br, ur, e2);
                    Bi[j] = two_sum(bi, ui, e3);
                }
                Alr[j] = e0; Ali[j] = e1; Blr[j] = e2; Bli[j] = e3;
            }
        }
        // lane 0 publishes its A(0), lane 31 its B(CPL - 1)
        {
            R2 *slot;
            if constexpr (kStaged)
                slot = st_own[nslot];
            else
                slot = bnd + (nslot * nwarps + warp) * NB + (is_first ? 0 : 1);
            const bool pub = is_first || is_last;
            if constexpr (kPredBnd) {
                st_shared_if(pub, slot, is_first ? Ar[0] : Br[CPL - 1],
                             is_first ? Ai[0] : Bi[CPL - 1]);
                if constexpr (COMP)
                    st_shared_if(pub, slot + 2,
                                 is_first ? Alr[0] : Blr[CPL - 1],
                                 is_first ? Ali[0] : Bli[CPL - 1]);
            } else if (pub) {
                slot[0] = is_first ? R2{Ar[0], Ai[0]}
                                   : R2{Br[CPL - 1], Bi[CPL - 1]};
                if constexpr (COMP)
                    slot[2] = is_first ? R2{Alr[0], Ali[0]}
                                       : R2{Blr[CPL - 1], Bli[CPL - 1]};
            }
        }
        // The stage of step k + 1 (DIRECT) or k + 2 (CONVERT) is complete
        // and, after the barrier, visible to every thread.
        if (stage == ST_DIRECT && !kBulk) cp_async_wait<1>();
        else if (stage == ST_CONVERT) cp_async_wait<0>();
        __syncthreads();
    };
    if constexpr (kStaged) {
        int k = 0;
        unsigned phase = 0;
        for (; k + 3 <= nsteps; k += 3, phase ^= 1u) {
            step(k, RingIdx<0>{}, phase);
            step(k + 1, RingIdx<1>{}, phase);
            step(k + 2, RingIdx<2>{}, phase);
        }
        if (k < nsteps) step(k, RingIdx<0>{}, phase);
        if (k + 1 < nsteps) step(k + 1, RingIdx<1>{}, phase);
    } else {
        int ring = 0;
        for (int k = 0; k < nsteps; ++k) {
            step(k, ring, 0u);
            ring = ring == 2 ? 0 : ring + 1;
        }
    }
    if (stage != ST_COMPUTE && !kBulk) cp_async_wait<0>();
    // Every issued row was waited for inside its step (and every thread is
    // past the last step's barrier): the barriers can be released for the
    // next use of this shared memory.
    if (kBulk && tid == 0)
        for (int st = 0; st < 3; ++st) row_bar_inval(&bars[st]);
    if (!bulk_ok && a.err) atomicExch(a.err, 1);

    // ---------------------------------------------------------- output
    if (ie_raw >= a.n_e) return;
    const double2 S = __ldg(a.scale + ie);
    R2 *out = reinterpret_cast<R2 *>(a.out) + ((size_t)ie * a.Ny + iy) * Nx;
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int x = L * CPL + j;
        if (x < Nx) {
            double br = (double)Br[j], bi = (double)Bi[j];
            if constexpr (COMP) { br += (double)Blr[j]; bi += (double)Bli[j]; }
            // a row copy that never completed: the wave reads NaN
            if (!bulk_ok) br = bi = __longlong_as_double(0x7ff8000000000000LL);
            out[x] = R2{(R)(S.x * br - S.y * bi), (R)(S.x * bi + S.y * br)};
        }
    }
}

// One CTA per (row, angle group) of one solve.
template <typename R, int CPL, int HT, bool COMP>
__global__ void laue_march_kernel(const MarchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int row_blk = blockIdx.x / a.n_groups;
    march_block<R, CPL, HT, COMP>(a, row_blk,
                                  blockIdx.x - row_blk * a.n_groups, smem);
}

// The same with at most 80 registers a thread: the fused single-precision
// marches at 5 columns per lane run two 320-thread CTAs per multiprocessor
// at 80 registers, and the compiler's own allocation for them moves with
// small changes to the phase code and can cost that second CTA.
template <typename R, int CPL, int HT, bool COMP>
__global__ void __maxnreg__(80) laue_march_kernel_r80(const MarchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int row_blk = blockIdx.x / a.n_groups;
    march_block<R, CPL, HT, COMP>(a, row_blk,
                                  blockIdx.x - row_blk * a.n_groups, smem);
}

template <typename R, int CPL, int HT, bool COMP>
constexpr bool march_capped() {
    return sizeof(R) == 4 && CPL == 5 && (HT == HT_SEG || HT == HT_SEG64);
}

template <typename R, int CPL, int HT, bool COMP>
constexpr auto march_kernel() {
    if constexpr (march_capped<R, CPL, HT, COMP>())
        return laue_march_kernel_r80<R, CPL, HT, COMP>;
    else
        return laue_march_kernel<R, CPL, HT, COMP>;
}

// Host launch of one instantiation; returns cudaError_t.  Also reports the
// instantiation's maximum block size and register count.
template <typename R, int CPL, int HT, bool COMP>
cudaError_t launch_march(const MarchArgs &a, int grid, int block, size_t smem,
                         cudaStream_t stream) {
    auto *k = march_kernel<R, CPL, HT, COMP>();
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k<<<grid, block, smem, stream>>>(a);
    count_launch(1);
    return cudaGetLastError();
}

template <typename R, int CPL, int HT, bool COMP>
cudaError_t attr_march(cudaFuncAttributes *attr) {
    return cudaFuncGetAttributes(attr, march_kernel<R, CPL, HT, COMP>());
}

using MarchLaunch = cudaError_t (*)(const MarchArgs &, int, int, size_t,
                                    cudaStream_t);
using MarchAttr = cudaError_t (*)(cudaFuncAttributes *);

struct MarchEntry {
    MarchLaunch launch;
    MarchAttr attr;
};

// Defined in laue_f64.cu / laue_f32.cu; return {nullptr, nullptr} for an
// instantiation that does not exist.
MarchEntry march_entry_f64(int cpl, int ht);
MarchEntry march_entry_f32_plain(int cpl, int ht);
MarchEntry march_entry_f32_comp(int cpl, int ht);
extern const int kCplF64[];
extern const int kNumCplF64;
constexpr int kCplF32[] = {5, 7, 9, 11, 13};
constexpr int kNumCplF32 = 5;

}  // namespace dyfox
