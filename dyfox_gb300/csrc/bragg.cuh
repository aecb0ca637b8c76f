// Building blocks of the Bragg (reflection) shooting solve, one CTA per
// system (y-plane x deviation parameter):
//   * complex helpers and CTA-wide reductions (warp shuffles + one shared
//     slot per warp, fixed order, so results are deterministic);
//   * the down-march of DYFOX bragg/solver.py:28-35 (the GMRES matvec), in
//     double and in single precision (the inner products of the mixed
//     solve);
//   * a mixed-radix Stockham FFT in shared memory for the perfect-crystal
//     preconditioner ifft(fft(w) / T22s) of bragg/solver.py:167-168, in
//     double and in single precision.
#pragma once
#include <string.h>

#include "common.cuh"

namespace dyfox {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
    return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) {
    return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 cmulz(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ double2 cdotz(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cscale(double s, double2 a) {
    return make_double2(s * a.x, s * a.y);
}
__device__ __forceinline__ double2 cconj(double2 a) {
    return make_double2(a.x, -a.y);
}
__device__ __forceinline__ double cabs2(double2 a) {
    return a.x * a.x + a.y * a.y;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ float2 cmulz(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) {
    return make_float2(a.x, -a.y);
}
__device__ __forceinline__ float2 cscale(float s, float2 a) {
    return make_float2(s * a.x, s * a.y);
}

// Sum of v over the CTA.  red: shared scratch of >= 33 double2.  Every
// thread returns the total.  Two barriers.
__device__ __forceinline__ double2 block_sum(double2 v, double2 *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double2 t = lane < nw ? red[lane] : make_double2(0.0, 0.0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            t.x += __shfl_down_sync(0xffffffffu, t.x, o);
            t.y += __shfl_down_sync(0xffffffffu, t.y, o);
        }
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

// Maximum over the CTA of a non-negative double.
__device__ __forceinline__ double block_max(double v, double2 *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) red[warp].x = v;
    __syncthreads();
    if (warp == 0) {
        double t = lane < nw ? red[lane].x : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            t = fmax(t, __shfl_down_sync(0xffffffffu, t, o));
        if (lane == 0) red[32].x = t;
    }
    __syncthreads();
    return red[32].x;
}

// ---------------------------------------------------------------------------
// Down-march (bragg/solver.py:28-35): for k = 0 .. Nz-2
//   D0'[x] = e0 (D0[x-1] + ds Cb[k][x-1] Dg[x-1])      (roll +1, periodic)
//   Dg'[x] = (Dg[x+1] - ds Ch[k][x+1] D0[x+1]) / eg     (roll -1, periodic)
// cb, ch: this plane's (Nz, Nx) couplings with ds folded in.  Column x is
// held by thread x % nt in register slot x / nt; the shifted values pass
// through the two shared exchange rows.  d0_in / dg_in NULL means zero.
// Dg(t) is written to out (shared or global).
template <int CPL>
__device__ void bragg_march(const double2 *__restrict__ cb,
                            const double2 *__restrict__ ch, double2 e0,
                            double2 ieg, int Nz, int Nx,
                            const double2 *d0_in, const double2 *dg_in,
                            double2 *ex0, double2 *ex1, double2 *out) {
    const int tid = threadIdx.x, nt = blockDim.x;
    double2 D0[CPL], Dg[CPL];
#pragma unroll
    for (int i = 0; i < CPL; ++i) {
        const int x = tid + i * nt;
        D0[i] = make_double2(0.0, 0.0);
        Dg[i] = make_double2(0.0, 0.0);
        if (x < Nx) {
            if (d0_in) D0[i] = d0_in[x];
            if (dg_in) Dg[i] = dg_in[x];
        }
    }
    for (int k = 0; k < Nz - 1; ++k) {
        const double2 *cbk = cb + (size_t)k * Nx, *chk = ch + (size_t)k * Nx;
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            const int x = tid + i * nt;
            if (x < Nx) {
                const double2 b = __ldg(cbk + x), h = __ldg(chk + x);
                const double2 u = cadd(D0[i], cmulz(b, Dg[i]));
                const double2 v = cmulz(csub(Dg[i], cmulz(h, D0[i])), ieg);
                ex0[x + 1 == Nx ? 0 : x + 1] = cmulz(e0, u);
                ex1[x == 0 ? Nx - 1 : x - 1] = v;
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            const int x = tid + i * nt;
            if (x < Nx) {
                D0[i] = ex0[x];
                Dg[i] = ex1[x];
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < CPL; ++i) {
        const int x = tid + i * nt;
        if (x < Nx) out[x] = Dg[i];
    }
    __syncthreads();
}

// The march in single precision, for the inner (Arnoldi) products of the
// mixed-precision solve, in the depth-scaled form A_k = e0^-k D0_k:
//   A'(x+1) = A(x) + cb'_k(x) Dg(x),  Dg'(x-1) = (Dg(x) - ch'_k(x) A(x)) ieg
// with cb'_k = e0^-k cb_k and ch'_k = e0^k ch_k folded into the couplings
// (e0 does not depend on the deviation parameter), so a column-step costs
// two complex products and one multiplication by ieg; Dg, and so the
// result Dg(t), are unchanged.  Couplings and ieg in float, the inputs
// rounded to float (NULL means zero), the result widened into out.
//   Thread t holds the CPL contiguous columns [t CPL, (t+1) CPL) of the row
// in registers (threads past column Nx - 1 hold padding, kept zero).  The
// one-column shifts move in registers, across lanes by warp shuffle, and
// across warps and around the periodic ends (column Nx - 1 to 0 and back)
// through a few shared slots at the start of ex0, double-buffered by the
// step's parity: one barrier a step.  ex1 is unused.
template <int CPL>
__device__ void bragg_march32(const float2 *__restrict__ cb,
                              const float2 *__restrict__ ch, float2 ieg,
                              int Nz, int Nx, const double2 *d0_in,
                              const double2 *dg_in, float2 *ex0, float2 *ex1,
                              double2 *out) {
    (void)ex1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nw = blockDim.x >> 5;
    const int x0 = tid * CPL;
    const int last = (Nx - 1) / CPL, jl = Nx - 1 - last * CPL;
    const bool is_last = tid == last, is_first = tid == 0;
    // sU[p][w]: the last column's u of warp w; sV[p][w]: the first column's
    // v of warp w; sW[p]: (u of column Nx - 1, v of column 0)
    float2 *sU = ex0, *sV = ex0 + 2 * nw, *sW = ex0 + 4 * nw;
    const float2 z = make_float2(0.f, 0.f);
    bool valid[CPL];
    float2 A[CPL], G[CPL], b[CPL], h[CPL];
    const int ns = Nz - 1;
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int x = x0 + j;
        valid[j] = x < Nx;
        A[j] = z;
        G[j] = z;
        b[j] = z;
        h[j] = z;
        if (valid[j]) {
            if (d0_in) {
                const double2 v = d0_in[x];
                A[j] = make_float2((float)v.x, (float)v.y);
            }
            if (dg_in) {
                const double2 v = dg_in[x];
                G[j] = make_float2((float)v.x, (float)v.y);
            }
            if (ns > 0) {
                b[j] = __ldg(cb + x);
                h[j] = __ldg(ch + x);
            }
        }
    }
    for (int k = 0; k < ns; ++k) {
        const int p = k & 1;
        float2 u[CPL], v[CPL];
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            u[j] = cadd(A[j], cmulz(b[j], G[j]));
            v[j] = cmulz(csub(G[j], cmulz(h[j], A[j])), ieg);
        }
        // the couplings of step k + 1
        if (k + 1 < ns) {
            const float2 *cbn = cb + (size_t)(k + 1) * Nx + x0;
            const float2 *chn = ch + (size_t)(k + 1) * Nx + x0;
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                if (valid[j]) {
                    b[j] = __ldg(cbn + j);
                    h[j] = __ldg(chn + j);
                }
            }
        }
        float2 uin, vin;
        uin.x = __shfl_up_sync(0xffffffffu, u[CPL - 1].x, 1);
        uin.y = __shfl_up_sync(0xffffffffu, u[CPL - 1].y, 1);
        vin.x = __shfl_down_sync(0xffffffffu, v[0].x, 1);
        vin.y = __shfl_down_sync(0xffffffffu, v[0].y, 1);
        if (lane == 31) sU[p * nw + warp] = u[CPL - 1];
        if (lane == 0) sV[p * nw + warp] = v[0];
        if (is_last) {
            float2 ul = u[0];
#pragma unroll
            for (int j = 1; j < CPL; ++j)
                if (j == jl) ul = u[j];
            sW[2 * p] = ul;
        }
        if (is_first) sW[2 * p + 1] = v[0];
        __syncthreads();
        if (lane == 0) uin = is_first ? sW[2 * p] : sU[p * nw + warp - 1];
        if (lane == 31 && tid < last) vin = sV[p * nw + warp + 1];
#pragma unroll
        for (int j = CPL - 1; j >= 1; --j) A[j] = valid[j] ? u[j - 1] : z;
        A[0] = valid[0] ? uin : z;
#pragma unroll
        for (int j = 0; j + 1 < CPL; ++j) G[j] = valid[j] ? v[j + 1] : z;
        G[CPL - 1] = valid[CPL - 1] ? vin : z;
        if (is_last) {
            const float2 w = sW[2 * p + 1];
#pragma unroll
            for (int j = 0; j < CPL; ++j)
                if (j == jl) G[j] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < CPL; ++j)
        if (valid[j]) out[x0 + j] = make_double2(G[j].x, G[j].y);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Float-float ("double-single") complex arithmetic, for the right-hand side
// and the true residuals of the mixed-precision solve.  A real number is
// hi + lo (|lo| <= ulp(hi) / 2); a complex number is the float4 (re.hi,
// re.lo, im.hi, im.lo).  Products are Dekker's (the FMA residual of the
// high parts) with the first-order cross terms, sums Knuth's two-sum:
// relative error about 2^-44 a step, against 2^-53 in double, at several
// times less pipe time on a part whose double rate is 1/64 of single.
// __fmul_rn / __fadd_rn keep the compiler from contracting the products
// whose rounding error is being captured.
__device__ __forceinline__ float2 ff_of(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ float4 ffc_of(double2 v) {
    const float2 r = ff_of(v.x), i = ff_of(v.y);
    return make_float4(r.x, r.y, i.x, i.y);
}
__device__ __forceinline__ double2 ffc_to(float4 v) {
    return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}

// c + a1 b1 + a2 b2, real float-float.
__device__ __forceinline__ float2 ff_dot2(float2 a1, float2 b1, float2 a2,
                                          float2 b2, float2 c) {
    const float p1 = __fmul_rn(a1.x, b1.x), p2 = __fmul_rn(a2.x, b2.x);
    float e = __fadd_rn(fmaf(a1.x, b1.x, -p1), fmaf(a2.x, b2.x, -p2));
    e = fmaf(a1.x, b1.y, e);
    e = fmaf(a1.y, b1.x, e);
    e = fmaf(a2.x, b2.y, e);
    e = fmaf(a2.y, b2.x, e);
    float s = __fadd_rn(c.x, p1);
    float v = __fsub_rn(s, c.x);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(c.x, __fsub_rn(s, v)), __fsub_rn(p1, v)));
    const float s2 = __fadd_rn(s, p2);
    v = __fsub_rn(s2, s);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(s2, v)), __fsub_rn(p2, v)));
    e = __fadd_rn(e, c.y);
    const float t = __fadd_rn(s2, e);
    return make_float2(t, __fsub_rn(e, __fsub_rn(t, s2)));
}

// c + a b, complex float-float.
__device__ __forceinline__ float4 ffc_fma(float4 a, float4 b, float4 c) {
    const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
    const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
    const float2 re = ff_dot2(ar, br, make_float2(-a.z, -a.w), bi,
                              make_float2(c.x, c.y));
    const float2 im = ff_dot2(ar, bi, ai, br, make_float2(c.z, c.w));
    return make_float4(re.x, re.y, im.x, im.y);
}

// a1 b1 + a2 b2, real float-float (ff_dot2 with no addend: one two-sum).
__device__ __forceinline__ float2 ff_dot2z(float2 a1, float2 b1, float2 a2,
                                           float2 b2) {
    const float p1 = __fmul_rn(a1.x, b1.x), p2 = __fmul_rn(a2.x, b2.x);
    float e = __fadd_rn(fmaf(a1.x, b1.x, -p1), fmaf(a2.x, b2.x, -p2));
    e = fmaf(a1.x, b1.y, e);
    e = fmaf(a1.y, b1.x, e);
    e = fmaf(a2.x, b2.y, e);
    e = fmaf(a2.y, b2.x, e);
    const float s = __fadd_rn(p1, p2);
    const float v = __fsub_rn(s, p1);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(p1, __fsub_rn(s, v)), __fsub_rn(p2, v)));
    const float t = __fadd_rn(s, e);
    return make_float2(t, __fsub_rn(e, __fsub_rn(t, s)));
}

// a b, complex float-float.
__device__ __forceinline__ float4 ffc_mul(float4 a, float4 b) {
    const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
    const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
    const float2 re = ff_dot2z(ar, br, make_float2(-a.z, -a.w), bi);
    const float2 im = ff_dot2z(ar, bi, ai, br);
    return make_float4(re.x, re.y, im.x, im.y);
}

// Column layout of the float-float march: column x = tid + i blockDim.x of
// a thread, its periodic neighbours x + 1 and x - 1, and whether it exists
// (x < Nx), formed once per march.
template <int CPL>
struct MarchCols {
    int x[CPL], xp[CPL], xm[CPL];
    bool ok[CPL];
    __device__ __forceinline__ MarchCols(int Nx) {
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            const int c = threadIdx.x + i * blockDim.x;
            ok[i] = c < Nx;
            x[i] = ok[i] ? c : 0;
            xp[i] = c + 1 >= Nx ? 0 : c + 1;
            xm[i] = c == 0 ? Nx - 1 : c - 1;
        }
    }
};

// The march of bragg_march32 in float-float, for the right-hand side and
// the true residuals of the mixed-precision solve: the depth-scaled form
// with the folded couplings as hi (cb, ch) and lo (cbl, chl) float2
// planes, ieg as float-float, inputs (NULL: zero) and the result in
// double.  ex0, ex1: float4 exchange rows of Nx (two barriers a step).
template <int CPL>
__device__ void bragg_march_ff(const float2 *__restrict__ cb,
                               const float2 *__restrict__ cbl,
                               const float2 *__restrict__ ch,
                               const float2 *__restrict__ chl, float4 ieg,
                               int Nz, int Nx, const double2 *d0_in,
                               const double2 *dg_in, float4 *ex0,
                               float4 *ex1, double2 *out) {
    const MarchCols<CPL> mc(Nx);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 A[CPL], G[CPL];
#pragma unroll
    for (int i = 0; i < CPL; ++i) {
        A[i] = z4;
        G[i] = z4;
        if (mc.ok[i]) {
            if (d0_in) A[i] = ffc_of(d0_in[mc.x[i]]);
            if (dg_in) G[i] = ffc_of(dg_in[mc.x[i]]);
        }
    }
    for (int k = 0; k < Nz - 1; ++k) {
        const size_t row = (size_t)k * Nx;
        const float2 *cbk = cb + row, *cblk = cbl + row;
        const float2 *chk = ch + row, *chlk = chl + row;
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            if (mc.ok[i]) {
                const int x = mc.x[i];
                const float2 bh = __ldg(cbk + x), bl = __ldg(cblk + x);
                const float2 hh = __ldg(chk + x), hl = __ldg(chlk + x);
                const float4 b = make_float4(bh.x, bl.x, bh.y, bl.y);
                const float4 nh = make_float4(-hh.x, -hl.x, -hh.y, -hl.y);
                ex0[mc.xp[i]] = ffc_fma(b, G[i], A[i]);
                ex1[mc.xm[i]] = ffc_mul(ffc_fma(nh, A[i], G[i]), ieg);
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            if (mc.ok[i]) {
                A[i] = ex0[mc.x[i]];
                G[i] = ex1[mc.x[i]];
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < CPL; ++i)
        if (mc.ok[i]) out[mc.x[i]] = ffc_to(G[i]);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Mixed-radix Stockham FFT (Govindaraju et al., SC'08 formulation): stage of
// radix R over butterflies j in [0, N/R), Ns = product of earlier radices;
// input index j + r N/R, output index (j / Ns) Ns R + j % Ns + q Ns.  The
// twiddle exp(-+2 pi i r (j % Ns) / (Ns R)) and the radix-R DFT kernel both
// come from the table tw[m] = exp(-2 pi i m / N).  Radix 2 and 4 use
// explicit butterflies; other radices evaluate each output as an R-term sum
// (N R complex products per stage).  inverse: conjugate twiddles, no scale.
struct FftPlan {
    int n;
    int nfac;
    int fac[24];
    // Per pass f: ceil(2^32 / Ns_f) and ceil(2^32 / (n / fac[f])), or 0
    // where the divisor is 1.  __umulhi(i, magic) is then i / divisor,
    // exactly for i < 2^16 and divisors below 2^16 (n <= 2^16).
    unsigned ns_magic[24], nb_magic[24];
};

inline unsigned fft_magic(unsigned d) {
    return d > 1 ? (unsigned)(((1ull << 32) + d - 1) / d) : 0u;
}

// Radices of an N-point transform: 4s, then 2s, then odd factors.
// N <= 65536 (the magic divisions; callers check).
inline FftPlan make_fft_plan(int N) {
    FftPlan p;
    memset(&p, 0, sizeof p);
    p.n = N;
    int n = N;
    while (n % 4 == 0 && p.nfac < 24) { p.fac[p.nfac++] = 4; n /= 4; }
    while (n % 2 == 0 && p.nfac < 24) { p.fac[p.nfac++] = 2; n /= 2; }
    for (int f = 3; n > 1 && p.nfac < 24; f += 2)
        while (n % f == 0 && p.nfac < 24) { p.fac[p.nfac++] = f; n /= f; }
    unsigned Ns = 1;
    for (int f = 0; f < p.nfac; ++f) {
        p.ns_magic[f] = fft_magic(Ns);
        p.nb_magic[f] = fft_magic((unsigned)(N / p.fac[f]));
        Ns *= (unsigned)p.fac[f];
    }
    return p;
}

template <typename C>
__device__ __forceinline__ C twid(const C *tw, int m, bool inv) {
    C w = __ldg(tw + m);
    return inv ? cconj(w) : w;
}

__device__ __forceinline__ int fft_div(int i, unsigned magic) {
    return magic ? (int)__umulhi((unsigned)i, magic) : i;
}

// One radix-R pass (R odd, 3..13) of `count` transforms: one thread per
// butterfly.  Inputs are twiddled once, then the R-point DFT uses the
// conjugate pairs r, R - r: with a_r = x_r + x_{R-r}, b_r = x_r - x_{R-r},
// y_q = x_0 + sum a_r cos(2 pi r q / R) -+ i sum b_r sin(2 pi r q / R) and
// y_{R-q} the other sign (forward / inverse), about half the products of
// the plain sum.  cos and sin come from the N-point table at multiples of
// N / R.
template <int R, typename C>
__device__ __forceinline__ void fft_odd_pass(const C *src, C *dst, int N,
                                             int nb, int Ns, int step,
                                             unsigned ns_mg, unsigned nb_mg,
                                             int count, int stride,
                                             const C *tw, bool inv) {
    constexpr int H = (R - 1) / 2;
    const int unit = N / R;
    const int items = nb * count;
    for (int t = threadIdx.x; t < items; t += blockDim.x) {
        const int c = count > 1 ? fft_div(t, nb_mg) : 0;
        const int j = t - c * nb;
        const C *sc = src + (size_t)c * stride;
        C *dc = dst + (size_t)c * stride;
        const int q = fft_div(j, ns_mg), k = j - q * Ns;
        C x[R];
        x[0] = sc[j];
#pragma unroll
        for (int r = 1; r < R; ++r) {
            C v = sc[j + r * nb];
            if (k) v = cmulz(v, twid(tw, r * k * step, inv));
            x[r] = v;
        }
        C a[H], b[H];
        C y0 = x[0];
#pragma unroll
        for (int r = 1; r <= H; ++r) {
            a[r - 1] = cadd(x[r], x[R - r]);
            b[r - 1] = csub(x[r], x[R - r]);
            y0 = cadd(y0, a[r - 1]);
        }
        const int d = q * Ns * R + k;
        dc[d] = y0;
#pragma unroll
        for (int qq = 1; qq <= H; ++qq) {
            C P = x[0], Q;
            Q.x = 0; Q.y = 0;
#pragma unroll
            for (int r = 1; r <= H; ++r) {
                const C w = __ldg(tw + ((r * qq) % R) * unit);  // (cos, -sin)
                P.x += a[r - 1].x * w.x;
                P.y += a[r - 1].y * w.x;
                Q.x -= b[r - 1].x * w.y;
                Q.y -= b[r - 1].y * w.y;
            }
            // forward: y_qq = P - iQ, y_{R-qq} = P + iQ; inverse swaps.
            C m, pl;
            m.x = P.x + Q.y; m.y = P.y - Q.x;
            pl.x = P.x - Q.y; pl.y = P.y + Q.x;
            dc[d + qq * Ns] = inv ? pl : m;
            dc[d + (R - qq) * Ns] = inv ? m : pl;
        }
    }
}

// Stockham FFT of `count` N-point transforms, transform c at offset
// c * stride (stride >= N; 0: N), between two buffers.  Returns the buffer
// holding the result (src or dst).  All threads call.  C is double2 or
// float2 (the table tw has the same type).  count * (N / 2)^2 < 2^32 keeps
// the magic division of the item index by N / R exact.
// BIG_ODD: register butterflies also for radices 11 and 13 (the imaging
// kernels in single precision: 4% on 544 x 1056 images; the Bragg kernels
// keep them off, where they would raise every kernel's register count).
// 17 and 19 stay plain sums: their butterflies cost the imaging kernels
// more in occupancy (128 registers) than they save.
template <typename C, bool BIG_ODD = false>
__device__ C *fft_run(C *src, C *dst, const FftPlan &p,
                      const C *__restrict__ tw, bool inv, int count = 1,
                      int stride = 0) {
    const int N = p.n, tid = threadIdx.x, nt = blockDim.x;
    if (stride == 0) stride = N;
    int Ns = 1;
    for (int f = 0; f < p.nfac; ++f) {
        const int R = p.fac[f];
        const int nb = N / R;
        const int step = N / (Ns * R);
        const unsigned ns_mg = p.ns_magic[f], nb_mg = p.nb_magic[f];
        const int items = nb * count;
        if (R == 2) {
            for (int t = tid; t < items; t += nt) {
                const int c = count > 1 ? fft_div(t, nb_mg) : 0;
                const int j = t - c * nb;
                const C *sc = src + (size_t)c * stride;
                C *dc = dst + (size_t)c * stride;
                const int q = fft_div(j, ns_mg), k = j - q * Ns;
                C a = sc[j], b = sc[j + nb];
                if (k) b = cmulz(b, twid(tw, k * step, inv));
                const int d = q * Ns * 2 + k;
                dc[d] = cadd(a, b);
                dc[d + Ns] = csub(a, b);
            }
        } else if (R == 4) {
            for (int t = tid; t < items; t += nt) {
                const int c = count > 1 ? fft_div(t, nb_mg) : 0;
                const int j = t - c * nb;
                const C *sc = src + (size_t)c * stride;
                C *dc = dst + (size_t)c * stride;
                const int q = fft_div(j, ns_mg), k = j - q * Ns;
                C v0 = sc[j], v1 = sc[j + nb], v2 = sc[j + 2 * nb],
                  v3 = sc[j + 3 * nb];
                if (k) {
                    v1 = cmulz(v1, twid(tw, k * step, inv));
                    v2 = cmulz(v2, twid(tw, 2 * k * step, inv));
                    v3 = cmulz(v3, twid(tw, 3 * k * step, inv));
                }
                const C s02 = cadd(v0, v2), d02 = csub(v0, v2);
                const C s13 = cadd(v1, v3), d13 = csub(v1, v3);
                // -i d13 forward, +i d13 inverse
                C rot;
                rot.x = inv ? -d13.y : d13.y;
                rot.y = inv ? d13.x : -d13.x;
                const int d = q * Ns * 4 + k;
                dc[d] = cadd(s02, s13);
                dc[d + Ns] = cadd(d02, rot);
                dc[d + 2 * Ns] = csub(s02, s13);
                dc[d + 3 * Ns] = csub(d02, rot);
            }
        } else if (R == 3) {
            fft_odd_pass<3>(src, dst, N, nb, Ns, step, ns_mg, nb_mg, count, stride, tw, inv);
        } else if (R == 5) {
            fft_odd_pass<5>(src, dst, N, nb, Ns, step, ns_mg, nb_mg, count, stride, tw, inv);
        } else if (R == 7) {
            fft_odd_pass<7>(src, dst, N, nb, Ns, step, ns_mg, nb_mg, count, stride, tw, inv);
        } else if (BIG_ODD && R == 11) {
            fft_odd_pass<11>(src, dst, N, nb, Ns, step, ns_mg, nb_mg, count, stride, tw, inv);
        } else if (BIG_ODD && R == 13) {
            fft_odd_pass<13>(src, dst, N, nb, Ns, step, ns_mg, nb_mg, count, stride, tw, inv);
        } else {
            // Other odd factors (17, 19, ...; 11 and 13 without BIG_ODD):
            // one output per thread, the plain sum over the R inputs.
            for (int it = tid; it < N * count; it += nt) {
                const int c = count > 1 ? it / N : 0, o = it - c * N;
                const C *sc = src + (size_t)c * stride;
                C *dc = dst + (size_t)c * stride;
                const int q = o / nb, j = o - q * nb;
                const int jq = fft_div(j, ns_mg), k = j - jq * Ns;
                // sum_r src[j + r nb] W^(r (k step + q nb))
                int base = k * step + q * nb;
                if (base >= N) base -= N;
                C acc = sc[j];
                int m = base;
                for (int r = 1; r < R; ++r) {
                    acc = cadd(acc, cmulz(sc[j + r * nb], twid(tw, m, inv)));
                    m += base;
                    if (m >= N) m -= N;
                }
                dc[jq * Ns * R + k + q * Ns] = acc;
            }
        }
        __syncthreads();
        C *t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    return src;
}

// w <- ifft(fft(w) * iT) with iT = 1 / T22s; a, b are scratch rows.
__device__ inline void precond_apply(double2 *w, double2 *a, double2 *b,
                              const FftPlan &p,
                              const double2 *__restrict__ tw,
                              const double2 *__restrict__ iT) {
    const int N = p.n, tid = threadIdx.x, nt = blockDim.x;
    for (int x = tid; x < N; x += nt) a[x] = w[x];
    __syncthreads();
    double2 *f = fft_run(a, b, p, tw, false);
    for (int x = tid; x < N; x += nt) f[x] = cmulz(f[x], __ldg(iT + x));
    __syncthreads();
    double2 *o = f == a ? b : a;
    double2 *g = fft_run(f, o, p, tw, true);
    const double inv_n = 1.0 / N;
    for (int x = tid; x < N; x += nt) w[x] = cscale(inv_n, g[x]);
    __syncthreads();
}

// The same preconditioner in single precision: w (double) is rounded to
// float, transformed with the float table, and widened back.  a, b: float2
// scratch rows of N.
__device__ inline void precond_apply32(double2 *w, float2 *a, float2 *b,
                                const FftPlan &p,
                                const float2 *__restrict__ tw,
                                const float2 *__restrict__ iT) {
    const int N = p.n, tid = threadIdx.x, nt = blockDim.x;
    for (int x = tid; x < N; x += nt)
        a[x] = make_float2((float)w[x].x, (float)w[x].y);
    __syncthreads();
    float2 *f = fft_run(a, b, p, tw, false);
    for (int x = tid; x < N; x += nt) f[x] = cmulz(f[x], __ldg(iT + x));
    __syncthreads();
    float2 *o = f == a ? b : a;
    float2 *g = fft_run(f, o, p, tw, true);
    const double inv_n = 1.0 / N;
    for (int x = tid; x < N; x += nt)
        w[x] = make_double2(inv_n * g[x].x, inv_n * g[x].y);
    __syncthreads();
}

// Device-side arguments of the Bragg solve of one call (or one instance of
// a batch): sizes, crystal, and pointers into the workspace.
struct BraggArgs {
    int Nx, Nz, n_y, n_s;
    double ds, s0r, s0i, shr, shi, sbr, sbi;
    const double *s_dev;          // (n_s)
    const double2 *cb, *ch;       // (n_y, Nz, Nx): ds sigma e^{+-iH}
    const double2 *e0h;           // (n_y, Nx): e^{-iH(z=0)}
    const double2 *inc;           // (Nx): incident D0
    const double2 *iT;            // (n_s, Nx): 1 / T22s
    const double2 *tw;            // (Nx): exp(-2 pi i m / Nx)
    const float2 *cb32, *ch32;    // e0^-k cb, e0^k ch rounded to float:
                                  // the mixed form's depth-scaled march
    const float2 *cbl32, *chl32;  // their remainders rounded to float: the
                                  // float-float couplings (mixed form)
    const float2 *iT32, *tw32;    // FP32 copies of iT, tw (mixed form)
    FftPlan plan;
    double2 *V;                   // (n_sys, m + 1, Nx)
    double2 *Hh;                  // (n_sys, m, m + 1)
    double2 *X, *B;               // (n_sys, Nx)
    double2 *out;                 // (n_s, n_y, Nx)
    double *info;                 // (n_sys, 4)
    double tol;
    int restart, maxiter, use_x0;
    int force_resume;             // DYFOX_BRAGG_FORCE_RESUME (checks)
};

}  // namespace dyfox
