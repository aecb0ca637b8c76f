// The Bragg GMRES solve of one system on one CTA and the kernels around it
// (single calls, parity-check operators, batches), shared by the
// translation units that instantiate them: bragg_k64.cu (double),
// bragg_k32.cu (mixed precision), bragg_kb64.cu and bragg_kb32.cu
// (batches).  The algorithm is described at the top of bragg.cu.
#pragma once
#include <math.h>
#include <string.h>

#include "bragg.cuh"
#include "volterra.cuh"

namespace dyfox {

__device__ __forceinline__ void step_factors(const BraggArgs &a, int is,
                                             double2 &e0, double2 &ieg) {
    const double alpha = -2.0 * kPi * a.s_dev[is];
    const double er = exp(a.s0r * a.ds);
    double sn, c;
    sincos(a.s0i * a.ds, &sn, &c);
    e0 = make_double2(er * c, er * sn);
    sincos((a.s0i + alpha) * a.ds, &sn, &c);
    // 1 / eg = exp(-(s0 + i alpha) ds)
    ieg = make_double2(c / er, -sn / er);
}

// Shared memory of the GMRES kernel: three Nx rows (exchange / FFT scratch
// and the Arnoldi vector), the reduction slots, S, y and the rotations.
__host__ __device__ inline size_t gmres_smem(int Nx, int m) {
    return (size_t)3 * Nx * sizeof(double2) + 34 * sizeof(double2) +
           (size_t)2 * (m + 1) * sizeof(double2) +
           (size_t)m * (sizeof(double2) + sizeof(double)) + 64;
}

// LAPACK zlartg: c real, s complex, r with [c s; -conj(s) c] [f; g] = [r; 0].
__device__ inline void lartg(double2 f, double2 g, double &c, double2 &s,
                      double2 &r) {
    const double fa = hypot(f.x, f.y), ga = hypot(g.x, g.y);
    if (ga == 0.0) {
        c = 1.0; s = make_double2(0.0, 0.0); r = f;
    } else if (fa == 0.0) {
        c = 0.0; s = make_double2(g.x / ga, -g.y / ga); r = make_double2(ga, 0.0);
    } else {
        const double d = hypot(fa, ga);
        c = fa / d;
        const double2 fu = make_double2(f.x / fa, f.y / fa);   // f / |f|
        s = cscale(1.0 / d, cmulz(fu, cconj(g)));
        r = cscale(d, fu);
    }
}

// Drop of the estimated (preconditioned) residual after which a restart
// cycle of the mixed form ends its inner iteration.
constexpr double kMixedInnerDrop = 1e-5;

// The solve of system `sys` (deviation parameter sys / n_y, plane
// sys % n_y) of `a` by the calling CTA.  smem: gmres_smem(Nx, restart).
// warm: start from the X already in place (else from a.use_x0's rule);
// inner0: inner iterations already spent on this system.  Returns -1 when
// the solve ended (result and info written); a MIXED solve that did not
// converge returns its inner iteration count instead and writes nothing,
// and the caller continues in double from the X reached so far.
template <int CPL, bool MIXED>
__device__ __forceinline__ int gmres_system(const BraggArgs &a, int sys,
                                            unsigned char *smem, bool warm,
                                            int inner0) {
    const int Nx = a.Nx, m = a.restart;
    double2 *A0 = reinterpret_cast<double2 *>(smem);
    double2 *A1 = A0 + Nx;
    double2 *W = A1 + Nx;
    double2 *red = W + Nx;     // [0, 33): block_sum; [33]: presid
    double2 *S = red + 34;
    double2 *yv = S + (m + 1);
    double2 *gs = yv + (m + 1);
    double *gc = reinterpret_cast<double *>(gs + m);
    int *flags = reinterpret_cast<int *>(gc + m);          // [0] stop

    const int is = sys / a.n_y, iy = sys - is * a.n_y;
    const int tid = threadIdx.x, nt = blockDim.x;
    const double2 *cb = a.cb + (size_t)iy * a.Nz * Nx;
    const double2 *ch = a.ch + (size_t)iy * a.Nz * Nx;
    const double2 *iT = a.iT + (size_t)is * Nx;
    double2 *V = a.V + (size_t)sys * (m + 1) * Nx;
    double2 *Hh = a.Hh + (size_t)sys * m * (m + 1);
    double2 *X = a.X + (size_t)sys * Nx;
    double2 *B = a.B + (size_t)sys * Nx;
    double2 e0, ieg;
    step_factors(a, is, e0, ieg);
    const float2 iegf = make_float2((float)ieg.x, (float)ieg.y);
    const float2 *cb32 = MIXED ? a.cb32 + (size_t)iy * a.Nz * Nx : nullptr;
    const float2 *ch32 = MIXED ? a.ch32 + (size_t)iy * a.Nz * Nx : nullptr;
    const float2 *cbl32 = MIXED ? a.cbl32 + (size_t)iy * a.Nz * Nx : nullptr;
    const float2 *chl32 = MIXED ? a.chl32 + (size_t)iy * a.Nz * Nx : nullptr;
    const float4 iegff = ffc_of(ieg);
    const float2 *iT32 = MIXED ? a.iT32 + (size_t)is * Nx : nullptr;
    const double eps = 2.220446049250313e-16;

    auto norm2 = [&](const double2 *v) {
        double2 t = make_double2(0.0, 0.0);
        for (int x = tid; x < Nx; x += nt) t.x += cabs2(v[x]);
        return sqrt(block_sum(t, red).x);
    };
    // W <- A src (src NULL: particular solution from the incident beam); in
    // float-float when MIXED (the right-hand side and the true residuals).
    auto matvec = [&](const double2 *src) {
        if (MIXED) {
            bragg_march_ff<CPL>(cb32, cbl32, ch32, chl32, iegff, a.Nz,
                                Nx, src ? nullptr : a.inc, src,
                                reinterpret_cast<float4 *>(A0),
                                reinterpret_cast<float4 *>(A1), W);
        } else if (src) {
            bragg_march<CPL>(cb, ch, e0, ieg, a.Nz, Nx, nullptr, src, A0, A1,
                             W);
        } else {
            bragg_march<CPL>(cb, ch, e0, ieg, a.Nz, Nx, a.inc, nullptr, A0,
                             A1, W);
        }
    };
    // The Arnoldi operator: W <- M A src, in single precision when MIXED.
    auto inner_op = [&](const double2 *src) {
        if (MIXED) {
            bragg_march32<CPL>(cb32, ch32, iegf, a.Nz, Nx, nullptr, src,
                               reinterpret_cast<float2 *>(A0),
                               reinterpret_cast<float2 *>(A1), W);
        } else {
            matvec(src);
        }
    };
    auto precond = [&]() {
        if (MIXED)
            precond_apply32(W, reinterpret_cast<float2 *>(A0),
                            reinterpret_cast<float2 *>(A1), a.plan, a.tw32,
                            iT32);
        else
            precond_apply(W, A0, A1, a.plan, a.tw, iT);
    };

    // b = -d
    matvec(nullptr);
    for (int x = tid; x < Nx; x += nt) {
        B[x] = make_double2(-W[x].x, -W[x].y);
        if (!a.use_x0 && !warm) X[x] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    const double bnrm2 = norm2(B);
    double *info = a.info + (size_t)sys * 4;
    double rnorm = 0.0;
    int inner = 0, code = 0;
    if (bnrm2 == 0.0) {
        for (int x = tid; x < Nx; x += nt) X[x] = make_double2(0.0, 0.0);
    } else {
        const double atol = a.tol * bnrm2;
        for (int x = tid; x < Nx; x += nt) W[x] = B[x];
        __syncthreads();
        precond();
        const double Mb_nrm2 = norm2(W);
        double ptol_max_factor = 1.0;
        double ptol = Mb_nrm2 * fmin(ptol_max_factor, atol / bnrm2);
        double presid = 0.0;
        // r = b - A x0 (b when x0 is zero)
        bool nonzero = false;
        if (a.use_x0 || warm) {
            double2 t = make_double2(0.0, 0.0);
            for (int x = tid; x < Nx; x += nt) t.x += cabs2(X[x]);
            nonzero = block_sum(t, red).x > 0.0;
        }
        if (nonzero) {
            matvec(X);
            for (int x = tid; x < Nx; x += nt) W[x] = csub(B[x], W[x]);
        } else {
            for (int x = tid; x < Nx; x += nt) W[x] = B[x];
        }
        __syncthreads();
        rnorm = norm2(W);
        code = a.maxiter;
        if (rnorm < atol) {
            code = 0;
        } else {
            for (int iter = 0; iter < a.maxiter; ++iter) {
                // v0 = M r / |M r|, S = (|M r|, 0, ...)
                precond();
                const double tmp = norm2(W);
                // inner stopping level of this cycle
                const double pstop =
                    MIXED ? fmax(ptol, kMixedInnerDrop * tmp) : ptol;
                for (int x = tid; x < Nx; x += nt) V[x] = cscale(1.0 / tmp, W[x]);
                for (int j = tid; j <= m; j += nt)
                    S[j] = make_double2(j == 0 ? tmp : 0.0, 0.0);
                __syncthreads();
                bool breakdown = false;
                int col = 0;
                for (col = 0; col < m; ++col) {
                    inner_op(V + (size_t)col * Nx);
                    precond();
                    const double h0 = norm2(W);
                    // Modified Gram-Schmidt, one pass per basis vector:
                    // subtract the previous projection, accumulate the next.
                    double2 hprev = make_double2(0.0, 0.0);
                    for (int k = 0; k <= col; ++k) {
                        const double2 *vk = V + (size_t)k * Nx;
                        const double2 *vp = k ? V + (size_t)(k - 1) * Nx : vk;
                        double2 t = make_double2(0.0, 0.0);
                        for (int x = tid; x < Nx; x += nt) {
                            double2 w = W[x];
                            if (k) w = csub(w, cmulz(hprev, vp[x]));
                            W[x] = w;
                            const double2 d = cdotz(vk[x], w);
                            t.x += d.x;
                            t.y += d.y;
                        }
                        const double2 h = block_sum(t, red);
                        if (tid == 0) Hh[(size_t)col * (m + 1) + k] = h;
                        hprev = h;
                    }
                    {
                        const double2 *vp = V + (size_t)col * Nx;
                        for (int x = tid; x < Nx; x += nt)
                            W[x] = csub(W[x], cmulz(hprev, vp[x]));
                    }
                    __syncthreads();
                    const double h1 = norm2(W);
                    double2 *vn = V + (size_t)(col + 1) * Nx;
                    if (h1 <= eps * h0) {
                        breakdown = true;
                        for (int x = tid; x < Nx; x += nt) vn[x] = W[x];
                    } else {
                        for (int x = tid; x < Nx; x += nt)
                            vn[x] = cscale(1.0 / h1, W[x]);
                    }
                    if (tid == 0) {
                        double2 *hc = Hh + (size_t)col * (m + 1);
                        hc[col + 1] = make_double2(breakdown ? 0.0 : h1, 0.0);
                        for (int k = 0; k < col; ++k) {
                            const double c = gc[k];
                            const double2 s = gs[k];
                            const double2 n0 = hc[k], n1 = hc[k + 1];
                            hc[k] = cadd(cscale(c, n0), cmulz(s, n1));
                            hc[k + 1] = cadd(cscale(-1.0, cmulz(cconj(s), n0)),
                                             cscale(c, n1));
                        }
                        double c;
                        double2 s, r;
                        lartg(hc[col], hc[col + 1], c, s, r);
                        gc[col] = c;
                        gs[col] = s;
                        hc[col] = r;
                        hc[col + 1] = make_double2(0.0, 0.0);
                        const double2 t = cscale(-1.0, cmulz(cconj(s), S[col]));
                        S[col] = cscale(c, S[col]);
                        S[col + 1] = t;
                        red[33].x = hypot(t.x, t.y);
                    }
                    __syncthreads();
                    presid = red[33].x;
                    ++inner;
                    __syncthreads();
                    if (presid <= pstop || breakdown) break;
                }
                if (col == m) col = m - 1;
                // y = R^{-1} S (back substitution; R[row][c] = Hh[c][row])
                if (tid == 0) {
                    const double2 *Hc = Hh;
                    if (Hc[(size_t)col * (m + 1) + col].x == 0.0 &&
                        Hc[(size_t)col * (m + 1) + col].y == 0.0)
                        S[col] = make_double2(0.0, 0.0);
                    for (int k = 0; k <= col; ++k) yv[k] = S[k];
                    for (int k = col; k > 0; --k) {
                        if (yv[k].x != 0.0 || yv[k].y != 0.0) {
                            const double2 hkk = Hc[(size_t)k * (m + 1) + k];
                            const double d = cabs2(hkk);
                            yv[k] = cscale(1.0 / d, cmulz(yv[k], cconj(hkk)));
                            const double2 tk = yv[k];
                            for (int i = 0; i < k; ++i)
                                yv[i] = csub(yv[i],
                                             cmulz(tk, Hc[(size_t)k * (m + 1) + i]));
                        }
                    }
                    if (yv[0].x != 0.0 || yv[0].y != 0.0) {
                        const double2 h00 = Hc[0];
                        yv[0] = cscale(1.0 / cabs2(h00), cmulz(yv[0], cconj(h00)));
                    }
                }
                __syncthreads();
                for (int x = tid; x < Nx; x += nt) {
                    double2 acc = X[x];
                    for (int k = 0; k <= col; ++k)
                        acc = cadd(acc, cmulz(yv[k], V[(size_t)k * Nx + x]));
                    X[x] = acc;
                }
                __syncthreads();
                matvec(X);
                for (int x = tid; x < Nx; x += nt) W[x] = csub(B[x], W[x]);
                __syncthreads();
                rnorm = norm2(W);
                if (rnorm <= atol) { code = 0; break; }
                if (breakdown) break;
                if (presid <= ptol)
                    ptol_max_factor = fmax(eps, 0.25 * ptol_max_factor);
                else
                    ptol_max_factor = fmin(1.0, 1.5 * ptol_max_factor);
                ptol = presid * fmin(ptol_max_factor, atol / rnorm);
            }
            if (rnorm <= atol) code = 0;
        }
    }
    // A mixed solve that did not converge (single precision not accurate
    // enough for this system) is handed over to the double continuation.
    if (MIXED && (code != 0 || a.force_resume)) return inner0 + inner;
    // exit wave v e^{-iH(0)}
    double2 *out = a.out + ((size_t)is * a.n_y + iy) * Nx;
    const double2 *e0h = a.e0h + (size_t)iy * Nx;
    for (int x = tid; x < Nx; x += nt) out[x] = cmulz(X[x], __ldg(e0h + x));
    if (tid == 0) {
        info[0] = bnrm2 > 0.0 ? rnorm / bnrm2 : 0.0;
        info[1] = inner0 + inner;
        info[2] = code;
        info[3] = bnrm2;
    }
    (void)flags;
    return -1;
}

// A system in the requested precision.  A mixed solve that stalls leaves
// its solution so far in X and marks the system (code -1, iterations spent
// in info[1]) for bragg_resume_kernel, which finishes it in double; the
// double path is a separate launch so that the single-precision kernel
// carries none of it.
template <int CPL, bool MIXED>
__device__ __forceinline__ void solve_system(const BraggArgs &a, int sys,
                                             unsigned char *smem) {
    const int spent = gmres_system<CPL, MIXED>(a, sys, smem, false, 0);
    if (MIXED && spent >= 0 && threadIdx.x == 0) {
        double *info = a.info + (size_t)sys * 4;
        info[1] = spent;
        info[2] = -1.0;
    }
}

// Continuation in double of the systems a mixed solve marked.
template <int CPL>
__device__ __forceinline__ void resume_system(const BraggArgs &a, int sys,
                                              unsigned char *smem) {
    const double *info = a.info + (size_t)sys * 4;
    if (info[2] != -1.0) return;          // uniform over the CTA
    gmres_system<CPL, false>(a, sys, smem, true, (int)info[1]);
}

// The GMRES kernels carry no launch bounds: the compiler's own choice
// (about 100 registers for the 4-column mixed kernel) measured fastest on
// the 20 um Bragg scan (Nx 456, Nz 90, 21 x 64 systems).  Bounds of
// (128, 5) forced 96 registers and lost 18%; bounds of
// (NT, 1) let it take 212 registers and lost 40% to occupancy.

// One CTA of NT threads per system of one solve call.
template <int CPL, bool MIXED, int NT>
__global__ void
bragg_gmres_kernel(const BraggArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    solve_system<CPL, MIXED>(a, blockIdx.x, smem);
}

// The mixed 4-column, 128-thread kernel (the shape of the 20 um scan's
// 456-column planes) with bounds that keep 5 CTAs per SM (96 registers
// instead of 122: 4% on that scan).  Bounds
// on every instantiation would let the others take 186-234 registers.
// (a template so that only the unit that launches it compiles it)
template <int NT>
__global__ void __launch_bounds__(NT, 5)
bragg_gmres_mixed4_kernel(const BraggArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    solve_system<4, true>(a, blockIdx.x, smem);
}

// After a mixed launch: one CTA per system, returning at once unless the
// system was marked.
template <int CPL, int NT>
__global__ void
bragg_resume_kernel(const BraggArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    resume_system<CPL>(a, blockIdx.x, smem);
}

// Matvec / preconditioner for parity checks: one CTA per system.
// mode 0: out = march(d0, dg); mode 1: out = M in.  MIXED: the
// single-precision operators of the mixed form.
template <int CPL, bool MIXED>
__global__ void bragg_apply_kernel(const BraggArgs a, int mode,
                                   const double2 *d0, const double2 *dg,
                                   double2 *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int Nx = a.Nx;
    double2 *A0 = reinterpret_cast<double2 *>(smem);
    double2 *A1 = A0 + Nx;
    double2 *W = A1 + Nx;
    const int sys = blockIdx.x, is = sys / a.n_y, iy = sys - is * a.n_y;
    const size_t off = (size_t)sys * Nx;
    if (mode == 2) {
        // the float-float march of the mixed form's residuals
        double2 e0, ieg;
        step_factors(a, is, e0, ieg);
        if (MIXED)
            bragg_march_ff<CPL>(a.cb32 + (size_t)iy * a.Nz * Nx,
                                a.cbl32 + (size_t)iy * a.Nz * Nx,
                                a.ch32 + (size_t)iy * a.Nz * Nx,
                                a.chl32 + (size_t)iy * a.Nz * Nx,
                                ffc_of(ieg), a.Nz, Nx,
                                d0 ? d0 + off : nullptr,
                                dg ? dg + off : nullptr,
                                reinterpret_cast<float4 *>(A0),
                                reinterpret_cast<float4 *>(A1), W);
    } else if (mode == 0) {
        double2 e0, ieg;
        step_factors(a, is, e0, ieg);
        if (MIXED)
            bragg_march32<CPL>(a.cb32 + (size_t)iy * a.Nz * Nx,
                               a.ch32 + (size_t)iy * a.Nz * Nx,
                               make_float2((float)ieg.x, (float)ieg.y), a.Nz,
                               Nx, d0 ? d0 + off : nullptr,
                               dg ? dg + off : nullptr,
                               reinterpret_cast<float2 *>(A0),
                               reinterpret_cast<float2 *>(A1), W);
        else
            bragg_march<CPL>(a.cb + (size_t)iy * a.Nz * Nx,
                             a.ch + (size_t)iy * a.Nz * Nx, e0, ieg, a.Nz, Nx,
                             d0 ? d0 + off : nullptr, dg ? dg + off : nullptr,
                             A0, A1, W);
    } else {
        for (int x = threadIdx.x; x < Nx; x += blockDim.x) W[x] = d0[off + x];
        __syncthreads();
        if (MIXED)
            precond_apply32(W, reinterpret_cast<float2 *>(A0),
                            reinterpret_cast<float2 *>(A1), a.plan, a.tw32,
                            a.iT32 + (size_t)is * Nx);
        else
            precond_apply(W, A0, A1, a.plan, a.tw, a.iT + (size_t)is * Nx);
    }
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) out[off + x] = W[x];
}

// cudaErrorLaunchOutOfResources unless one CTA of `threads` threads and
// `smem` bytes fits on an SM.
template <typename K>
static cudaError_t resident(K *k, int threads, size_t smem) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, k, threads, smem);
    if (e) return e;
    return occ >= 1 ? cudaSuccess : cudaErrorLaunchOutOfResources;
}

// The kernel of CPL columns a thread for `threads` (128 or 256) threads:
// CPL 1, 2 only occur with 128 threads, 8 and 16 only with 256.
template <int CPL, bool MIXED>
static void (*gmres_kernel_for(int threads))(const BraggArgs) {
    if constexpr (CPL == 4 && MIXED) {
        if (threads == 128) return bragg_gmres_mixed4_kernel<128>;
    }
    if constexpr (CPL <= 2) {
        return bragg_gmres_kernel<CPL, MIXED, 128>;
    } else if constexpr (CPL >= 8) {
        return bragg_gmres_kernel<CPL, MIXED, 256>;
    } else {
        return threads == 128 ? bragg_gmres_kernel<CPL, MIXED, 128>
                              : bragg_gmres_kernel<CPL, MIXED, 256>;
    }
}

template <int CPL>
static void (*resume_kernel_for(int threads))(const BraggArgs) {
    if constexpr (CPL <= 2) {
        return bragg_resume_kernel<CPL, 128>;
    } else if constexpr (CPL >= 8) {
        return bragg_resume_kernel<CPL, 256>;
    } else {
        return threads == 128 ? bragg_resume_kernel<CPL, 128>
                              : bragg_resume_kernel<CPL, 256>;
    }
}

template <int CPL, bool MIXED>
static cudaError_t launch_gmres(const BraggArgs &a, int threads, size_t smem,
                                int grid, cudaStream_t stream) {
    auto *k = gmres_kernel_for<CPL, MIXED>(threads);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e) return e;
    }
    if (cudaError_t e = resident(k, threads, smem)) return e;
    if (MIXED) {
        auto *r = resume_kernel_for<CPL>(threads);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(
                r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e) return e;
        }
        k<<<grid, threads, smem, stream>>>(a);
        r<<<grid, threads, smem, stream>>>(a);
        count_launch(2);
        return cudaGetLastError();
    }
    k<<<grid, threads, smem, stream>>>(a);
    count_launch(1);
    return cudaGetLastError();
}

template <int CPL, bool MIXED>
static cudaError_t launch_apply(const BraggArgs &a, int threads, size_t smem,
                                int grid, int mode, const double2 *d0,
                                const double2 *dg, double2 *out,
                                cudaStream_t stream) {
    auto *k = bragg_apply_kernel<CPL, MIXED>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e) return e;
    }
    if (cudaError_t e = resident(k, threads, smem)) return e;
    k<<<grid, threads, smem, stream>>>(a, mode, d0, dg, out);
    count_launch(1);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Pieces used by the batched launcher (batch.cu): one CTA per system of
// many instances, the instances' arguments in a device array.
template <int CPL, int NT>
__global__ void
bragg_batch_resume_kernel(const BraggArgs *__restrict__ insts,
                          const int2 *__restrict__ systems) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ BraggArgs a;
    const int2 w = systems[blockIdx.x];
    if (threadIdx.x == 0) a = insts[w.x];
    __syncthreads();
    resume_system<CPL>(a, w.y, smem);
}

template <int CPL, bool MIXED, int NT>
__global__ void
bragg_batch_kernel(const BraggArgs *__restrict__ insts,
                   const int2 *__restrict__ systems) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ BraggArgs a;
    const int2 w = systems[blockIdx.x];
    if (threadIdx.x == 0) a = insts[w.x];
    __syncthreads();
    solve_system<CPL, MIXED>(a, w.y, smem);
}

template <int CPL, bool MIXED>
static void (*batch_kernel_for(int threads))(const BraggArgs *,
                                             const int2 *) {
    if constexpr (CPL <= 2) {
        return bragg_batch_kernel<CPL, MIXED, 128>;
    } else if constexpr (CPL >= 8) {
        return bragg_batch_kernel<CPL, MIXED, 256>;
    } else {
        return threads == 128 ? bragg_batch_kernel<CPL, MIXED, 128>
                              : bragg_batch_kernel<CPL, MIXED, 256>;
    }
}

template <int CPL>
static void (*batch_resume_for(int threads))(const BraggArgs *,
                                             const int2 *) {
    if constexpr (CPL <= 2) {
        return bragg_batch_resume_kernel<CPL, 128>;
    } else if constexpr (CPL >= 8) {
        return bragg_batch_resume_kernel<CPL, 256>;
    } else {
        return threads == 128 ? bragg_batch_resume_kernel<CPL, 128>
                              : bragg_batch_resume_kernel<CPL, 256>;
    }
}

template <int CPL, bool MIXED>
static cudaError_t launch_bragg_batch_t(const BraggArgs *insts,
                                        const int2 *systems, int n_sys,
                                        int threads, size_t smem,
                                        cudaStream_t stream) {
    batch_kernel_for<CPL, MIXED>(threads)<<<n_sys, threads, smem, stream>>>(
        insts, systems);
    count_launch(1);
    if (MIXED) {
        batch_resume_for<CPL>(threads)<<<n_sys, threads, smem, stream>>>(
            insts, systems);
        count_launch(1);
    }
    return cudaGetLastError();
}

template <int CPL, bool MIXED>
static cudaError_t set_smem_t(size_t smem, int threads) {
    auto *k = batch_kernel_for<CPL, MIXED>(threads);
    cudaError_t e = cudaFuncSetAttribute(
        k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!e) e = resident(k, threads, smem);
    if (!e && MIXED) {
        auto *r = batch_resume_for<CPL>(threads);
        e = cudaFuncSetAttribute(
            r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    return e;
}

// Per-precision entry points (one translation unit each): the solve
// launch (with the double resume after a mixed launch), the parity-check
// operators, and the batch kernels.
cudaError_t bragg_launch_solve64(int cpl, const BraggArgs &a, int threads,
                                 size_t smem, int grid, cudaStream_t stream);
cudaError_t bragg_launch_solve32(int cpl, const BraggArgs &a, int threads,
                                 size_t smem, int grid, cudaStream_t stream);
cudaError_t bragg_launch_apply64(int cpl, const BraggArgs &a, int threads,
                                 size_t smem, int grid, int mode,
                                 const double2 *d0, const double2 *dg,
                                 double2 *out, cudaStream_t stream);
cudaError_t bragg_launch_apply32(int cpl, const BraggArgs &a, int threads,
                                 size_t smem, int grid, int mode,
                                 const double2 *d0, const double2 *dg,
                                 double2 *out, cudaStream_t stream);
cudaError_t bragg_batch_smem64(int cpl, size_t smem, int threads);
cudaError_t bragg_batch_smem32(int cpl, size_t smem, int threads);
cudaError_t bragg_batch_launch64(const BraggArgs *insts, const int2 *systems,
                                 int n_sys, int threads, int cpl, size_t smem,
                                 cudaStream_t stream);
cudaError_t bragg_batch_launch32(const BraggArgs *insts, const int2 *systems,
                                 int n_sys, int threads, int cpl, size_t smem,
                                 cudaStream_t stream);

}  // namespace dyfox
