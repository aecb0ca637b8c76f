// Laue march: per-angle constants, the general (interpolating) march, the
// launch planner and the C entry points dyfox_laue_workspace_bytes /
// dyfox_laue_solve (replacing laue/solver.py:34-118 and the three kernels of
// laue/kernels.py).
#include <math.h>
#include <string.h>

#include "laue_march.cuh"
#include "laue_pair.cuh"

namespace dyfox {

// cs staging, defined in volterra.cu.
cudaError_t launch_cs_stage(bool single, bool sum64, const double *segs,
                            int n_seg, int Nx, int Ny, int Nz, double dx,
                            double dz, const VolterraConsts &vc, int row0,
                            int n_rows, void *out, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Per-(angle, step) constants of the interaction picture, in double:
// kappa12_k, kappa21_k and the final factor M22^(Nz-1).  The step constants
// cg, sg, e_p follow kernels.py:91-103.
__device__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ void laue_setup_item(
    long idx, const double *__restrict__ s_dev, int n_e, int nsteps,
    double ds, double s0r, double s0i, double shr, double shi, double sbr,
    double sbi, Kappa *kappa, float4 *kappa32, double2 *scale, float *kpair) {
    if (idx >= (long)n_e * nsteps) return;
    const int ie = (int)(idx / nsteps), k = (int)(idx - (long)ie * nsteps);
    const double alpha = -2.0 * kPi * s_dev[ie];
    const double gam = sqrt((shr * shr + shi * shi) + alpha * alpha * 0.25);
    double cg, sg;
    if (gam > 1e-30) {
        cg = cos(gam * ds);
        sg = sin(gam * ds) / gam;
    } else {
        cg = 1.0;
        sg = ds;
    }
    const double p22i = alpha * 0.5 * sg;
    const double rho = hypot(cg, p22i);
    const double th = atan2(p22i, cg);
    // e^{i (2k+1) th}: the product is split exactly (fma residual) so the
    // phase carries no rounding growing with k.
    const double m = 2.0 * k + 1.0;
    const double ph = m * th;
    const double pe = fma(m, th, -ph);
    double sp, cp;
    sincos(ph, &sp, &cp);
    const double wr = cp - sp * pe, wi = sp + cp * pe;
    const double f = sg / rho;
    Kappa kp;
    kp.k12 = make_double2(f * (sbr * wr - sbi * wi), f * (sbr * wi + sbi * wr));
    kp.k21 = make_double2(f * (shr * wr + shi * wi), f * (shi * wr - shr * wi));
    kappa[idx] = kp;
    kappa32[idx] = make_float4((float)kp.k12.x, (float)kp.k12.y,
                               (float)kp.k21.x, (float)kp.k21.y);
    if (kpair) {
        // This angle's half of its pair's KPair (laue_pair.cuh); the last
        // angle of an odd count fills both halves.
        const float k12r = (float)kp.k12.x, k12i = (float)kp.k12.y;
        const float k21r = (float)kp.k21.x, k21i = (float)kp.k21.y;
        float *q = kpair + ((size_t)(ie >> 1) * nsteps + k) * 16;
        const int t0 = ie & 1, t1 = (ie == n_e - 1 && t0 == 0) ? 1 : t0;
        for (int t = t0; t <= t1; ++t) {
            q[0 + t] = k12r;   q[2 + t] = k12i;
            q[4 + t] = -k12i;  q[6 + t] = -k12r;
            q[8 + t] = k21r;   q[10 + t] = k21i;
            q[12 + t] = -k21r; q[14 + t] = -k21i;
        }
    }
    if (k == 0) {
        const double exp_pr = exp(s0r * ds);
        const double pi_ = (s0i + alpha * 0.5) * ds;
        const double2 ep = make_double2(exp_pr * cos(pi_), exp_pr * sin(pi_));
        double2 base = cmul(ep, make_double2(cg, p22i));
        double2 acc = make_double2(1.0, 0.0);
        for (int n = nsteps; n > 0; n >>= 1) {
            if (n & 1) acc = cmul(acc, base);
            base = cmul(base, base);
        }
        scale[ie] = acc;
    }
}

__global__ void laue_setup_kernel(const double *__restrict__ s_dev, int n_e,
                                  int nsteps, double ds, double s0r,
                                  double s0i, double shr, double shi,
                                  double sbr, double sbi, Kappa *kappa,
                                  float4 *kappa32, double2 *scale,
                                  float *kpair) {
    laue_setup_item(blockIdx.x * (long)blockDim.x + threadIdx.x, s_dev, n_e,
                    nsteps, ds, s0r, s0i, shr, shi, sbr, sbi, kappa, kappa32,
                    scale, kpair);
}

// e^{iH(kk, x)} from a cheap source, for the general march.
template <typename R>
__device__ __forceinline__ typename RT<R>::R2 eval_cs(const MarchArgs &a,
                                                      int iy, int row_blk,
                                                      int kk, int x,
                                                      const typename RT<R>::R2 *an_cs) {
    const int Nx = a.Nx, Nz = a.Nz;
    switch (a.hsrc) {
    case HS_GRID64:
        return CS<R>::of_f64(__ldg((const double *)a.hgrid +
                                   ((size_t)iy * Nz + kk) * Nx + x));
    case HS_GRID32:
        return CS<R>::of_f32(__ldg((const float *)a.hgrid +
                                   ((size_t)iy * Nz + kk) * Nx + x));
    case HS_CS32:
        return CS<R>::of_cs(__ldg((const float2 *)a.csgrid +
                                  ((size_t)row_blk * (Nz - 1) + kk) * Nx + x));
    case HS_CS64:
        return CS<R>::of_cs(__ldg((const double2 *)a.csgrid +
                                  ((size_t)row_blk * (Nz - 1) + kk) * Nx + x));
    case HS_ANALYTIC:
        return an_cs[kk];
    default: {
        typename RT<R>::R2 v;
        v.x = R(1);
        v.y = R(0);
        return v;
    }
    }
}

// General march for any shift_px (laue/kernels.py:122-135 bilinear transport
// with its edge rules), one CTA per (row, angle), state in shared memory,
// in the same interaction picture as the register-resident march.
template <typename R>
__global__ void laue_general_kernel(const MarchArgs a, R shift_px) {
    using R2 = typename RT<R>::R2;
    extern __shared__ __align__(16) unsigned char smem[];
    const int Nx = a.Nx, Nz = a.Nz, nsteps = Nz - 1, NP = Nx + 1;
    R *st = reinterpret_cast<R *>(smem);
    R2 *an_cs = reinterpret_cast<R2 *>(
        smem + ((2 * 4 * (size_t)NP * sizeof(R) + 15) & ~(size_t)15));
    const int row_blk = blockIdx.x / a.n_e, ie = blockIdx.x - row_blk * a.n_e;
    const int iy = a.row0 + row_blk;
    const int tid = threadIdx.x, nt = blockDim.x;
    const double y_pix = (iy - a.Ny / 2) * a.dx;
#define ST(b, c, i) st[((b) * 4 + (c)) * NP + (i)]
    for (int ix = tid; ix < Nx; ix += nt) {
        ST(0, 0, ix) = (R)beam_profile(ix, Nx, a.dx, a.sheet_hw);
        ST(0, 1, ix) = 0; ST(0, 2, ix) = 0; ST(0, 3, ix) = 0;
    }
    if (a.hsrc == HS_ANALYTIC)
        for (int k = tid; k < nsteps; k += nt)
            an_cs[k] = CS<R>::of_f64(analytic_h(a.an, y_pix, k, a.dz));
    __syncthreads();
    int cur = 0;
    const Kappa *kap = a.kappa + (size_t)ie * nsteps;
    for (int k = 0; k < nsteps; ++k) {
        const int nx = 1 - cur;
        const Kappa kk4 = ldg_kappa(kap + k);
        const R k12r = (R)kk4.k12.x, k12i = (R)kk4.k12.y;
        const R k21r = (R)kk4.k21.x, k21i = (R)kk4.k21.y;
        for (int ix = tid; ix < Nx; ix += nt) {
            const R2 e = eval_cs<R>(a, iy, row_blk, k, ix, an_cs);
            R src0 = (R)ix + shift_px;
            int i0 = (int)floor(src0);
            R f0 = src0 - (R)i0, ar, ai;
            if (i0 >= 0 && i0 + 1 < Nx) {
                ar = (1 - f0) * ST(cur, 0, i0) + f0 * ST(cur, 0, i0 + 1);
                ai = (1 - f0) * ST(cur, 1, i0) + f0 * ST(cur, 1, i0 + 1);
            } else if (i0 >= 0 && i0 < Nx) {
                ar = (1 - f0) * ST(cur, 0, i0);
                ai = (1 - f0) * ST(cur, 1, i0);
            } else {
                ar = 0; ai = 0;
            }
            R srcg = (R)ix - shift_px;
            int ig = (int)floor(srcg);
            R fg = srcg - (R)ig, br, bi;
            if (ig >= 0 && ig + 1 < Nx) {
                br = (1 - fg) * ST(cur, 2, ig) + fg * ST(cur, 2, ig + 1);
                bi = (1 - fg) * ST(cur, 3, ig) + fg * ST(cur, 3, ig + 1);
            } else if (ig >= 0 && ig < Nx) {
                br = (1 - fg) * ST(cur, 2, ig);
                bi = (1 - fg) * ST(cur, 3, ig);
            } else {
                br = 0; bi = 0;
            }
            const R m12r = k12r * e.x - k12i * e.y, m12i = k12r * e.y + k12i * e.x;
            const R m21r = k21r * e.x + k21i * e.y, m21i = k21i * e.x - k21r * e.y;
            ST(nx, 0, ix) = fmaR(m12r, br, fmaR(-m12i, bi, ar));
            ST(nx, 1, ix) = fmaR(m12r, bi, fmaR(m12i, br, ai));
            ST(nx, 2, ix) = fmaR(m21r, ar, fmaR(-m21i, ai, br));
            ST(nx, 3, ix) = fmaR(m21r, ai, fmaR(m21i, ar, bi));
        }
        __syncthreads();
        cur = nx;
    }
    const double2 S = __ldg(a.scale + ie);
    R2 *out = reinterpret_cast<R2 *>(a.out) + ((size_t)ie * a.Ny + iy) * Nx;
    for (int ix = tid; ix < Nx; ix += nt) {
        const double br = ST(cur, 2, ix), bi = ST(cur, 3, ix);
        out[ix] = R2{(R)(S.x * br - S.y * bi), (R)(S.x * bi + S.y * br)};
    }
#undef ST
}

// Rows with |y| >= fov_hy are written as zero (kernels.py:70-75).  Rows
// start on 8-byte boundaries (complex64 or complex128 elements), so the
// stores are 8 bytes wide; blocks stride over the (angle, row) pairs.
// Rows outside the beam of every angle set to zero; block b of nb.
__device__ __forceinline__ void zero_rows_blocks(char *out, int n_e, int Ny,
                                                 size_t row_bytes, int row0,
                                                 int n_rows, int b, int nb) {
    const int n_inactive = Ny - n_rows;
    const long pairs = (long)n_e * n_inactive;
    const size_t words = row_bytes / 8;
    for (long r = b; r < pairs; r += nb) {
        const int ie = (int)(r / n_inactive);
        const int j = (int)(r - (long)ie * n_inactive);
        const int iy = j < row0 ? j : j + n_rows;
        uint2 *p = reinterpret_cast<uint2 *>(out + ((size_t)ie * Ny + iy) * row_bytes);
        for (size_t i = threadIdx.x; i < words; i += blockDim.x)
            p[i] = make_uint2(0, 0);
    }
}

__global__ void zero_rows_kernel(char *out, int n_e, int Ny, size_t row_bytes,
                                 int row0, int n_rows) {
    zero_rows_blocks(out, n_e, Ny, row_bytes, row0, n_rows, blockIdx.x,
                     gridDim.x);
}

// The set-up of one solve in one launch: blocks [0, nz) zero the rows
// outside the beam, the next ns blocks compute the kappa tables, the last
// np blocks the segment pivots of a fused single-precision march.  The three
// are independent; as separate launches they ran one after another
// (about 60 us on the README workload, most of it double-precision latency).
struct PrologueArgs {
    // zero rows
    char *out; int n_e, Ny; size_t row_bytes; int row0, n_rows;
    // kappa tables
    const double *s_dev; int nsteps;
    double ds, s0r, s0i, shr, shi, sbr, sbi;
    Kappa *kappa; float4 *kappa32; double2 *scale; float *kpair;
    // pivots
    const double *segs; int n_seg, Nx; double dx, dz; float4 *piv;
    int nz, ns, np;
    int *err;                   // the march's wait status, zeroed here
};

__global__ void laue_prologue_kernel(const PrologueArgs a) {
    const int b = blockIdx.x;
    if (b == 0 && threadIdx.x == 0 && a.err) *a.err = 0;
    if (b < a.nz) {
        zero_rows_blocks(a.out, a.n_e, a.Ny, a.row_bytes, a.row0, a.n_rows, b,
                         a.nz);
    } else if (b < a.nz + a.ns) {
        laue_setup_item((long)(b - a.nz) * blockDim.x + threadIdx.x, a.s_dev,
                        a.n_e, a.nsteps, a.ds, a.s0r, a.s0i, a.shr, a.shi,
                        a.sbr, a.sbi, a.kappa, a.kappa32, a.scale, a.kpair);
    } else {
        const long total = (long)a.n_rows * a.nsteps * a.n_seg;
        for (long i = (long)(b - a.nz - a.ns) * blockDim.x + threadIdx.x;
             i < total; i += (long)a.np * blockDim.x)
            pivot_item(i, a.segs, a.n_seg, a.Nx, a.Ny, a.dx, a.dz, a.row0,
                       a.nsteps, a.piv);
    }
}

// ---------------------------------------------------------------------------
struct LauePlan {
    bool general = false;
    int hsrc = HS_NONE;      // source the march kernel reads
    int stage = 0;           // 0: none, 1: stage e^{iH} (CS32/CS64)
    int row0 = 0, n_rows = 0;
    size_t off_kappa = 0, off_k32 = 0, off_scale = 0, off_stage = 0,
           off_piv = 0, off_kpair = 0, off_err = 0, ws = 0;
};

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

static int validate(const dyfox_laue_desc *d) {
    if (!d) { set_error("descriptor is NULL"); return DYFOX_EINVAL; }
    if (d->Nx < 1 || d->Ny < 1 || d->Nz < 2 || d->n_e < 1) {
        set_error("bad sizes Nx=%d Ny=%d Nz=%d n_e=%d (need Nx, Ny, n_e >= 1, "
                  "Nz >= 2)", d->Nx, d->Ny, d->Nz, d->n_e);
        return DYFOX_EINVAL;
    }
    if (d->precision != DYFOX_FP64 && d->precision != DYFOX_FP32) {
        set_error("precision is DYFOX_FP64 or DYFOX_FP32, not %d", d->precision);
        return DYFOX_EINVAL;
    }
    if (!(d->dx > 0) || !(d->dz > 0) || !(d->ds > 0) || !(d->shift_px > 0) ||
        !isfinite(d->shift_px) || !isfinite(d->sheet_hw) || d->sheet_hw == 0.0) {
        set_error("bad grid scalars dx=%g dz=%g ds=%g shift_px=%g sheet_hw=%g",
                  d->dx, d->dz, d->ds, d->shift_px, d->sheet_hw);
        return DYFOX_EINVAL;
    }
    if (d->h_source < DYFOX_H_NONE || d->h_source > DYFOX_H_ANALYTIC) {
        set_error("unknown h_source %d", d->h_source);
        return DYFOX_EINVAL;
    }
    if (d->h_source == DYFOX_H_SEGMENTS && d->n_seg < 0) {
        set_error("n_seg < 0");
        return DYFOX_EINVAL;
    }
    const double *sc[] = {d->sig0, d->sig_h, d->sig_hbar};
    for (int i = 0; i < 3; ++i)
        if (!isfinite(sc[i][0]) || !isfinite(sc[i][1])) {
            set_error("non-finite crystal coupling");
            return DYFOX_ENAN;
        }
    return DYFOX_OK;
}

static void active_rows(const dyfox_laue_desc *d, int *row0, int *n_rows) {
    int first = -1, count = 0;
    for (int iy = 0; iy < d->Ny; ++iy) {
        double y_pix = (iy - d->Ny / 2) * d->dx;
        if (fabs(y_pix) < d->fov_hy) {
            if (first < 0) first = iy;
            ++count;
        }
    }
    *row0 = first < 0 ? 0 : first;
    *n_rows = count;
}

// Angles one CTA of the register-resident march holds at this Nx: fusing
// the Volterra phase into the march pays only when every angle of a row
// shares one evaluation, i.e. one CTA holds them all.
static int fused_angle_limit(const dyfox_laue_desc *d) {
    const bool single = d->precision == DYFOX_FP32;
    const int *cpls = single ? kCplF32 : kCplF64;
    const int ncpl = single ? kNumCplF32 : kNumCplF64;
    int best = 1 << 30;
    for (int i = 0; i < ncpl; ++i) {
        if (d->cols_per_lane && cpls[i] != d->cols_per_lane) continue;
        const int wa = div_up(d->Nx, 32 * cpls[i]);
        if (wa <= 16 && wa < best) best = wa;
    }
    if (best == 1 << 30) return 1;
    const int a = 512 / (32 * best);
    return a < 8 ? (a < 1 ? 1 : a) : 8;
}

static int make_plan(const dyfox_laue_desc *d, LauePlan *p) {
    int st = validate(d);
    if (st) return st;
    active_rows(d, &p->row0, &p->n_rows);
    const bool exact = d->shift_px == 1.0;
    p->general = !exact || (d->flags & DYFOX_FLAG_GENERAL);
    const bool single = d->precision == DYFOX_FP32;
    switch (d->h_source) {
    case DYFOX_H_NONE: p->hsrc = HS_NONE; break;
    case DYFOX_H_GRID_F64: p->hsrc = HS_GRID64; break;
    case DYFOX_H_GRID_F32: p->hsrc = HS_GRID32; break;
    case DYFOX_H_ANALYTIC: p->hsrc = HS_ANALYTIC; break;
    default: {
        bool fused;
        if (d->flags & DYFOX_FLAG_FUSED) fused = true;
        else if (d->flags & DYFOX_FLAG_STAGED) fused = false;
        else fused = d->n_e <= fused_angle_limit(d);
        if (p->general) fused = false;
        if (d->n_seg == 0) { p->hsrc = HS_NONE; break; }
        p->hsrc = fused ? HS_SEG : (single ? HS_CS32 : HS_CS64);
        p->stage = fused ? 0 : 1;
    }
    }
    size_t off = 0;
    p->off_kappa = off;
    off = align256(off + (size_t)d->n_e * (d->Nz - 1) * sizeof(Kappa));
    p->off_k32 = off;
    off = align256(off + (size_t)d->n_e * (d->Nz - 1) * sizeof(float4));
    p->off_scale = off;
    off = align256(off + (size_t)d->n_e * sizeof(double2));
    p->off_stage = off;
    if (p->stage)
        off = align256(off + (size_t)p->n_rows * (d->Nz - 1) * d->Nx *
                                 (single ? sizeof(float2) : sizeof(double2)));
    p->off_piv = off;
    if (p->hsrc == HS_SEG && single)
        off = align256(off + (size_t)p->n_rows * (d->Nz - 1) * d->n_seg *
                                 sizeof(float4));
    p->off_kpair = off;
    if (single)
        off = align256(off + (size_t)((d->n_e + 1) / 2) * (d->Nz - 1) *
                                 sizeof(KPair));
    p->off_err = off;
    off = align256(off + sizeof(int));
    p->ws = off;
    return DYFOX_OK;
}

struct FastConfig {
    MarchEntry entry;
    int cpl, WA, A, block;
    int regs = 0;            // registers per thread of the chosen kernel
    size_t smem;
    int stage = ST_COMPUTE, raw_elem = 0;
    bool pairs = false;      // A counts angle pairs
};

// The packed-pair march (laue_pair.cuh) applies to compensated single
// precision with the fused segment phase or staged float2 e^{iH} rows, at
// two or more deviation parameters; DYFOX_FLAG_PAIRS selects it there (a
// cols_per_lane it does not have keeps the scalar march).
static bool use_pairs(const dyfox_laue_desc *d, const LauePlan &p,
                      const FastConfig &fc) {
    if (d->precision != DYFOX_FP32 || (d->flags & DYFOX_FLAG_NO_COMP) ||
        !(d->flags & DYFOX_FLAG_PAIRS) || (d->flags & DYFOX_FLAG_SCALAR) ||
        d->n_e < 2)
        return false;
    if (!(p.hsrc == HS_SEG || (p.hsrc == HS_CS32 && fc.stage == ST_DIRECT)))
        return false;
    if (d->cols_per_lane) {
        bool have = false;
        for (int i = 0; i < kNumCplPair; ++i)
            have = have || kCplPair[i] == d->cols_per_lane;
        if (!have) return false;
    }
    return true;
}

static int choose_fast(const dyfox_laue_desc *d, const LauePlan &p,
                       FastConfig *fc) {
    const bool single = d->precision == DYFOX_FP32;
    const bool comp = single && !(d->flags & DYFOX_FLAG_NO_COMP);
    const int ht_gen = p.hsrc != HS_SEG ? HT_GENERIC
                       : (single && (d->flags & DYFOX_FLAG_H_FP64)) ? HT_SEG64
                                                                    : HT_SEG;
    fc->pairs = use_pairs(d, p, *fc);
    // A source staged in the march's own precision, read in place: the
    // compile-time staged march (the pair march keeps its generic form).
    const int ht = (ht_gen == HT_GENERIC && fc->stage == ST_DIRECT &&
                    !fc->pairs) ? HT_STAGED : ht_gen;
    const int *cpls = fc->pairs ? kCplPair : single ? kCplF32 : kCplF64;
    const int ncpl = fc->pairs ? kNumCplPair : single ? kNumCplF32 : kNumCplF64;
    // Columns per lane: the fewest padded columns; ties go to more columns
    // per lane (fewer warps per angle).
    int best = -1, best_pad = 1 << 30;
    for (int i = 0; i < ncpl; ++i) {
        int c = cpls[i];
        if (d->cols_per_lane && c != d->cols_per_lane) continue;
        int wa = div_up(d->Nx, 32 * c);
        int pad = wa * 32 * c - d->Nx;
        if (wa > 32) continue;
        if (pad < best_pad || (pad == best_pad && c > best)) {
            best = c;
            best_pad = pad;
        }
    }
    if (best < 0) {
        set_error("no register-resident configuration for Nx=%d "
                  "(cols_per_lane=%d)", d->Nx, d->cols_per_lane);
        return DYFOX_ENOSYS;
    }
    fc->cpl = best;
    fc->WA = div_up(d->Nx, 32 * best);
    fc->entry = fc->pairs ? march_entry_f32_pair(best, ht)
                : single ? (comp ? march_entry_f32_comp(best, ht)
                                 : march_entry_f32_plain(best, ht))
                         : march_entry_f64(best, ht);
    if (!fc->entry.launch) {
        set_error("missing instantiation cpl=%d", best);
        return DYFOX_ENOSYS;
    }
    cudaFuncAttributes attr;
    cudaError_t e = fc->entry.attr(&attr);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncGetAttributes(march)");
    fc->regs = attr.numRegs;
    int max_threads = attr.maxThreadsPerBlock < 1024 ? attr.maxThreadsPerBlock
                                                     : 1024;
    int cap = 512 < max_threads ? 512 : max_threads;
    int amax = cap / (32 * fc->WA);
    if (amax < 1) amax = max_threads / (32 * fc->WA);
    if (amax < 1) {
        set_error("Nx=%d needs %d warps per angle, above the block limit",
                  d->Nx, fc->WA);
        return DYFOX_ENOSYS;
    }
    // Angles (pairs of angles for the pair march) per CTA.
    const int units = fc->pairs ? (d->n_e + 1) / 2 : d->n_e;
    int A = d->angles_per_cta > 0
                ? (fc->pairs ? (d->angles_per_cta + 1) / 2 : d->angles_per_cta)
                : units;
    if (A > amax) A = amax;
    if (A > units) A = units;
    if (A * 32 * fc->WA > max_threads) {
        set_error("angles_per_cta=%d exceeds the block limit", A);
        return DYFOX_EINVAL;
    }
    fc->A = A;
    fc->block = 32 * fc->WA * A;
    if (fc->pairs) {
        fc->smem = pair_smem(best, fc->WA, A, d->n_seg, p.hsrc == HS_SEG).total;
        return DYFOX_OK;
    }
    MarchSmem sm = single
        ? march_smem<float>(best, fc->WA, A, d->Nz, p.hsrc, d->n_seg, comp,
                            fc->stage, fc->raw_elem)
        : march_smem<double>(best, fc->WA, A, d->Nz, p.hsrc, d->n_seg, false,
                             fc->stage, fc->raw_elem);
    fc->smem = sm.total;
    return DYFOX_OK;
}

// CTAs of the chosen march resident on the whole device (0 when unknown):
// the blocks a multiprocessor holds by registers (allocated per warp in
// units of 256), shared memory (1 KB reserved a block), threads and the
// 32-block limit, times the multiprocessor count.
static int resident_ctas(const FastConfig &fc) {
    int dev = 0, sms = 0, smem_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm,
                               cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                               dev) != cudaSuccess ||
        fc.regs <= 0 || fc.block <= 0)
        return 0;
    const int warps = (fc.block + 31) / 32;
    const int warp_regs = (fc.regs * 32 + 255) / 256 * 256;
    int per = 65536 / (warp_regs * warps);
    const int by_smem = (int)((size_t)smem_sm / (fc.smem + 1024));
    if (by_smem < per) per = by_smem;
    if (2048 / fc.block < per) per = 2048 / fc.block;
    if (per > 32) per = 32;
    return per > 0 ? per * sms : 0;
}

// Staging mode of a grid source: rows are copied with 16-byte cp.async, so
// the base must be 16-byte aligned and a row a multiple of 16 bytes.
static void choose_stage(const dyfox_laue_desc *d, const LauePlan &p,
                         const void *base, FastConfig *fc) {
    const bool single = d->precision == DYFOX_FP32;
    fc->stage = ST_COMPUTE;
    fc->raw_elem = 0;
    int elem = 0;
    switch (p.hsrc) {
    case HS_GRID64: elem = 8; break;
    case HS_GRID32: elem = 4; break;
    case HS_CS32: elem = 8; break;
    case HS_CS64: elem = 16; break;
    default: return;
    }
    if (((uintptr_t)base & 15) || ((size_t)d->Nx * elem) % 16) return;
    fc->raw_elem = elem;
    fc->stage = ((p.hsrc == HS_CS32 && single) || (p.hsrc == HS_CS64 && !single))
                    ? ST_DIRECT : ST_CONVERT;
}

static int smem_limit(size_t need) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&optin,
                                   cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return cuda_status(e, "device query");
    if (need > (size_t)optin) {
        set_error("kernel needs %zu bytes of shared memory per block, the device "
                  "allows %d", need, optin);
        return DYFOX_ESMEM;
    }
    return DYFOX_OK;
}

// ---------------------------------------------------------------------------
// Pieces of a solve used by the batched launcher (batch.cu).
int laue_check_desc(const dyfox_laue_desc *d) { return validate(d); }

void laue_active_rows(const dyfox_laue_desc *d, int *row0, int *n_rows) {
    active_rows(d, row0, n_rows);
}

cudaError_t launch_laue_setup(const dyfox_laue_desc *d, const double *s_dev,
                              Kappa *kappa, float4 *kappa32, double2 *scale,
                              float4 *kpair, cudaStream_t stream) {
    const int nsteps = d->Nz - 1;
    const long n = (long)d->n_e * nsteps;
    laue_setup_kernel<<<(int)((n + 255) / 256), 256, 0, stream>>>(
        s_dev, d->n_e, nsteps, d->ds, d->sig0[0], d->sig0[1], d->sig_h[0],
        d->sig_h[1], d->sig_hbar[0], d->sig_hbar[1], kappa, kappa32, scale,
        reinterpret_cast<float *>(kpair));
    count_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_zero_rows(const dyfox_laue_desc *d, void *out, size_t elem,
                             int row0, int n_rows, cudaStream_t stream) {
    if (n_rows >= d->Ny) return cudaSuccess;
    const size_t row_bytes = (size_t)d->Nx * elem;
    const long pairs = (long)d->n_e * (d->Ny - n_rows);
    const int grid = pairs < 152L * 16 ? (int)pairs : 152 * 16;
    zero_rows_kernel<<<grid, 256, 0, stream>>>((char *)out, d->n_e, d->Ny,
                                               row_bytes, row0, n_rows);
    count_launch(1);
    return cudaGetLastError();
}

}  // namespace dyfox

using namespace dyfox;

extern "C" size_t dyfox_laue_workspace_bytes(const dyfox_laue_desc *d) {
    LauePlan p;
    if (make_plan(d, &p)) return 0;
    return p.ws;
}

// The solve of dyfox_laue_solve and dyfox_laue_solve_to_host.  host_out
// non-NULL: the active rows are marched in n_chunks row chunks (0: about
// 8, in whole waves of CTAs), all
// deviation parameters in one launch per chunk, and after each chunk's
// march its rows of every wave are copied into host_out on copy_stream,
// behind an event on `stream`.
static int laue_solve_impl(const dyfox_laue_desc *d, const double *s_dev,
                           const void *h_grid, const double *seg_table,
                           void *out, void *workspace,
                           size_t workspace_bytes, void *stream_,
                           void *host_out, int n_chunks,
                           cudaStream_t copy_stream) {
    set_error("");
    LauePlan p;
    int st = make_plan(d, &p);
    if (st) return st;
    if (!s_dev || !out) {
        set_error("s_dev and out must be device pointers");
        return DYFOX_EINVAL;
    }
    if ((d->h_source == DYFOX_H_GRID_F64 || d->h_source == DYFOX_H_GRID_F32) &&
        !h_grid) {
        set_error("h_source is a grid but h_grid is NULL");
        return DYFOX_EINVAL;
    }
    if (d->h_source == DYFOX_H_SEGMENTS && d->n_seg > 0 && !seg_table) {
        set_error("h_source is segments but seg_table is NULL");
        return DYFOX_EINVAL;
    }
    if (workspace_bytes < p.ws || (p.ws && !workspace)) {
        set_error("workspace of %zu bytes, %zu needed", workspace_bytes, p.ws);
        return DYFOX_ENOMEM;
    }
    cudaStream_t stream = (cudaStream_t)stream_;
    const bool single = d->precision == DYFOX_FP32;
    const size_t elem = single ? sizeof(float2) : sizeof(double2);
    char *ws = (char *)workspace;
    const int nsteps = d->Nz - 1;

    MarchArgs a;
    memset(&a, 0, sizeof a);
    a.Nx = d->Nx; a.Ny = d->Ny; a.Nz = d->Nz; a.n_e = d->n_e;
    a.row0 = p.row0; a.n_rows = p.n_rows;
    a.dx = d->dx; a.dz = d->dz; a.sheet_hw = d->sheet_hw;
    a.hsrc = p.hsrc;
    a.hgrid = h_grid;
    a.segs = seg_table;
    a.n_seg = d->h_source == DYFOX_H_SEGMENTS ? d->n_seg : 0;
    a.vc = volterra_consts(d->nu, d->a_core);
    memcpy(a.an, d->analytic, sizeof a.an);
    a.kappa = (const Kappa *)(ws + p.off_kappa);
    a.kappa32 = (const float4 *)(ws + p.off_k32);
    a.scale = (const double2 *)(ws + p.off_scale);
    a.out = out;
    a.csgrid = ws + p.off_stage;
    a.piv = (const float4 *)(ws + p.off_piv);
    a.kpair = single ? (const float4 *)(ws + p.off_kpair) : nullptr;
    a.err = (int *)(ws + p.off_err);

    cudaError_t e;
    // Rows [r0, r0 + nr) of every angle of out into host_out on
    // copy_stream, after the work queued so far on `stream` (one strided
    // copy: n_e slices of nr rows).
    auto copy_rows = [&](int r0, int nr) -> int {
        if (!host_out || nr <= 0) return DYFOX_OK;
        cudaEvent_t ev;
        cudaError_t ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (ce) return cuda_status(ce, "copy event");
        ce = cudaEventRecord(ev, stream);
        if (!ce) ce = cudaStreamWaitEvent(copy_stream, ev, 0);
        if (!ce) {
            const size_t pitch = (size_t)d->Nx * elem;
            cudaMemcpy3DParms cp;
            memset(&cp, 0, sizeof cp);
            cp.srcPtr = make_cudaPitchedPtr(out, pitch, d->Nx, d->Ny);
            cp.dstPtr = make_cudaPitchedPtr(host_out, pitch, d->Nx, d->Ny);
            cp.srcPos = make_cudaPos(0, (size_t)r0, 0);
            cp.dstPos = make_cudaPos(0, (size_t)r0, 0);
            cp.extent = make_cudaExtent(pitch, (size_t)nr, (size_t)d->n_e);
            cp.kind = cudaMemcpyDeviceToHost;
            ce = cudaMemcpy3DAsync(&cp, copy_stream);
        }
        cudaEventDestroy(ev);
        return ce ? cuda_status(ce, "exit-wave copy") : DYFOX_OK;
    };
    laue_mark(0, stream);
    // Rows outside the beam are zero; kappa tables; pivots (one launch).
    {
        PrologueArgs pa;
        memset(&pa, 0, sizeof pa);
        pa.out = (char *)out; pa.n_e = d->n_e; pa.Ny = d->Ny;
        pa.row_bytes = (size_t)d->Nx * elem; pa.row0 = p.row0;
        pa.n_rows = p.n_rows;
        pa.s_dev = s_dev; pa.nsteps = nsteps;
        pa.ds = d->ds; pa.s0r = d->sig0[0]; pa.s0i = d->sig0[1];
        pa.shr = d->sig_h[0]; pa.shi = d->sig_h[1];
        pa.sbr = d->sig_hbar[0]; pa.sbi = d->sig_hbar[1];
        pa.kappa = (Kappa *)(ws + p.off_kappa);
        pa.kappa32 = (float4 *)(ws + p.off_k32);
        pa.scale = (double2 *)(ws + p.off_scale);
        pa.kpair = single ? (float *)(ws + p.off_kpair) : nullptr;
        pa.segs = seg_table; pa.n_seg = d->n_seg; pa.Nx = d->Nx;
        pa.dx = d->dx; pa.dz = d->dz; pa.piv = (float4 *)(ws + p.off_piv);
        pa.err = (int *)(ws + p.off_err);
        const long zpairs = p.n_rows < d->Ny ? (long)d->n_e * (d->Ny - p.n_rows)
                                              : 0;
        pa.nz = (int)(zpairs < 152L * 16 ? zpairs : 152L * 16);
        pa.ns = p.n_rows ? (int)(((long)d->n_e * nsteps + 255) / 256) : 0;
        long pv = 0;
        if (p.n_rows && p.hsrc == HS_SEG && single) {
            pv = ((long)p.n_rows * nsteps * d->n_seg + 255) / 256;
            if (pv > 152L * 32) pv = 152L * 32;
        }
        pa.np = (int)pv;
        const int blocks = pa.nz + pa.ns + pa.np;
        if (blocks > 0) {
            laue_prologue_kernel<<<blocks, 256, 0, stream>>>(pa);
            count_launch(1);
            if ((e = cudaGetLastError())) return cuda_status(e, "prologue");
        } else if ((e = cudaMemsetAsync(pa.err, 0, sizeof(int), stream))) {
            return cuda_status(e, "status reset");
        }
    }
    laue_mark(1, stream);
    // the rows outside the beam (zero) go to the host at once
    if ((st = copy_rows(0, p.row0))) return st;
    if ((st = copy_rows(p.row0 + p.n_rows, d->Ny - p.row0 - p.n_rows)))
        return st;
    if (p.n_rows == 0) {
        laue_mark(2, stream);
        laue_mark(3, stream);
        return DYFOX_OK;
    }
    if (p.stage) {
        e = launch_cs_stage(single, (d->flags & DYFOX_FLAG_H_FP64) != 0,
                            seg_table, d->n_seg, d->Nx, d->Ny,
                            d->Nz, d->dx, d->dz, a.vc, p.row0, p.n_rows,
                            ws + p.off_stage, stream);
        if (e) return cuda_status(e, "cs_stage");
    }
    laue_mark(2, stream);

    if (p.general) {
        size_t smem = ((2 * 4 * (size_t)(d->Nx + 1) * (single ? 4 : 8) + 15) &
                       ~(size_t)15) +
                      (p.hsrc == HS_ANALYTIC ? (size_t)d->Nz * elem : 0);
        if ((st = smem_limit(smem))) return st;
        a.n_groups = d->n_e;
        a.A = 1;
        int grid = p.n_rows * d->n_e;
        if (single) {
            auto *k = laue_general_kernel<float>;
            if (smem > 48 * 1024 &&
                (e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem)))
                return cuda_status(e, "general smem");
            k<<<grid, 256, smem, stream>>>(a, (float)d->shift_px);
            count_launch(1);
        } else {
            auto *k = laue_general_kernel<double>;
            if (smem > 48 * 1024 &&
                (e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem)))
                return cuda_status(e, "general smem");
            k<<<grid, 256, smem, stream>>>(a, d->shift_px);
            count_launch(1);
        }
        if ((e = cudaGetLastError())) return cuda_status(e, "laue_general");
        laue_mark(3, stream);
        return copy_rows(p.row0, p.n_rows);
    }

    FastConfig fc;
    choose_stage(d, p, p.stage ? (const void *)a.csgrid : h_grid, &fc);
    if ((st = choose_fast(d, p, &fc))) return st;
    if ((st = smem_limit(fc.smem))) return st;
    a.WA = fc.WA;
    a.A = fc.A;
    a.ncols = 32 * fc.WA * fc.cpl;
    a.stage = fc.stage;
    a.raw_elem = fc.raw_elem;
    a.n_groups = div_up(fc.pairs ? (d->n_e + 1) / 2 : d->n_e, fc.A);
    // Row chunks (copies to the host), else one launch; the row-relative
    // tables (staged e^{iH}, pivots) start at the chunk's first row.
    int nc = host_out ? (n_chunks > 0 ? n_chunks : 8) : 1;
    if (nc > 64) nc = 64;
    if (nc > p.n_rows / 8) nc = p.n_rows / 8 > 1 ? p.n_rows / 8 : 1;
    int rc = div_up(p.n_rows, nc);
    if (nc > 1 && n_chunks <= 0) {
        // Chunks of whole waves of CTAs (the remainder rows last, so that
        // the copy left after the march is short).
        const int wave = resident_ctas(fc);
        if (wave > 0) {
            int g = a.n_groups, w = wave;
            while (w) { const int t = g % w; g = w; w = t; }
            const int unit = wave / g;           // rows per whole wave
            if (unit <= p.n_rows / 4) {
                const int want = p.n_rows / nc;
                rc = unit * (want / unit > 0 ? want / unit : 1);
            }
        }
    }
    const size_t stage_row = (size_t)nsteps * d->Nx * elem;
    for (int r0 = 0; r0 < p.n_rows; r0 += rc) {
        const int nr = p.n_rows - r0 < rc ? p.n_rows - r0 : rc;
        MarchArgs ac = a;
        ac.row0 = p.row0 + r0;
        ac.n_rows = nr;
        if (p.stage) ac.csgrid = ws + p.off_stage + (size_t)r0 * stage_row;
        ac.piv = a.piv + (size_t)r0 * nsteps * d->n_seg;
        e = fc.entry.launch(ac, nr * ac.n_groups, fc.block, fc.smem, stream);
        if (e) return cuda_status(e, "laue_march");
        if ((st = copy_rows(p.row0 + r0, nr))) return st;
    }
    laue_mark(3, stream);
    return DYFOX_OK;
}

extern "C" int dyfox_laue_solve(const dyfox_laue_desc *d, const double *s_dev,
                                const void *h_grid, const double *seg_table,
                                void *out, void *workspace,
                                size_t workspace_bytes, void *stream) {
    return laue_solve_impl(d, s_dev, h_grid, seg_table, out, workspace,
                           workspace_bytes, stream, nullptr, 0, nullptr);
}

extern "C" int dyfox_laue_solve_status(const dyfox_laue_desc *d,
                                       const void *workspace,
                                       size_t workspace_bytes, void *stream) {
    set_error("");
    LauePlan p;
    int st = make_plan(d, &p);
    if (st) return st;
    if (!workspace || workspace_bytes < p.ws) {
        set_error("workspace of %zu bytes, %zu needed", workspace_bytes, p.ws);
        return DYFOX_ENOMEM;
    }
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, (const char *)workspace + p.off_err,
                                    sizeof(int), cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (!e) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e) return cuda_status(e, "solve status");
    if (err) {
        set_error("a staged row's copy into shared memory did not complete "
                  "within its bounded wait; its exit waves read NaN");
        return DYFOX_ETIMEOUT;
    }
    return DYFOX_OK;
}

extern "C" int dyfox_laue_solve_to_host(
    const dyfox_laue_desc *d, const double *s_dev, const void *h_grid,
    const double *seg_table, void *out, void *host_out, void *workspace,
    size_t workspace_bytes, int n_chunks, void *stream,
    void *copy_stream) {
    if (!host_out) {
        set_error("host_out must be host memory (pinned for the copies to "
                  "overlap the march)");
        return DYFOX_EINVAL;
    }
    return laue_solve_impl(d, s_dev, h_grid, seg_table, out, workspace,
                           workspace_bytes, stream, host_out, n_chunks,
                           copy_stream ? (cudaStream_t)copy_stream
                                       : (cudaStream_t)stream);
}
