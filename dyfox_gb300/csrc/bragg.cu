// Bragg (reflection) shooting solve: couplings, the perfect-crystal
// symbol, and one persistent GMRES per system (y-plane x deviation
// parameter), replacing DYFOX bragg/solver.py:28-60 and 135-379.
//
// Shooting form (bragg/solver.py:1-20): march D0, Dg down from z = 0 with
// D_g(0) = v unknown; the back-face condition D_g(t) = 0 gives A v = -d,
// A v = march(0, v), d = march(incident, 0).  Each system is solved with
// restarted GMRES, left-preconditioned by M w = ifft(fft(w) / T22s), in the
// published algorithm of SciPy 1.18's scipy.sparse.linalg.gmres (modified
// Gram-Schmidt Arnoldi, Givens rotations (LAPACK lartg), adaptive inner
// tolerance, true residual at every restart).  The exit wave is
// v e^{-iH(z=0)}.
//
// Precision DYFOX_FP32 is a mixed-precision form of the same solve: the
// Arnoldi products (march and preconditioner) run in single precision, b
// and every true residual come from a float-float march (FP64-class, at a
// fraction of the double pipe's time), and the Gram-Schmidt coefficients,
// the Givens rotations and the solution stay in double.  Each restart is
// then one step of iterative refinement on that residual, so the solve
// still stops at true relative residual <= tol; a restart cycle
// stops its inner iteration once the estimated residual has dropped by
// kMixedInnerDrop, below which the single-precision operator's own error
// makes further inner steps useless.  A system the mixed solve does not
// converge within maxiter restarts (single precision not accurate enough
// for it) is finished in double, from the solution reached, by a separate
// resume launch.  The test sits after the restart loop: any test inside it
// (of the cycle's true-residual reduction) measured 30% slower on the 20 um
// Bragg scan (Nx 456, Nz 90, 21 x 64 systems) even when it never fired.
#include <math.h>
#include <string.h>

#include "bragg_solve.cuh"

namespace dyfox {


// Couplings of every plane: cb = ds (sigma_hbar e^{+iH}), ch = ds (sigma_h
// e^{-iH}) with H the Volterra phase at (x_i, y_p, z_k) summed in segment
// order; e0h = e^{-iH} at k = 0.  One thread per voxel.
// cb32, ch32 (may be NULL): the couplings of the mixed form's depth-scaled
// march, e0^-k cb and e0^k ch with e0^k = exp(k s0 ds) formed in double,
// rounded to float; cbl32, chl32: the remainders, rounded to float
// (float-float couplings).
__global__ void bragg_couple_kernel(const double *__restrict__ segs,
                                    int n_seg, int Nx, int Nz, double dx,
                                    double dz, VolterraConsts vc,
                                    const double *__restrict__ y, int n_y,
                                    double ds, double s0r, double s0i,
                                    double shr, double shi,
                                    double sbr, double sbi, double2 *cb,
                                    double2 *ch, double2 *e0h, float2 *cb32,
                                    float2 *ch32, float2 *cbl32,
                                    float2 *chl32) {
    const long total = (long)n_y * Nz * Nx;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
         idx += (long)gridDim.x * blockDim.x) {
        const int x = (int)(idx % Nx);
        const long t = idx / Nx;
        const int k = (int)(t % Nz);
        const int p = (int)(t / Nz);
        const double X0 = __dmul_rn((double)x - 0.5 * Nx, dx);
        const double zv = __dmul_rn((double)k, dz);
        double H = 0.0;
        for (int s = 0; s < n_seg; ++s) {
            const double *sg = segs + (size_t)s * DYFOX_SEG_STRIDE;
            H = __dadd_rn(H, h_seg_f64(sg, __dsub_rn(X0, __ldg(sg + SEG_CX)),
                                       __dsub_rn(y[p], __ldg(sg + SEG_CY)),
                                       __dsub_rn(zv, __ldg(sg + SEG_CZ)), vc));
        }
        double sn, c;
        sincos(H, &sn, &c);
        // sigma e^{-+iH}, then ds times each part (solver.py:260-261, 31-32)
        const double2 a = make_double2(shr * c + shi * sn, shi * c - shr * sn);
        const double2 b = make_double2(sbr * c - sbi * sn, sbi * c + sbr * sn);
        const double2 vb = make_double2(ds * b.x, ds * b.y);
        const double2 vh = make_double2(ds * a.x, ds * a.y);
        cb[idx] = vb;
        ch[idx] = vh;
        if (cb32) {
            // e0^k = m (cos q, sin q); e0^-k = (cos q, -sin q) / m
            const double m = exp(k * s0r * ds);
            double sq, cq;
            sincos(k * s0i * ds, &sq, &cq);
            const double im = 1.0 / m;
            const double2 fb = make_double2(im * (vb.x * cq + vb.y * sq),
                                            im * (vb.y * cq - vb.x * sq));
            const double2 fh = make_double2(m * (vh.x * cq - vh.y * sq),
                                            m * (vh.y * cq + vh.x * sq));
            const float2 b32 = make_float2((float)fb.x, (float)fb.y);
            const float2 h32 = make_float2((float)fh.x, (float)fh.y);
            cb32[idx] = b32;
            ch32[idx] = h32;
            cbl32[idx] = make_float2((float)(fb.x - (double)b32.x),
                                     (float)(fb.y - (double)b32.y));
            chl32[idx] = make_float2((float)(fh.x - (double)h32.x),
                                     (float)(fh.y - (double)h32.y));
        }
        if (k == 0) e0h[(size_t)p * Nx + x] = make_double2(c, -sn);
    }
}

// exp(-2 pi i m / N) for m in [0, N); tw32 (may be NULL) rounded to float.
__global__ void twiddle_kernel(double2 *tw, float2 *tw32, int N) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= N) return;
    double sn, c;
    sincospi(-2.0 * m / N, &sn, &c);
    tw[m] = make_double2(c, sn);
    if (tw32) tw32[m] = make_float2((float)c, (float)sn);
}

// perfect_symbol (bragg/solver.py:38-60): per Fourier mode the 2 x 2 chain
// of the unstrained down-march; T22 floored at 1e-8 max|T22| (164-165,
// 277-278) and inverted into iT (and into iT32, rounded to float, when
// not NULL).  One CTA per deviation parameter.
__global__ void bragg_symbol_kernel(const double *__restrict__ s_dev, int Nx,
                                    int Nz, double ds, double s0r, double s0i,
                                    double shr, double shi, double sbr,
                                    double sbi, double2 *T21, double2 *T22,
                                    double2 *iT, float2 *iT32) {
    __shared__ double2 red[33];
    const int is = blockIdx.x;
    const double alpha = -2.0 * kPi * s_dev[is];
    const double er = exp(s0r * ds);
    double sn, c;
    sincos(s0i * ds, &sn, &c);
    const double2 e0 = make_double2(er * c, er * sn);
    sincos((s0i + alpha) * ds, &sn, &c);
    const double2 eg = make_double2(er * c, er * sn);
    const double2 ieg = make_double2(c / er, -sn / er);
    const double2 sh = make_double2(shr, shi), sb = make_double2(sbr, sbi);
    double mx = 0.0;
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        // fftfreq: m = x for x < ceil(N/2), else x - N
        const int m = x < (Nx + 1) / 2 ? x : x - Nx;
        double ps, pc;
        sincospi(-2.0 * m / Nx, &ps, &pc);
        const double2 p = make_double2(pc, ps), pi = make_double2(pc, -ps);
        const double2 a11 = cmulz(e0, p);
        const double2 a12 = cmulz(cscale(ds, a11), sb);
        const double2 a21 = cmulz(cmulz(cscale(-ds, pi), sh), ieg);
        const double2 a22 = cmulz(pi, ieg);
        double2 t11 = make_double2(1, 0), t12 = make_double2(0, 0);
        double2 t21 = make_double2(0, 0), t22 = make_double2(1, 0);
        for (int k = 0; k < Nz - 1; ++k) {
            const double2 n11 = cadd(cmulz(a11, t11), cmulz(a12, t21));
            const double2 n12 = cadd(cmulz(a11, t12), cmulz(a12, t22));
            const double2 n21 = cadd(cmulz(a21, t11), cmulz(a22, t21));
            const double2 n22 = cadd(cmulz(a21, t12), cmulz(a22, t22));
            t11 = n11; t12 = n12; t21 = n21; t22 = n22;
        }
        if (T21) T21[(size_t)is * Nx + x] = t21;
        if (T22) T22[(size_t)is * Nx + x] = t22;
        if (iT) iT[(size_t)is * Nx + x] = t22;
        mx = fmax(mx, hypot(t22.x, t22.y));
    }
    (void)eg;
    if (!iT) return;
    const double floor_ = 1e-8 * block_max(mx, red);
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        double2 t = iT[(size_t)is * Nx + x];
        if (hypot(t.x, t.y) < floor_) t = make_double2(floor_, 0.0);
        const double d = t.x * t.x + t.y * t.y;
        const double2 v = make_double2(t.x / d, -t.y / d);
        iT[(size_t)is * Nx + x] = v;
        if (iT32)
            iT32[(size_t)is * Nx + x] = make_float2((float)v.x, (float)v.y);
    }
}

// ---------------------------------------------------------------------------

struct BraggPlan {
    int threads, cpl;
    bool mixed;
    size_t off_cb, off_ch, off_e0h, off_inc, off_iT, off_tw, off_y;
    size_t off_cb32, off_ch32, off_cbl32, off_chl32, off_iT32, off_tw32;
    size_t off_V, off_H, off_X, off_B, off_info, ws;
};

static size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

static int bragg_validate(const dyfox_bragg_desc *d) {
    if (!d) { set_error("descriptor is NULL"); return DYFOX_EINVAL; }
    if (d->Nx < 2 || d->Nz < 2 || d->n_y < 1 || d->n_s < 1 || d->n_seg < 0) {
        set_error("bad sizes Nx=%d Nz=%d n_y=%d n_s=%d n_seg=%d", d->Nx, d->Nz,
                  d->n_y, d->n_s, d->n_seg);
        return DYFOX_EINVAL;
    }
    if (d->Nx > 16 * 256) {
        set_error("Nx=%d above the supported 4096", d->Nx);
        return DYFOX_ENOSYS;
    }
    if (!(d->ds > 0) || !(d->dx > 0) || !(d->dz > 0) || !(d->tol > 0) ||
        d->restart < 1 || d->maxiter < 1 || d->restart > 1024) {
        set_error("bad scalars ds=%g dx=%g dz=%g tol=%g restart=%d maxiter=%d",
                  d->ds, d->dx, d->dz, d->tol, d->restart, d->maxiter);
        return DYFOX_EINVAL;
    }
    if (d->precision != DYFOX_FP64 && d->precision != DYFOX_FP32) {
        set_error("precision %d is neither DYFOX_FP64 nor DYFOX_FP32",
                  d->precision);
        return DYFOX_EINVAL;
    }
    if (d->flags & ~DYFOX_BRAGG_FORCE_RESUME) {
        set_error("unknown Bragg flags 0x%x", d->flags);
        return DYFOX_EINVAL;
    }
    return DYFOX_OK;
}

static int bragg_plan(const dyfox_bragg_desc *d, BraggPlan *p) {
    int st = bragg_validate(d);
    if (st) return st;
    const size_t Nx = d->Nx, plane = (size_t)d->Nz * Nx * sizeof(double2);
    const size_t nsys = (size_t)d->n_y * d->n_s;
    const int m = d->restart;
    // Columns per thread of the march: a power of two <= 16 (Nx <= 4096);
    // 256 threads at most, so that the 16-column kernels (up to 255
    // registers a thread) stay resident.
    p->threads = Nx <= 512 ? 128 : 256;
    p->cpl = (int)((Nx + p->threads - 1) / p->threads);
    int c = 1;
    while (c < p->cpl) c *= 2;
    p->cpl = c;
    size_t o = 0;
    p->off_cb = o; o = a256(o + d->n_y * plane);
    p->off_ch = o; o = a256(o + d->n_y * plane);
    p->off_e0h = o; o = a256(o + d->n_y * Nx * sizeof(double2));
    p->off_inc = o; o = a256(o + Nx * sizeof(double2));
    p->off_iT = o; o = a256(o + d->n_s * Nx * sizeof(double2));
    p->off_tw = o; o = a256(o + Nx * sizeof(double2));
    p->off_y = o; o = a256(o + d->n_y * sizeof(double));
    p->mixed = d->precision == DYFOX_FP32;
    const size_t f32 = p->mixed ? 1 : 0;
    const size_t plane32 = (size_t)d->Nz * Nx * sizeof(float2) * f32;
    p->off_cb32 = o; o = a256(o + d->n_y * plane32);
    p->off_ch32 = o; o = a256(o + d->n_y * plane32);
    p->off_cbl32 = o; o = a256(o + d->n_y * plane32);
    p->off_chl32 = o; o = a256(o + d->n_y * plane32);
    p->off_iT32 = o; o = a256(o + f32 * d->n_s * Nx * sizeof(float2));
    p->off_tw32 = o; o = a256(o + f32 * Nx * sizeof(float2));
    p->off_V = o; o = a256(o + nsys * (m + 1) * Nx * sizeof(double2));
    p->off_H = o; o = a256(o + nsys * m * (m + 1) * sizeof(double2));
    p->off_X = o; o = a256(o + nsys * Nx * sizeof(double2));
    p->off_B = o; o = a256(o + nsys * Nx * sizeof(double2));
    p->off_info = o; o = a256(o + nsys * 4 * sizeof(double));
    p->ws = o;
    return DYFOX_OK;
}

__global__ void incident_kernel(double2 *inc, int Nx, double dx, int beam,
                                double thickness, double centre) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= Nx) return;
    double v = 1.0;
    if (beam) {
        const double xp = (x - Nx / 2.0) * dx;
        v = fabs(xp - centre) < 0.5 * thickness ? 1.0 : 0.0;
    }
    inc[x] = make_double2(v, 0.0);
}

// Couplings, incident beam, twiddles and the preconditioner for `d`.
// y_src: the planes' y, on the host (copied into the workspace), or on the
// device when y_on_device.
static int bragg_prepare(const dyfox_bragg_desc *d, const BraggPlan &p,
                         const double *seg_table, const double *y_src,
                         bool y_on_device, const double *s_dev, char *ws,
                         cudaStream_t stream, BraggArgs *a) {
    memset(a, 0, sizeof *a);
    a->Nx = d->Nx; a->Nz = d->Nz; a->n_y = d->n_y; a->n_s = d->n_s;
    a->ds = d->ds;
    a->s0r = d->sig0[0]; a->s0i = d->sig0[1];
    a->shr = d->sig_h[0]; a->shi = d->sig_h[1];
    a->sbr = d->sig_hbar[0]; a->sbi = d->sig_hbar[1];
    a->s_dev = s_dev;
    a->cb = (double2 *)(ws + p.off_cb);
    a->ch = (double2 *)(ws + p.off_ch);
    a->e0h = (double2 *)(ws + p.off_e0h);
    a->inc = (double2 *)(ws + p.off_inc);
    a->iT = (double2 *)(ws + p.off_iT);
    a->tw = (double2 *)(ws + p.off_tw);
    if (p.mixed) {
        a->cb32 = (const float2 *)(ws + p.off_cb32);
        a->ch32 = (const float2 *)(ws + p.off_ch32);
        a->cbl32 = (const float2 *)(ws + p.off_cbl32);
        a->chl32 = (const float2 *)(ws + p.off_chl32);
        a->iT32 = (const float2 *)(ws + p.off_iT32);
        a->tw32 = (const float2 *)(ws + p.off_tw32);
    }
    a->plan = make_fft_plan(d->Nx);
    a->V = (double2 *)(ws + p.off_V);
    a->Hh = (double2 *)(ws + p.off_H);
    a->X = (double2 *)(ws + p.off_X);
    a->B = (double2 *)(ws + p.off_B);
    a->info = (double *)(ws + p.off_info);
    a->tol = d->tol;
    a->restart = d->restart;
    a->maxiter = d->maxiter;
    a->force_resume = (d->flags & DYFOX_BRAGG_FORCE_RESUME) ? 1 : 0;
    cudaError_t e;
    const double *y = y_src;
    if (!y_on_device) {
        double *yw = (double *)(ws + p.off_y);
        if ((e = cudaMemcpyAsync(yw, y_src, sizeof(double) * d->n_y,
                                 cudaMemcpyHostToDevice, stream)))
            return cuda_status(e, "y upload");
        y = yw;
    }
    const long total = (long)d->n_y * d->Nz * d->Nx;
    long blocks = (total + 255) / 256;
    if (blocks > 152L * 64) blocks = 152L * 64;
    bragg_couple_kernel<<<(int)blocks, 256, 0, stream>>>(
        seg_table, d->n_seg, d->Nx, d->Nz, d->dx, d->dz,
        volterra_consts(d->nu, d->a_core), y, d->n_y, d->ds, a->s0r, a->s0i,
        a->shr, a->shi,
        a->sbr, a->sbi, (double2 *)a->cb, (double2 *)a->ch, (double2 *)a->e0h,
        (float2 *)a->cb32, (float2 *)a->ch32, (float2 *)a->cbl32,
        (float2 *)a->chl32);
    incident_kernel<<<div_up(d->Nx, 256), 256, 0, stream>>>(
        (double2 *)a->inc, d->Nx, d->dx, d->beam, d->beam_thickness,
        d->beam_centre);
    twiddle_kernel<<<div_up(d->Nx, 256), 256, 0, stream>>>(
        (double2 *)a->tw, (float2 *)a->tw32, d->Nx);
    bragg_symbol_kernel<<<d->n_s, 256, 0, stream>>>(
        s_dev, d->Nx, d->Nz, d->ds, a->s0r, a->s0i, a->shr, a->shi, a->sbr,
        a->sbi, nullptr, nullptr, (double2 *)a->iT, (float2 *)a->iT32);
    count_launch(4);
    return cuda_status(cudaGetLastError(), "bragg prepare");
}

// Dynamic shared memory of the batch kernel, and a check that one CTA fits
// (before any launch or capture).
cudaError_t set_bragg_batch_smem(int cpl, bool mixed, size_t smem,
                                 int threads) {
    return mixed ? bragg_batch_smem32(cpl, smem, threads)
                 : bragg_batch_smem64(cpl, smem, threads);
}

cudaError_t launch_bragg_batch(const BraggArgs *insts, const int2 *systems,
                               int n_sys, int threads, int cpl, bool mixed,
                               size_t smem, cudaStream_t stream) {
    if (n_sys == 0) return cudaSuccess;
    return mixed ? bragg_batch_launch32(insts, systems, n_sys, threads, cpl,
                                        smem, stream)
                 : bragg_batch_launch64(insts, systems, n_sys, threads, cpl,
                                        smem, stream);
}

// Workspace bytes, threads and columns per thread of one instance
// (0 bytes: invalid descriptor, error set).
size_t bragg_instance_bytes(const dyfox_bragg_desc *d, int *threads,
                            int *cpl) {
    BraggPlan p;
    if (bragg_plan(d, &p)) return 0;
    if (threads) *threads = p.threads;
    if (cpl) *cpl = p.cpl;
    return p.ws;
}

size_t bragg_instance_smem(const dyfox_bragg_desc *d) {
    return gmres_smem(d->Nx, d->restart);
}

// Set-up kernels of one instance on `stream` (y already on the device) and
// its arguments; out / info are the instance's results (info NULL: kept in
// the workspace).
int bragg_instance_prepare(const dyfox_bragg_desc *d, const double *seg_table,
                           const double *y_dev, const double *s_dev,
                           void *out, double *info, char *ws,
                           cudaStream_t stream, BraggArgs *a) {
    BraggPlan p;
    int st = bragg_plan(d, &p);
    if (st) return st;
    if ((st = bragg_prepare(d, p, seg_table, y_dev, true, s_dev, ws, stream,
                            a)))
        return st;
    a->out = (double2 *)out;
    if (info) a->info = info;
    return DYFOX_OK;
}

static int smem_ok(size_t need) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (!e) e = cudaDeviceGetAttribute(&optin,
                                       cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e) return cuda_status(e, "device query");
    if (need > (size_t)optin) {
        set_error("Bragg kernel needs %zu bytes of shared memory, the device "
                  "allows %d", need, optin);
        return DYFOX_ESMEM;
    }
    return DYFOX_OK;
}

}  // namespace dyfox

using namespace dyfox;

extern "C" size_t dyfox_bragg_workspace_bytes(const dyfox_bragg_desc *d) {
    BraggPlan p;
    if (bragg_plan(d, &p)) return 0;
    return p.ws;
}

extern "C" int dyfox_bragg_solve(const dyfox_bragg_desc *d,
                                 const double *seg_table,
                                 const double *y_values, const double *s_dev,
                                 const void *x0, void *out, double *info,
                                 void *workspace, size_t workspace_bytes,
                                 void *stream_) {
    set_error("");
    BraggPlan p;
    int st = bragg_plan(d, &p);
    if (st) return st;
    if (!y_values || !s_dev || !out || (d->n_seg > 0 && !seg_table)) {
        set_error("NULL argument to dyfox_bragg_solve");
        return DYFOX_EINVAL;
    }
    if (workspace_bytes < p.ws || !workspace) {
        set_error("workspace of %zu bytes, %zu needed", workspace_bytes, p.ws);
        return DYFOX_ENOMEM;
    }
    const size_t smem = gmres_smem(d->Nx, d->restart);
    if ((st = smem_ok(smem))) return st;
    cudaStream_t stream = (cudaStream_t)stream_;
    char *ws = (char *)workspace;
    BraggArgs a;
    if ((st = bragg_prepare(d, p, seg_table, y_values, false, s_dev, ws,
                            stream, &a)))
        return st;
    const size_t nsys = (size_t)d->n_y * d->n_s;
    cudaError_t e;
    if (x0) {
        if ((e = cudaMemcpyAsync(a.X, x0, nsys * d->Nx * sizeof(double2),
                                 cudaMemcpyDeviceToDevice, stream)))
            return cuda_status(e, "x0 copy");
        a.use_x0 = 1;
    }
    a.out = (double2 *)out;
    const int g = (int)nsys;
    e = p.mixed ? bragg_launch_solve32(p.cpl, a, p.threads, smem, g, stream)
                : bragg_launch_solve64(p.cpl, a, p.threads, smem, g, stream);
    if (e) return cuda_status(e, "bragg_gmres");
    if (info) {
        if ((e = cudaMemcpyAsync(info, a.info, nsys * 4 * sizeof(double),
                                 cudaMemcpyDeviceToDevice, stream)))
            return cuda_status(e, "info copy");
    }
    return DYFOX_OK;
}

extern "C" int dyfox_bragg_apply(const dyfox_bragg_desc *d, int mode,
                                 const double *seg_table,
                                 const double *y_values, const double *s_dev,
                                 const void *in0, const void *in1, void *out,
                                 void *workspace, size_t workspace_bytes,
                                 void *stream_) {
    set_error("");
    BraggPlan p;
    int st = bragg_plan(d, &p);
    if (st) return st;
    if (mode < 0 || mode > 2 || (mode == 2 && !p.mixed)) {
        set_error("mode is 0 (march), 1 (preconditioner) or, with precision "
                  "DYFOX_FP32, 2 (float-float march)");
        return DYFOX_EINVAL;
    }
    if (!y_values || !s_dev || !out || (mode == 1 && !in0) ||
        (d->n_seg > 0 && !seg_table)) {
        set_error("NULL argument to dyfox_bragg_apply");
        return DYFOX_EINVAL;
    }
    if (workspace_bytes < p.ws || !workspace) {
        set_error("workspace of %zu bytes, %zu needed", workspace_bytes, p.ws);
        return DYFOX_ENOMEM;
    }
    const size_t smem = (size_t)3 * d->Nx * sizeof(double2) + 64;
    if ((st = smem_ok(smem))) return st;
    cudaStream_t stream = (cudaStream_t)stream_;
    BraggArgs a;
    if ((st = bragg_prepare(d, p, seg_table, y_values, false, s_dev,
                            (char *)workspace, stream, &a)))
        return st;
    const int nsys = d->n_y * d->n_s;
    cudaError_t e;
    const double2 *i0 = (const double2 *)in0, *i1 = (const double2 *)in1;
    double2 *o = (double2 *)out;
    e = p.mixed ? bragg_launch_apply32(p.cpl, a, p.threads, smem, nsys, mode,
                                       i0, i1, o, stream)
                : bragg_launch_apply64(p.cpl, a, p.threads, smem, nsys, mode,
                                       i0, i1, o, stream);
    return cuda_status(e, "bragg_apply");
}

extern "C" int dyfox_bragg_symbol(const dyfox_bragg_desc *d,
                                  const double *s_dev, void *T21, void *T22,
                                  void *stream_) {
    set_error("");
    int st = bragg_validate(d);
    if (st) return st;
    if (!s_dev || (!T21 && !T22)) {
        set_error("NULL argument to dyfox_bragg_symbol");
        return DYFOX_EINVAL;
    }
    bragg_symbol_kernel<<<d->n_s, 256, 0, (cudaStream_t)stream_>>>(
        s_dev, d->Nx, d->Nz, d->ds, d->sig0[0], d->sig0[1], d->sig_h[0],
        d->sig_h[1], d->sig_hbar[0], d->sig_hbar[1], (double2 *)T21,
        (double2 *)T22, nullptr, nullptr);
    count_launch(1);
    return cuda_status(cudaGetLastError(), "bragg_symbol");
}
