// Imaging of exit waves through a pupil, replacing DYFOX optics.py
// (Optics.pupil 64-118, object_spectrum / image_from_spectrum /
// image_intensity 170-207), and the centre-of-mass reduction of a rocking
// scan, replacing the accumulation of analysis/rocking.py:37-83 (com_maps).
//
// For even Ny and Nx the reference's shifted transforms reduce to
//   I = |ifft2(fft2(u) * ifftshift(P))|^2
// (fftshift is then its own inverse, and a half-period shift in one domain
// is a sign alternation in the other, which cancels between the forward
// and the inverse transform), so the GPU path runs no shift pass: a
// forward FFT along x per row, a column pass (FFT along y, product with the
// pupil read in natural frequency order, inverse FFT along y), and a last
// pass per row (inverse FFT along x, |.|^2) that writes the image or adds
// phi(s) I and I into the scan's double-precision sums.  Transforms are the
// mixed-radix Stockham FFT of the Bragg preconditioner, in the stack's
// precision.
#include <math.h>
#include <string.h>

#include "bragg.cuh"

namespace dyfox {

// Pupil on the fftshifted frequency grid: frequency fx = (ix - Nx/2) /
// (Nx dx); aperture disc of radius aperture_f about (ax, ay); for ell != 0
// a spiral phase ell atan2(fy - sy, fx - sx), quantised to `levels` steps
// when levels > 0; the origin bin zeroed when zero_dc.  Double arithmetic.
__global__ void pupil_kernel(int Nx, int Ny, double fx_step, double fy_step,
                             double aperture_f, int ell, double ax,
                             double ay, double sx, double sy, int zero_dc,
                             int levels, int single, void *out) {
    const long total = (long)Nx * Ny;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int iy = (int)(i / Nx), ix = (int)(i - (long)iy * Nx);
        const double fx = __dmul_rn((double)(ix - Nx / 2), fx_step);
        const double fy = __dmul_rn((double)(iy - Ny / 2), fy_step);
        const double rx = fx - ax, ry = fy - ay;
        // separate roundings, as the reference's (fx-ax)**2 + (fy-ay)**2
        const double rad = sqrt(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)));
        const double circ = rad <= aperture_f ? 1.0 : 0.0;
        double re = circ, im = 0.0;
        if (ell != 0) {
            double ph = ell * atan2(fy - sy, fx - sx);
            if (levels > 0) {
                const double step = 2.0 * kPi / levels;
                double m = fmod(ph, 2.0 * kPi);
                if (m < 0.0) m += 2.0 * kPi;
                ph = floor(m / step) * step;
            }
            double sn, c;
            sincos(ph, &sn, &c);
            re = circ * c;
            im = circ * sn;
            if (zero_dc && iy == Ny / 2 && ix == Nx / 2) re = im = 0.0;
        }
        if (single)
            ((float2 *)out)[i] = make_float2((float)re, (float)im);
        else
            ((double2 *)out)[i] = make_double2(re, im);
    }
}

// exp(-2 pi i m / N), m < N, in the transform's precision.
template <typename C>
__global__ void optics_twiddle_kernel(C *tw, int N) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= N) return;
    double sn, c;
    sincospi(-2.0 * m / N, &sn, &c);
    C v;
    v.x = c;
    v.y = sn;
    tw[m] = v;
}

// Register butterflies for radices 11 and 13 in the row passes in single
// precision only (in double, and in the column pass that holds a block of
// columns in shared memory, the extra registers cost more occupancy than
// the butterflies save).
template <typename C> constexpr bool kBigOdd = false;
template <> constexpr bool kBigOdd<float2> = true;

// Copy of the stack with every row transformed along x (forward).  One CTA
// per (image, row).
template <typename C>
__global__ void fft_rows_kernel(const C *__restrict__ in, C *out, int Nx,
                                FftPlan plan, const C *__restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smem[];
    C *a = reinterpret_cast<C *>(smem), *b = a + Nx;
    const size_t row = (size_t)blockIdx.x * Nx;
    // The exit waves are read once: a streaming load keeps them from
    // displacing the spectra that the next two passes reread from L2.
    for (int x = threadIdx.x; x < Nx; x += blockDim.x)
        a[x] = __ldcs(in + row + x);
    __syncthreads();
    C *r = fft_run<C, kBigOdd<C>>(a, b, plan, tw, false);
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) out[row + x] = r[x];
}

// Column pass, in place: for CB adjacent columns of one image, forward FFT
// along y, product with the pupil (read from its fftshifted layout at the
// natural-order frequency), inverse FFT along y.
template <typename C>
__global__ void cols_pupil_kernel(C *data, int Ny, int Nx, int CB,
                                  FftPlan plan, const C *__restrict__ tw,
                                  const C *__restrict__ pupil) {
    extern __shared__ __align__(16) unsigned char smem[];
    // Column c of the block at a[c * S + y]; S = Ny + 1 (odd) keeps the
    // transposing loads and stores free of bank conflicts.
    const int S = Ny + 1;
    C *a = reinterpret_cast<C *>(smem), *b = a + (size_t)CB * S;
    const int nblk = (Nx + CB - 1) / CB;
    const int img = blockIdx.x / nblk, x0 = (blockIdx.x - img * nblk) * CB;
    const int nc = Nx - x0 < CB ? Nx - x0 : CB;
    C *base = data + (size_t)img * Ny * Nx;
    for (int t = threadIdx.x; t < Ny * CB; t += blockDim.x) {
        const int y = t / CB, c = t - y * CB;
        if (c < nc) a[c * S + y] = base[(size_t)y * Nx + x0 + c];
    }
    __syncthreads();
    // The nc columns are transformed together (one barrier per pass).
    C *res = fft_run<C, false>(a, b, plan, tw, false, nc, S);
    for (int t = threadIdx.x; t < Ny * CB; t += blockDim.x) {
        const int y = t / CB, c = t - y * CB;
        if (c >= nc) continue;
        const int kx = x0 + c;
        const C p = __ldg(pupil + (size_t)((y + Ny / 2) % Ny) * Nx +
                          (kx + Nx / 2) % Nx);
        res[c * S + y] = cmulz(res[c * S + y], p);
    }
    __syncthreads();
    C *other = res == a ? b : a;
    C *fin = fft_run<C, false>(res, other, plan, tw, true, nc, S);
    for (int t = threadIdx.x; t < Ny * CB; t += blockDim.x) {
        const int y = t / CB, c = t - y * CB;
        if (c < nc) base[(size_t)y * Nx + x0 + c] = fin[c * S + y];
    }
}

template <typename C> struct RealOf;
template <> struct RealOf<double2> { using T = double; };
template <> struct RealOf<float2> { using T = float; };

// Last pass, one CTA per row y over the n images: inverse FFT along x and
// I = |.|^2 / (Nx Ny)^2.  img != NULL: I is written (n, Ny, Nx).  sum_I !=
// NULL: sum_I[y][x] += I, sum_wI[y][x] += phi[e] I and rock_part[e][y] =
// sum_x I, in double, the images taken in order (each pixel owned by one
// thread: deterministic).
template <typename C>
__global__ void rows_intensity_kernel(const C *__restrict__ data, int n,
                                      int Ny, int Nx, FftPlan plan,
                                      const C *__restrict__ tw, double scale,
                                      typename RealOf<C>::T *img,
                                      const double *__restrict__ phi,
                                      double *sum_wI, double *sum_I,
                                      double *rock_part) {
    using R = typename RealOf<C>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    C *a = reinterpret_cast<C *>(smem), *b = a + Nx;
    double2 *red = reinterpret_cast<double2 *>(b + Nx);
    const int y = blockIdx.x;
    for (int e = 0; e < n; ++e) {
        const size_t row = ((size_t)e * Ny + y) * Nx;
        // The last read of this spectrum row (streaming).
        for (int x = threadIdx.x; x < Nx; x += blockDim.x)
            a[x] = __ldcs(data + row + x);
        __syncthreads();
        const C *r = fft_run<C, kBigOdd<C>>(a, b, plan, tw, true);
        double part = 0.0;
        for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
            // |.|^2 in the stack's precision, as the reference's abs()**2.
            const R vr = r[x].x, vi = r[x].y;
            const R I = (vr * vr + vi * vi) * (R)scale;
            if (img) img[row + x] = I;
            if (sum_I) {
                const size_t p = (size_t)y * Nx + x;
                sum_I[p] += (double)I;
                sum_wI[p] += phi[e] * (double)I;
                part += (double)I;
            }
        }
        if (sum_I) {
            const double tot = block_sum(make_double2(part, 0.0), red).x;
            if (threadIdx.x == 0) rock_part[(size_t)e * Ny + y] = tot;
        }
        __syncthreads();
    }
}

// rock[e] = sum_y rock_part[e][y].
__global__ void rock_reduce_kernel(const double *part, int n, int Ny,
                                   double *rock) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    double s = 0.0;
    for (int y = 0; y < Ny; ++y) s += part[(size_t)e * Ny + y];
    rock[e] = s;
}

struct ImagePlan {
    size_t csize, off_stack, off_twx, off_twy, off_rock, ws, smem_rows,
        smem_cols, smem_last;
    int CB;
    int chunk;   // images per pass sequence
};

// Images per pass sequence: the three passes run over chunks of images
// whose intermediate spectra (chunk x Ny x Nx) fit in 24 MB, so that the
// spectra written by one pass are read by the next from L2 rather than
// from HBM; chunks of equal size.
static int image_chunk(int n, int Ny, int Nx, size_t cs) {
    const size_t one = (size_t)Ny * Nx * cs;
    const size_t cap = (size_t)24 << 20;
    const int cmax = one >= cap ? 1 : (int)(cap / one);
    const int nchunks = (n + cmax - 1) / cmax;
    return (n + nchunks - 1) / nchunks;
}

static size_t al256o(size_t v) { return (v + 255) & ~(size_t)255; }

static int image_plan(int n, int Ny, int Nx, int precision, ImagePlan *p) {
    if (n < 1 || Ny < 2 || Nx < 2 || (Ny & 1) || (Nx & 1)) {
        set_error("imaging needs n >= 1 and even Ny, Nx (got %d, %d, %d)", n,
                  Ny, Nx);
        return DYFOX_EINVAL;
    }
    if (precision != DYFOX_FP64 && precision != DYFOX_FP32) {
        set_error("precision %d is neither DYFOX_FP64 nor DYFOX_FP32",
                  precision);
        return DYFOX_EINVAL;
    }
    const size_t cs = precision == DYFOX_FP64 ? sizeof(double2) : sizeof(float2);
    p->csize = cs;
    size_t o = 0;
    p->chunk = image_chunk(n, Ny, Nx, cs);
    p->off_stack = o; o = al256o(o + (size_t)p->chunk * Ny * Nx * cs);
    p->off_twx = o; o = al256o(o + (size_t)Nx * cs);
    p->off_twy = o; o = al256o(o + (size_t)Ny * cs);
    p->off_rock = o; o = al256o(o + (size_t)n * Ny * sizeof(double));
    p->ws = o;
    p->smem_rows = 2 * (size_t)Nx * cs;
    p->smem_last = 2 * (size_t)Nx * cs + 34 * sizeof(double2);
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (!e) e = cudaDeviceGetAttribute(&optin,
                                       cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                       dev);
    if (e) return cuda_status(e, "device query");
    if (Nx > 65536 || Ny > 65536) {
        set_error("image of %d x %d: transforms are limited to 65536 points",
                  Ny, Nx);
        return DYFOX_EINVAL;
    }
    // Columns per block of the column pass: 4 (against 8: 3% faster on
    // 544 x 1056 images, twice the resident blocks per SM), fewer where they
    // would not fit in half the shared memory or would break the exactness
    // of the batched transform's index division (CB (Ny / 2)^2 < 2^32).
    p->CB = 4;
    while (p->CB > 1 &&
           (2 * (size_t)p->CB * (Ny + 1) * cs > (size_t)optin / 2 ||
            (unsigned long long)p->CB * (Ny / 2) * (Ny / 2) >= (1ull << 32)))
        p->CB /= 2;
    p->smem_cols = 2 * (size_t)p->CB * (Ny + 1) * cs;
    if (p->smem_cols > (size_t)optin || p->smem_last > (size_t)optin) {
        set_error("image of %d x %d needs more shared memory than the device "
                  "has", Ny, Nx);
        return DYFOX_ESMEM;
    }
    return DYFOX_OK;
}

template <typename K>
static cudaError_t smem_attr(K *k, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

template <typename C>
static int run_image(const ImagePlan &p, const void *stack, int n, int Ny,
                     int Nx, const void *pupil, void *img, const double *phi,
                     double *sum_wI, double *sum_I, double *rock, char *ws,
                     cudaStream_t s) {
    using R = typename RealOf<C>::T;
    cudaError_t e;
    C *buf = (C *)(ws + p.off_stack);
    C *twx = (C *)(ws + p.off_twx), *twy = (C *)(ws + p.off_twy);
    double *rock_part = (double *)(ws + p.off_rock);
    const FftPlan px = make_fft_plan(Nx), py = make_fft_plan(Ny);
    optics_twiddle_kernel<C><<<div_up(Nx, 256), 256, 0, s>>>(twx, Nx);
    optics_twiddle_kernel<C><<<div_up(Ny, 256), 256, 0, s>>>(twy, Ny);
    count_launch(2);
    if ((e = smem_attr(fft_rows_kernel<C>, p.smem_rows)) ||
        (e = smem_attr(cols_pupil_kernel<C>, p.smem_cols)) ||
        (e = smem_attr(rows_intensity_kernel<C>, p.smem_last)))
        return cuda_status(e, "imaging shared memory");
    const int nblk = (Nx + p.CB - 1) / p.CB;
    const double scale = 1.0 / ((double)Nx * Ny * (double)Nx * Ny);
    const size_t plane = (size_t)Ny * Nx;
    // The sums take the images in order across chunks, as in one pass.
    for (int e0 = 0; e0 < n; e0 += p.chunk) {
        const int c = n - e0 < p.chunk ? n - e0 : p.chunk;
        fft_rows_kernel<C><<<c * Ny, 256, p.smem_rows, s>>>(
            (const C *)stack + e0 * plane, buf, Nx, px, twx);
        cols_pupil_kernel<C><<<c * nblk, 256, p.smem_cols, s>>>(
            buf, Ny, Nx, p.CB, py, twy, (const C *)pupil);
        rows_intensity_kernel<C><<<Ny, 256, p.smem_last, s>>>(
            buf, c, Ny, Nx, px, twx, scale,
            img ? (R *)img + e0 * plane : nullptr, phi ? phi + e0 : nullptr,
            sum_wI, sum_I, rock_part + (size_t)e0 * Ny);
        count_launch(3);
    }
    if (sum_I && rock) {
        rock_reduce_kernel<<<div_up(n, 128), 128, 0, s>>>(rock_part, n, Ny,
                                                          rock);
        count_launch(1);
    }
    return cuda_status(cudaGetLastError(), "imaging");
}

}  // namespace dyfox

using namespace dyfox;

extern "C" int dyfox_pupil(int Nx, int Ny, double dx, double aperture_f,
                           int ell, double aperture_fx, double aperture_fy,
                           double singularity_fx, double singularity_fy,
                           int dc_zero, int levels, int precision,
                           void *pupil, void *stream) {
    set_error("");
    if (Nx < 1 || Ny < 1 || !(dx > 0) || !(aperture_f >= 0) || !pupil ||
        levels < 0 || (precision != DYFOX_FP64 && precision != DYFOX_FP32)) {
        set_error("bad pupil arguments (Nx=%d Ny=%d dx=%g aperture=%g "
                  "levels=%d precision=%d)", Nx, Ny, dx, aperture_f, levels,
                  precision);
        return DYFOX_EINVAL;
    }
    const long total = (long)Nx * Ny;
    long blocks = (total + 255) / 256;
    if (blocks > 152L * 32) blocks = 152L * 32;
    pupil_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(
        Nx, Ny, 1.0 / (Nx * dx), 1.0 / (Ny * dx), aperture_f, ell,
        aperture_fx, aperture_fy, singularity_fx, singularity_fy,
        dc_zero ? 1 : 0, levels, precision == DYFOX_FP32 ? 1 : 0, pupil);
    count_launch(1);
    return cuda_status(cudaGetLastError(), "pupil");
}

extern "C" int dyfox_image_workspace_bytes(int n, int Ny, int Nx,
                                           int precision, size_t *bytes) {
    set_error("");
    if (!bytes) {
        set_error("NULL bytes");
        return DYFOX_EINVAL;
    }
    ImagePlan p;
    int st = image_plan(n, Ny, Nx, precision, &p);
    *bytes = st ? 0 : p.ws;
    return st;
}

extern "C" int dyfox_image(const void *stack, int n, int Ny, int Nx,
                           int precision, const void *pupil, void *out,
                           const double *phi, double *sum_wI, double *sum_I,
                           double *rock, void *workspace,
                           size_t workspace_bytes, void *stream) {
    set_error("");
    ImagePlan p;
    int st = image_plan(n, Ny, Nx, precision, &p);
    if (st) return st;
    if (!stack || !pupil || (!out && !sum_I) ||
        (sum_I && (!sum_wI || !phi))) {
        set_error("NULL argument to dyfox_image");
        return DYFOX_EINVAL;
    }
    if (!workspace || workspace_bytes < p.ws) {
        set_error("workspace of %zu bytes, %zu needed", workspace_bytes, p.ws);
        return DYFOX_ENOMEM;
    }
    cudaStream_t s = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    if (precision == DYFOX_FP64)
        return run_image<double2>(p, stack, n, Ny, Nx, pupil, out, phi, sum_wI,
                                  sum_I, rock, ws, s);
    return run_image<float2>(p, stack, n, Ny, Nx, pupil, out, phi, sum_wI,
                             sum_I, rock, ws, s);
}
