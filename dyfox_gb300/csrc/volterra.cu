// Volterra displacement phase: the segment table (host), the H grid and H
// rows kernels (replacing dislocations.compute_H_grid / H_plane), and the
// staging of e^{iH} for marches over many deviation parameters.
#include <math.h>
#include <string.h>

#include "volterra.cuh"

namespace dyfox {

// H of n_rows planes of constant y.  y_dev != NULL gives the planes' y;
// otherwise plane r is grid row r at y = (r - Ny/2) dx.  A CTA takes
// kHPairs consecutive (plane, depth) pairs at a time, its threads their
// columns: the pairs' offsets from every segment core (Y - cy, Z - cz) and
// their products with the line direction are formed once per pair in
// shared memory, the column coordinates once per CTA, so that a voxel's
// double work is the column-dependent part of the field (each value
// rounded as the reference's per-voxel evaluation rounds it).  Segments
// are taken in tiles of `tile`; between tiles a thread keeps its voxels'
// partial sums in `out` (the same values and order as one pass).  XTAB
// (all segments in one tile, few enough to fit): the column terms
// X = X0 - cx and X xi0 of every segment are formed once per CTA too.
constexpr int kHPairs = 4;

template <bool F32OUT, bool XTAB>
__global__ void h_rows_kernel(const double *__restrict__ segs, int n_seg,
                              int tile, int Nx, int Nz, double dx, double dz,
                              VolterraConsts vc,
                              const double *__restrict__ y_dev, int Ny,
                              long n_rows, void *out) {
    extern __shared__ __align__(16) double hsm[];
    // Nx: X0 of each column; XTAB: n_seg x 2 x Nx: X0 - cx, (X0 - cx) xi0
    double *x0 = hsm;
    const size_t ncol = XTAB ? (size_t)2 * n_seg * Nx : (size_t)Nx;
    double *yz = hsm + ncol;           // kHPairs x tile x 4: Y, Z, Y xi1, Z xi2
    const int tid = threadIdx.x, nt = blockDim.x;
    if (XTAB) {
        for (int i = tid; i < n_seg * Nx; i += nt) {
            const int s = i / Nx, x = i - s * Nx;
            const double *sg = segs + (size_t)s * DYFOX_SEG_STRIDE;
            const double X = __dsub_rn(__dmul_rn((double)x - 0.5 * Nx, dx),
                                       __ldg(sg + SEG_CX));
            x0[(size_t)2 * s * Nx + x] = X;
            x0[(size_t)(2 * s + 1) * Nx + x] = __dmul_rn(X, __ldg(sg + SEG_XI));
        }
    } else {
        for (int x = tid; x < Nx; x += nt)
            x0[x] = __dmul_rn((double)x - 0.5 * Nx, dx);
    }
    const long pairs = n_rows * (long)Nz;
    const long groups = (pairs + kHPairs - 1) / kHPairs;
    for (long gi = blockIdx.x; gi < groups; gi += gridDim.x) {
        const long rk0 = gi * kHPairs;
        const int np = pairs - rk0 < kHPairs ? (int)(pairs - rk0) : kHPairs;
        // (one pass with no segment writes zeros)
        for (int s0 = 0; s0 < n_seg || s0 == 0; s0 += tile) {
            const int ns = n_seg - s0 < tile ? n_seg - s0 : tile;
            const double *sg0 = segs + (size_t)s0 * DYFOX_SEG_STRIDE;
            __syncthreads();           // the previous tile's readers
            for (int it = tid; it < np * ns; it += nt) {
                const int pp = it / ns, s = it - pp * ns;
                const long rk = rk0 + pp;
                const long r = rk / Nz;
                const int k = (int)(rk - r * Nz);
                const double yv =
                    y_dev ? y_dev[r] : __dmul_rn((double)r - 0.5 * Ny, dx);
                const double zv = __dmul_rn((double)k, dz);
                const double *sg = sg0 + (size_t)s * DYFOX_SEG_STRIDE;
                const double Y = __dsub_rn(yv, __ldg(sg + SEG_CY));
                const double Z = __dsub_rn(zv, __ldg(sg + SEG_CZ));
                double *q = yz + ((size_t)pp * tile + s) * 4;
                q[0] = Y;
                q[1] = Z;
                q[2] = __dmul_rn(Y, __ldg(sg + SEG_XI + 1));
                q[3] = __dmul_rn(Z, __ldg(sg + SEG_XI + 2));
            }
            __syncthreads();
            for (int it = tid; it < np * Nx; it += nt) {
                const int pp = it / Nx, x = it - pp * Nx;
                const double X0 = XTAB ? 0.0 : x0[x];
                const size_t idx = (size_t)(rk0 + pp) * Nx + x;
                const double *q = yz + (size_t)pp * tile * 4;
                double acc = 0.0;
                float accf = 0.0f;
                if (s0) {
                    if (F32OUT) accf = ((const float *)out)[idx];
                    else acc = ((const double *)out)[idx];
                }
                for (int s = 0; s < ns; ++s) {
                    const double *sg = sg0 + (size_t)s * DYFOX_SEG_STRIDE;
                    double X, Xx0;
                    if (XTAB) {
                        X = x0[(size_t)2 * s * Nx + x];
                        Xx0 = x0[(size_t)(2 * s + 1) * Nx + x];
                    } else {
                        X = __dsub_rn(X0, __ldg(sg + SEG_CX));
                        Xx0 = __dmul_rn(X, __ldg(sg + SEG_XI));
                    }
                    const double h = h_seg_f64h(
                        sg, X, q[4 * s], q[4 * s + 1], Xx0, q[4 * s + 2],
                        q[4 * s + 3], vc);
                    if (F32OUT) accf = __fadd_rn(accf, __double2float_rn(h));
                    else acc = __dadd_rn(acc, h);
                }
                if (F32OUT) ((float *)out)[idx] = accf;
                else ((double *)out)[idx] = acc;
            }
        }
    }
}

// Threads per CTA of h_rows_kernel: the multiple of 32 in [128, 256] that
// leaves the fewest idle threads over a row of Nx columns (ties: more).
static int h_rows_threads(int Nx) {
    int best = 256, waste = 1 << 30;
    for (int t = 256; t >= 128; t -= 32) {
        const int w = (Nx + t - 1) / t * t - Nx;
        if (w < waste) { waste = w; best = t; }
    }
    return best;
}

static int launch_h_rows(bool f32out, const double *segs, int n_seg, int Nx,
                         int Nz, double dx, double dz, const VolterraConsts &vc,
                         const double *y_dev, int Ny, long n_rows, void *out,
                         cudaStream_t stream) {
    const long pairs = n_rows * (long)Nz;
    if (pairs == 0 || Nx == 0) return DYFOX_OK;
    // Shared memory: the column coordinates and a tile of segments for
    // kHPairs pairs, within 48 KB where the columns leave room for 64
    // segments, else up to 200 KB.
    const size_t per_seg = 4 * kHPairs * sizeof(double),
                 cols = (size_t)Nx * sizeof(double);
    const size_t budget = cols + 64 * per_seg <= 48 * 1024 ? 48 * 1024
                                                           : 200 * 1024;
    if (cols + per_seg > budget) {
        set_error("H rows of %d columns need more shared memory than 200 KB",
                  Nx);
        return DYFOX_ESMEM;
    }
    const long fit = (long)((budget - cols) / per_seg);
    const int tile = n_seg < 1 ? 1 : (n_seg < fit ? n_seg : (int)fit);
    // Column tables per segment where they fit in 40 KB with the tile (a
    // few segments: several CTAs per SM still fit).
    const size_t xtab = (size_t)2 * n_seg * cols + (size_t)n_seg * per_seg;
    const bool use_xtab = n_seg >= 1 && tile == n_seg && xtab <= 40 * 1024;
    const size_t smem = use_xtab ? xtab : cols + (size_t)tile * per_seg;
    const int threads = h_rows_threads(Nx);
    const long groups = (pairs + kHPairs - 1) / kHPairs;
    const long blocks = groups < 152L * 16 ? groups : 152L * 16;
    auto go = [&](auto kernel) {
        cudaError_t err = cudaSuccess;
        if (smem > 48 * 1024)
            err = cudaFuncSetAttribute(
                kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                (int)smem);
        if (!err)
            kernel<<<(int)blocks, threads, smem, stream>>>(
                segs, n_seg, tile, Nx, Nz, dx, dz, vc, y_dev, Ny, n_rows, out);
        return err;
    };
    const cudaError_t e =
        f32out ? (use_xtab ? go(h_rows_kernel<true, true>)
                           : go(h_rows_kernel<true, false>))
               : (use_xtab ? go(h_rows_kernel<false, true>)
                           : go(h_rows_kernel<false, false>));
    if (e) return cuda_status(e, "h_rows_kernel shared memory");
    count_launch(1);
    return cuda_status(cudaGetLastError(), "h_rows_kernel");
}

// ---------------------------------------------------------------------------
// e^{iH} of rows [row0, row0 + n_rows) for the depth steps 0 .. Nz-2, for a
// march over many deviation parameters (computed once, read by every angle
// group).  One CTA per (row, KB steps).  Double: reference-order H and
// sincos.  Single: pivot set-up per (row, step, segment) in double, segment
// terms in single, their sum and the 2 pi reduction in float-float (or in
// double when SUM64).
constexpr int kStageKB = 4;

template <bool SINGLE, bool SUM64>
__global__ void cs_stage_kernel(const double *__restrict__ segs, int n_seg,
                                int Nx, int Ny, int Nz, double dx, double dz,
                                VolterraConsts vc, int row0, int n_rows,
                                void *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nsteps = Nz - 1;
    const int kchunks = (nsteps + kStageKB - 1) / kStageKB;
    const int r = blockIdx.x / kchunks;
    const int k0 = (blockIdx.x - r * kchunks) * kStageKB;
    const int kn = nsteps - k0 < kStageKB ? nsteps - k0 : kStageKB;
    const int iy = row0 + r;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (SINGLE) {
        stage_chunk32(segs, n_seg, Nx, Ny, dx, dz, iy, k0, kn, SUM64,
                      (float2 *)out + (size_t)r * nsteps * Nx, smem);
    } else {
        const double yv = __dmul_rn((double)iy - 0.5 * Ny, dx);
        for (int j = tid; j < kn * Nx; j += nt) {
            const int kb = j / Nx, x = j - kb * Nx;
            const double X0 = __dmul_rn((double)x - 0.5 * Nx, dx);
            const double zv = __dmul_rn((double)(k0 + kb), dz);
            double acc = 0.0;
            for (int s = 0; s < n_seg; ++s) {
                const double *sg = segs + (size_t)s * DYFOX_SEG_STRIDE;
                acc = __dadd_rn(acc, h_seg_f64(sg, __dsub_rn(X0, __ldg(sg + SEG_CX)),
                                               __dsub_rn(yv, __ldg(sg + SEG_CY)),
                                               __dsub_rn(zv, __ldg(sg + SEG_CZ)), vc));
            }
            double sn, c;
            sincos(acc, &sn, &c);
            ((double2 *)out)[((size_t)r * nsteps + k0 + kb) * Nx + x] =
                make_double2(c, sn);
        }
    }
}

cudaError_t launch_cs_stage(bool single, bool sum64, const double *segs,
                            int n_seg, int Nx, int Ny, int Nz, double dx,
                            double dz,
                            const VolterraConsts &vc, int row0, int n_rows,
                            void *out, cudaStream_t stream) {
    const int nsteps = Nz - 1;
    const int kchunks = (nsteps + kStageKB - 1) / kStageKB;
    const long grid = (long)n_rows * kchunks;
    if (grid == 0) return cudaSuccess;
    if (single) {
        size_t smem = stage_chunk32_smem(n_seg, kStageKB);
        auto *k = sum64 ? cs_stage_kernel<true, true> : cs_stage_kernel<true, false>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(
                k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        k<<<(int)grid, 256, smem, stream>>>(segs, n_seg, Nx, Ny, Nz, dx, dz,
                                            vc, row0, n_rows, out);
        count_launch(1);
    } else {
        cs_stage_kernel<false, true><<<(int)grid, 256, 0, stream>>>(
            segs, n_seg, Nx, Ny, Nz, dx, dz, vc, row0, n_rows, out);
        count_launch(1);
    }
    return cudaGetLastError();
}

}  // namespace dyfox

using namespace dyfox;

static double dot3(const double *a, const double *b) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

static void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// The segment frame of dislocations.py:68-90 (volterra_frame): screw part
// b.xi, edge direction e1 along b_perp (or the lab axis furthest from the
// line for pure screw), e2 = xi x e1; plus the constants of 130-142 and
// those of the single-precision evaluator.
extern "C" int dyfox_segment_table(const double *segs, int n_seg,
                                   const double g[3], double nu,
                                   double a_core, double dx, double *table,
                                   int *n_valid) {
    set_error("");
    if (n_seg < 0 || (n_seg > 0 && (!segs || !table)) || !g || !n_valid) {
        set_error("bad arguments to dyfox_segment_table");
        return DYFOX_EINVAL;
    }
    if (!(dx > 0) || !(a_core > 0) || !(nu < 1.0) || !isfinite(nu)) {
        set_error("bad scalars dx=%g a_core=%g nu=%g", dx, a_core, nu);
        return DYFOX_EINVAL;
    }
    const double onu = 1.0 - nu;
    const double kl = (1 - 2 * nu) / (4 * onu);
    int kept = 0;
    for (int s = 0; s < n_seg; ++s) {
        const double *ra = segs + 9 * s, *rb = ra + 3, *bv = ra + 6;
        for (int i = 0; i < 9; ++i)
            if (!isfinite(ra[i])) {
                set_error("segment %d has a non-finite coordinate", s);
                return DYFOX_ENAN;
            }
        double t[3] = {rb[0] - ra[0], rb[1] - ra[1], rb[2] - ra[2]};
        double L = sqrt(dot3(t, t));
        if (L < 1e-20) continue;
        double *o = table + (size_t)DYFOX_SEG_STRIDE * kept;
        memset(o, 0, sizeof(double) * DYFOX_SEG_STRIDE);
        double xi[3] = {t[0] / L, t[1] / L, t[2] / L};
        double b_screw = dot3(bv, xi);
        double bp[3] = {bv[0] - b_screw * xi[0], bv[1] - b_screw * xi[1],
                        bv[2] - b_screw * xi[2]};
        double b_perp = sqrt(dot3(bp, bp));
        double e1[3], e2[3];
        if (b_perp > 1e-20) {
            for (int i = 0; i < 3; ++i) e1[i] = bp[i] / b_perp;
        } else if (fabs(xi[2]) > 0.9) {
            e1[0] = 1.0; e1[1] = 0.0; e1[2] = 0.0;
        } else {
            double ax[3] = {0, 0, 0};
            if (fabs(xi[0]) < 0.9) ax[0] = 1.0; else ax[1] = 1.0;
            cross3(xi, ax, e1);
            double m = sqrt(dot3(e1, e1));
            for (int i = 0; i < 3; ++i) e1[i] /= m;
        }
        cross3(xi, e1, e2);
        for (int i = 0; i < 3; ++i) {
            o[SEG_CX + i] = (ra[i] + rb[i]) / 2.0;
            o[SEG_XI + i] = xi[i];
            o[SEG_E1 + i] = e1[i];
            o[SEG_E2 + i] = e2[i];
        }
        const double ge1 = dot3(g, e1), ge2 = dot3(g, e2);
        o[SEG_CATAN] = ge1 * b_perp + dot3(g, xi) * b_screw;
        o[SEG_GE1] = ge1;
        o[SEG_GE2] = ge2;
        o[SEG_BPERP] = b_perp;
        if (b_perp > 1e-20) {
            // 2 pi c1 = b_perp
            o[SEG_KX] = ge1 * b_perp / (2 * onu);
            o[SEG_KL] = -ge2 * b_perp * kl;
            o[SEG_KQ] = -ge2 * b_perp / (4 * onu);
            o[SEG_HCONST] = o[SEG_KL] * log(dx * dx);
        }
        o[SEG_C1] = b_perp / (2 * kPi);
        o[SEG_A2PX] = (a_core / dx) * (a_core / dx);
        o[SEG_SLOPE1] = e1[0] - xi[0] * dot3(xi, e1);
        o[SEG_SLOPE2] = e2[0] - xi[0] * dot3(xi, e2);
        ++kept;
    }
    *n_valid = kept;
    return DYFOX_OK;
}

extern "C" int dyfox_h_grid(const double *seg_table, int n_seg, int Nx,
                            int Ny, int Nz, double dx, double dz, double nu,
                            double a_core, int precision, void *out,
                            void *stream) {
    set_error("");
    if (Nx < 1 || Ny < 1 || Nz < 1 || n_seg < 0 || !out ||
        (n_seg > 0 && !seg_table)) {
        set_error("bad arguments to dyfox_h_grid");
        return DYFOX_EINVAL;
    }
    if (precision != DYFOX_FP64 && precision != DYFOX_FP32) {
        set_error("precision is DYFOX_FP64 or DYFOX_FP32, not %d", precision);
        return DYFOX_EINVAL;
    }
    return launch_h_rows(precision == DYFOX_FP32, seg_table, n_seg, Nx, Nz, dx,
                         dz, volterra_consts(nu, a_core), nullptr, Ny, Ny, out,
                         (cudaStream_t)stream);
}

extern "C" int dyfox_h_rows(const double *seg_table, int n_seg, int Nx,
                            int Nz, double dx, double dz, double nu,
                            double a_core, const double *y_values, int n_rows,
                            double *out, void *stream) {
    set_error("");
    if (Nx < 1 || Nz < 1 || n_rows < 0 || n_seg < 0 || !out || !y_values ||
        (n_seg > 0 && !seg_table)) {
        set_error("bad arguments to dyfox_h_rows");
        return DYFOX_EINVAL;
    }
    return launch_h_rows(false, seg_table, n_seg, Nx, Nz, dx, dz,
                         volterra_consts(nu, a_core), y_values, 0, n_rows, out,
                         (cudaStream_t)stream);
}
