/*
 * dyfox_gb300 -- C ABI of the GB300 (sm_103a) diffraction hot path of DYFOX.
 *
 * Plain pointers and sizes only.  Every "device" pointer is CUDA device
 * memory owned by the caller; `stream` is a cudaStream_t (NULL = legacy
 * default stream).  Calls are asynchronous on `stream` and allocate no
 * device memory: scratch space is a caller-provided `workspace` whose size
 * the matching *_workspace_bytes() query returns.  Every entry returns a
 * dyfox_status; dyfox_last_error() gives a human-readable reason for the
 * last failure on the calling thread.
 *
 * Each entry names the DYFOX interface it replaces (file:line within the
 * DYFOX repository).
 */
#ifndef DYFOX_GB300_H
#define DYFOX_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DYFOX_ABI_VERSION 1

typedef enum dyfox_status {
    DYFOX_OK = 0,
    DYFOX_EINVAL = 1,      /* bad argument (ValueError in the shims)       */
    DYFOX_ENOMEM = 2,      /* workspace too small (MemoryError)            */
    DYFOX_ESMEM = 3,       /* shared memory above the device limit         */
    DYFOX_EMAXITER = 4,    /* iterative solve hit its iteration cap        */
    DYFOX_ENAN = 5,        /* non-finite value met                         */
    DYFOX_ECUDA = 6,       /* CUDA runtime error                           */
    DYFOX_ENOSYS = 7       /* configuration not supported                  */
} dyfox_status;

/* Precision of a march.  FP64: plain double everywhere (parity mode).
 * FP32: single-precision march in the interaction picture with two-sum
 * compensated amplitude updates; per-segment Volterra terms and sincos in
 * single precision with offsets set up in double; the segment sum kept in
 * float-float (two-sum) and reduced mod 2 pi exactly (Cody-Waite), or in
 * double with DYFOX_FLAG_H_FP64. */
#define DYFOX_FP64 0
#define DYFOX_FP32 1

/* Where the displacement phase H = 2 pi g.u of a Laue march comes from. */
#define DYFOX_H_NONE 0         /* perfect crystal (tt3d_pristine_batch)     */
#define DYFOX_H_GRID_F64 1     /* caller's (Ny, Nz, Nx) double grid         */
#define DYFOX_H_GRID_F32 2     /* caller's (Ny, Nz, Nx) float grid          */
#define DYFOX_H_SEGMENTS 3     /* Volterra field of a segment table         */
#define DYFOX_H_ANALYTIC 4     /* one line along x: closed form per (y, z)  */

/* dyfox_laue_desc.flags */
#define DYFOX_FLAG_FUSED 1u    /* H_SEGMENTS: evaluate H inside the march   */
#define DYFOX_FLAG_STAGED 2u   /* H_SEGMENTS: stage e^{iH} in the workspace */
#define DYFOX_FLAG_NO_COMP 4u  /* FP32: plain (uncompensated) updates       */
#define DYFOX_FLAG_GENERAL 8u  /* use the shared-memory general march even
                                  when shift_px == 1 (cross-checks)          */
#define DYFOX_FLAG_H_FP64 16u  /* FP32 + H_SEGMENTS: sum the segment terms and
                                  reduce mod 2 pi in double instead of in
                                  float-float (two-sum) arithmetic           */

/* Doubles per entry of a segment table (dyfox_segment_table). */
#define DYFOX_SEG_STRIDE 24

/* Build the per-segment Volterra frame table on the host.
 * Replaces the frame set-up loop of compute_H_grid (dislocations.py:130-142,
 * volterra_frame 68-90).  segs: n_seg x 9 doubles (r_start, r_end, b) in
 * lab metres; g: reciprocal vector (1/m, no 2 pi); dx: pixel pitch used to
 * scale the single-precision terms.  Segments shorter than 1e-20 m are
 * dropped as the reference drops them; *n_valid receives the count kept.
 * table: n_seg x DYFOX_SEG_STRIDE doubles, host memory. */
int dyfox_segment_table(const double *segs, int n_seg, const double g[3],
                        double nu, double a_core, double dx, double *table,
                        int *n_valid);

/* H on the whole (Ny, Nz, Nx) Laue volume.
 * Replaces dislocations.compute_H_grid (dislocations.py:113-168): segments
 * summed in table order from zero; FP64 keeps each term in double, FP32
 * rounds each segment's double value to float before a float sum, as the
 * reference does (dislocations.py:166).  out: device, Ny*Nz*Nx doubles
 * (precision FP64) or floats (FP32). */
int dyfox_h_grid(const double *seg_table, int n_seg, int Nx, int Ny, int Nz,
                 double dx, double dz, double nu, double a_core,
                 int precision, void *out, void *stream);

/* H (FP64) on n_rows planes of constant y: out[r][k][i] at x_i =
 * (i - Nx/2) dx, z_k = k dz, y = y_values[r] (device array).
 * Replaces dislocations.H_plane (dislocations.py:171-211). */
int dyfox_h_rows(const double *seg_table, int n_seg, int Nx, int Nz,
                 double dx, double dz, double nu, double a_core,
                 const double *y_values, int n_rows, double *out,
                 void *stream);

typedef struct dyfox_laue_desc {
    double sig0[2], sig_h[2], sig_hbar[2];   /* (re, im), 1/m              */
    int Nx, Ny, Nz;                          /* LaueGrid.geometry(), Nz    */
    double dx, dz, ds, shift_px;
    double sheet_hw;                         /* >0 top-hat half-width,
                                                <0 minus Gaussian sigma    */
    double fov_hy;                           /* beam_width / 2             */
    int n_e;                                 /* deviation parameters       */
    int precision;                           /* DYFOX_FP64 / DYFOX_FP32    */
    int h_source;                            /* DYFOX_H_*                  */
    int n_seg;                               /* H_SEGMENTS                 */
    double nu, a_core;                       /* H_SEGMENTS                 */
    double analytic[12];                     /* H_ANALYTIC: y0 z0 e1y e1z
                                                e2y e2z C_atan ge1 ge2
                                                b_perp nu a2               */
    unsigned flags;                          /* DYFOX_FLAG_*               */
    int angles_per_cta;                      /* 0 = automatic              */
    int cols_per_lane;                       /* 0 = automatic              */
} dyfox_laue_desc;

/* Size of the fixed scratch array of dyfox_laue_solve_noalloc. */
#define DYFOX_NOALLOC_SCRATCH_BYTES (32u << 20)

/* Workspace bytes dyfox_laue_solve needs for this descriptor. */
size_t dyfox_laue_workspace_bytes(const dyfox_laue_desc *d);

/* Exit waves D_g(z = t) of a Laue march for n_e deviation parameters.
 * Replaces the launches of tt3d_fullfield_batch / tt3d_analytic_batch /
 * tt3d_pristine_batch (laue/kernels.py:48-352) made by solve_dislocation
 * and solve_pristine (laue/solver.py:34-118), including the angle batch
 * loop and the planar-to-complex pack (solver.py:62-90).
 * s_dev: device, n_e doubles (1/m, finite).
 * h_grid: device (Ny, Nz, Nx) grid for H_GRID_F64 / H_GRID_F32, else NULL.
 * seg_table: device copy of dyfox_segment_table's output for H_SEGMENTS.
 * out: device, (n_e, Ny, Nx) interleaved complex: complex128 for FP64,
 * complex64 for FP32.  Rows with |y| >= fov_hy are written as zero. */
int dyfox_laue_solve(const dyfox_laue_desc *d, const double *s_dev,
                     const void *h_grid, const double *seg_table, void *out,
                     void *workspace, size_t workspace_bytes, void *stream);

/* dyfox_laue_solve for callers that cannot allocate device memory when
 * they solve (no counterpart in the DYFOX reference).  Examples: a real-time
 * acquisition or reconstruction loop that reserves its device memory once
 * and must not fail on an allocation mid-run, a plugin host that forbids
 * allocations after start-up, or a C/Fortran caller with no device
 * allocator of its own.  Same arguments and results as dyfox_laue_solve,
 * without the workspace: the scratch is a fixed array of
 * DYFOX_NOALLOC_SCRATCH_BYTES (32 MiB) in the library's device memory, held
 * by every GPU that loads the library until the process exits.  Problems
 * whose dyfox_laue_workspace_bytes exceeds it return DYFOX_ENOMEM.  The
 * first call on each device looks the array's address up with that device
 * current (cudaGetSymbolAddress); make that first call before any stream
 * capture.  All calls share the array, which keeps the last call's contents
 * (nothing in it has to start at zero); calls whose work overlaps on the GPU
 * race on it and must be serialised.  Allocates no device memory. */
int dyfox_laue_solve_noalloc(const dyfox_laue_desc *d, const double *s_dev,
                             const void *h_grid, const double *seg_table,
                             void *out, void *stream);

typedef struct dyfox_bragg_desc {
    double sig0[2], sig_h[2], sig_hbar[2];   /* (re, im), 1/m              */
    int Nx, Nz;                              /* BraggConfig.Nx, .Nz        */
    double dx, dz, ds;                       /* BraggConfig.dx, .dz, .ds   */
    int n_y;                                 /* y-planes per deviation     */
    int n_s;                                 /* deviation parameters       */
    int n_seg;                               /* segment table entries      */
    double nu, a_core;
    int beam;                                /* 0 plane wave, 1 top hat    */
    double beam_thickness, beam_centre;      /* top hat (BraggConfig)      */
    double tol;                              /* GMRES rtol (true residual) */
    int restart, maxiter;                    /* GMRES restart, maxiter     */
    int precision;                           /* DYFOX_FP64 / DYFOX_FP32    */
    unsigned flags;                          /* reserved, 0                */
} dyfox_bragg_desc;

/* Workspace bytes of dyfox_bragg_solve / dyfox_bragg_apply. */
size_t dyfox_bragg_workspace_bytes(const dyfox_bragg_desc *d);

/* Surface exit waves of n_s x n_y independent shooting problems (every
 * deviation parameter on every y-plane), each solved by its own
 * left-preconditioned restarted GMRES to true relative residual <= tol.
 * Replaces solve_surface_batch and solve_bragg_stable (bragg/solver.py:
 * 135-379) including the Volterra phase of each plane (H_plane, dislocations
 * .py:171-211), the couplings (solver.py:256-261), the particular march
 * (263-265), the perfect-crystal preconditioner (270-278) and the phase
 * restoration v e^{-iH(0)} (362-373).
 * seg_table: device; y_values: HOST, n_y doubles; s_dev: device, n_s;
 * x0: device (n_s, n_y, Nx) complex128 warm start, or NULL for zero;
 * out: device (n_s, n_y, Nx) complex128; info: device (n_s * n_y, 4)
 * doubles per system: true relative residual, inner iterations, code (0
 * converged, else maxiter), |b|; or NULL.
 * precision DYFOX_FP32: mixed-precision solve.  The Arnoldi products (march
 * and preconditioner) run in single precision; b, every true residual, the
 * Gram-Schmidt coefficients, the rotations and the solution stay in double,
 * so the stopping test is the same double-precision true residual <= tol.
 * Inputs and outputs keep their complex128 layout.  The workspace grows by
 * the single-precision couplings. */
int dyfox_bragg_solve(const dyfox_bragg_desc *d, const double *seg_table,
                      const double *y_values, const double *s_dev,
                      const void *x0, void *out, double *info,
                      void *workspace, size_t workspace_bytes, void *stream);

/* One operator application per system, for parity checks.
 * mode 0: out = down-march of (D0(0), Dg(0)) = (in0, in1) to D_g(t)
 *         (bragg/solver.py:28-35; NULL input = zero);
 * mode 1: out = ifft(fft(in0) / T22s) (solver.py:167-168, 297-300).
 * in0, in1, out: device (n_s, n_y, Nx) complex128.  precision DYFOX_FP32
 * applies the single-precision operators of the mixed solve. */
int dyfox_bragg_apply(const dyfox_bragg_desc *d, int mode,
                      const double *seg_table, const double *y_values,
                      const double *s_dev, const void *in0, const void *in1,
                      void *out, void *workspace, size_t workspace_bytes,
                      void *stream);

/* Fourier symbol of the perfect-crystal shooting operator per deviation
 * parameter: T21, T22 (device, (n_s, Nx) complex128; either may be NULL).
 * Replaces bragg.perfect_symbol (bragg/solver.py:38-60). */
int dyfox_bragg_symbol(const dyfox_bragg_desc *d, const double *s_dev,
                       void *T21, void *T22, void *stream);

/* Diagnostic (not part of any DYFOX interface): measured FMA throughput
 * of this GPU in TFLOP/s (2 flops per FMA) for DYFOX_FP64 or DYFOX_FP32,
 * the denominator of the arithmetic-bound kernels' roofline.  Synchronises
 * `stream`; allocates one scalar of device memory for the call. */
int dyfox_pipe_peak(int precision, int iters, double *tflops, void *stream);

/* Number of kernels this library has launched since it was loaded. */
unsigned long long dyfox_launch_count(void);

/* Human-readable name of a status code. */
const char *dyfox_status_string(int status);
/* Reason for the last failure on the calling thread ("" if none). */
const char *dyfox_last_error(void);
/* DYFOX_ABI_VERSION of the library. */
int dyfox_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DYFOX_GB300_H */
