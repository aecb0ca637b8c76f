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
    DYFOX_ENOSYS = 7,      /* configuration not supported                  */
    DYFOX_ETIMEOUT = 8     /* a bounded device wait ran out (the kernel
                              returned; its results are not valid)         */
} dyfox_status;

/* Precision of a march.  FP64: plain double everywhere (parity mode).
 * FP32: single-precision march in the interaction picture with compensated
 * amplitude updates (Dekker Fast2Sum); per-segment Volterra terms and sincos in
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
#define DYFOX_FLAG_H_FP64 16u  /* FP32 + H_SEGMENTS: sum the segment terms
                                  exactly (each rounded to 2^-66 rad) and
                                  round the total to double (in double, in
                                  order, where the terms' magnitudes sum to
                                  2^17 rad or more) and reduce mod 2 pi in
                                  double, instead of in float-float
                                  (two-sum) arithmetic                       */
#define DYFOX_FLAG_PAIRS 32u   /* FP32 compensated, fused segments or staged
                                  e^{iH}, n_e >= 2: march two deviation
                                  parameters per thread in packed f32x2
                                  arithmetic (same results bit for bit)      */
#define DYFOX_FLAG_SCALAR 64u  /* FP32: one deviation parameter per thread
                                  (overrides DYFOX_FLAG_PAIRS)               */

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
 * (precision FP64) or floats (FP32).  DYFOX_ESMEM for rows of more than
 * about 25,000 columns (a row's coordinates are kept in shared memory). */
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

/* Device status of the last dyfox_laue_solve or dyfox_laue_solve_to_host
 * queued on `stream` with this workspace:
 * synchronises `stream`, then DYFOX_OK, or DYFOX_ETIMEOUT when a staged
 * row's copy into shared memory did not complete within its bounded wait
 * (about 2 s; the march then wrote that row's exit waves as NaN and
 * returned instead of waiting longer). */
int dyfox_laue_solve_status(const dyfox_laue_desc *d, const void *workspace,
                            size_t workspace_bytes, void *stream);

/* dyfox_laue_solve with the exit waves also copied into host memory while
 * the march proceeds: the active rows are marched in n_chunks row chunks
 * (at most 64 and one per 8 rows; 0: about 8, each a whole number of
 * waves of resident CTAs with the remainder rows last), every deviation
 * parameter in one launch per chunk, and after each chunk's march its rows of every wave
 * are copied into host_out (same layout; pinned, for the copies to
 * overlap) on copy_stream (NULL: `stream`), behind an event on `stream`;
 * the rows outside the beam are copied at once.  Returns once the work is
 * queued; host_out is complete when copy_stream is.  No DYFOX counterpart
 * (DYFOX returns device arrays): the copy of a 256-angle scan's 1.2 GB of
 * waves hides behind its march. */
int dyfox_laue_solve_to_host(const dyfox_laue_desc *d, const double *s_dev,
                             const void *h_grid, const double *seg_table,
                             void *out, void *host_out, void *workspace,
                             size_t workspace_bytes, int n_chunks,
                             void *stream, void *copy_stream);

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
 * capture.  Under CUDA's default lazy module loading the array's memory is
 * reserved at that first call on each device, which can therefore still
 * fail for lack of device memory: callers that must not fail mid-run make
 * one call during start-up (under CUDA_MODULE_LOADING=EAGER it is reserved
 * when the library loads).  The address is kept for the process: do not
 * call this entry point after a cudaDeviceReset.  All calls share the
 * array, which keeps the last call's contents (nothing in it has to start
 * at zero); calls whose work overlaps on the GPU race on it and must be
 * serialised.  Later calls allocate no device memory. */
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
    unsigned flags;                          /* DYFOX_BRAGG_* or 0         */
} dyfox_bragg_desc;

/* dyfox_bragg_desc.flags: for checks, a DYFOX_FP32 solve hands every system
 * over to its double-precision continuation (the path of a system the
 * mixed solve does not converge within maxiter restarts). */
#define DYFOX_BRAGG_FORCE_RESUME 1u

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
 * and preconditioner) run in single precision; b and every true residual
 * come from a float-float march (about 2^-44 relative a step); the
 * Gram-Schmidt coefficients, the rotations and the solution stay in
 * double, so the stopping test is the same true residual <= tol.  Inputs
 * and outputs keep their complex128 layout.  The workspace grows by the
 * single-precision couplings and their remainders. */
int dyfox_bragg_solve(const dyfox_bragg_desc *d, const double *seg_table,
                      const double *y_values, const double *s_dev,
                      const void *x0, void *out, double *info,
                      void *workspace, size_t workspace_bytes, void *stream);

/* One operator application per system, for parity checks.
 * mode 0: out = down-march of (D0(0), Dg(0)) = (in0, in1) to D_g(t)
 *         (bragg/solver.py:28-35; NULL input = zero);
 * mode 1: out = ifft(fft(in0) / T22s) (solver.py:167-168, 297-300);
 * mode 2 (precision DYFOX_FP32 only): mode 0 in the float-float arithmetic
 *         of the mixed solve's right-hand side and residuals.
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

/* ---- Batched uneven instances --------------------------------------------
 * No single DYFOX counterpart: a set of independent Laue and Bragg solves of
 * different sizes (what a caller would otherwise issue as one
 * solve_dislocation / solve_surface_batch call per instance) planned once
 * and replayed as one CUDA graph:
 *   * every Laue instance's per-angle set-up, then ONE persistent march
 *     launch over a cost-sorted queue of (instance, row) items: the CTA that
 *     takes an item stages e^{iH} of that row once into its own slab and
 *     marches every angle group of the instance through it;
 *   * every Bragg instance's couplings / symbol set-up, then one CTA per
 *     (instance, deviation parameter, plane) system, longest first: one
 *     launch per launch shape present (precision, threads, columns per
 *     thread, as a single solve of the instance would choose them).
 * Laue items: precision DYFOX_FP32 (compensated march), h_source
 * DYFOX_H_SEGMENTS or DYFOX_H_NONE, shift_px == 1, Nx even and at most
 * 32 * cols_per_lane * warps; flags DYFOX_FLAG_H_FP64 sums the segment
 * terms and reduces mod 2 pi in double (else float-float).  Output
 * (n_e, Ny, Nx) complex64.  Bragg items: as dyfox_bragg_solve (either
 * precision; x0 = 0), output (n_s, n_y, Nx) complex128, y_values on the
 * HOST (uploaded by dyfox_batch_create). */
#define DYFOX_BATCH_LAUE 0
#define DYFOX_BATCH_BRAGG 1

typedef struct dyfox_batch_item {
    int kind;                     /* DYFOX_BATCH_LAUE / DYFOX_BATCH_BRAGG     */
    dyfox_laue_desc laue;         /* kind LAUE                                */
    dyfox_bragg_desc bragg;       /* kind BRAGG                               */
    const double *s_dev;          /* device: n_e (Laue) / n_s (Bragg)         */
    const double *seg_table;      /* device: n_seg x DYFOX_SEG_STRIDE, or NULL*/
    const double *y_values;       /* BRAGG: HOST, n_y doubles                 */
    void *out;                    /* device output (see above)                */
    double *info;                 /* BRAGG: device (n_s * n_y, 4), or NULL    */
} dyfox_batch_item;

typedef struct dyfox_batch_opts {
    int laue_cols_per_lane;       /* 5, 7, 9 or 11; 0: 5                     */
    int laue_warps;               /* warps per CTA of the Laue march: 4, 8 or
                                     16; 0: 8                                 */
    int laue_ctas_per_sm;         /* resident CTAs per SM; 0: occupancy max   */
    unsigned flags;               /* DYFOX_FLAG_H_FP64                        */
} dyfox_batch_opts;

typedef struct dyfox_batch dyfox_batch;     /* opaque plan + CUDA graph */

/* Workspace bytes of a batch into *bytes; a status (invalid or unsupported
 * items: see dyfox_last_error). */
int dyfox_batch_workspace_bytes(const dyfox_batch_item *items, int n,
                                const dyfox_batch_opts *opts, size_t *bytes);

/* Plans the batch, uploads its tables (synchronously, on `stream`), and
 * captures and instantiates its CUDA graph.  The workspace, items' inputs
 * and outputs must stay valid until dyfox_batch_destroy; opts may be NULL. */
int dyfox_batch_create(const dyfox_batch_item *items, int n,
                       const dyfox_batch_opts *opts, void *workspace,
                       size_t workspace_bytes, void *stream,
                       dyfox_batch **batch);

/* Replays the batch's graph on `stream` (asynchronous). */
int dyfox_batch_launch(dyfox_batch *batch, void *stream);

/* Kernel launches one replay makes (the graph's kernel nodes). */
int dyfox_batch_kernel_count(const dyfox_batch *batch);

/* Device status of the last replay queued on `stream`: synchronises
 * `stream`, then DYFOX_OK, or DYFOX_ETIMEOUT when a staged row's copy into
 * shared memory did not complete within its bounded wait (that row's exit
 * waves read NaN). */
int dyfox_batch_status(const dyfox_batch *batch, void *stream);

/* Frees the graph and the plan (not the workspace). */
int dyfox_batch_destroy(dyfox_batch *batch);

/* ---- Imaging and rocking-scan maps -----------------------------------------
 * Pupil of an objective on the fftshifted frequency grid (replaces
 * Optics.pupil, optics.py:64-118): frequency (i - N/2) / (N dx) per axis;
 * the aperture disc of radius aperture_f (NA / lambda) about (aperture_fx,
 * aperture_fy); for ell != 0 the spiral phase ell atan2(fy - sy, fx - sx)
 * about (singularity_fx, singularity_fy), quantised to `levels` steps when
 * levels > 0; dc_zero != 0 zeroes the origin bin (the caller applies the
 * reference's "exact" / "half_bin" / "never" policy).  pupil: device
 * (Ny, Nx) complex128 (FP64) or complex64 (FP32). */
int dyfox_pupil(int Nx, int Ny, double dx, double aperture_f, int ell,
                double aperture_fx, double aperture_fy, double singularity_fx,
                double singularity_fy, int dc_zero, int levels, int precision,
                void *pupil, void *stream);

/* Workspace bytes of dyfox_image for n images of Ny x Nx (even sizes). */
int dyfox_image_workspace_bytes(int n, int Ny, int Nx, int precision,
                                size_t *bytes);

/* Image-plane intensity of n exit waves through one pupil (replaces
 * image_intensity / object_spectrum / image_from_spectrum, optics.py:
 * 170-207): I = |ifft2(fft2(u) ifftshift(P))|^2, equal to the reference's
 * shifted composition for even Ny, Nx.  stack: device (n, Ny, Nx) complex
 * of `precision` (unchanged); pupil: as dyfox_pupil, same precision.
 * out (may be NULL): device (n, Ny, Nx) float64 / float32.  With sum_I !=
 * NULL the images are also reduced as com_maps does (analysis/rocking.py:
 * 37-83): sum_I[y][x] += I, sum_wI[y][x] += phi[e] I (device (Ny, Nx)
 * doubles, accumulated across calls, images in order: deterministic), and
 * rock (device n doubles, may be NULL) receives sum_xy I per image; phi:
 * device n doubles. */
int dyfox_image(const void *stack, int n, int Ny, int Nx, int precision,
                const void *pupil, void *out, const double *phi,
                double *sum_wI, double *sum_I, double *rock, void *workspace,
                size_t workspace_bytes, void *stream);

/* ---- Learned shooting guess (no DYFOX counterpart) ------------------------
 * A 4-level U-Net, 32 base channels, bfloat16 storage and FP32 accumulation
 * (the 3x3 convolutions are implicit GEMMs on the tensor cores), mapping
 * (cos, sin) of H on the first 8 depth slices of a set of y-planes plus the
 * deviation parameter (input (n, H, W, 32) bf16, channels 17..31 zero) to
 * the shooting unknown D_g(0) minus its perfect-crystal value ((n, H, W, 2)
 * float32, Re and Im).  The Bragg solve takes it as x0 (dyfox_bragg_solve)
 * and keeps its own residual test.  Parameters: FP32, flat, in the order of
 * the layer list (per 3x3 convolution W[Cout][3][3][Cin] then b[Cout]:
 * e0a e0b e1a e1b e2a e2b ba bb d2a d2b d1a d1b d0a d0b; then the 1x1 head
 * W[2][32], b[2]).  All buffers live in one caller workspace (256-byte
 * aligned). */
typedef struct dyfox_unet dyfox_unet;

size_t dyfox_unet_param_count(void);
int dyfox_unet_workspace_bytes(int batch, int H, int W, size_t *bytes);
int dyfox_unet_create(int batch, int H, int W, void *workspace,
                      size_t workspace_bytes, dyfox_unet **net);
int dyfox_unet_destroy(dyfox_unet *net);
/* Device pointers of the FP32 parameters and of their gradients. */
int dyfox_unet_params(dyfox_unet *net, float **params, float **grads);
/* He-normal weights from a counter-based generator, zero biases and Adam
 * state. */
int dyfox_unet_init(dyfox_unet *net, unsigned long long seed, void *stream);
/* Refresh the bfloat16 weight copies after the FP32 parameters changed. */
int dyfox_unet_refresh(dyfox_unet *net, void *stream);
/* Forward pass of n <= batch samples; y (device, may be NULL) receives the
 * (n, H, W, 2) output.  Keeps the activations for dyfox_unet_backward. */
int dyfox_unet_forward(dyfox_unet *net, const void *x, int n, float *y,
                       void *stream);
/* Gradients of L = sum((y - t)^2) / (2 * 2 n H W) after a forward pass;
 * loss (device float, may be NULL) receives L. */
int dyfox_unet_backward(dyfox_unet *net, const float *target, float *loss,
                        void *stream);
/* One Adam step on the gradients, then refresh of the bfloat16 copies. */
int dyfox_unet_adam(dyfox_unet *net, float lr, float beta1, float beta2,
                    float eps, void *stream);
/* Network input from the top 8 depth slices of H: h_top (n_y, 8, Nx)
 * doubles, columns (col0 + x) mod Nx for x < W (the lateral grid is
 * periodic), s_values (n_s doubles, already scaled); x_out (n_s, n_y, W,
 * 32) bfloat16. */
int dyfox_unet_features(const double *h_top, int n_y, int Nx, int col0,
                        int W, const double *s_values, int n_s, void *x_out,
                        void *stream);
/* Error code recorded by a tcgen05 convolution whose bounded wait expired
 * (0 none, 1 a load, 2 a stage release, 3 the accumulator); clear != 0
 * resets it.  Synchronises the device. */
int dyfox_unet_tc_error(int *code, int clear);

/* Device buffer of the last forward / backward pass, for checks: which 0
 * conv output `index` (bf16), 1 pooled tensor (bf16), 2 concatenated input
 * of d2a / d1a / d0a (bf16), 3 gradient of conv output `index` (float);
 * sized for the network's batch, NHWC. */
int dyfox_unet_buffer(dyfox_unet *net, int which, int index, void **ptr,
                      size_t *bytes);
/* One 3x3 convolution product, for checks: mode 0 out = bf16(relu(conv(X,
 * Wk) + bias)) (Wk [Cout][9][Cin]); mode 1 out = data gradient of G
 * (float, (N, H, W, Cin); Wk the transposed weights [Cin][9][Cout]); mode
 * 2 out = weight gradient [Cout][9][Cin] (float) of X and G, with the
 * split partials in the workspace.  Channels multiples of 32.  All three
 * run on the tcgen05 tensor cores (TMEM accumulators, TMA-staged tiles)
 * when rows hold 128 pixels or divide 128 (mode 2 also needs a workspace
 * of at least 9 Cin Cout floats); mode | DYFOX_CONV_MMA_SYNC runs the
 * mma.sync implicit GEMM instead (cross-checks). */
#define DYFOX_CONV_MMA_SYNC 16
int dyfox_unet_conv(int mode, const void *X, const void *G, const void *Wk,
                    const float *bias, void *out, int N, int H, int W,
                    int Cin, int Cout, void *workspace,
                    size_t workspace_bytes, void *stream);

/* Diagnostic (not part of any DYFOX interface): measured FMA throughput
 * of this GPU in TFLOP/s (2 flops per FMA) for DYFOX_FP64 or DYFOX_FP32,
 * the denominator of the arithmetic-bound kernels' roofline.  Synchronises
 * `stream`; allocates one scalar of device memory for the call. */
int dyfox_pipe_peak(int precision, int iters, double *tflops, void *stream);

/* Diagnostic (not part of any DYFOX interface): the single-precision
 * building blocks of the fused Volterra phase beside CUDA's correctly
 * rounded operations, elementwise over n device floats a (and b) into out:
 * op 0 the Newton-refined reciprocal of a, 1 __frcp_rn(a), 2 the
 * residual-corrected quotient a / b, 3 __fdiv_rn(a, b) (float out); op 4
 * the integer-built widening of a to double used by the FP64 segment sum,
 * 5 the hardware conversion (double out). */
int dyfox_arith_probe(int op, const float *a, const float *b, void *out,
                      int n, void *stream);
/* The same for the double-precision blocks of the FP64 Volterra field:
 * op 0 the table-driven atan2(a, b), 1 CUDA's atan2(a, b), 2 the
 * table-driven log(a), 3 CUDA's log(a), 4 the Newton-refined reciprocal of
 * a, 5 __drcp_rn(a); n device doubles a (and b) into out. */
int dyfox_arith_probe64(int op, const double *a, const double *b,
                        double *out, int n, void *stream);
/* The FP64 segment sum of the FP32 march (the sum exact on a 2^-66 grid
 * rounded to double, or in double in order past its range) over each of n
 * groups of m device floats (terms, n * m of them) into n device doubles
 * out. */
int dyfox_seg_sum_probe(const float *terms, int m, double *out, int n,
                        void *stream);

/* Diagnostic (not part of any DYFOX interface): with on != 0, each later
 * dyfox_laue_solve on the calling thread records CUDA events on its stream
 * around its kernels; dyfox_laue_kernel_ms then gives the last such solve's
 * kernel durations in ms: [0] the prologue (zero rows, per-angle tables,
 * pivots), [1] the e^{iH} staging (0 when not staged), [2] the march.
 * dyfox_laue_kernel_ms synchronises on the last event. */
int dyfox_kernel_timing(int on);
int dyfox_laue_kernel_ms(float ms[3]);

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
