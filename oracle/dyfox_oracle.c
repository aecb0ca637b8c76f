/*
 * ORACLE -- test infrastructure only.  This file is the CPU checker of the
 * dyfox_gb300 CUDA path and the timed CPU baseline of bench.py; nothing in
 * the product links it.  Parity is pinned: tests/test_oracle_pins.py checks
 * every function here against the golden vectors of tests/golden/ (made
 * from the DYFOX reference itself by tests/golden/make_golden.py) and, when
 * oracle/_ref is built, against the reference kernel source compiled for
 * the CPU.
 *
 * Plain C restatement of DYFOX's diffraction hot path:
 *   oracle_segment_frames   dislocations.py:68-90   (volterra_frame) and the
 *                           per-segment constants of dislocations.py:130-142
 *   oracle_h_rows           dislocations.py:113-168 (compute_H_grid) and
 *                           171-211 (H_plane): H = 2 pi g.u summed over the
 *                           segments in list order, FP64, one y per row
 *   oracle_laue_march       laue/kernels.py:48-150  (tt3d_fullfield_batch),
 *                           154-266 (tt3d_analytic_batch) and 269-352
 *                           (tt3d_pristine_batch), one block at a time
 *
 * Every arithmetic expression keeps the operation order of the reference.
 * Build with -ffp-contract=off so x86 and aarch64 give the same bits.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PI 3.14159265358979323846

/* One segment after volterra_frame: 16 doubles.
 * [0..2] core  [3..5] xi  [6..8] e1  [9..11] e2
 * [12] C_atan  [13] ge1  [14] ge2  [15] b_perp                              */
#define OSEG 16

static double dot3(const double *a, const double *b) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

static double norm3(const double *a) { return sqrt(dot3(a, a)); }

static void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* dislocations.py:68-90 plus the constants of compute_H_grid (130-142).
 * segs: n x 9 (r_start, r_end, b).  Segments shorter than 1e-20 m are
 * skipped (dislocations.py:134-135).  Returns the number kept.            */
int oracle_segment_frames(const double *segs, int n, const double *g,
                          double *out) {
    int kept = 0;
    for (int s = 0; s < n; ++s) {
        const double *ra = segs + 9 * s, *rb = ra + 3, *bv = ra + 6;
        double t[3] = {rb[0] - ra[0], rb[1] - ra[1], rb[2] - ra[2]};
        double L = norm3(t);
        if (L < 1e-20) continue;
        double *o = out + OSEG * kept;
        double xi[3] = {t[0] / L, t[1] / L, t[2] / L};
        double core[3] = {(ra[0] + rb[0]) / 2.0, (ra[1] + rb[1]) / 2.0,
                          (ra[2] + rb[2]) / 2.0};
        double b_screw = dot3(bv, xi);
        double bp[3] = {bv[0] - b_screw * xi[0], bv[1] - b_screw * xi[1],
                        bv[2] - b_screw * xi[2]};
        double b_perp = norm3(bp);
        double e1[3], e2[3];
        if (b_perp > 1e-20) {
            e1[0] = bp[0] / b_perp; e1[1] = bp[1] / b_perp;
            e1[2] = bp[2] / b_perp;
        } else if (fabs(xi[2]) > 0.9) {
            e1[0] = 1.0; e1[1] = 0.0; e1[2] = 0.0;
        } else {
            double ax[3] = {0, 0, 0};
            if (fabs(xi[0]) < 0.9) ax[0] = 1.0; else ax[1] = 1.0;
            cross3(xi, ax, e1);
            double m = norm3(e1);
            e1[0] /= m; e1[1] /= m; e1[2] /= m;
        }
        cross3(xi, e1, e2);
        double ge1 = dot3(g, e1), ge2 = dot3(g, e2);
        memcpy(o, core, sizeof core);
        memcpy(o + 3, xi, sizeof xi);
        memcpy(o + 6, e1, sizeof e1);
        memcpy(o + 9, e2, sizeof e2);
        o[12] = ge1 * b_perp + dot3(g, xi) * b_screw;
        o[13] = ge1;
        o[14] = ge2;
        o[15] = b_perp;
        ++kept;
    }
    return kept;
}

/* H of one segment at lab point offsets (X, Y, Z) = r - core, in the
 * operation order of dislocations.py:148-164.                              */
static double h_one(const double *sg, double X, double Y, double Z,
                    double nu, double a_core) {
    const double *xi = sg + 3, *e1 = sg + 6, *e2 = sg + 9;
    double eta = (X * xi[0] + Y * xi[1]) + Z * xi[2];
    double Px = X - eta * xi[0], Py = Y - eta * xi[1], Pz = Z - eta * xi[2];
    double d1 = (Px * e1[0] + Py * e1[1]) + Pz * e1[2];
    double d2 = (Px * e2[0] + Py * e2[1]) + Pz * e2[2];
    double r2 = d1 * d1 + d2 * d2;
    double a2 = a_core * a_core;
    double r2c = r2 > a2 ? r2 : a2;
    double H = sg[12] * atan2(d2, d1);
    double b_perp = sg[15];
    if (b_perp > 1e-20) {
        double onu = 1.0 - nu;
        double c1 = b_perp / (2 * ORACLE_PI);
        double ux = c1 * d1 * d2 / ((2 * onu) * r2c);
        double uy = -c1 * ((1 - 2 * nu) / (4 * onu) * log(r2c)
                           + (d1 * d1 - d2 * d2) / ((4 * onu) * r2c));
        H = H + (2 * ORACLE_PI) * (sg[13] * ux + sg[14] * uy);
    }
    return H;
}

/* H on rows of constant y: out[r][k][i] for y = y_values[r], x_i =
 * (i - Nx/2) dx, z_k = k dz.  Segments are summed in list order starting
 * from zero (dislocations.py:139, 166; 181, 210).  cast_fp32 != 0 gives
 * compute_H_grid(precision=FP32): each segment's FP64 value is rounded to
 * float before a float accumulation; the result is stored widened.       */
void oracle_h_rows(const double *frames, int n_seg, double nu, double a_core,
                   int Nx, int Nz, double dx, double dz,
                   const double *y_values, int n_rows, int cast_fp32,
                   double *out) {
    #pragma omp parallel for collapse(2) schedule(static)
    for (int r = 0; r < n_rows; ++r)
        for (int k = 0; k < Nz; ++k) {
            double z = k * dz;
            for (int i = 0; i < Nx; ++i) {
                double x = (i - Nx / 2.0) * dx;
                double acc = 0.0;
                float accf = 0.0f;
                for (int s = 0; s < n_seg; ++s) {
                    const double *sg = frames + OSEG * s;
                    double h = h_one(sg, x - sg[0], y_values[r] - sg[1],
                                     z - sg[2], nu, a_core);
                    if (cast_fp32) accf = accf + (float)h;
                    else acc = acc + h;
                }
                out[((size_t)r * Nz + k) * Nx + i] = cast_fp32 ? accf : acc;
            }
        }
}

/* Closed-form parameters of tt3d_analytic_batch (dislocations.py:214-242):
 * y0 z0 e1y e1z e2y e2z C_atan ge1 ge2 b_perp nu a2                        */
enum { AN_Y0, AN_Z0, AN_E1Y, AN_E1Z, AN_E2Y, AN_E2Z, AN_C, AN_GE1, AN_GE2,
       AN_BP, AN_NU, AN_A2 };

/* The Laue march of laue/kernels.py, one (row, angle) block at a time.
 * mode 0 = pristine (269-352), 1 = full field with H_rows (48-150),
 * 2 = analytic (154-266).  rows lists the y indices to compute (NULL: all
 * Ny); H_rows is indexed by position in that list: [r][k][i].  Outputs are
 * complex interleaved, [e][r][i].                                          */
void oracle_laue_march(int mode, double s0r, double s0i, double shr,
                       double shi, double sbr, double sbi,
                       const double *s_dev, int n_e, double dz,
                       double shift_px, double ds, double dx, int Nz,
                       int Nx, int Ny, double sheet_hw, double fov_hy,
                       const double *H_rows, const double *an,
                       const int *rows, int n_rows, double *out) {
    if (!rows) n_rows = Ny;
    #pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int e = 0; e < n_e; ++e)
        for (int r = 0; r < n_rows; ++r) {
            int iy = rows ? rows[r] : r;
            double *o = out + 2 * ((size_t)e * n_rows + r) * Nx;
            double y_pix = (iy - Ny / 2) * dx;
            if (fabs(y_pix) >= fov_hy) {
                for (int i = 0; i < 2 * Nx; ++i) o[i] = 0.0;
                continue;
            }
            double *cur = malloc(sizeof(double) * 4 * (Nx + 1));
            double *nxt = malloc(sizeof(double) * 4 * (Nx + 1));
#define S(b, a, i) (b)[(a) * (Nx + 1) + (i)]
            for (int ix = 0; ix < Nx; ++ix) {
                double x_pos = (ix - Nx / 2) * dx;
                double beam = sheet_hw > 0.0
                    ? (fabs(x_pos) < sheet_hw ? 1.0 : 0.0)
                    : exp(-x_pos * x_pos / (2.0 * sheet_hw * sheet_hw));
                S(cur, 0, ix) = beam; S(cur, 1, ix) = 0.0;
                S(cur, 2, ix) = 0.0;  S(cur, 3, ix) = 0.0;
            }
            double alpha = -2.0 * ORACLE_PI * s_dev[e];
            double gam = sqrt((shr * shr + shi * shi) + alpha * alpha * 0.25);
            double exp_pr = exp(s0r * ds);
            double cg, sg;
            if (gam > 1e-30) { cg = cos(gam * ds); sg = sin(gam * ds) / gam; }
            else { cg = 1.0; sg = ds; }
            double P11r = cg, P11i = -alpha * 0.5 * sg;
            double P22r = cg, P22i = alpha * 0.5 * sg;
            double pi_ = (s0i + alpha * 0.5) * ds;
            double epr = exp_pr * cos(pi_), epi = exp_pr * sin(pi_);
            double M11r = epr * P11r - epi * P11i, M11i = epr * P11i + epi * P11r;
            double M22r = epr * P22r - epi * P22i, M22i = epr * P22i + epi * P22r;
            double dy = 0, c1 = 0, onu = 0;
            if (mode == 2) {
                dy = y_pix - an[AN_Y0];
                onu = 1.0 - an[AN_NU];
                c1 = an[AN_BP] / (2.0 * ORACLE_PI);
            }
            for (int k = 0; k < Nz - 1; ++k) {
                double Ha = 0.0;
                if (mode == 2) {
                    double dzv = k * dz - an[AN_Z0];
                    double d1 = dy * an[AN_E1Y] + dzv * an[AN_E1Z];
                    double d2 = dy * an[AN_E2Y] + dzv * an[AN_E2Z];
                    double r2 = d1 * d1 + d2 * d2;
                    double r2c = r2 > an[AN_A2] ? r2 : an[AN_A2];
                    Ha = an[AN_C] * atan2(d2, d1);
                    if (an[AN_BP] > 0.0) {
                        double nu = an[AN_NU];
                        double ux = c1 * d1 * d2 / (2.0 * onu * r2c);
                        double uy = -c1 * ((1.0 - 2.0 * nu) / (4.0 * onu) * log(r2c)
                                           + (d1 * d1 - d2 * d2) / (4.0 * onu * r2c));
                        Ha += 2.0 * ORACLE_PI * (an[AN_GE1] * ux + an[AN_GE2] * uy);
                    }
                }
                for (int ix = 0; ix < Nx; ++ix) {
                    double M12r, M12i, M21r, M21i;
                    if (mode == 0) {
                        double P12r = sbr * sg, P12i = sbi * sg;
                        double P21r = shr * sg, P21i = shi * sg;
                        M12r = epr * P12r - epi * P12i; M12i = epr * P12i + epi * P12r;
                        M21r = epr * P21r - epi * P21i; M21i = epr * P21i + epi * P21r;
                    } else {
                        double H = mode == 1
                            ? H_rows[((size_t)r * Nz + k) * Nx + ix] : Ha;
                        double cH = cos(H), sH = sin(H);
                        double P12r = (sbr * cH - sbi * sH) * sg;
                        double P12i = (sbi * cH + sbr * sH) * sg;
                        double P21r = (shr * cH + shi * sH) * sg;
                        double P21i = (shi * cH - shr * sH) * sg;
                        M12r = epr * P12r - epi * P12i; M12i = epr * P12i + epi * P12r;
                        M21r = epr * P21r - epi * P21i; M21i = epr * P21i + epi * P21r;
                    }
                    double src0 = (double)ix + shift_px;
                    int i0 = (int)floor(src0);
                    double f0 = src0 - (double)i0, d0r, d0i;
                    if (i0 >= 0 && i0 + 1 < Nx) {
                        d0r = (1 - f0) * S(cur, 0, i0) + f0 * S(cur, 0, i0 + 1);
                        d0i = (1 - f0) * S(cur, 1, i0) + f0 * S(cur, 1, i0 + 1);
                    } else if (i0 >= 0 && i0 < Nx) {
                        d0r = (1 - f0) * S(cur, 0, i0); d0i = (1 - f0) * S(cur, 1, i0);
                    } else { d0r = 0; d0i = 0; }
                    double srcg = (double)ix - shift_px;
                    int ig = (int)floor(srcg);
                    double fg = srcg - (double)ig, dgr, dgi;
                    if (ig >= 0 && ig + 1 < Nx) {
                        dgr = (1 - fg) * S(cur, 2, ig) + fg * S(cur, 2, ig + 1);
                        dgi = (1 - fg) * S(cur, 3, ig) + fg * S(cur, 3, ig + 1);
                    } else if (ig >= 0 && ig < Nx) {
                        dgr = (1 - fg) * S(cur, 2, ig); dgi = (1 - fg) * S(cur, 3, ig);
                    } else { dgr = 0; dgi = 0; }
                    S(nxt, 0, ix) = M11r * d0r - M11i * d0i + M12r * dgr - M12i * dgi;
                    S(nxt, 1, ix) = M11r * d0i + M11i * d0r + M12r * dgi + M12i * dgr;
                    S(nxt, 2, ix) = M21r * d0r - M21i * d0i + M22r * dgr - M22i * dgi;
                    S(nxt, 3, ix) = M21r * d0i + M21i * d0r + M22r * dgi + M22i * dgr;
                }
                double *t = cur; cur = nxt; nxt = t;
            }
            for (int ix = 0; ix < Nx; ++ix) {
                o[2 * ix] = S(cur, 2, ix);
                o[2 * ix + 1] = S(cur, 3, ix);
            }
#undef S
            free(cur);
            free(nxt);
        }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
