/* Error model of the compensated single-precision Laue march (test-side).
 *
 * A scalar C restatement of the arithmetic of laue_march_kernel<float,...>
 * (dyfox_gb300/csrc/laue_march.cuh, the step loop) and of its per-angle
 * tables (laue_setup_item in dyfox_gb300/csrc/laue.cu), with one change:
 * the phase factor e^{iH} of each voxel is the correctly rounded float of
 * cos H and sin H from a double H.  Comparing it with the double-precision
 * oracle therefore measures what the single-precision march arithmetic
 * itself costs, separately from the single-precision Volterra terms.
 *
 * Built with -ffp-contract=off: every fused multiply-add below is an
 * explicit fmaf, as in the kernel, and nothing else is contracted.
 *
 *   march_f32_model(comp, sig[6], s, ds, Nz, Nx, dx, sheet_hw, H, out)
 *     comp   1: Fast2Sum-compensated amplitudes (the library's default)
 *            0: plain single-precision updates
 *     H      (Nz, Nx) doubles, row k the phase of step k
 *     out    Nx complex doubles (re, im), the exit D_g as the kernel
 *            writes it (rounded to float)
 */
#include <math.h>
#include <stdlib.h>

static float fast2sum(float a, float b, float *err) {
    const float s = a + b;
    *err = b - (s - a);
    return s;
}

int march_f32_model(int comp, const double *sig, double s, double ds, int Nz,
                    int Nx, double dx, double sheet_hw, const double *H,
                    double *out) {
    const double s0r = sig[0], s0i = sig[1], shr = sig[2], shi = sig[3];
    const double sbr = sig[4], sbi = sig[5];
    const double pi = 3.14159265358979323846;
    const double alpha = -2.0 * pi * s;
    const double gam = sqrt((shr * shr + shi * shi) + alpha * alpha * 0.25);
    const double cg = cos(gam * ds), sg = sin(gam * ds) / gam;
    const double p22i = alpha * 0.5 * sg;
    const double rho = hypot(cg, p22i), th = atan2(p22i, cg);
    const int nsteps = Nz - 1;

    /* A, B and their low words; one zero column past each edge. */
    float *v = calloc((size_t)8 * (Nx + 2), sizeof(float));
    if (!v) return 1;
    float *Ar = v + 1, *Ai = Ar + Nx + 2, *Br = Ai + Nx + 2, *Bi = Br + Nx + 2;
    float *Alr = Bi + Nx + 2, *Ali = Alr + Nx + 2, *Blr = Ali + Nx + 2,
          *Bli = Blr + Nx + 2;
    for (int x = 0; x < Nx; ++x) {
        const double xp = (x - Nx / 2) * dx;
        Ar[x] = (float)(sheet_hw > 0 ? (fabs(xp) < sheet_hw ? 1.0 : 0.0)
                                     : exp(-xp * xp / (2.0 * sheet_hw * sheet_hw)));
    }
    for (int k = 0; k < nsteps; ++k) {
        /* kappa_12, kappa_21 of step k in double, then rounded */
        const double m = 2.0 * k + 1.0, ph = m * th, pe = fma(m, th, -ph);
        const double sp = sin(ph), cp = cos(ph);
        const double wr = cp - sp * pe, wi = sp + cp * pe, f = sg / rho;
        const float k12r = (float)(f * (sbr * wr - sbi * wi));
        const float k12i = (float)(f * (sbr * wi + sbi * wr));
        const float k21r = (float)(f * (shr * wr + shi * wi));
        const float k21i = (float)(f * (shi * wr - shr * wi));
        float pbr = 0, pbi = 0, pblr = 0, pbli = 0;   /* B, low of x - 1 */
        for (int x = 0; x < Nx; ++x) {
            const double h = H[(size_t)k * Nx + x];
            const float ex = (float)cos(h), ey = (float)sin(h);
            const float ar = Ar[x + 1], ai = Ai[x + 1];
            const float alr = Alr[x + 1], ali = Ali[x + 1];
            const float br = pbr, bi = pbi, blr = pblr, bli = pbli;
            pbr = Br[x]; pbi = Bi[x]; pblr = Blr[x]; pbli = Bli[x];
            const float m12r = fmaf(k12r, ex, -k12i * ey);
            const float m12i = fmaf(k12r, ey, k12i * ex);
            const float m21r = fmaf(k21r, ex, k21i * ey);
            const float m21i = fmaf(k21i, ex, -k21r * ey);
            if (comp) {
                const float tr = fmaf(m12r, br, fmaf(-m12i, bi, alr));
                const float ti = fmaf(m12r, bi, fmaf(m12i, br, ali));
                const float ur = fmaf(m21r, ar, fmaf(-m21i, ai, blr));
                const float ui = fmaf(m21r, ai, fmaf(m21i, ar, bli));
                Ar[x] = fast2sum(ar, tr, &Alr[x]);
                Ai[x] = fast2sum(ai, ti, &Ali[x]);
                Br[x] = fast2sum(br, ur, &Blr[x]);
                Bi[x] = fast2sum(bi, ui, &Bli[x]);
            } else {
                Ar[x] = fmaf(m12r, br, fmaf(-m12i, bi, ar));
                Ai[x] = fmaf(m12r, bi, fmaf(m12i, br, ai));
                Br[x] = fmaf(m21r, ar, fmaf(-m21i, ai, br));
                Bi[x] = fmaf(m21r, ai, fmaf(m21i, ar, bi));
            }
        }
    }
    /* the free propagation factored out of the interaction picture:
     * (e^{(sigma_0 + i alpha / 2) ds} (cos g ds + i alpha / 2 sin(g ds)/g))^N */
    const double er = exp(s0r * ds), pim = (s0i + alpha * 0.5) * ds;
    double br_ = er * cos(pim) * cg - er * sin(pim) * p22i;
    double bi_ = er * cos(pim) * p22i + er * sin(pim) * cg;
    double Sr = 1.0, Si = 0.0;
    for (int n = nsteps; n > 0; n >>= 1) {
        if (n & 1) {
            const double t = Sr * br_ - Si * bi_;
            Si = Sr * bi_ + Si * br_;
            Sr = t;
        }
        const double t = br_ * br_ - bi_ * bi_;
        bi_ = 2.0 * br_ * bi_;
        br_ = t;
    }
    for (int x = 0; x < Nx; ++x) {
        double b0 = Br[x], b1 = Bi[x];
        if (comp) { b0 += Blr[x]; b1 += Bli[x]; }
        out[2 * x] = (float)(Sr * b0 - Si * b1);
        out[2 * x + 1] = (float)(Sr * b1 + Si * b0);
    }
    free(v);
    return 0;
}
