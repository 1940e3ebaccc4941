/* fftgal_oracle -- CPU FP64 restatement of the reference's power-spectrum path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library (fftgal_gb300/)
 * links, loads or calls this file; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it, as the checker.
 *
 * Each function restates one reference function, in plain C99 FP64 with the
 * same operation order, so that (built with -ffp-contract=off) it reproduces
 * the reference's own arithmetic bit for bit when both use the same FFT.  The
 * FFT is oracle/fft64.c (FFTW's conventions; FFTW itself is not available).
 * Differences from the reference, all deliberate:
 *   - no file I/O and no assert(): results are returned in arrays and misuse
 *     returns a negative status;
 *   - the mode-count closure check uses `long` (the reference's
 *     `Ng*Ng*Ng-1` is an int expression and overflows at Ng = 2048);
 *   - Pmu takes the wedge count Nmu as a parameter (the reference fixes 3).
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "fft64.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846264338328
#endif
#define OG_SQRT3 1.73205080756887729352744634151

typedef struct og_grid {
    int Ng, Ng_pad;
    long Ng3_pad;
    double L;
    double offset[3];
    double *f;
} og_grid;

#define OF(g, i, j, k) ((g)->f[((long)(i) * (g)->Ng + (j)) * (g)->Ng_pad + (k)])
#define ORE(g, i, j, k) OF(g, i, j, 2 * (k))
#define OIM(g, i, j, k) OF(g, i, j, 2 * (k) + 1)

static inline double sq(double x) { return x * x; }
static inline double cube(double x) { return x * x * x; }
static inline double quart(double x) { double x2 = x * x; return x2 * x2; }

/* allocation part of fft_init (src/fft.c:13-24) */
og_grid *og_grid_new(int Ng, double L) {
    if (Ng < 1) return NULL;
    og_grid *g = (og_grid *)calloc(1, sizeof(og_grid));
    if (!g) return NULL;
    g->Ng = Ng;
    g->L = L;
    g->Ng_pad = 2 * (Ng / 2 + 1);
    g->Ng3_pad = (long)Ng * Ng * g->Ng_pad;
    g->f = (double *)calloc((size_t)g->Ng3_pad, sizeof(double));
    if (!g->f) { free(g); return NULL; }
    return g;
}

void og_grid_free(og_grid *g) {
    if (g) { free(g->f); free(g); }
}

double *og_grid_data(og_grid *g) { return g->f; }
long og_grid_size(og_grid *g) { return g->Ng3_pad; }
void og_grid_offset(og_grid *g, double out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = g->offset[i];
}

/* cubic B-spline (PCS) weights for fractional offset d (src/fft.c:83-88) */
static inline void pcs_weights(double d, double w[4]) {
    w[0] = cube(1 - d) / 6;
    w[1] = ((3 * d - 6) * sq(d) + 4) / 6;
    w[2] = (((-3 * d + 3) * d + 3) * d + 1) / 6;
    w[3] = cube(d) / 6;
}

/* base cell and the four periodic stencil cells (src/fft.c:68-82) */
static inline double pcs_cells(double u, int Ng, int c[4]) {
    int g1 = floor(u);
    double d = u - g1;
    g1 = (g1 % Ng + Ng) % Ng;
    c[0] = (g1 - 1 + Ng) % Ng;
    c[1] = g1;
    c[2] = (g1 + 1) % Ng;
    c[3] = (g1 + 2) % Ng;
    return d;
}

static void paint(og_grid *g, long Np, const double *x, const double *y,
                  const double *z, double Hinv, double alpha, int sub) {
    const int Ng = g->Ng;
    for (long p = 0; p < Np; ++p) {
        int ci[4], cj[4], ck[4];
        double wx[4], wy[4], wz[4];
        pcs_weights(pcs_cells(x[p] * Hinv - g->offset[0], Ng, ci), wx);
        pcs_weights(pcs_cells(y[p] * Hinv - g->offset[1], Ng, cj), wy);
        pcs_weights(pcs_cells(z[p] * Hinv - g->offset[2], Ng, ck), wz);
        for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c) {
            if (sub)
                OF(g, ci[a], cj[b], ck[c]) -= alpha * wx[a] * wy[b] * wz[c];
            else
                OF(g, ci[a], cj[b], ck[c]) += wx[a] * wy[b] * wz[c];
        }
    }
}

/* fft_p2g (src/fft.c:57-131): PCS mass assignment of a catalog (and of its
 * optional randoms, weighted by -alpha) onto the periodic grid, then scaled
 * to n/nbar.  `offset` is reduced with remainder() and written back. */
void og_p2g(og_grid *g, long Np, double V, const double *x, const double *y,
            const double *z, long Nr, const double *xr, const double *yr,
            const double *zr, double offset[3]) {
    const int Ng = g->Ng;
    for (int i = 0; i < 3; ++i) {
        offset[i] = remainder(offset[i], Ng);
        g->offset[i] = offset[i];
    }
    memset(g->f, 0, (size_t)g->Ng3_pad * sizeof(double));
    double Hinv = Ng / g->L;
    paint(g, Np, x, y, z, Hinv, 0, 0);
    if (Nr > 0 && xr) {
        double alpha = (double)Np / Nr;
        paint(g, Nr, xr, yr, zr, Hinv, alpha, 1);
    }
    double H3 = cube(g->L / Ng);
    double nbar = Np / V;
    double Npcinv = 1 / nbar / H3;
    for (long q = 0; q < g->Ng3_pad; ++q)
        g->f[q] *= Npcinv;
}

/* fft_offset_phase (src/fft.c:196-233), including its Nyquist behaviour: the
 * table entry for n = Ng/2 is written and then overwritten by its conjugate. */
int og_offset_phase(og_grid *g, int onoff) {
    if (onoff == 0) return -1;
    onoff = onoff > 0 ? 1 : -1;
    const int Ng = g->Ng;
    double *ph = (double *)malloc(sizeof(double) * 3 * Ng * 2);
    if (!ph) return -2;
#define PH(a, n, c) ph[((a) * Ng + (n)) * 2 + (c)]
    for (int a = 0; a < 3; ++a) { PH(a, 0, 0) = 1; PH(a, 0, 1) = 0; }
    for (int a = 0; a < 3; ++a)
    for (int n = 1; n <= Ng / 2; ++n) {
        double arg = -onoff * 2 * M_PI * n / Ng * g->offset[a];
        PH(a, n, 0) = cos(arg);
        PH(a, n, 1) = sin(arg);
        PH(a, Ng - n, 0) = PH(a, n, 0);
        PH(a, Ng - n, 1) = -PH(a, n, 1);
    }
    for (int i = 0; i < Ng; ++i)
    for (int j = 0; j < Ng; ++j)
    for (int k = 0; k <= Ng / 2; ++k) {
        double ar = PH(0, i, 0), ai = PH(0, i, 1);
        double br = PH(1, j, 0), bi = PH(1, j, 1);
        double cr = PH(2, k, 0), ci = PH(2, k, 1);
        double pr = ar * br * cr - ar * bi * ci - ai * br * ci - ai * bi * cr;
        double pi = ai * br * cr + ar * bi * cr + ar * br * ci - ai * bi * ci;
        double fr = ORE(g, i, j, k), fi = OIM(g, i, j, k);
        ORE(g, i, j, k) = fr * pr - fi * pi;
        OIM(g, i, j, k) = fr * pi + fi * pr;
    }
#undef PH
    free(ph);
    return 0;
}

/* fft_x2k (src/fft.c:172-181): forward r2c, times H^3, optional phase */
void og_x2k(og_grid *g, int offset_phase_on) {
    long nh = g->Ng / 2 + 1;
    fft64_r2c_3d(g->Ng, g->Ng, g->Ng, g->f, 2 * nh, g->f, nh);
    double H3 = cube(g->L / g->Ng);
    for (long q = 0; q < g->Ng3_pad; ++q)
        g->f[q] *= H3;
    if (offset_phase_on)
        og_offset_phase(g, 1);
}

/* fft_k2x (src/fft.c:184-193): backward c2r, times 1/L^3, optional phase */
void og_k2x(og_grid *g, int offset_phase_off) {
    long nh = g->Ng / 2 + 1;
    fft64_c2r_3d(g->Ng, g->Ng, g->Ng, g->f, nh, g->f, 2 * nh);
    double L3inv = 1 / cube(g->L);
    for (long q = 0; q < g->Ng3_pad; ++q)
        g->f[q] *= L3inv;
    if (offset_phase_off)
        og_offset_phase(g, -1);
}

/* fft_deconv (src/fft.c:236-254): divide by the PCS window sinc^4 per axis */
void og_deconv(og_grid *g) {
    const int Ng = g->Ng;
    double *Winv = (double *)malloc(sizeof(double) * Ng);
    Winv[0] = 1;
    for (int n = 1; n <= Ng / 2; ++n) {
        double arg = M_PI * n / Ng;
        Winv[n] = quart(arg / sin(arg));
        Winv[Ng - n] = Winv[n];
    }
    for (int i = 0; i < Ng; ++i)
    for (int j = 0; j < Ng; ++j)
    for (int k = 0; k <= Ng / 2; ++k) {
        double W3 = Winv[i] * Winv[j] * Winv[k];
        ORE(g, i, j, k) *= W3;
        OIM(g, i, j, k) *= W3;
    }
    free(Winv);
}

/* fft_p2k (src/fft.c:257-276): interlaced paint + FFT, average, deconvolve */
void og_p2k(og_grid *g, long Np, double V, const double *x, const double *y,
            const double *z, long Nr, const double *xr, const double *yr,
            const double *zr) {
    double off_dual[3] = {0.5, 0.5, 0.5};
    og_p2g(g, Np, V, x, y, z, Nr, xr, yr, zr, off_dual);
    og_x2k(g, 1);
    double *f_dual = (double *)malloc((size_t)g->Ng3_pad * sizeof(double));
    memcpy(f_dual, g->f, (size_t)g->Ng3_pad * sizeof(double));
    double off_none[3] = {0, 0, 0};
    og_p2g(g, Np, V, x, y, z, Nr, xr, yr, zr, off_none);
    og_x2k(g, 0);
    for (long q = 0; q < g->Ng3_pad; ++q)
        g->f[q] = 0.5 * (f_dual[q] + g->f[q]);
    og_deconv(g);
    free(f_dual);
}

/* fft_g2p (src/fft.c:134-169), reproducing the reference exactly: its inner
 * statement assigns (`=`) instead of accumulating, so each output is the last
 * stencil term F(c3,c3,c3) * wx[3] * wy[3] * wz[3]. */
void og_g2p(og_grid *g, long Np, const double *x, const double *y,
            const double *z, double *out) {
    const int Ng = g->Ng;
    double Hinv = Ng / g->L;
    for (long p = 0; p < Np; ++p) {
        int ci[4], cj[4], ck[4];
        double wx[4], wy[4], wz[4];
        pcs_weights(pcs_cells(x[p] * Hinv - g->offset[0], Ng, ci), wx);
        pcs_weights(pcs_cells(y[p] * Hinv - g->offset[1], Ng, cj), wy);
        pcs_weights(pcs_cells(z[p] * Hinv - g->offset[2], Ng, ck), wz);
        for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c)
            out[p] = OF(g, ci[a], cj[b], ck[c]) * wx[a] * wy[b] * wz[c];
    }
}

/* P (src/power.c:12-27): in place |delta|^2/V - Pshot, imaginary parts and
 * the DC mode zeroed. */
void og_power(og_grid *g, long Np, double V, long Nr) {
    const int Ng = g->Ng;
    double Vinv = 1 / V;
    double alpha = (Nr <= 0) ? 0 : (double)Np / Nr;
    double Pshot = (1 + alpha) * V / Np;
    ORE(g, 0, 0, 0) = OIM(g, 0, 0, 0) = 0;
    for (int i = 0; i < Ng; ++i)
    for (int j = 0; j < Ng; ++j)
    for (int k = (i == 0 && j == 0); k <= Ng / 2; ++k) {
        double d2 = sq(ORE(g, i, j, k)) + sq(OIM(g, i, j, k));
        ORE(g, i, j, k) = d2 * Vinv - Pshot;
        OIM(g, i, j, k) = 0;
    }
}

/* hat() of src/gal.h:19-26 */
void og_hat(double v[3]) {
    double amp = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (amp > 1e-7) { v[0] /= amp; v[1] /= amp; v[2] /= amp; }
}

/* number of k bins used by Pl and Pmu (src/power.c:34-36) */
int og_nk(int Ng, double L, double dK) {
    double KF = 2 * M_PI / L;
    double dKinv = KF / dK;
    return (int)floor(OG_SQRT3 * (Ng / 2) * dKinv) + 1;
}

static void kval_table(int Ng, double *Kval) {
    Kval[0] = 0;
    for (int n = 1; n <= Ng / 2; ++n) { Kval[n] = n; Kval[Ng - n] = -n; }
}

/* Pl (src/power.c:30-101) without the file output: multipoles l = 0,2,4,6.
 * K[NK], N[NK], P[NK*4] are written; empty bins give NaN as in the reference.
 * Returns 0, or -1 if a mode falls outside [0, NK), -2 if the mode-count
 * closure sum(N) == Ng^3 - 1 fails. */
int og_pl(og_grid *g, double los[3], double dK, double *K, long *N, double *P) {
    const int Ng = g->Ng;
    og_hat(los);
    double KF = 2 * M_PI / g->L;
    double dKinv = KF / dK;
    int NK = (int)floor(OG_SQRT3 * (Ng / 2) * dKinv) + 1;
    const int Nl = 4;
    for (int b = 0; b < NK; ++b) {
        K[b] = 0; N[b] = 0;
        for (int l = 0; l < Nl; ++l) P[b * Nl + l] = 0;
    }
    double *Kval = (double *)malloc(sizeof(double) * Ng);
    kval_table(Ng, Kval);
    int bad = 0;
    for (int i = 0; i < Ng; ++i)
    for (int j = 0; j < Ng; ++j)
    for (int k = (i == 0 && j == 0); k <= Ng / 2; ++k) {
        int count = 1 + (2 * k % Ng > 0);
        double d2 = ORE(g, i, j, k);
        d2 *= count;
        double Kamp = sqrt(sq(Kval[i]) + sq(Kval[j]) + sq(Kval[k]));
        int iK = floor(Kamp * dKinv);
        double mu2 = sq((Kval[i] * los[0] + Kval[j] * los[1] + Kval[k] * los[2]) / Kamp);
        if (iK < 0 || iK >= NK) { bad = 1; continue; }
        K[iK] += count * Kamp;
        N[iK] += count;
        P[iK * Nl + 0] += d2;
        P[iK * Nl + 1] += d2 * (1.5 * mu2 - 0.5);
        P[iK * Nl + 2] += d2 * ((4.375 * mu2 - 3.75) * mu2 + 0.375);
        P[iK * Nl + 3] += d2 * (((14.4375 * mu2 - 19.6875) * mu2 + 6.5625) * mu2 - 0.3125);
    }
    free(Kval);
    long Ntot = 0;
    for (int b = 0; b < NK; ++b) {
        K[b] *= KF / N[b];
        for (int l = 0; l < Nl; ++l)
            P[b * Nl + l] *= (4 * l + 1.0) / N[b];
        Ntot += N[b];
    }
    if (bad) return -1;
    if (Ntot != (long)Ng * Ng * Ng - 1) return -2;
    return 0;
}

/* Pmu (src/power.c:104-178) without the file output, with Nmu wedges.
 * K, N, P are [NK][Nmu]; the mu = 1 corner (imu == Nmu) is merged into the
 * last wedge; empty wedges stay 0 (the reference guards N > 0 there). */
int og_pmu(og_grid *g, double los[3], double dK, int Nmu, double *K, long *N,
           double *P) {
    const int Ng = g->Ng;
    og_hat(los);
    double KF = 2 * M_PI / g->L;
    double dKinv = KF / dK;
    int NK = (int)floor(OG_SQRT3 * (Ng / 2) * dKinv) + 1;
    int W = Nmu + 1;
    double *Kb = (double *)calloc((size_t)NK * W, sizeof(double));
    double *Pb = (double *)calloc((size_t)NK * W, sizeof(double));
    long *Nb = (long *)calloc((size_t)NK * W, sizeof(long));
    double *Kval = (double *)malloc(sizeof(double) * Ng);
    kval_table(Ng, Kval);
    int bad = 0;
    for (int i = 0; i < Ng; ++i)
    for (int j = 0; j < Ng; ++j)
    for (int k = (i == 0 && j == 0); k <= Ng / 2; ++k) {
        int count = 1 + (2 * k % Ng > 0);
        double d2 = ORE(g, i, j, k);
        d2 *= count;
        double Kamp = sqrt(sq(Kval[i]) + sq(Kval[j]) + sq(Kval[k]));
        int iK = floor(Kamp * dKinv);
        double mu = (Kval[i] * los[0] + Kval[j] * los[1] + Kval[k] * los[2]) / Kamp;
        int imu = floor(fabs(mu * Nmu));
        if (iK < 0 || iK >= NK || imu < 0 || imu > Nmu) { bad = 1; continue; }
        Kb[iK * W + imu] += count * Kamp;
        Nb[iK * W + imu] += count;
        Pb[iK * W + imu] += d2;
    }
    free(Kval);
    for (int b = 0; b < NK; ++b) {
        Kb[b * W + Nmu - 1] += Kb[b * W + Nmu];
        Nb[b * W + Nmu - 1] += Nb[b * W + Nmu];
        Pb[b * W + Nmu - 1] += Pb[b * W + Nmu];
    }
    long Ntot = 0;
    for (int b = 0; b < NK; ++b)
        for (int m = 0; m < Nmu; ++m) {
            double kk = Kb[b * W + m], pp = Pb[b * W + m];
            long nn = Nb[b * W + m];
            if (nn) {
                kk *= KF / nn;
                pp /= nn;
                Ntot += nn;
            }
            K[b * Nmu + m] = kk; N[b * Nmu + m] = nn; P[b * Nmu + m] = pp;
        }
    free(Kb); free(Pb); free(Nb);
    if (bad) return -1;
    if (Ntot != (long)Ng * Ng * Ng - 1) return -2;
    return 0;
}

/* gal_wrap (src/gal.c:51-60) */
void og_wrap(long Np, double *x, double *y, double *z, double L) {
    double Linv = 1 / L;
    for (long p = 0; p < Np; ++p) {
        x[p] -= L * floor(x[p] * Linv);
        y[p] -= L * floor(y[p] * Linv);
        z[p] -= L * floor(z[p] * Linv);
    }
}

/* gal_rsd (src/gal.c:63-77): plane-parallel redshift-space displacement */
void og_rsd(long Np, const double *x, const double *y, const double *z,
            const double *vx, const double *vy, const double *vz,
            double los[3], double aH, double *xo, double *yo, double *zo) {
    og_hat(los);
    double aHinv = 1 / aH;
    for (long p = 0; p < Np; ++p) {
        double vdl = los[0] * vx[p] + los[1] * vy[p] + los[2] * vz[p];
        xo[p] = x[p] + aHinv * vdl * los[0];
        yo[p] = y[p] + aHinv * vdl * los[1];
        zo[p] = z[p] + aHinv * vdl * los[2];
    }
}

/* sub-box window deconvolution of the real-space grid, the host loop of
 * src/app/Psb.c:76-83 (also :126-133): cells (i, j, k) in (-Ngsub, Ngsub)^3,
 * wrapped mod Ng, times Ngsub^3 / ((Ngsub-|i|)(Ngsub-|j|)(Ngsub-|k|)) */
void og_window_box(og_grid *g, int Ngsub) {
    const int Ng = g->Ng;
    double Ngsub3 = (double)Ngsub * Ngsub * Ngsub;
    for (int i = -Ngsub + 1; i < Ngsub; ++i)
        for (int j = -Ngsub + 1; j < Ngsub; ++j)
            for (int k = -Ngsub + 1; k < Ngsub; ++k) {
                double Winv = Ngsub3 / ((double)(Ngsub - abs(i)) * (Ngsub - abs(j)) * (Ngsub - abs(k)));
                OF(g, (i + Ng) % Ng, (j + Ng) % Ng, (k + Ng) % Ng) *= Winv;
            }
}

/* sub-sphere window deconvolution, the host loop of src/app/Pss.c:72-84:
 * cells with d2 = i^2 + j^2 + k^2 < 0.99 * 3 Ngsub^2 over (-Ngbnd, Ngbnd)^3,
 * Ngbnd = ceil(sqrt(3) Ngsub), wrapped mod Ng (an index range wider than
 * Ng/2 reaches some cells twice, each time multiplying again), times
 * 1 / ((1 - dD)^2 (1 + dD/2)), dD = sqrt(d2 / D2) */
void og_window_sphere(og_grid *g, int Ngsub) {
    const int Ng = g->Ng;
    double D2 = 3.0 * Ngsub * Ngsub;
    int Ngbnd = (int)ceil(sqrt(D2));
    for (int i = -Ngbnd + 1; i < Ngbnd; ++i)
        for (int j = -Ngbnd + 1; j < Ngbnd; ++j)
            for (int k = -Ngbnd + 1; k < Ngbnd; ++k) {
                double d2 = (double)i * i + (double)j * j + (double)k * k;
                if (d2 < 0.99 * D2) {
                    double dD = sqrt(d2 / D2);
                    double Winv = 1 / ((1 - dD) * (1 - dD) * (1 + 0.5 * dD));
                    OF(g, (i + Ng) % Ng, (j + Ng) % Ng, (k + Ng) % Ng) *= Winv;
                }
            }
}

/* super-sample modes of sub-volumes, the loop body of src/app/DLsb.c:56-92
 * (box, sphere = 0) and src/app/DLss.c:54-90 (sphere = 1) for one line of
 * sight and one multipole iL: the grid holds the unfiltered k-space field on
 * entry; F(k) <- L_iL(mu^2) W(k) F(k) (the k = 0 real part zeroed), c2r
 * (fft_k2x without phase), then out[(isub*Nsub + jsub)*Nsub + ksub] =
 * F(isub*Ngsub, jsub*Ngsub, ksub*Ngsub) / bias.  los is normalised here. */
static double og_tophat(double KR) { return 3 * (sin(KR) - KR * cos(KR)) / cube(KR); }

void og_dl(og_grid *g, int sphere, int Nsub, const double los_in[3], int iL, double bias, double *out) {
    const int Ng = g->Ng, Ngsub = Ng / Nsub;
    double los[3] = {los_in[0], los_in[1], los_in[2]};
    og_hat(los);
    double *Wamp = (double *)malloc(sizeof(double) * Ng);
    double *Wph = (double *)malloc(sizeof(double) * 6 * Ng);
    double *Kval = (double *)malloc(sizeof(double) * Ng);
    Wamp[0] = 1;
    for (int i = 1; i < Ng; ++i) Wamp[i] = sin(M_PI * i / Nsub) / sin(M_PI * i / Ng) / Ngsub;
    for (int i = 0; i < 3 * Ng; ++i) {
        Wph[2 * i] = cos(M_PI * i * (Ngsub - 1) / Ng);
        Wph[2 * i + 1] = sin(M_PI * i * (Ngsub - 1) / Ng);
    }
    Kval[0] = 0;
    for (int i = 1; i <= Ng / 2; ++i) {
        Kval[i] = i;
        Kval[Ng - i] = -i;
    }
    g->f[0] = 0;
    for (int i = 0; i < Ng; ++i)
        for (int j = 0; j < Ng; ++j)
            for (int k = (i == 0 && j == 0); k <= Ng / 2; ++k) {
                double Kamp = sqrt(sq(Kval[i]) + sq(Kval[j]) + sq(Kval[k]));
                double mu2 = sq((Kval[i] * los[0] + Kval[j] * los[1] + Kval[k] * los[2]) / Kamp);
                double Legendre[3] = {1, 1.5 * mu2 - 0.5, (4.375 * mu2 - 3.75) * mu2 + 0.375};
                if (sphere) {
                    double W = og_tophat(Kamp * M_PI * OG_SQRT3 / Nsub);
                    ORE(g, i, j, k) *= Legendre[iL] * W;
                    OIM(g, i, j, k) *= Legendre[iL] * W;
                } else {
                    double Wamp3 = Wamp[i] * Wamp[j] * Wamp[k];
                    double W_re = Wph[2 * (i + j + k)] * Wamp3;
                    double W_im = Wph[2 * (i + j + k) + 1] * Wamp3;
                    double f_re = ORE(g, i, j, k);
                    double f_im = OIM(g, i, j, k);
                    ORE(g, i, j, k) = Legendre[iL] * (f_re * W_re - f_im * W_im);
                    OIM(g, i, j, k) = Legendre[iL] * (f_re * W_im + f_im * W_re);
                }
            }
    og_k2x(g, 0);
    for (int isub = 0; isub < Nsub; ++isub)
        for (int jsub = 0; jsub < Nsub; ++jsub)
            for (int ksub = 0; ksub < Nsub; ++ksub)
                out[(isub * Nsub + jsub) * Nsub + ksub] = OF(g, isub * Ngsub, jsub * Ngsub, ksub * Ngsub) / bias;
    free(Wamp);
    free(Wph);
    free(Kval);
}
