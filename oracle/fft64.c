/* fft64 -- double-precision FFT for the CPU oracle.  See fft64.h for the
 * conventions (FFTW's r2c/c2r sign, normalisation and in-place layout, which
 * the reference relies on at src/fft.c:26-45,174,186). */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "fft64.h"

struct fft64_1d {
    int n, sign, nfac;
    int fac[64];
    double *tw;   /* tw[2t], tw[2t+1] = cos, sin of sign * 2 pi t / n */
};

static void factorize(fft64_1d *p) {
    int n = p->n, k = 0;
    while (n % 4 == 0) { p->fac[k++] = 4; n /= 4; }
    while (n % 2 == 0) { p->fac[k++] = 2; n /= 2; }
    for (int f = 3; f * f <= n; f += 2)
        while (n % f == 0) { p->fac[k++] = f; n /= f; }
    if (n > 1) p->fac[k++] = n;
    p->nfac = k;
}

fft64_1d *fft64_1d_plan(int n, int sign) {
    fft64_1d *p = (fft64_1d *)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->n = n;
    p->sign = sign < 0 ? -1 : 1;
    factorize(p);
    p->tw = (double *)malloc(2 * (size_t)n * sizeof(double));
    if (!p->tw) { free(p); return NULL; }
    for (int t = 0; t < n; ++t) {
        /* reduce the angle to the first octant-free form t/n in [0,1) so the
         * table is exact to the last ulp of cos/sin */
        double a = 2.0 * M_PI * (double)t / (double)n;
        p->tw[2 * t] = cos(a);
        p->tw[2 * t + 1] = p->sign * sin(a);
    }
    return p;
}

void fft64_1d_free(fft64_1d *p) {
    if (p) { free(p->tw); free(p); }
}

/* one Stockham pass of radix R: src -> dst, Ns = product of earlier radices */
static void stockham_pass(const fft64_1d *p, int R, int Ns,
                          const double *src, double *dst) {
    const int n = p->n, m = n / R, tstep = n / (Ns * R);
    const double *tw = p->tw;
    double vr[64], vi[64], wr[64], wi[64];
    double *bvr = vr, *bvi = vi, *bwr = wr, *bwi = wi;
    if (R > 64) {  /* large prime radix: heap buffers */
        bvr = (double *)malloc(4 * (size_t)R * sizeof(double));
        bvi = bvr + R; bwr = bvi + R; bwi = bwr + R;
    }
    for (int j = 0; j < m; ++j) {
        int jm = j % Ns;
        for (int r = 0; r < R; ++r) {
            double xr = src[2 * (j + r * m)], xi = src[2 * (j + r * m) + 1];
            int t = r * jm * tstep;
            double cr = tw[2 * t], ci = tw[2 * t + 1];
            bvr[r] = xr * cr - xi * ci;
            bvi[r] = xr * ci + xi * cr;
        }
        if (R == 2) {
            bwr[0] = bvr[0] + bvr[1]; bwi[0] = bvi[0] + bvi[1];
            bwr[1] = bvr[0] - bvr[1]; bwi[1] = bvi[0] - bvi[1];
        } else if (R == 4) {
            double ar = bvr[0] + bvr[2], ai = bvi[0] + bvi[2];
            double br = bvr[0] - bvr[2], bi = bvi[0] - bvi[2];
            double cr = bvr[1] + bvr[3], ci = bvi[1] + bvi[3];
            double er = bvr[1] - bvr[3], ei = bvi[1] - bvi[3];
            /* d = e * (sign * i) */
            double dr = -p->sign * ei, di = p->sign * er;
            bwr[0] = ar + cr; bwi[0] = ai + ci;
            bwr[2] = ar - cr; bwi[2] = ai - ci;
            bwr[1] = br + dr; bwi[1] = bi + di;
            bwr[3] = br - dr; bwi[3] = bi - di;
        } else {
            const int step = n / R;
            for (int q = 0; q < R; ++q) {
                double sr = 0, si = 0;
                for (int r = 0; r < R; ++r) {
                    int t = (int)(((long)r * q) % R) * step;
                    double cr = tw[2 * t], ci = tw[2 * t + 1];
                    sr += bvr[r] * cr - bvi[r] * ci;
                    si += bvr[r] * ci + bvi[r] * cr;
                }
                bwr[q] = sr; bwi[q] = si;
            }
        }
        int d = (j / Ns) * Ns * R + jm;
        for (int r = 0; r < R; ++r) {
            dst[2 * (d + r * Ns)] = bwr[r];
            dst[2 * (d + r * Ns) + 1] = bwi[r];
        }
    }
    if (R > 64) free(bvr);
}

void fft64_1d_exec(const fft64_1d *p, double *data, double *work) {
    double *src = data, *dst = work;
    int Ns = 1;
    for (int s = 0; s < p->nfac; ++s) {
        int R = p->fac[s];
        stockham_pass(p, R, Ns, src, dst);
        Ns *= R;
        double *t = src; src = dst; dst = t;
    }
    if (src != data)
        memcpy(data, src, 2 * (size_t)p->n * sizeof(double));
}

/* ---- 3D transforms in the FFTW in-place layout ------------------------- */

#define COLBLK 16

/* complex transform along one of the two leading axes for all columns.
 * nrow = length of the transformed axis, stride = distance (in complex
 * values) between consecutive elements of a column, ncol = number of columns
 * per "slab", nslab/slabstride = repetition over the other leading axis. */
static void c2c_columns(const fft64_1d *p, double *a, int nlen, long stride,
                        long ncol, long nslab, long slabstride) {
    double *buf = (double *)malloc(2 * (size_t)nlen * COLBLK * sizeof(double));
    double *work = (double *)malloc(2 * (size_t)nlen * sizeof(double));
    for (long s = 0; s < nslab; ++s) {
        double *base = a + 2 * s * slabstride;
        for (long c0 = 0; c0 < ncol; c0 += COLBLK) {
            int nb = (int)((ncol - c0) < COLBLK ? (ncol - c0) : COLBLK);
            for (int e = 0; e < nlen; ++e) {
                const double *row = base + 2 * ((long)e * stride + c0);
                for (int b = 0; b < nb; ++b) {
                    buf[2 * ((long)b * nlen + e)] = row[2 * b];
                    buf[2 * ((long)b * nlen + e) + 1] = row[2 * b + 1];
                }
            }
            for (int b = 0; b < nb; ++b)
                fft64_1d_exec(p, buf + 2 * (long)b * nlen, work);
            for (int e = 0; e < nlen; ++e) {
                double *row = base + 2 * ((long)e * stride + c0);
                for (int b = 0; b < nb; ++b) {
                    row[2 * b] = buf[2 * ((long)b * nlen + e)];
                    row[2 * b + 1] = buf[2 * ((long)b * nlen + e) + 1];
                }
            }
        }
    }
    free(buf); free(work);
}

/* real row (n reals) -> n/2+1 complex, forward */
static void r2c_row(const fft64_1d *half, const fft64_1d *full, int n,
                    const double *x, double *X, double *z, double *work) {
    if (n % 2 == 0 && n >= 2) {
        int h = n / 2;
        for (int m = 0; m < h; ++m) { z[2 * m] = x[2 * m]; z[2 * m + 1] = x[2 * m + 1]; }
        fft64_1d_exec(half, z, work);
        /* X[k] = E[k] + W^k O[k], E = (Z[k] + conj Z[h-k])/2, O = (Z[k] - conj Z[h-k])/(2i) */
        for (int k = 0; k <= h; ++k) {
            int k1 = k % h, k2 = (h - k) % h;
            double zr = z[2 * k1], zi = z[2 * k1 + 1];
            double cr = z[2 * k2], ci = -z[2 * k2 + 1];
            double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
            double dr = zr - cr, di = zi - ci;          /* = 2i O */
            double or_ = 0.5 * di, oi = -0.5 * dr;       /* O = (d)/(2i) */
            double a = 2.0 * M_PI * (double)k / (double)n;
            double wr = cos(a), wi = -sin(a);
            X[2 * k] = er + (wr * or_ - wi * oi);
            X[2 * k + 1] = ei + (wr * oi + wi * or_);
        }
    } else {
        for (int m = 0; m < n; ++m) { z[2 * m] = x[m]; z[2 * m + 1] = 0; }
        fft64_1d_exec(full, z, work);
        for (int k = 0; k <= n / 2; ++k) { X[2 * k] = z[2 * k]; X[2 * k + 1] = z[2 * k + 1]; }
    }
}

/* n/2+1 complex -> n reals, backward (FFTW c2r: Im X[0], Im X[n/2] ignored) */
static void c2r_row(const fft64_1d *half, const fft64_1d *full, int n,
                    const double *X, double *x, double *z, double *work) {
    if (n % 2 == 0 && n >= 2) {
        int h = n / 2;
        for (int k = 0; k < h; ++k) {
            /* A = X[k] + X[k+h], B = (X[k] - X[k+h]) e^{+2 pi i k/n},
             * X[k+h] = conj X[h-k] (Hermitian); Im X[0], Im X[h] dropped */
            double xr = X[2 * k], xi = (k == 0) ? 0 : X[2 * k + 1];
            double yr = X[2 * (h - k)], yi = (h - k == h) ? 0 : -X[2 * (h - k) + 1];
            if (k == 0) yi = 0;  /* X[h] real part only */
            double ar = xr + yr, ai = xi + yi;
            double br0 = xr - yr, bi0 = xi - yi;
            double a = 2.0 * M_PI * (double)k / (double)n;
            double wr = cos(a), wi = sin(a);
            double br = br0 * wr - bi0 * wi, bi = br0 * wi + bi0 * wr;
            z[2 * k] = ar - bi;        /* Z = A + iB */
            z[2 * k + 1] = ai + br;
        }
        fft64_1d_exec(half, z, work);
        for (int m = 0; m < h; ++m) { x[2 * m] = z[2 * m]; x[2 * m + 1] = z[2 * m + 1]; }
    } else {
        int h = n / 2;
        for (int k = 0; k <= h; ++k) {
            z[2 * k] = X[2 * k];
            z[2 * k + 1] = (k == 0) ? 0 : X[2 * k + 1];
        }
        for (int k = h + 1; k < n; ++k) {
            z[2 * k] = X[2 * (n - k)];
            z[2 * k + 1] = -X[2 * (n - k) + 1];
        }
        fft64_1d_exec(full, z, work);
        for (int m = 0; m < n; ++m) x[m] = z[2 * m];
    }
}

void fft64_r2c_3d(int n0, int n1, int n2, double *in, long in_pitch,
                  double *out, long out_pitch) {
    int nh = n2 / 2 + 1;
    fft64_1d *half = (n2 % 2 == 0) ? fft64_1d_plan(n2 / 2, -1) : NULL;
    fft64_1d *full = fft64_1d_plan(n2, -1);
    double *row = (double *)malloc(sizeof(double) * (size_t)(n2 + 2));
    double *z = (double *)malloc(2 * sizeof(double) * (size_t)(n2 + 2));
    double *work = (double *)malloc(2 * sizeof(double) * (size_t)(n2 + 2));
    double *X = (double *)malloc(2 * sizeof(double) * (size_t)nh);
    for (long r = 0; r < (long)n0 * n1; ++r) {
        memcpy(row, in + r * in_pitch, (size_t)n2 * sizeof(double));
        r2c_row(half, full, n2, row, X, z, work);
        memcpy(out + 2 * r * out_pitch, X, 2 * (size_t)nh * sizeof(double));
    }
    free(row); free(z); free(work); free(X);
    fft64_1d_free(half); fft64_1d_free(full);
    /* axis 1 (j): columns are the nh complex entries of each row */
    fft64_1d *p1 = fft64_1d_plan(n1, -1);
    c2c_columns(p1, out, n1, out_pitch, nh, n0, (long)n1 * out_pitch);
    fft64_1d_free(p1);
    /* axis 0 (i) */
    fft64_1d *p0 = fft64_1d_plan(n0, -1);
    c2c_columns(p0, out, n0, (long)n1 * out_pitch, (long)n1 * out_pitch, 1, 0);
    fft64_1d_free(p0);
}

void fft64_c2r_3d(int n0, int n1, int n2, double *in, long in_pitch,
                  double *out, long out_pitch) {
    int nh = n2 / 2 + 1;
    fft64_1d *p0 = fft64_1d_plan(n0, +1);
    c2c_columns(p0, in, n0, (long)n1 * in_pitch, (long)n1 * in_pitch, 1, 0);
    fft64_1d_free(p0);
    fft64_1d *p1 = fft64_1d_plan(n1, +1);
    c2c_columns(p1, in, n1, in_pitch, nh, n0, (long)n1 * in_pitch);
    fft64_1d_free(p1);
    fft64_1d *half = (n2 % 2 == 0) ? fft64_1d_plan(n2 / 2, +1) : NULL;
    fft64_1d *full = fft64_1d_plan(n2, +1);
    double *X = (double *)malloc(2 * sizeof(double) * (size_t)nh);
    double *z = (double *)malloc(2 * sizeof(double) * (size_t)(n2 + 2));
    double *work = (double *)malloc(2 * sizeof(double) * (size_t)(n2 + 2));
    double *row = (double *)malloc(sizeof(double) * (size_t)(n2 + 2));
    for (long r = 0; r < (long)n0 * n1; ++r) {
        memcpy(X, in + 2 * r * in_pitch, 2 * (size_t)nh * sizeof(double));
        c2r_row(half, full, n2, X, row, z, work);
        memcpy(out + r * out_pitch, row, (size_t)n2 * sizeof(double));
    }
    free(X); free(z); free(work); free(row);
    fft64_1d_free(half); fft64_1d_free(full);
}
