/* FFTW3 API shim implementation (oracle only): plans record the array shape
 * and pointers; execution calls the FP64 transforms of oracle/fft64.c with
 * FFTW's in-place padded layout. Wisdom files hold a one-line marker. */
#include <stdio.h>
#include <stdlib.h>
#include "fftw3.h"
#include "../fft64.h"

struct fftw_plan_s { int n0, n1, n2, dir; double *in, *out; };

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

static fftw_plan mk(int n0, int n1, int n2, int dir, double *in, double *out) {
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    p->n0 = n0; p->n1 = n1; p->n2 = n2; p->dir = dir; p->in = in; p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags) {
    (void)flags;
    return mk(n0, n1, n2, -1, in, (double *)out);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags) {
    (void)flags;
    return mk(n0, n1, n2, +1, (double *)in, out);
}

void fftw_execute(const fftw_plan p) {
    long nh = p->n2 / 2 + 1;
    /* in-place when in == out: real pitch 2*nh doubles; out-of-place: n2 */
    long rpitch = (p->in == p->out) ? 2 * nh : p->n2;
    if (p->dir < 0)
        fft64_r2c_3d(p->n0, p->n1, p->n2, p->in, rpitch, p->out, nh);
    else
        fft64_c2r_3d(p->n0, p->n1, p->n2, p->in, nh, p->out, rpitch);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

int fftw_import_wisdom_from_filename(const char *filename) {
    FILE *fp = fopen(filename, "r");
    if (!fp) return 0;
    fclose(fp);
    return 1;
}

int fftw_export_wisdom_to_filename(const char *filename) {
    FILE *fp = fopen(filename, "w");
    if (!fp) return 0;
    fprintf(fp, "(oracle-fft64-wisdom)\n");
    fclose(fp);
    return 1;
}
