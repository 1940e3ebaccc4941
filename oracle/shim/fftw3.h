/* Minimal FFTW3 API shim for building the reference's own C sources as a CPU
 * oracle (test infrastructure only).  It declares exactly the FFTW symbols the
 * reference uses (src/fft.h:6,17 and src/fft.c:26-45,174,186) and routes them
 * to the project's FP64 FFT in oracle/fft64.c.  FFTW itself (double precision,
 * version unpinned in the reference Makefile) is not installed here. */
#ifndef ORACLE_SHIM_FFTW3_H
#define ORACLE_SHIM_FFTW3_H
#include <stddef.h>

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
int fftw_import_wisdom_from_filename(const char *filename);
int fftw_export_wisdom_to_filename(const char *filename);
#endif
