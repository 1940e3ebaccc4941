/* fft64 -- double-precision FFT used only by the CPU oracle (test infrastructure).
 *
 * The reference delegates its transforms to FFTW3 (double precision, version
 * unpinned; call sites src/fft.c:26-45 plan, src/fft.c:174,186 execute).  FFTW
 * is not available here, so this file restates the discrete Fourier transform
 * from its definition with FFTW's conventions:
 *   forward r2c:  X[k] = sum_n x[n] exp(-2 pi i n k / N), unnormalised,
 *   backward c2r: x[n] = sum_k X[k] exp(+2 pi i n k / N), unnormalised,
 * using Hermitian symmetry along the last axis (FFTW ignores Im X[0] and
 * Im X[N/2] of each last-axis row, and so does this code).
 * In-place layout: row-major [n0][n1][2*(n2/2+1)] doubles, i.e. the real row
 * is padded to hold n2/2+1 complex values (src/fft.h:10-21).
 *
 * Algorithm: self-sorting mixed-radix Stockham passes (radices 4, 2, 3, 5 and
 * a generic odd prime), twiddles from an exactly indexed table exp(-2 pi i t/N).
 * Nothing under oracle/ is part of the shipped library.
 */
#ifndef ORACLE_FFT64_H
#define ORACLE_FFT64_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fft64_1d fft64_1d;

/* 1D complex plan of length n (any n >= 1). sign = -1 forward, +1 backward. */
fft64_1d *fft64_1d_plan(int n, int sign);
void fft64_1d_free(fft64_1d *p);
/* transform `howmany` interleaved complex vectors stored contiguously
 * (vector v at data + 2*n*v); work must hold 2*n doubles. */
void fft64_1d_exec(const fft64_1d *p, double *data, double *work);

/* 3D real-to-half-complex forward transform (unnormalised).  `in` holds the
 * real array with row pitch `in_pitch` doubles along the last axis; `out`
 * receives complex rows of n2/2+1 values with row pitch `out_pitch` complex.
 * in and out may alias (FFTW in-place layout: in_pitch = 2*(n2/2+1),
 * out_pitch = n2/2+1). */
void fft64_r2c_3d(int n0, int n1, int n2, double *in, long in_pitch,
                  double *out, long out_pitch);
/* inverse of the above without normalisation (FFTW c2r semantics). The complex
 * input is overwritten (as FFTW's c2r does). */
void fft64_c2r_3d(int n0, int n1, int n2, double *in, long in_pitch,
                  double *out, long out_pitch);

#ifdef __cplusplus
}
#endif
#endif
