/* grid data type -- drop-in replacement for the reference's src/fft.h.
 *
 * Same macros, struct fields and prototypes (src/fft.h:9-49) so the
 * reference's drivers (src/app/P.c, Psb.c, Pss.c, DLsb.c, DLss.c,
 * src/tests/octet.c) compile and link unchanged.  Differences:
 *   - no <fftw3.h>: the two plan handles are opaque pointers owned by the
 *     GPU library (the canonical grid lives in GPU memory);
 *   - `f` is a host view of the grid in double precision.  Under the default
 *     host-view mode ("sync") every call leaves `f` equal to the device grid
 *     and re-reads it on entry, so host code may read and write F() between
 *     calls exactly as with the reference.  Under "lazy" (FFTGAL_HOST_VIEW=lazy
 *     or fftgal_set_host_view) `f` is only refreshed by fftgal_sync_host().
 * Grid precision on the GPU is FP32 by default; FFTGAL_PRECISION=f64 selects
 * FP64 (see fftgal_gb300.h).  Errors print a message and abort(), as the
 * reference's assert() does. */
#ifndef FFT_H
#define FFT_H

#include "gal.h"

/* field value in configuration space */
#define F(self,i,j,k) (self->f[((long)(i) * self->Ng + (j)) * self->Ng_pad + (k)])
/* field value in Fourier space */
#define F_Re(self,i,j,k) F(self,i,j,2*k)
#define F_Im(self,i,j,k) F(self,i,j,2*k+1)

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fft {
    void *x2k, *k2x;  /* opaque GPU state (the reference holds FFTW plans here) */
    double *f;  /* host view; in-place: fk = (complex *)fx */
    int Ng;
    int Ng_pad;  /* 2 * (Ng/2 + 1) for the in-place r2c layout */
    long Ng3_pad;  /* sizeof(f) / sizeof(double) */
    double L;  /* [Mpc/h] */
    double offset[3];  /* grid (Dirac comb) wrt boundary [0,L)^3 in grid unit */
} fft_t;


/* src/fft.c:13-47; `wisdom` names the plan cache file ("FFTW_ESTIMATE" = built-in plans) */
fft_t *fft_init(int Ng, double L, char *wisdom);
/* src/fft.c:50-54 */
void fft_free(fft_t *self);

/* PCS paint (src/fft.c:57-131); offset is reduced with remainder() and written back */
void fft_p2g(fft_t *self, gal_t *part, double offset[3]);
/* PCS readout (src/fft.c:134-169), reproducing the reference's result exactly */
double *fft_g2p(fft_t *self, gal_t *pos);

/* forward r2c, times H^3, optional offset phase (src/fft.c:172-181) */
void fft_x2k(fft_t *self, int offset_phase_on);
/* backward c2r, times 1/L^3, optional offset phase removal (src/fft.c:184-193) */
void fft_k2x(fft_t *self, int offset_phase_off);
/* apply (onoff>0) or remove applied (onoff<0) offset phase (src/fft.c:196-233) */
void fft_offset_phase(fft_t *self, int onoff);

/* PCS window deconvolution (src/fft.c:236-254) */
void fft_deconv(fft_t *self);

/* simple interlacing interface = (paint + FFT) x 2 + average + deconvolve
 * (src/fft.c:257-276) */
void fft_p2k(fft_t *self, gal_t *part);

/* snapshot to a malloc'd buffer the caller free()s / restore (src/fft.c:279-289) */
double *fft_exportf(fft_t *self);
void fft_importf(fft_t *self, double *src);

#ifdef __cplusplus
}
#endif
#endif
