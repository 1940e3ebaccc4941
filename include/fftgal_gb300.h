/* fftgal_gb300.h -- extensions of the GB300 power-spectrum library beyond the
 * reference's own C API (include/fft.h, include/power.h, include/gal.h).
 *
 * All functions return 0 on success or a negative FFTGAL_ERR_* status; the
 * message of the last failure on the calling thread is in fftgal_last_error().
 * Nothing here has a counterpart in the reference unless a citation says so.
 */
#ifndef FFTGAL_GB300_H
#define FFTGAL_GB300_H

#include "fft.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FFTGAL_OK 0
#define FFTGAL_ERR_ARG (-1)
#define FFTGAL_ERR_CUDA (-2)
#define FFTGAL_ERR_NOMEM (-3)
#define FFTGAL_ERR_UNSUPPORTED (-4)
#define FFTGAL_ERR_RANGE (-5)
#define FFTGAL_ERR_STATE (-6)
#define FFTGAL_ERR_IO (-7)

/* host-view modes of fft_t.f (see include/fft.h) */
#define FFTGAL_VIEW_SYNC 0
#define FFTGAL_VIEW_LAZY 1

/* where caller buffers live */
#define FFTGAL_MEM_HOST 0
#define FFTGAL_MEM_DEVICE 1

int fftgal_version(void);
/* status and message of the last failure on this thread */
int fftgal_last_status(void);
const char *fftgal_last_error(void);

/* bytes per grid value on the GPU: 4 (FP32, default) or 8 (FP64).  Chosen at
 * fft_init from FFTGAL_PRECISION ("f32" | "f64"). */
int fftgal_grid_precision(const fft_t *grid);
/* host-view policy; FFTGAL_HOST_VIEW ("sync" | "lazy") sets the default */
int fftgal_set_host_view(fft_t *grid, int mode);
/* copy the device grid into grid->f / grid->f into the device grid */
int fftgal_sync_host(fft_t *grid);
int fftgal_sync_device(fft_t *grid);
/* run the grid's work on an existing CUDA stream (cudaStream_t), or NULL to
 * return to the library's own non-blocking stream (for the legacy default
 * stream pass cudaStreamLegacy, not 0) */
int fftgal_set_stream(fft_t *grid, void *cuda_stream);
void *fftgal_get_stream(fft_t *grid);
/* suppress (1) or restore (0) the per-call timing lines on stderr; the
 * FFTGAL_QUIET environment variable sets the default */
int fftgal_set_quiet(fft_t *grid, int quiet);
/* device pointer of the canonical grid (Ng*Ng*Ng_pad values) */
void *fftgal_device_grid(fft_t *grid);
/* copy Ng3_pad values of the grid's precision between the canonical grid and
 * a caller buffer (host or device, any CUDA-visible pointer):
 * to_grid = 1 copies buf -> grid, 0 copies grid -> buf.  The copy waits for
 * the grid's stream, runs on the legacy default stream and is complete when
 * the call returns; work that fills `buf` on other non-blocking streams must
 * be complete first. */
int fftgal_copy_grid(fft_t *grid, void *buf, int to_grid);
/* wait for all queued work of the grid */
int fftgal_synchronize(fft_t *grid);

/* number of k bins of Pl/Pmu for (Ng, L, dK) (src/power.c:34-36) */
int fftgal_nk(int Ng, double L, double dK);

/* Interlaced power spectrum of one catalog with FP32 positions in one call:
 * PCS paint of both interlacing grids in a single particle pass, r2c FFT of
 * both, offset phase + average + window deconvolution, then multipoles and
 * Nmu wedges.  Results equal fft_p2k + P + Pl + Pmu (src/fft.c:257-276,
 * src/power.c:12-178) on the same catalog, with Pmu generalised to Nmu wedges.
 *   x, y, z   positions [Mpc/h], FP32, on the host or the device (`where`)
 *   V         catalog volume (shot noise V/Np, normalisation 1/V)
 *   los       line of sight (normalised internally, not modified)
 * Outputs (host, any may be NULL): K[NK], N[NK], Pl[NK*4] (l=0,2,4,6);
 * Kmu[NK*Nmu], Nmu_count[NK*Nmu], Pmu[NK*Nmu].  Bins are normalised exactly as
 * Pl()/Pmu() normalise them (empty multipole bins are NaN).  With the sync
 * host view the grid is left holding the deconvolved density field in k space
 * (as after fft_p2k, grid->f and the device grid); with the lazy view the
 * finished field is binned without being stored (4.3 GB fewer writes at
 * Ng = 1024) and the device grid's contents are unspecified until the next
 * paint, import or copy.  The same holds for fftgal_power_batch_f32 and
 * fftgal_power_rsd_f32.  Requires an FP32 grid. */
int fftgal_power_f32(fft_t *grid, const float *x, const float *y, const float *z, long Np,
                     double V, int where, const double los[3], double dK, int Nmu,
                     double *K, long *N, double *Pl, double *Kmu, long *Nmu_count,
                     double *Pmu);

/* Sub-volume window deconvolution of the real-space grid on the GPU, the
 * host loops of src/app/Psb.c:76-83 (sub-box: cells (i,j,k) in (-Ngsub,
 * Ngsub)^3 wrapped mod Ng, times Ngsub^3 / ((Ngsub-|i|)(Ngsub-|j|)(Ngsub-|k|)))
 * and src/app/Pss.c:72-84 (sub-sphere: d2 < 0.99 * 3 Ngsub^2 over
 * (-ceil(sqrt(3) Ngsub), ceil(sqrt(3) Ngsub))^3 wrapped mod Ng, times
 * 1 / ((1 - dD)^2 (1 + dD/2)), a cell reached by several wrapped indices
 * multiplied once per index, as the loop does).  Call after fft_k2x, in
 * place of the loop over grid->f; FP64 grids reproduce the loop bit for bit.
 * 1 <= Ngsub <= Ng/2. */
int fftgal_window_box(fft_t *grid, int Ngsub);
int fftgal_window_sphere(fft_t *grid, int Ngsub);

/* Super-sample modes of sub-volumes, the per-line-of-sight loop of
 * src/app/DLsb.c:56-92 (sphere = 0: sub-box window) and src/app/DLss.c:54-90
 * (sphere = 1: top-hat sphere of radius sqrt(3) L / (2 Nsub)).  On entry the
 * grid holds the unfiltered k-space field (fft_p2g + fft_x2k(grid, 0), as the
 * drivers prepare it).  For each of the nlos lines of sight los[3*l..3*l+2]
 * and each multipole iL = 0, 1, 2 the field is multiplied by L_iL(mu^2) W(k),
 * transformed to configuration space (fft_k2x without phase) and sampled at
 * the sub-volume corners: DeltaL[(3*l + iL)*Nsub^3 + (isub*Nsub + jsub)*Nsub +
 * ksub] = F(isub*Ngsub, jsub*Ngsub, ksub*Ngsub) / bias.  The unfiltered field
 * stays on the GPU between the 3 * nlos filters (no exportf/importf round
 * trips); on return the grid holds the last filtered configuration-space
 * field, as after the drivers' loop.  Nsub >= 2 must divide Ng. */
int fftgal_dl_sub(fft_t *grid, int sphere, int Nsub, int nlos, const double *los, double bias,
                  double *DeltaL);

/* fftgal_power_f32 over a list of ncat catalogs with FP32 positions in host
 * (or device) memory (x[c], y[c], z[c], Np[c] particles, volume V[c]): while
 * catalog c is
 * painted and transformed, catalog c + 1 is copied to the GPU on a second
 * stream, so with page-locked host arrays the host-to-device copies hide
 * behind the computation.  Outputs are the fftgal_power_f32 outputs of each
 * catalog one after another: K[ncat*NK], N[ncat*NK], Pl[ncat*NK*4],
 * Kmu/Nmu_count/Pmu[ncat*NK*Nmu] (any may be NULL).  Holds two device buffers
 * of 3 * (max(Np) + max(Np)/8) floats until fft_free (later batches of up to
 * that many particles per catalog reuse them).
 * By default (FFTGAL_GRAPHS unset or not "0", or fftgal_set_graphs(grid, 1))
 * each catalog's device work runs as one CUDA graph launch: the sequence is
 * captured once per upload buffer (again when a catalog outgrows the buffers,
 * or the bins or a buffer change) with the kernels reading each catalog's count and scales
 * from device memory; the host waits once per batch, not once per catalog.
 * Per-stage timers (fftgal_stage_times) are not recorded in that mode. */
int fftgal_set_graphs(fft_t *grid, int on);
int fftgal_power_batch_f32(fft_t *grid, int ncat, const float *const *x, const float *const *y,
                           const float *const *z, const long *Np, const double *V,
                           const double los[3], double dK, int Nmu, double *K, long *N,
                           double *Pl, double *Kmu, long *Nmu_count, double *Pmu);

/* Interlaced power spectra of a list of catalogs of mixed grid sizes, box
 * lengths (fold factors: L[c] = L_box / fold, src/app/P.c:35-36) and bin
 * widths in one call, e.g. a covariance set of mocks with uneven particle
 * counts.  Catalog c: FP32 positions x[c], y[c], z[c] (host or device),
 * Np[c] particles, volume V[c], grid Ng[c], box L[c], bin width dK[c]; its
 * outputs go to K[c][NK_c], N[c][NK_c], Pl[c][NK_c*4], Kmu[c], Nmu_count[c],
 * Pmu[c][NK_c*Nmu] with NK_c = fftgal_nk(Ng[c], L[c], dK[c]) (any array of
 * pointers, or any pointer in it, may be NULL).  Catalogs with the same
 * (Ng, L, dK) run together through fftgal_power_batch_f32 (uploads overlapped,
 * each catalog one captured graph launch) on an FP32 grid kept per (device,
 * Ng, L) between calls with device memory only, released by
 * fftgal_power_mixed_release.  Results equal fftgal_power_f32 on each
 * catalog.  No counterpart in the reference (its job scripts run one process
 * per mock, src/app/job_P.sh:22-26).  Not thread-safe with itself. */
int fftgal_power_mixed_f32(int ncat, const float *const *x, const float *const *y, const float *const *z,
                           const long *Np, const double *V, const int *Ng, const double *L,
                           const double los[3], const double *dK, int Nmu, double *const *K,
                           long *const *N, double *const *Pl, double *const *Kmu, long *const *Nmu_count,
                           double *const *Pmu);
int fftgal_power_mixed_release(void);

/* fftgal_power_f32 without interlacing: one paint, r2c, PCS deconvolution,
 * multipoles and wedges -- the sequence fft_p2g(offset 0) -> fft_x2k(0) ->
 * fft_deconv -> P -> Pl -> Pmu (src/fft.c:57-131,172-181,236-254,
 * src/power.c:12-178).  Half the paint and FFT work of the interlaced call;
 * aliasing is not suppressed.  With the sync host view the grid then holds
 * the deconvolved field (grid->f and the device grid); with the lazy view the
 * deconvolution is applied only while binning and the device grid's contents
 * are unspecified until the next paint, import or copy. */
int fftgal_power_single_f32(fft_t *grid, const float *x, const float *y, const float *z, long Np,
                            double V, int where, const double los[3], double dK, int Nmu,
                            double *K, long *N, double *Pl, double *Kmu, long *Nmu_count,
                            double *Pmu);

/* Learned aliasing correction (no counterpart in the reference): a
 * 5 -> 64 -> 64 -> 64 -> 3 tanh perceptron, FP32, mapping the single-paint
 * multipoles of a k bin to the interlaced ones.  Features of bin b (den =
 * |P0| + Pshot): k / k_Nyq, Pshot / den, P2 / den, P4 / den and the local
 * slope d ln den / d ln k; outputs (P_l^interlaced - P_l^single) / den, l = 0,
 * 2, 4.  Parameters: fftgal_mlp_nparams() floats, W1[5][64] b1 W2[64][64] b2
 * W3[64][64] b3 W4[64][3] b4.  The training and forward kernels take device
 * pointers; fftgal_mlp_grad accumulates into grad and loss (the caller clears
 * them) the gradient and value of the mean squared error over n samples
 * (X[n][5], T[n][3]); fftgal_mlp_adam takes one Adam step (beta 0.9, 0.999). */
int fftgal_mlp_nparams(void);
int fftgal_mlp_grad(const float *params, const float *X, const float *T, long n, float *grad,
                    float *loss, void *stream);
int fftgal_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr,
                    void *stream);
int fftgal_mlp_forward(const float *params, const float *X, long n, float *Y, void *stream);
/* features X[NK][5] of single-paint multipoles P[NK][4] (host arrays; empty
 * bins give zeros) */
int fftgal_alias_features(int NK, const double *K, const double *P, double Pshot, double kNyq,
                          float *X);
/* e(u) = u^6 / (1 + u^6), u = k / k_Nyq: the scale of the perceptron's
 * outputs, P_l^interlaced - P_l^single = (|P0| + Pshot) e(u) y_l */
double fftgal_alias_envelope(double u);
/* Plan cache (the counterpart of FFTW wisdom, src/fft.c:26-45).  fft_init(Ng,
 * L, path) with a file name instead of "FFTW_ESTIMATE" takes the launch shapes
 * of the FP32 r2c passes (k-pass rows per CTA, j- and i-pass log2 columns per
 * CTA) from the file's entry for this device (compute capability and SM count),
 * Ng and precision; without one it measures every valid shape on the new grid
 * (the FFTW_MEASURE step) and writes the entry back, keeping the file's other
 * lines.  Shapes change no result: every shape computes each row and column
 * with the same operations.  Grids whose FFT has no tunable shapes (FP64,
 * Ng not a power of two in [4, 1024]) use the built-in plans. */
#define FFTGAL_PLAN_BUILTIN 0  /* "FFTW_ESTIMATE", or nothing to tune */
#define FFTGAL_PLAN_MEASURED 1 /* measured by this fft_init */
#define FFTGAL_PLAN_FILE 2     /* imported from the plan file */
#define FFTGAL_PLAN_CACHE 3    /* measured earlier in this process */
/* the grid's shapes (tune[0] k rows, tune[1] j, tune[2] i log2 columns; 0 / -1
 * = built-in), where they came from, and the measured times (ms, 0 unless
 * measured) */
int fftgal_plan_info(fft_t *grid, int tune[3], int *source, double ms[3]);
/* measure now (clears the grid) and keep the fastest shapes on this grid */
int fftgal_plan_autotune(fft_t *grid, double ms[3]);
/* Launch shapes of the tile paint and of the finish + binning kernel of an
 * FP32 grid (power-of-two Ng): shapes[0] = persistent paint CTAs per SM
 * (1 or 2), shapes[1] = binning CTAs per SM (1-3, fewer when its shared
 * accumulators do not fit), shapes[2] = binning blocks between the folds of
 * its FP32 sums into FP64 (0: built-in, 8 or FFTGAL_BIN_FOLD).  With a plan
 * file, fft_init imports them from the file's "fftgal_gb300-launch" line for
 * this device and Ng, or times every shape (binning on zero grids, the paint
 * on a uniform catalog of Ng^3/10 particles; built-in kept unless another is
 * more than 2 % faster) and writes the line; `source` as fftgal_plan_info,
 * ms = the chosen paint and binning times (0 unless measured). */
int fftgal_launch_shapes(fft_t *grid, int shapes[3], int *source, double ms[2]);
/* in-place unnormalised FFTs of length N (a power of two from 4 to 2048) along
 * strided columns of complex FP32 data in GPU memory, with the kernels of the
 * grid's j and i passes: element n of column c (c < ncols) of batch b
 * (b < nbatch) is data[b * bs + n * es + c] (complex units); sign -1
 * forward, +1 backward; shape: -1 for the built-in launch shape, else a
 * j/i-pass shape of the plan (log2 columns per CTA); stream as cudaStream_t
 * (NULL: legacy default).  Returns after the transforms are done. */
int fftgal_fft_columns_f32(int N, void *data, int ncols, long es, long bs, long nbatch, int sign,
                           int shape, void *stream);
/* host-only plan file access: 1 and tune[] if `path` holds an entry for the
 * key, 0 if not (or no file); store replaces the key's entry */
int fftgal_plan_lookup(const char *path, int cc, int sms, int Ng, int prec, int tune[3]);
int fftgal_plan_store(const char *path, int cc, int sms, int Ng, int prec, const int tune[3],
                      const double ms[3], const char *device_name);
/* 1 if `shape` is launchable for pass 0 (k), 1 (j) or 2 (i) at Ng */
int fftgal_plan_valid(int Ng, int pass, int shape);

/* fftgal_power_single_f32 with P_0,2,4 corrected by the perceptron with host
 * parameters mlp_params (wedges and P_6 as measured): one paint and one FFT
 * instead of two of each. */
int fftgal_power_learned_f32(fft_t *grid, const float *x, const float *y, const float *z, long Np,
                             double V, int where, const double los[3], double dK, int Nmu,
                             const float *mlp_params, double *K, long *N, double *Pl, double *Kmu,
                             long *Nmu_count, double *Pmu);

/* Learned mode over a list of catalogs (x[c], y[c], z[c], Np[c], V[c]; host or
 * device memory per `where`) checked against the interlaced estimator, with
 * fallback: every holdout_every-th catalog (c % holdout_every == 0; 0 = none)
 * is measured both ways and its interlaced result is reported, with
 * disagreement[c] = the largest |P_l^learned - P_l^interlaced| /
 * (|P_0^interlaced| + Pshot) over l = 0, 2, 4 and the bins with modes below
 * 0.8 k_Nyq; once a disagreement exceeds tol, every later catalog runs
 * interlaced.  used[c]: 0 learned, 1 interlaced (checked), 2 interlaced
 * (fallback); disagreement (may be NULL) is NaN where not checked.  Outputs as
 * fftgal_power_batch_f32, one catalog after another. */
int fftgal_power_learned_checked_f32(fft_t *grid, int ncat, const float *const *x,
                                     const float *const *y, const float *const *z, const long *Np,
                                     const double *V, int where, const double los[3], double dK,
                                     int Nmu, const float *mlp_params, int holdout_every, double tol,
                                     double *K, long *N, double *Pl, double *Kmu, long *Nmu_count,
                                     double *Pmu, int *used, double *disagreement);

/* fftgal_power_f32 of the redshift-space catalog: every particle is
 * displaced along the line of sight while it is painted, x + (v . los) / aH
 * los, as gal_rsd forms it (src/gal.c:63-77), so the P.c sequence
 * gal_rsd -> fft_p2k -> P -> Pl -> Pmu (src/app/P.c:50-66) is one call with no
 * displaced copy of the catalog.  vx, vy, vz: FP32 velocities in the same
 * memory as x, y, z (`where`); los (normalised internally) is both the
 * displacement direction and the multipole axis. */
int fftgal_power_rsd_f32(fft_t *grid, const float *x, const float *y, const float *z,
                         const float *vx, const float *vy, const float *vz, long Np, double V,
                         int where, const double los[3], double aH, double dK, int Nmu,
                         double *K, long *N, double *Pl, double *Kmu, long *Nmu_count,
                         double *Pmu);

/* Per-stage device times (ms) of the last fftgal_power_f32 call, measured with
 * CUDA events on the grid's stream: [0] position upload, [1] paint key +
 * histogram, [2] histogram scan, [3] scatter, [4] tile paint, [5] FFT k pass,
 * [6] FFT j pass, [7] FFT i pass, [8] nothing (the interlacing finish --
 * offset phase, average, deconvolution -- runs inside [9]), [9] finish +
 * binning, [10] total.  Enabled with fftgal_set_timing(grid, 1). */
#define FFTGAL_NSTAGES 11
int fftgal_set_timing(fft_t *grid, int on);
int fftgal_stage_times(fft_t *grid, double out_ms[FFTGAL_NSTAGES]);
/* number of kernel launches the library has issued in this process */
long fftgal_launch_count(void);

/* PCS readout that sums the 64 stencil terms (the reference's fft_g2p,
 * src/fft.c:134-169, assigns instead of summing; fft_g2p here reproduces
 * that).  out[Np] on the host. */
int fftgal_g2p_sum(fft_t *grid, const gal_t *pos, double *out);

/* bytes of GPU memory held by the grid (grids, scratch, tables) */
long fftgal_device_bytes(fft_t *grid);

/* Multipoles and wedges of a deconvolved FP32 k-space grid that is already in
 * GPU memory, without allocating GPU memory.  No counterpart in the
 * reference: it serves callers that cannot allocate -- a host framework that
 * owns all device memory through its own pool, code that must not call
 * cudaMalloc/cudaFree because they synchronise the device, or a process whose
 * device memory is committed in advance.  It calls no cudaMalloc, cudaFree or
 * allocating library routine.
 *   fk         Ng*Ng*(Ng/2+1) complex FP32 values in the layout of the
 *              canonical grid (rows of Ng+2 floats), e.g. fftgal_device_grid()
 *              after fft_p2k on an FP32 grid (or after fftgal_power_f32 with
 *              the sync host view)
 *   V, Np      P = |fk|^2 / V - V / Np (src/power.c:55)
 *   los, dK, Nmu, outputs: as fftgal_power_f32 (outputs on the host)
 *   stream     cudaStream_t to run on (NULL: the legacy default stream); the
 *              call returns after the results are on the host
 * Scratch is one fixed array of about 1.8 MB in the library's device memory,
 * shared by all calls: it holds the k-bin limits, per-bin sums and counts of
 * the last call and is cleared at the start of each.  Calls whose GPU work
 * overlaps (from several host threads, or on several streams) race on it.
 * The call waits for `stream` (cudaStreamSynchronize) and copies the tables
 * to the caller's host arrays before it returns.
 * Limits: NK <= 2048 k bins, 1 <= Nmu <= 16, Ng <= 4096, and the per-block
 * shared accumulators NK * (36 + 16 * Nmu) + 8 <= 225280 bytes (220 KB):
 * NK <= 2048 up to Nmu = 5, NK <= 1149 at Nmu = 10, NK <= 771 at Nmu = 16
 * (Ng = 1024 with dK = 2 pi / L has NK = 887).  Larger requests return
 * FFTGAL_ERR_RANGE (NK) or FFTGAL_ERR_UNSUPPORTED (shared memory).
 * The first call on each device looks up the scratch's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the life
 * of the process; make that first call before any stream capture.  A
 * cudaDeviceReset of that device after its first call is not supported (the
 * kept address would be stale). */
int fftgal_power_bins_noalloc(const float *fk, int Ng, double L, double V, long Np,
                              const double los[3], double dK, int Nmu, double *K,
                              long *N, double *Pl, double *Kmu, long *Nmu_count,
                              double *Pmu, void *stream);

#ifdef __cplusplus
}
#endif
#endif
