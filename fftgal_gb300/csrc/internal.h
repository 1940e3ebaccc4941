// Internal declarations shared by the CUDA translation units of
// libfftgal_gb300.so.  Nothing here is part of the public C ABI
// (include/fft.h, include/power.h, include/gal.h, include/fftgal_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace fg {

// ---- status / errors ------------------------------------------------------
enum Status {
    OK = 0,
    ERR_ARG = -1,
    ERR_CUDA = -2,
    ERR_NOMEM = -3,
    ERR_UNSUPPORTED = -4,
    ERR_RANGE = -5,
    ERR_STATE = -6,
    ERR_IO = -7,
};

// records a status with a message (thread-local); returns the status
int set_error(int status, const char *fmt, ...);
int cuda_check(cudaError_t e, const char *what);

#define FG_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t fg_e_ = (call);                                     \
        if (fg_e_ != cudaSuccess) return ::fg::cuda_check(fg_e_, #call); \
    } while (0)

// every kernel launch site reports here (counted for the benchmark's
// launch tally) and checks the launch
void note_launches(int n);
long launch_count();
#define FG_LAUNCHED(n)                                                      \
    do {                                                                    \
        ::fg::note_launches(n);                                             \
        cudaError_t fg_e_ = cudaGetLastError();                             \
        if (fg_e_ != cudaSuccess) return ::fg::cuda_check(fg_e_, "launch"); \
    } while (0)

#define FG_TRY(expr)                  \
    do {                              \
        int fg_s_ = (expr);           \
        if (fg_s_ != 0) return fg_s_; \
    } while (0)

// ---- FFT plans -------------------------------------------------------------
constexpr int kMaxRadixPasses = 16;

struct Fft1dPlan {
    int n = 0;                    // complex length
    int nrad = 0;
    int rad[kMaxRadixPasses] = {};
    void *tw = nullptr;           // device: exp(-2 pi i t / n), t < n (float2 or double2)
};

struct FftPlan {
    int prec = 4;                 // 4 = float, 8 = double
    int Ng = 0, nh = 0;
    bool even = true;
    Fft1dPlan axis;               // length Ng (j and i axes; odd-Ng k axis)
    Fft1dPlan half;               // length Ng/2 (k axis, even Ng)
    void *rtw = nullptr;          // device: exp(-2 pi i k / Ng), k <= Ng/2 (r2c split)
    // launch shapes chosen by the planner
    int cols = 16, col_threads = 256;      // column kernel: columns per CTA
    int rows = 16, row_threads = 256;      // k-axis kernel: rows per CTA
    size_t col_smem = 0, row_smem = 0;
    // launch shapes of the two-level FP32 kernels (fft2.cu), set by the
    // autotuner or a plan file: [0] k-pass rows per CTA (0 = built-in),
    // [1] j-pass and [2] i-pass log2 columns per CTA (-1 = built-in)
    int tune[3] = {0, -1, -1};
};

int fft_plan_create(FftPlan *p, int Ng, int prec);
void fft_plan_destroy(FftPlan *p);
// forward r2c (sign -1) of `ngrids` in-place padded grids, unnormalised
int fft_r2c(const FftPlan *p, void *const *grids, int ngrids, cudaStream_t s);
// backward c2r (sign +1), unnormalised
int fft_c2r(const FftPlan *p, void *const *grids, int ngrids, cudaStream_t s);
// the three passes separately (used by the fused pipeline)
int fft_pass_k_r2c(const FftPlan *p, void *const *grids, int ngrids, cudaStream_t s);
int fft_pass_j(const FftPlan *p, void *const *grids, int ngrids, int sign, cudaStream_t s);
int fft_pass_i(const FftPlan *p, void *const *grids, int ngrids, int sign, cudaStream_t s);

// two-level FP32 kernels (fft2.cu) for power-of-two Ng in [4, 1024]
bool fft2_supported(int Ng, int prec);
int fft2_cols(int N, const void *W, void *g0, void *g1, int ngrids, int ncols, long es, long bs,
              long nbatch, int sign, cudaStream_t s, int logC_req = -1);
int fft2_k_r2c(int Ng, const void *W, const void *rtw, void *g0, void *g1, int ngrids, cudaStream_t s,
               int R_req = 0);
// launch shape `v` of pass `which` (0 = k rows per CTA, 1 = j / 2 = i log2
// columns per CTA) is launchable for Ng; the built-in choice of each pass
bool fft2_valid_shape(int Ng, int which, int v);
int fft2_default_shape(int Ng, int which);
// device twiddle tables of the two-level kernels (built once per device)
int fft2_prepare();
// TMA-staged strided pass along i of FP32 grids (Ng = 512 or 1024; selected by
// FFTGAL_TMA=1): the i pass of fft_pass_i; fft2_tma_check reports (and
// clears) a time-out of its bounded mbarrier waits -- call it after a sync
bool fft2_tma_supported(int Ng, int prec);
int fft2_cols_tma(int Ng, const void *W, void *g0, void *g1, int ngrids, int sign, cudaStream_t s);
int fft2_tma_check();
// time every valid launch shape of the three r2c passes on `grid` (one FP32
// grid of the plan's size; its contents are transformed in place) and keep the
// fastest in p->tune; ms[3] = the chosen shapes' times
int fft2_autotune(FftPlan *p, void *grid, cudaStream_t s, double ms[3]);
// plan cache (plan.cu): the entry of `path` for this device and the plan's
// size, else the in-process cache, else fft2_autotune on `grid`; writes the
// entry back to `path`.  *source: FFTGAL_PLAN_*; ms: measured times or 0.
int plan_resolve(FftPlan *p, void *grid, cudaStream_t s, const char *path, bool quiet, int *source, double ms[3]);
// Launch shapes of the paint and binning kernels of an FP32 grid, kept in the
// same plan file on lines of their own ("fftgal_gb300-launch 1 ...") per
// (compute capability, SM count, Ng).  0 = built-in.
struct LaunchTune {
    int paint_cta = 0;  // persistent tile-paint CTAs per SM
    int bin_cta = 0;    // binning CTAs per SM
    int bin_fold = 0;   // binning blocks between folds
};
int plan_device_key(int *cc, int *sms, char *name, size_t len);
int launch_lookup(const char *path, int cc, int sms, int Ng, LaunchTune *t);
int launch_store(const char *path, int cc, int sms, int Ng, const LaunchTune &t, const double ms[2], const char *dev);

// ---- paint -----------------------------------------------------------------
struct PaintTiling {
    int Ng = 0;
    int nt[3] = {0, 0, 0};        // tiles along i, j, k
    int tmax[3] = {0, 0, 0};      // largest tile extent along i, j, k
    int *d_tables = nullptr;      // device, per axis a: tile_of[Ng], then start[nt[a]+1]
    int tab_off[3] = {0, 0, 0};   // offset of axis a's tables in d_tables
    long nkeys = 0;               // nt0*nt1*nt2 * 27
    int cta_per_sm = 0;           // persistent FP32 tile-paint CTAs per SM (1 or 2; 0: built-in 2)
    // tiles of up to 32 x 16 x 32 cells for FP32 paints of one grid (owned;
    // null where Ng < 64): the one grid's accumulators fill the shared memory
    // that two grids of 16 x 16 x 32 take
    PaintTiling *one = nullptr;
};

struct PaintScratch {
    long cap_particles = 0;
    void *sorted = nullptr;       // [cap] sorted records (float4 or double x3)
    long cap_keys = 0;
    uint32_t *hist = nullptr;     // [nkeys + 1] counts -> exclusive offsets
    uint32_t *cursor = nullptr;   // [nkeys + 1] next free slot per key while scattering
    uint32_t *scan_tmp = nullptr; // block sums for the scan
    size_t bytes = 0;
};

struct PaintGridSpec {
    void *out = nullptr;          // padded real grid (float or double)
    double offset[3] = {0, 0, 0}; // already reduced with remainder()
    double scale = 1.0;           // Npcinv (times -alpha for randoms)
    int accumulate = 0;           // 0: overwrite (and zero padding), 1: out += value
};

int paint_tiling_create(PaintTiling *t, int Ng);
void paint_tiling_destroy(PaintTiling *t);
void paint_scratch_free(PaintScratch *s);

// Redshift-space displacement applied while painting (FP32 positions only):
// x + (v . los) / aH * los per particle, as src/gal.c:63-77 (gal_rsd) forms it.
struct PaintRsd {
    const float *v[3] = {nullptr, nullptr, nullptr};  // device velocities, or null: no displacement
    double los[3] = {0, 0, 0};                         // already normalised with hat()
    double aHinv = 0;
};

// Per-catalog scalars that the kernels read from device memory instead of
// their launch arguments, so that one captured CUDA graph serves catalogs of
// any size (graph-captured batches): the particle count, the paint scales of
// the two grids, and the binning's 1/V and shot noise.
struct DevScalars {
    long Np;
    double scale[2];
    float Vinv, Pshot;
};

// Paint one catalog onto 1 or 2 grids (same tiling, offsets within 1 cell of
// each other).  pos_prec: 4 (float x,y,z) or 8 (double x,y,z); device pointers.
// `ev` (optional, 4 events) is recorded after the key, scan, scatter and
// tile-paint kernels.  With `ds` (device, FP32 only) the kernels take Np and
// the grids' scales from *ds; Np is then the capacity (the largest count).
int paint(const PaintTiling *t, PaintScratch *s, int grid_prec,
          const void *x, const void *y, const void *z, int pos_prec, long Np,
          double Hinv, const PaintGridSpec *grids, int ngrids, cudaStream_t st,
          cudaEvent_t *ev = nullptr, const PaintRsd *rsd = nullptr, const DevScalars *ds = nullptr);
// scratch for catalogs of up to Np particles (no allocation in later paints)
int paint_reserve(const PaintTiling *t, PaintScratch *s, long Np);

// ---- spectral elementwise ----------------------------------------------------
int scale_grid(void *f, long n, int prec, double s, cudaStream_t st);
// offset phase with the reference's Nyquist behaviour; tab = [3][Ng] complex (double)
int build_phase_table(double *host_tab, int Ng, const double offset[3], int onoff);
int apply_phase(void *f, int Ng, int prec, const void *d_tab, cudaStream_t st);
int build_winv_table(double *host_tab, int Ng);
int apply_deconv(void *f, int Ng, int prec, const void *d_winv, cudaStream_t st);
int interlace_average(void *f, const void *fdual, long n, int prec, cudaStream_t st);
// A <- deconv(0.5 * (phase(B * H3) + A * H3)) in one pass; d_tab is the
// [3][Ng] phase table of B's offset, d_winv the [Ng] deconvolution table
int interlace_finish(void *A, const void *B, int Ng, int prec, double H3, const void *d_tab,
                     const void *d_winv, cudaStream_t st);
int power_inplace(void *f, int Ng, int prec, double Vinv, double Pshot, cudaStream_t st);
// real-space sub-volume window deconvolutions of src/app/Psb.c:76-83 and Pss.c:72-84
int window_box(void *f, int Ng, int prec, int Ngsub, cudaStream_t st);
int window_sphere(void *f, int Ng, int prec, int Ngsub, cudaStream_t st);
// super-sample filters of src/app/DLsb.c:67-85 / DLss.c:65-81 (los normalised) and the
// corner samples of their c2r output
int dl_filter(void *dst, const void *src, int Ng, int prec, int sphere, const double *d_tab, const double los[3],
              int iL, cudaStream_t st);
int dl_sample(const void *f, int Ng, int prec, int Nsub, double bias, double *d_out, cudaStream_t st);
int convert_grid(void *dst, int dst_prec, const void *src, int src_prec, long n, cudaStream_t st);

// ---- binning -----------------------------------------------------------------
struct BinSpec {
    int Ng = 0;
    double L = 0, dK = 0;
    double los[3] = {0, 0, 0};    // already normalised with hat()
    int Nmu = 3;
    int NK = 0;
    double KF = 0, dKinv = 0;
};

struct BinGeometry {               // data-independent part, cached
    BinSpec spec;
    bool valid = false;
    long *N = nullptr;            // host [NK]
    double *K = nullptr;          // host [NK] (sum count*Kamp)
    long *Nw = nullptr;           // host [NK][Nmu+1]
    double *Kw = nullptr;         // host [NK][Nmu+1]
    uint32_t *d_thr = nullptr;    // device: n2 thresholds of the k bins [NK+1]
    double *d_acc = nullptr;      // device accumulators (per call)
    size_t acc_len = 0;
    int bad = 0;
    // FP32 binning launch shape (0: built-in): CTAs per SM, blocks between folds
    int cta_per_sm = 0, fold = 0;
};

int bin_spec_init(BinSpec *b, int Ng, double L, double dK, const double los_hat[3], int Nmu);
int bin_geometry_build(BinGeometry *g, const BinSpec &spec, cudaStream_t st);
void bin_geometry_free(BinGeometry *g);
// interlacing finish fused into the FP32 binning pass (mode 2 of bin_power)
struct BinFinish {
    void *A = nullptr;           // canonical grid, finished in place
    const void *B = nullptr;     // interlacing grid
    const void *ph32 = nullptr;  // [3][Ng] float2 phase of the interlacing grid
    const void *w32 = nullptr;   // [Ng] float PCS window inverse
    double scale = 0;            // H^3 / 2
};
// power sums over the half spectrum.  mode 0: input holds P (F_Re = P, from P());
// mode 1: input holds delta (complex), P = |delta|^2 * Vinv - Pshot computed on the fly;
// mode 2 (FP32): `fin` names both interlacing grids, A <- (A + B phase) W^-1 H^3/2
// is written back and binned as in mode 1 (`f` unused); mode 3 (FP32): one grid,
// A <- A W^-1 scale (fin->B, ph32 unused); mode 4 (FP32): as 3 without
// writing A back (the deconvolved field exists only while it is binned);
// mode 5 (FP32): as 2 without writing A back.
// Results (host): Psum[NK][4] (count-weighted, times Legendre), Pw[NK][Nmu+1].
// `ev_end` (optional) is recorded right after the binning kernel
int bin_power(BinGeometry *g, const void *f, int prec, int mode, double Vinv, double Pshot,
              double *Psum, double *Pw, cudaStream_t st, cudaEvent_t *ev_end = nullptr,
              const BinFinish *fin = nullptr);
// the launches of bin_power (FP32, modes 2 to 5) without the read-back: the
// sums stay in g->d_acc ([NK][4 + Nmu + 1] doubles); with `ds` the kernel
// takes Vinv and Pshot from device memory
int bin_power_launch(BinGeometry *g, int mode, double Vinv, double Pshot, cudaStream_t st, const BinFinish *fin,
                     const DevScalars *ds);
// Psum / Pw of bin_power from a copy of g->d_acc
void bin_power_unpack(const BinGeometry *g, const double *acc, double *Psum, double *Pw);

// ---- misc -----------------------------------------------------------------------
int num_sms();
int device_max_smem();

}  // namespace fg
