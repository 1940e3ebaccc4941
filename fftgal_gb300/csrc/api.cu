// C ABI of libfftgal_gb300.so: the reference's fft.h / power.h functions
// (src/fft.h:27-49, src/power.h:7-13) on a GPU-resident grid, plus the
// extensions of include/fftgal_gb300.h.
//
// Each fft_t owns: the canonical grid in HBM (FP32 or FP64), a second grid for
// interlacing, FFT plans, paint tiling and scratch, spectral tables, the
// binning geometry cache and a CUDA stream.  The reference's `f` stays a host
// double array: under the "sync" host view it mirrors the device grid after
// every call (and is re-read at the start of every call that reads the grid),
// under "lazy" it is refreshed only on request.  Errors in reference-API calls
// print a message and abort(), as the reference's assert() does.
#include "internal.h"
#include "common.cuh"

#include "fft.h"
#include "power.h"
#include "fftgal_gb300.h"

#include <cmath>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace fg {

// ---- errors ----------------------------------------------------------------------
static thread_local int t_status = 0;
static thread_local char t_msg[1024] = "";

int set_error(int status, const char *fmt, ...) {
    t_status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return OK;
    return set_error(e == cudaErrorMemoryAllocation ? ERR_NOMEM : ERR_CUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

static std::atomic<long> g_launches{0};
void note_launches(int n) { g_launches += n; }
long launch_count() { return g_launches.load(); }

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

int device_max_smem() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

// ---- per-grid device state -----------------------------------------------------------
constexpr int kGeoCache = 8;
// timed stages of fftgal_power_f32: upload, key, scan, scatter, paint tile,
// fft k, fft j, fft i, finish (phase/average/deconv), bin
constexpr int kStages = 10;

struct Grid {
    int prec = 4;
    int Ng = 0, Ng_pad = 0, nh = 0;
    long Ng3_pad = 0;
    double L = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    void *d_f = nullptr, *d_aux = nullptr;
    int view = FFTGAL_VIEW_SYNC;
    bool pinned = false;
    int quiet = 0;
    FftPlan fft;
    PaintTiling tiling;
    PaintScratch scratch;
    void *d_pos = nullptr;  // 3 position arrays (float or double)
    size_t pos_cap = 0;     // bytes
    // fftgal_power_batch_f32: two device buffers of FP32 positions (one being
    // uploaded on copy_stream while the other is painted) and their events
    float *d_batch[2] = {nullptr, nullptr};
    size_t batch_cap = 0;  // floats per buffer
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t up_done[2] = {nullptr, nullptr}, buf_free[2] = {nullptr, nullptr};
    void *d_stage = nullptr;  // host-double staging for uploads
    size_t stage_cap = 0;
    double *d_tab = nullptr;  // [3][Ng] complex phase table, [Ng] winv, [3][Ng] offset-1/2 phase,
                              // then FP32 copies: [3][Ng] offset-1/2 phase, [Ng] winv
    BinGeometry geo[kGeoCache];
    int geo_next = 0;
    unsigned long version = 1;  // bumped whenever the grid changes
    // Pl -> Pmu reuse of the wedge sums from the same pass
    struct {
        unsigned long version = 0;
        BinSpec spec;
        std::vector<double> Pw;
    } wedge_cache;
    int timing = 0;
    cudaEvent_t ev[kStages + 1] = {};
    double stage_ms[kStages + 1] = {};
    int plan_source = FFTGAL_PLAN_BUILTIN;
    LaunchTune launch;  // paint / binning launch shapes (0: built-in)
    int launch_source = FFTGAL_PLAN_BUILTIN;
    double launch_ms[2] = {0, 0};
    double plan_ms[3] = {0, 0, 0};
    // graph-captured batches: one executable graph per upload buffer, the
    // per-catalog scalars it reads (device, one block per buffer; pinned
    // host ring, one block per catalog) and a pinned ring of bin sums
    int use_graphs = 1;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    std::vector<uint64_t> gkey;  // everything the captured graphs depend on
    int graph_kernels = 0;       // kernel nodes per graph
    DevScalars *d_scal = nullptr;
    DevScalars *h_scal = nullptr;
    size_t h_scal_cap = 0;
    double *h_acc = nullptr;
    size_t h_acc_cap = 0;
};

static Grid *G(const fft_t *f) { return f ? reinterpret_cast<Grid *>(f->x2k) : nullptr; }

static int env_precision() {
    const char *e = getenv("FFTGAL_PRECISION");
    if (!e) return 4;
    if (!strcmp(e, "f64") || !strcmp(e, "fp64") || !strcmp(e, "double") || !strcmp(e, "8")) return 8;
    return 4;
}

static int env_view() {
    const char *e = getenv("FFTGAL_HOST_VIEW");
    return (e && !strcmp(e, "lazy")) ? FFTGAL_VIEW_LAZY : FFTGAL_VIEW_SYNC;
}

static int env_graphs() {
    const char *e = getenv("FFTGAL_GRAPHS");
    return !(e && !strcmp(e, "0"));
}

static int env_quiet() {
    const char *e = getenv("FFTGAL_QUIET");
    return e && strcmp(e, "0") != 0;
}

[[noreturn]] static void die(const char *where) {
    fprintf(stderr, "%s: %s\n", where, t_msg[0] ? t_msg : "failure");
    fflush(stderr);
    abort();
}

#define FG_API(expr, where)              \
    do {                                 \
        if ((expr) != 0) die(where);     \
    } while (0)

static double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// ---- host view transfers -----------------------------------------------------------------
constexpr size_t kStageBytes = 64u << 20;

static int ensure_stage(Grid *g, size_t bytes) {
    if (bytes <= g->stage_cap) return OK;
    cudaFree(g->d_stage);
    g->d_stage = nullptr;
    FG_CUDA(cudaMalloc(&g->d_stage, bytes));
    g->stage_cap = bytes;
    return OK;
}

// device grid -> host double array (pinned: direct conversion; else staged)
static int device_to_host(Grid *g, double *host, bool host_pinned) {
    if (g->prec == 8) {
        FG_CUDA(cudaMemcpyAsync(host, g->d_f, sizeof(double) * g->Ng3_pad, cudaMemcpyDeviceToHost, g->stream));
    } else if (host_pinned) {
        FG_TRY(convert_grid(host, 8, g->d_f, 4, g->Ng3_pad, g->stream));
    } else {
        FG_TRY(ensure_stage(g, kStageBytes));
        const long chunk = kStageBytes / 8;
        for (long o = 0; o < g->Ng3_pad; o += chunk) {
            const long n = g->Ng3_pad - o < chunk ? g->Ng3_pad - o : chunk;
            FG_TRY(convert_grid(g->d_stage, 8, (const float *)g->d_f + o, 4, n, g->stream));
            FG_CUDA(cudaMemcpyAsync(host + o, g->d_stage, sizeof(double) * n, cudaMemcpyDeviceToHost, g->stream));
        }
    }
    FG_CUDA(cudaStreamSynchronize(g->stream));
    return OK;
}

static int host_to_device(Grid *g, const double *host, bool host_pinned) {
    if (g->prec == 8) {
        FG_CUDA(cudaMemcpyAsync(g->d_f, host, sizeof(double) * g->Ng3_pad, cudaMemcpyHostToDevice, g->stream));
    } else if (host_pinned) {
        FG_TRY(convert_grid(g->d_f, 4, host, 8, g->Ng3_pad, g->stream));
    } else {
        FG_TRY(ensure_stage(g, kStageBytes));
        const long chunk = kStageBytes / 8;
        for (long o = 0; o < g->Ng3_pad; o += chunk) {
            const long n = g->Ng3_pad - o < chunk ? g->Ng3_pad - o : chunk;
            FG_CUDA(cudaMemcpyAsync(g->d_stage, host + o, sizeof(double) * n, cudaMemcpyHostToDevice, g->stream));
            FG_TRY(convert_grid((float *)g->d_f + o, 4, g->d_stage, 8, n, g->stream));
        }
    }
    FG_CUDA(cudaStreamSynchronize(g->stream));
    ++g->version;
    return OK;
}

// entry/exit of reference-API calls under the host-view policy
static int enter(fft_t *self, bool reads_grid) {
    Grid *g = G(self);
    if (g->view == FFTGAL_VIEW_SYNC && reads_grid) FG_TRY(host_to_device(g, self->f, g->pinned));
    return OK;
}

static int leave(fft_t *self, bool modified) {
    Grid *g = G(self);
    if (modified) ++g->version;
    if (g->view == FFTGAL_VIEW_SYNC && modified) FG_TRY(device_to_host(g, self->f, g->pinned));
    FG_CUDA(cudaStreamSynchronize(g->stream));
    return fft2_tma_check();
}

// ---- helpers ------------------------------------------------------------------------------
static int ensure_aux(Grid *g) {
    if (g->d_aux) return OK;
    FG_CUDA(cudaMalloc(&g->d_aux, (size_t)g->prec * g->Ng3_pad));
    return OK;
}

static int ensure_tables(Grid *g) {
    if (g->d_tab) return OK;
    const size_t Ng = g->Ng;
    FG_CUDA(cudaMalloc(&g->d_tab, sizeof(double) * (17 * Ng)));
    std::vector<double> w(Ng);
    build_winv_table(w.data(), g->Ng);
    FG_CUDA(cudaMemcpy(g->d_tab + 6 * Ng, w.data(), sizeof(double) * Ng, cudaMemcpyHostToDevice));
    // phase table of the interlacing grid (offset 1/2 on every axis, applied)
    std::vector<double> ph(6 * Ng);
    const double half[3] = {remainder(0.5, g->Ng), remainder(0.5, g->Ng), remainder(0.5, g->Ng)};
    build_phase_table(ph.data(), g->Ng, half, 1);
    FG_CUDA(cudaMemcpy(g->d_tab + 7 * Ng, ph.data(), sizeof(double) * 6 * Ng, cudaMemcpyHostToDevice));
    // FP32 copies of both for the fused finish + binning pass
    std::vector<float> t32(7 * Ng);
    for (size_t e = 0; e < 6 * Ng; ++e) t32[e] = (float)ph[e];
    for (size_t e = 0; e < Ng; ++e) t32[6 * Ng + e] = (float)w[e];
    FG_CUDA(cudaMemcpy(g->d_tab + 13 * Ng, t32.data(), sizeof(float) * 7 * Ng, cudaMemcpyHostToDevice));
    return OK;
}

static const double *winv_tab(const Grid *g) { return g->d_tab + 6 * (size_t)g->Ng; }
static const double *dual_tab(const Grid *g) { return g->d_tab + 7 * (size_t)g->Ng; }
static const float *dual_tab32(const Grid *g) { return reinterpret_cast<const float *>(g->d_tab + 13 * (size_t)g->Ng); }
static const float *winv_tab32(const Grid *g) { return dual_tab32(g) + 6 * (size_t)g->Ng; }

static int phase(Grid *g, void *dst, const double offset[3], int onoff) {
    FG_TRY(ensure_tables(g));
    std::vector<double> tab(6 * (size_t)g->Ng);
    build_phase_table(tab.data(), g->Ng, offset, onoff);
    FG_CUDA(cudaMemcpyAsync(g->d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, g->stream));
    FG_TRY(apply_phase(dst, g->Ng, g->prec, g->d_tab, g->stream));
    // the host table must outlive the async copy
    FG_CUDA(cudaStreamSynchronize(g->stream));
    return OK;
}

static int deconv(Grid *g, void *dst) {
    FG_TRY(ensure_tables(g));
    return apply_deconv(dst, g->Ng, g->prec, g->d_tab + 6 * (size_t)g->Ng, g->stream);
}

// positions of a catalog (host doubles) -> device arrays in the grid's precision
static int upload_positions(Grid *g, const gal_t *part, void **px, void **py, void **pz) {
    const long Np = part->Np;
    const size_t need = (size_t)3 * (Np > 0 ? Np : 1) * g->prec;
    if (need > g->pos_cap) {
        cudaFree(g->d_pos);
        g->d_pos = nullptr;
        FG_CUDA(cudaMalloc(&g->d_pos, need));
        g->pos_cap = need;
    }
    char *base = (char *)g->d_pos;
    const double *src[3] = {part->x, part->y, part->z};
    void *dst[3];
    for (int a = 0; a < 3; ++a) dst[a] = base + (size_t)a * (Np > 0 ? Np : 1) * g->prec;
    if (Np > 0) {
        if (g->prec == 8) {
            for (int a = 0; a < 3; ++a)
                FG_CUDA(cudaMemcpyAsync(dst[a], src[a], sizeof(double) * Np, cudaMemcpyHostToDevice, g->stream));
        } else {
            FG_TRY(ensure_stage(g, kStageBytes));
            const long chunk = kStageBytes / 8;
            for (int a = 0; a < 3; ++a)
                for (long o = 0; o < Np; o += chunk) {
                    const long n = Np - o < chunk ? Np - o : chunk;
                    FG_CUDA(cudaMemcpyAsync(g->d_stage, src[a] + o, sizeof(double) * n, cudaMemcpyHostToDevice,
                                            g->stream));
                    FG_TRY(convert_grid((float *)dst[a] + o, 4, g->d_stage, 8, n, g->stream));
                }
        }
    }
    *px = dst[0];
    *py = dst[1];
    *pz = dst[2];
    return OK;
}

// paint `part` (and its randoms) onto the given grids of the same tiling
static int paint_catalog(Grid *g, const gal_t *part, void *const *outs, double (*offs)[3], int ngrids) {
    void *x, *y, *z;
    FG_TRY(upload_positions(g, part, &x, &y, &z));
    const double Hinv = g->Ng / g->L;
    const double H = g->L / g->Ng;
    const double H3r = H * H * H;  // gsl_pow_3(L/Ng) as the reference evaluates it
    const double nbar = part->Np / part->V;
    const double Npcinv = 1 / nbar / H3r;
    PaintGridSpec spec[2];
    for (int q = 0; q < ngrids; ++q) {
        spec[q].out = outs[q];
        for (int a = 0; a < 3; ++a) spec[q].offset[a] = offs[q][a];
        spec[q].scale = Npcinv;
        spec[q].accumulate = 0;
    }
    FG_TRY(paint(&g->tiling, &g->scratch, g->prec, x, y, z, g->prec, part->Np, Hinv, spec, ngrids, g->stream));
    if (part->rand) {
        const gal_t *r = part->rand;
        const double alpha = (double)part->Np / r->Np;
        FG_TRY(upload_positions(g, r, &x, &y, &z));
        for (int q = 0; q < ngrids; ++q) {
            spec[q].scale = -alpha * Npcinv;
            spec[q].accumulate = 1;
        }
        FG_TRY(paint(&g->tiling, &g->scratch, g->prec, x, y, z, g->prec, r->Np, Hinv, spec, ngrids, g->stream));
    }
    return OK;
}

static double H3_of(const Grid *g) {
    const double H = g->L / g->Ng;
    return H * H * H;
}

static BinGeometry *geometry(Grid *g, const BinSpec &s) {
    for (int q = 0; q < kGeoCache; ++q) {
        BinGeometry &c = g->geo[q];
        if (c.valid && c.spec.Ng == s.Ng && c.spec.L == s.L && c.spec.dK == s.dK && c.spec.Nmu == s.Nmu &&
            c.spec.los[0] == s.los[0] && c.spec.los[1] == s.los[1] && c.spec.los[2] == s.los[2])
            return &c;
    }
    BinGeometry &c = g->geo[g->geo_next];
    g->geo_next = (g->geo_next + 1) % kGeoCache;
    if (bin_geometry_build(&c, s, g->stream) != OK) return nullptr;
    c.cta_per_sm = g->launch.bin_cta;
    c.fold = g->launch.bin_fold;
    return &c;
}

// ---- launch shapes of the paint and binning kernels (autotuned) ----------------------------
// uniform FP32 positions in [0, L) from the splitmix64 stream of `seed`
__global__ void tune_uniform_kernel(float *x, long n, float L, unsigned long long seed) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const float u = (float)(z >> 40) * (1.0f / 16777216.0f);  // 24 bits: [0, 1)
        x[i] = L * u < L ? L * u : 0.f;
    }
}

// median of 3 timed runs after one untimed, CUDA events on st
template <typename F>
static int median_ms(cudaStream_t st, F run, double *ms) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FG_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_check(ce, "tune events");
    }
    int rc = run();
    float t[3] = {0, 0, 0};
    for (int r = 0; r < 3 && rc == OK; ++r) {
        rc = cuda_check(cudaEventRecord(e0, st), "tune");
        if (rc == OK) rc = run();
        if (rc == OK) rc = cuda_check(cudaEventRecord(e1, st), "tune");
        if (rc == OK) rc = cuda_check(cudaEventSynchronize(e1), "tune");
        if (rc == OK) rc = cuda_check(cudaEventElapsedTime(&t[r], e0, e1), "tune");
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FG_TRY(rc);
    std::sort(t, t + 3);
    *ms = t[1];
    return OK;
}

static std::mutex g_launch_mu;
static std::map<std::tuple<int, int, int>, LaunchTune> g_launch_cache;

// The counterpart of plan_resolve for the paint and binning launch shapes of
// an FP32 grid with the two-level FFT: the plan file's launch line for this
// device and Ng, else this process's earlier measurement, else timing every
// shape (binning: 1-3 CTAs per SM x fold every 8 or 32 blocks on zero grids;
// tile paint: 1 or 2 persistent CTAs per SM on a uniform catalog of Ng^3/10
// particles) and writing the line.  The built-in shape stays unless another
// is more than 2 % faster.  The grids are left zeroed.
static int tune_launch(fft_t *self, const char *path) {
    Grid *g = G(self);
    const int Ng = self->Ng;
    if (g->prec != 4 || !fft2_supported(Ng, 4)) return OK;
    int cc = 0, sms = 0;
    char name[256];
    FG_TRY(plan_device_key(&cc, &sms, name, sizeof(name)));
    LaunchTune t;
    const auto key = std::make_tuple(cc, sms, Ng);
    if (launch_lookup(path, cc, sms, Ng, &t)) {
        g->launch_source = FFTGAL_PLAN_FILE;
    } else {
        bool cached = false;
        {
            std::lock_guard<std::mutex> lk(g_launch_mu);
            auto it = g_launch_cache.find(key);
            if (it != g_launch_cache.end()) {
                t = it->second;
                cached = true;
            }
        }
        if (cached) {
            g->launch_source = FFTGAL_PLAN_CACHE;
        } else {
            cudaStream_t st = g->stream;
            FG_TRY(ensure_aux(g));
            FG_TRY(ensure_tables(g));
            const size_t gb = (size_t)4 * self->Ng3_pad;
            FG_CUDA(cudaMemsetAsync(g->d_f, 0, gb, st));
            FG_CUDA(cudaMemsetAsync(g->d_aux, 0, gb, st));
            // binning: the interlaced finish + binning of fftgal_power_f32 (lazy view)
            const double los[3] = {0, 0, 1};
            BinSpec bs;
            FG_TRY(bin_spec_init(&bs, Ng, self->L, 2 * M_PI / self->L, los, 3));
            BinGeometry *geo = geometry(g, bs);
            if (!geo) return t_status ? t_status : ERR_CUDA;
            BinFinish fin;
            fin.A = g->d_f;
            fin.B = g->d_aux;
            fin.ph32 = dual_tab32(g);
            fin.w32 = winv_tab32(g);
            fin.scale = 0.5 * H3_of(g);
            double best_b = 0, def_b = 0;
            t.bin_cta = 3;
            t.bin_fold = 8;
            for (int cta = 3; cta >= 1; --cta)
                for (int fold : {8, 32}) {
                    geo->cta_per_sm = cta;
                    geo->fold = fold;
                    double ms = 0;
                    FG_TRY(median_ms(st, [&]() { return bin_power_launch(geo, 5, 1.0, 0.0, st, &fin, nullptr); }, &ms));
                    if (cta == 3 && fold == 8) {
                        def_b = best_b = ms;
                    } else if (ms < best_b && ms < 0.98 * def_b) {
                        best_b = ms;
                        t.bin_cta = cta;
                        t.bin_fold = fold;
                    }
                }
            geo->cta_per_sm = t.bin_cta;
            geo->fold = t.bin_fold;
            // tile paint of both interlacing grids on a uniform catalog
            long Np = (long)Ng * Ng * Ng / 10;
            Np = Np < 100000 ? 100000 : (Np > 200000000 ? 200000000 : Np);
            float *pos = nullptr;
            FG_CUDA(cudaMalloc(&pos, sizeof(float) * 3 * (size_t)Np));
            for (int a = 0; a < 3; ++a)
                tune_uniform_kernel<<<num_sms() * 8, 256, 0, st>>>(pos + (size_t)a * Np, Np, (float)self->L,
                                                                   0x5EEDull + (unsigned long long)a);
            note_launches(3);
            PaintGridSpec spec[2];
            spec[0].out = g->d_f;
            spec[1].out = g->d_aux;
            for (int a = 0; a < 3; ++a) {
                spec[0].offset[a] = 0;
                spec[1].offset[a] = remainder(0.5, Ng);
            }
            double best_p = 0, def_p = 0;
            t.paint_cta = 2;
            int rc = cuda_check(cudaGetLastError(), "tune catalog");
            for (int cta = 2; cta >= 1 && rc == OK; --cta) {
                g->tiling.cta_per_sm = cta;
                double ms = 0;
                rc = median_ms(st, [&]() {
                    return paint(&g->tiling, &g->scratch, 4, pos, pos + Np, pos + 2 * (size_t)Np, 4, Np,
                                 Ng / self->L, spec, 2, st);
                }, &ms);
                if (rc != OK) break;
                if (cta == 2) {
                    def_p = best_p = ms;
                } else if (ms < 0.98 * def_p) {
                    best_p = ms;
                    t.paint_cta = cta;
                }
            }
            cudaFree(pos);
            FG_TRY(rc);
            FG_CUDA(cudaMemsetAsync(g->d_f, 0, gb, st));
            FG_CUDA(cudaMemsetAsync(g->d_aux, 0, gb, st));
            FG_CUDA(cudaStreamSynchronize(st));
            g->launch_ms[0] = best_p;
            g->launch_ms[1] = best_b;
            g->launch_source = FFTGAL_PLAN_MEASURED;
            {
                std::lock_guard<std::mutex> lk(g_launch_mu);
                g_launch_cache[key] = t;
            }
        }
        if (launch_store(path, cc, sms, Ng, t, g->launch_ms, name) != OK)
            fprintf(stderr, "fft_init() could not export the launch shapes to %s: %s\n", path, fftgal_last_error());
    }
    g->launch = t;
    g->tiling.cta_per_sm = t.paint_cta;
    for (auto &c : g->geo)
        if (c.valid) {
            c.cta_per_sm = t.bin_cta;
            c.fold = t.bin_fold;
        }
    return OK;
}

}  // namespace fg

using namespace fg;

// ======================================================================================
// reference API: src/fft.h
// ======================================================================================

// a grid and its device state; host_view: allocate fft_t.f (the drop-in
// API's host array), else f stays NULL and the grid runs with the lazy view.
// Returns NULL with the status set on failure.
static fft_t *grid_new(int Ng, double L, const char *wisdom, bool host_view, bool quiet) {
    if (Ng < 2) {
        set_error(ERR_ARG, "Ng must be >= 2");
        return nullptr;
    }
    fft_t *self = (fft_t *)calloc(1, sizeof(fft_t));
    if (!self) {
        set_error(ERR_NOMEM, "fft_t");
        return nullptr;
    }
    Grid *g = new Grid();
    self->x2k = g;
    self->k2x = nullptr;
    self->Ng = Ng;
    self->L = L;
    for (int i = 0; i < 3; ++i) self->offset[i] = 0;
    self->Ng_pad = 2 * (Ng / 2 + 1);
    self->Ng3_pad = (long)Ng * Ng * self->Ng_pad;
    g->prec = env_precision();
    g->view = host_view ? env_view() : FFTGAL_VIEW_LAZY;
    g->quiet = quiet ? 1 : env_quiet();
    g->use_graphs = env_graphs();
    g->Ng = Ng;
    g->Ng_pad = self->Ng_pad;
    g->nh = Ng / 2 + 1;
    g->Ng3_pad = self->Ng3_pad;
    g->L = L;
    auto fail = [&]() -> fft_t * {
        const int st = t_status;
        char msg[sizeof(t_msg)];
        memcpy(msg, t_msg, sizeof(msg));
        fft_free(self);
        t_status = st;
        memcpy(t_msg, msg, sizeof(msg));
        return nullptr;
    };
    if (cuda_check(cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking), "stream")) return fail();
    g->stream = g->own_stream;
    if (host_view) {
        // host view: pinned so the GPU converts straight into it
        void *hv = nullptr;
        if (cudaMallocHost(&hv, sizeof(double) * self->Ng3_pad) == cudaSuccess) {
            g->pinned = true;
        } else {
            cudaGetLastError();
            hv = malloc(sizeof(double) * self->Ng3_pad);
            if (!hv) {
                set_error(ERR_NOMEM, "host view of %ld doubles", self->Ng3_pad);
                return fail();
            }
        }
        self->f = (double *)hv;
        memset(self->f, 0, sizeof(double) * self->Ng3_pad);
    }
    if (cuda_check(cudaMalloc(&g->d_f, (size_t)g->prec * self->Ng3_pad), "grid")) return fail();
    if (cuda_check(cudaMemsetAsync(g->d_f, 0, (size_t)g->prec * self->Ng3_pad, g->stream), "grid")) return fail();
    if (fft_plan_create(&g->fft, Ng, g->prec)) return fail();
    if (paint_tiling_create(&g->tiling, Ng)) return fail();
    if (cuda_check(cudaStreamSynchronize(g->stream), "init")) return fail();
    if (!wisdom || !strcmp(wisdom, "FFTW_ESTIMATE")) {
        if (!g->quiet)
            fprintf(stderr, "fft_init() using built-in GPU plans (%s grid)\n", g->prec == 4 ? "FP32" : "FP64");
    } else if (plan_resolve(&g->fft, g->d_f, g->stream, wisdom, g->quiet != 0, &g->plan_source, g->plan_ms) ||
               tune_launch(self, wisdom)) {
        return fail();
    }
    return self;
}

extern "C" fft_t *fft_init(int Ng, double L, char *wisdom) {
    fprintf(stderr, "fft_init() making a %d^3 grid in a %g^3 box\n", Ng, L);
    fft_t *self = grid_new(Ng, L, wisdom, true, false);
    if (!self) die("fft_init()");
    return self;
}

extern "C" void fft_free(fft_t *self) {
    if (self != NULL) {
        Grid *g = G(self);
        if (g) {
            cudaStreamSynchronize(g->stream);
            cudaFree(g->d_f);
            cudaFree(g->d_aux);
            cudaFree(g->d_pos);
            for (int b = 0; b < 2; ++b) {
                cudaFree(g->d_batch[b]);
                if (g->up_done[b]) cudaEventDestroy(g->up_done[b]);
                if (g->buf_free[b]) cudaEventDestroy(g->buf_free[b]);
            }
            if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
            for (int b = 0; b < 2; ++b)
                if (g->gexec[b]) cudaGraphExecDestroy(g->gexec[b]);
            if (g->cap_stream) cudaStreamDestroy(g->cap_stream);
            cudaFree(g->d_scal);
            if (g->h_scal) cudaFreeHost(g->h_scal);
            if (g->h_acc) cudaFreeHost(g->h_acc);
            cudaFree(g->d_stage);
            cudaFree(g->d_tab);
            fft_plan_destroy(&g->fft);
            paint_tiling_destroy(&g->tiling);
            paint_scratch_free(&g->scratch);
            for (int q = 0; q < kGeoCache; ++q) bin_geometry_free(&g->geo[q]);
            for (auto &e : g->ev)
                if (e) cudaEventDestroy(e);
            if (g->own_stream) cudaStreamDestroy(g->own_stream);
            if (g->pinned)
                cudaFreeHost(self->f);
            else
                free(self->f);  // NULL for grids without a host view
            delete g;
        }
    }
    free(self);
}

extern "C" void fft_p2g(fft_t *self, gal_t *part, double offset[3]) {
    const double t = now_s();
    Grid *g = G(self);
    const int Ng = self->Ng;
    for (int i = 0; i < 3; ++i) {
        offset[i] = remainder(offset[i], Ng);
        self->offset[i] = offset[i];
    }
    FG_API(enter(self, false), "fft_p2g()");
    void *outs[1] = {g->d_f};
    double offs[1][3] = {{offset[0], offset[1], offset[2]}};
    FG_API(paint_catalog(g, part, outs, offs, 1), "fft_p2g()");
    FG_API(leave(self, true), "fft_p2g()");
    if (!g->quiet) fprintf(stderr, "fft_p2g() %.2fs\n", now_s() - t);
}

extern "C" void fft_x2k(fft_t *self, int offset_phase_on) {
    const double t = now_s();
    Grid *g = G(self);
    FG_API(enter(self, true), "fft_x2k()");
    void *grids[1] = {g->d_f};
    FG_API(fft_r2c(&g->fft, grids, 1, g->stream), "fft_x2k()");
    FG_API(scale_grid(g->d_f, self->Ng3_pad, g->prec, H3_of(g), g->stream), "fft_x2k()");
    if (offset_phase_on) FG_API(phase(g, g->d_f, self->offset, 1), "fft_x2k()");
    FG_API(leave(self, true), "fft_x2k()");
    if (!g->quiet) fprintf(stderr, "fft_x2k() %.2fs\n", now_s() - t);
}

extern "C" void fft_k2x(fft_t *self, int offset_phase_off) {
    const double t = now_s();
    Grid *g = G(self);
    FG_API(enter(self, true), "fft_k2x()");
    void *grids[1] = {g->d_f};
    FG_API(fft_c2r(&g->fft, grids, 1, g->stream), "fft_k2x()");
    const double L3 = self->L * self->L * self->L;
    FG_API(scale_grid(g->d_f, self->Ng3_pad, g->prec, 1 / L3, g->stream), "fft_k2x()");
    if (offset_phase_off) FG_API(phase(g, g->d_f, self->offset, -1), "fft_k2x()");
    FG_API(leave(self, true), "fft_k2x()");
    if (!g->quiet) fprintf(stderr, "fft_k2x() %.2fs\n", now_s() - t);
}

extern "C" void fft_offset_phase(fft_t *self, int onoff) {
    if (onoff == 0) {
        set_error(ERR_ARG, "onoff must be nonzero");
        die("fft_offset_phase()");
    }
    Grid *g = G(self);
    FG_API(enter(self, true), "fft_offset_phase()");
    FG_API(phase(g, g->d_f, self->offset, onoff), "fft_offset_phase()");
    FG_API(leave(self, true), "fft_offset_phase()");
}

extern "C" void fft_deconv(fft_t *self) {
    const double t = now_s();
    Grid *g = G(self);
    FG_API(enter(self, true), "fft_deconv()");
    FG_API(deconv(g, g->d_f), "fft_deconv()");
    FG_API(leave(self, true), "fft_deconv()");
    if (!g->quiet) fprintf(stderr, "fft_deconv() %.2fs\n", now_s() - t);
}

extern "C" void fft_p2k(fft_t *self, gal_t *part) {
    Grid *g = G(self);
    if (!g->quiet) fprintf(stderr, "fft_p2k() interlacing\n");
    const double t = now_s();
    FG_API(enter(self, false), "fft_p2k()");
    FG_API(ensure_aux(g), "fft_p2k()");
    // both interlacing grids painted in one particle pass: offset 0 -> f,
    // offset 1/2 -> aux (src/fft.c:260-269)
    const int Ng = self->Ng;
    double offs[2][3] = {{0, 0, 0}, {0.5, 0.5, 0.5}};
    for (int q = 0; q < 2; ++q)
        for (int a = 0; a < 3; ++a) offs[q][a] = remainder(offs[q][a], Ng);
    void *outs[2] = {g->d_f, g->d_aux};
    FG_API(paint_catalog(g, part, outs, offs, 2), "fft_p2k()");
    FG_API(fft_r2c(&g->fft, outs, 2, g->stream), "fft_p2k()");
    FG_API(ensure_tables(g), "fft_p2k()");
    FG_API(interlace_finish(g->d_f, g->d_aux, Ng, g->prec, H3_of(g), dual_tab(g), winv_tab(g), g->stream),
           "fft_p2k()");
    for (int a = 0; a < 3; ++a) self->offset[a] = offs[0][a];
    FG_API(leave(self, true), "fft_p2k()");
    if (!g->quiet) fprintf(stderr, "fft_p2k() %.2fs\n", now_s() - t);
}

extern "C" double *fft_exportf(fft_t *self) {
    Grid *g = G(self);
    double *dest = (double *)malloc(self->Ng3_pad * sizeof(double));
    if (!dest) {
        set_error(ERR_NOMEM, "export buffer");
        die("fft_exportf()");
    }
    if (g->view == FFTGAL_VIEW_SYNC)
        memcpy(dest, self->f, self->Ng3_pad * sizeof(double));
    else
        FG_API(device_to_host(g, dest, false), "fft_exportf()");
    return dest;
}

extern "C" void fft_importf(fft_t *self, double *src) {
    Grid *g = G(self);
    if (src == NULL) {
        set_error(ERR_ARG, "src is NULL");
        die("fft_importf()");
    }
    if (g->view == FFTGAL_VIEW_SYNC) {
        memcpy(self->f, src, self->Ng3_pad * sizeof(double));
        ++g->version;
    } else {
        FG_API(host_to_device(g, src, false), "fft_importf()");
    }
}

// PCS readout (src/fft.c:134-169)
namespace fg {
template <typename T>
__global__ void g2p_kernel(const T *__restrict__ f, int Ng, int Ng_pad, double Hinv, double o0, double o1,
                           double o2, const double *__restrict__ x, const double *__restrict__ y,
                           const double *__restrict__ z, long Np, int sum, double *__restrict__ out) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < Np; p += (long)gridDim.x * blockDim.x) {
        const double pos[3] = {x[p], y[p], z[p]};
        const double off[3] = {o0, o1, o2};
        int c[3][4];
        double w[3][4];
        for (int a = 0; a < 3; ++a) {
            const double u = __dsub_rn(__dmul_rn(pos[a], Hinv), off[a]);
            int g1 = (int)floor(u);
            const double d = __dsub_rn(u, (double)g1);
            g1 = (g1 % Ng + Ng) % Ng;
            c[a][0] = (g1 - 1 + Ng) % Ng;
            c[a][1] = g1;
            c[a][2] = (g1 + 1) % Ng;
            c[a][3] = (g1 + 2) % Ng;
            const double e = __dsub_rn(1.0, d), d2 = __dmul_rn(d, d);
            w[a][0] = __ddiv_rn(__dmul_rn(__dmul_rn(e, e), e), 6.0);
            w[a][1] = __ddiv_rn(__dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(3.0, d), 6.0), d2), 4.0), 6.0);
            w[a][2] = __ddiv_rn(
                __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(-3.0, d), 3.0), d), 3.0), d), 1.0), 6.0);
            w[a][3] = __ddiv_rn(__dmul_rn(d2, d), 6.0);
        }
        double acc = 0;
        if (sum) {
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j)
                    for (int k = 0; k < 4; ++k)
                        acc += (double)f[((long)c[0][i] * Ng + c[1][j]) * Ng_pad + c[2][k]] * w[0][i] * w[1][j] *
                               w[2][k];
        } else {
            // the reference assigns each term, so the last one remains
            acc = __dmul_rn(__dmul_rn(__dmul_rn((double)f[((long)c[0][3] * Ng + c[1][3]) * Ng_pad + c[2][3]],
                                                w[0][3]),
                                      w[1][3]),
                            w[2][3]);
        }
        out[p] = acc;
    }
}

static int g2p_run(fft_t *self, const gal_t *pos, int sum, double *host_out) {
    Grid *g = G(self);
    const long Np = pos->Np;
    if (Np <= 0) return OK;
    double *d = nullptr;
    FG_CUDA(cudaMalloc(&d, sizeof(double) * 4 * Np));
    cudaError_t e = cudaSuccess;
    for (int a = 0; a < 3 && e == cudaSuccess; ++a)
        e = cudaMemcpyAsync(d + a * Np, a == 0 ? pos->x : a == 1 ? pos->y : pos->z, sizeof(double) * Np,
                            cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) {
        long nb = ceil_div(Np, 256);
        if (nb > 64L * num_sms()) nb = 64L * num_sms();
        const double Hinv = self->Ng / self->L;
        if (g->prec == 4)
            g2p_kernel<float><<<(unsigned)nb, 256, 0, g->stream>>>((const float *)g->d_f, self->Ng, self->Ng_pad, Hinv,
                                                                   self->offset[0], self->offset[1], self->offset[2],
                                                                   d, d + Np, d + 2 * Np, Np, sum, d + 3 * Np);
        else
            g2p_kernel<double><<<(unsigned)nb, 256, 0, g->stream>>>((const double *)g->d_f, self->Ng, self->Ng_pad,
                                                                    Hinv, self->offset[0], self->offset[1],
                                                                    self->offset[2], d, d + Np, d + 2 * Np, Np, sum,
                                                                    d + 3 * Np);
        note_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_out, d + 3 * Np, sizeof(double) * Np, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(d);
    return cuda_check(e, "g2p");
}
}  // namespace fg

extern "C" double *fft_g2p(fft_t *self, gal_t *pos) {
    const double t = now_s();
    Grid *g = G(self);
    double *out = (double *)malloc((pos->Np > 0 ? pos->Np : 1) * sizeof(double));
    if (!out) die("fft_g2p()");
    FG_API(enter(self, true), "fft_g2p()");
    FG_API(g2p_run(self, pos, 0, out), "fft_g2p()");
    if (!g->quiet) fprintf(stderr, "fft_g2p() %.2fs\n", now_s() - t);
    return out;
}

// ======================================================================================
// reference API: src/power.h
// ======================================================================================

extern "C" void P(fft_t *grid, gal_t *part) {
    const double t = now_s();
    Grid *g = G(grid);
    FG_API(enter(grid, true), "P()");
    const double Vinv = 1 / part->V;
    const double alpha = (part->rand == NULL) ? 0 : (double)part->Np / part->rand->Np;
    const double Pshot = (1 + alpha) * part->V / part->Np;
    FG_API(power_inplace(g->d_f, grid->Ng, g->prec, Vinv, Pshot, g->stream), "P()");
    FG_API(leave(grid, true), "P()");
    if (!g->quiet) fprintf(stderr, "P() %.2fs\n", now_s() - t);
}

namespace fg {
// one binning pass for (los, dK, Nmu); fills the multipole and wedge sums and
// caches the wedge sums for a following Pmu on the same grid version
static int bin_pass(fft_t *grid, const double los_hat[3], double dK, int Nmu, BinGeometry **geo_out,
                    std::vector<double> &Psum, std::vector<double> &Pw, int mode, double Vinv, double Pshot,
                    cudaEvent_t *ev_end = nullptr, const BinFinish *fin = nullptr) {
    Grid *g = G(grid);
    BinSpec s;
    FG_TRY(bin_spec_init(&s, grid->Ng, grid->L, dK, los_hat, Nmu));
    BinGeometry *geo = geometry(g, s);
    if (!geo) return t_status ? t_status : ERR_CUDA;
    if (geo->bad)
        return set_error(ERR_RANGE, "a mode falls beyond the last of NK=%d k bins (dK too small for Ng)", s.NK);
    Psum.assign((size_t)s.NK * 4, 0.0);
    Pw.assign((size_t)s.NK * (Nmu + 1), 0.0);
    FG_TRY(bin_power(geo, g->d_f, g->prec, mode, Vinv, Pshot, Psum.data(), Pw.data(), g->stream, ev_end, fin));
    *geo_out = geo;
    return OK;
}

static void write_header(FILE *fp, int NK, double dK, const char *nlab, int nval, const fft_t *grid,
                         const gal_t *part, double alpha, const double los[3]) {
    fprintf(fp, "# NK %d\n", NK);
    fprintf(fp, "# dK %g\n", dK);
    fprintf(fp, "# %s %d\n", nlab, nval);
    fprintf(fp, "# Ng %d\n", grid->Ng);
    fprintf(fp, "# L %g\n", grid->L);
    fprintf(fp, "# Np %ld\n", part->Np);
    fprintf(fp, "# V %g\n", part->V);
    fprintf(fp, "# alpha %g\n", alpha);
    fprintf(fp, "# los[3] %g %g %g\n", los[0], los[1], los[2]);
}

// normalise multipole sums like src/power.c:69-76
static int finish_pl(const BinGeometry *geo, const std::vector<double> &Psum, double *K, long *N, double *P) {
    const BinSpec &s = geo->spec;
    long Ntot = 0;
    for (int b = 0; b < s.NK; ++b) {
        const long n = geo->N[b];
        if (K) K[b] = geo->K[b] * (s.KF / n);
        if (N) N[b] = n;
        if (P)
            for (int l = 0; l < 4; ++l) P[b * 4 + l] = Psum[(size_t)b * 4 + l] * ((4 * l + 1.0) / n);
        Ntot += n;
    }
    const long Ng = s.Ng;
    if (Ntot != Ng * Ng * Ng - 1) return set_error(ERR_RANGE, "mode count %ld != Ng^3-1", Ntot);
    return OK;
}

// merge the mu = 1 slot and normalise like src/power.c:139-153
static int finish_pmu(const BinGeometry *geo, const std::vector<double> &Pw, double *K, long *N, double *P) {
    const BinSpec &s = geo->spec;
    const int Nmu = s.Nmu, W = Nmu + 1;
    long Ntot = 0;
    for (int b = 0; b < s.NK; ++b) {
        std::vector<double> kk(W), pp(W);
        std::vector<long> nn(W);
        for (int m = 0; m < W; ++m) {
            kk[m] = geo->Kw[(size_t)b * W + m];
            nn[m] = geo->Nw[(size_t)b * W + m];
            pp[m] = Pw[(size_t)b * W + m];
        }
        kk[Nmu - 1] += kk[Nmu];
        nn[Nmu - 1] += nn[Nmu];
        pp[Nmu - 1] += pp[Nmu];
        for (int m = 0; m < Nmu; ++m) {
            double kv = kk[m], pv = pp[m];
            if (nn[m]) {
                kv *= s.KF / nn[m];
                pv /= nn[m];
                Ntot += nn[m];
            }
            if (K) K[b * Nmu + m] = kv;
            if (N) N[b * Nmu + m] = nn[m];
            if (P) P[b * Nmu + m] = pv;
        }
    }
    const long Ng = s.Ng;
    if (Ntot != Ng * Ng * Ng - 1) return set_error(ERR_RANGE, "mode count %ld != Ng^3-1", Ntot);
    return OK;
}
}  // namespace fg

extern "C" void Pl(fft_t *grid, gal_t *part, double los[3], double dK, char *file) {
    const double t = now_s();
    Grid *g = G(grid);
    FG_API(enter(grid, true), "Pl()");
    hat(los);
    const int Nmu = 3;
    BinGeometry *geo = nullptr;
    std::vector<double> Psum, Pw;
    FG_API(bin_pass(grid, los, dK, Nmu, &geo, Psum, Pw, 0, 0, 0), "Pl()");
    g->wedge_cache.version = g->version;
    g->wedge_cache.spec = geo->spec;
    g->wedge_cache.Pw = Pw;
    const int NK = geo->spec.NK, Nl = 4;
    std::vector<double> K(NK), Pv((size_t)NK * Nl);
    std::vector<long> N(NK);
    FG_API(finish_pl(geo, Psum, K.data(), N.data(), Pv.data()), "Pl()");
    const double alpha = (part->rand == NULL) ? 0 : (double)part->Np / part->rand->Np;
    FILE *fp = fopen(file, "w");
    if (!fp) {
        set_error(ERR_ARG, "cannot open %s", file);
        die("Pl()");
    }
    write_header(fp, NK, dK, "Nl", Nl, grid, part, alpha, los);
    fprintf(fp, "# K N");
    for (int il = 0; il < Nl; ++il) fprintf(fp, " P%d", 2 * il);
    fprintf(fp, "\n");
    for (int iK = 0; iK < NK; ++iK) {
        fprintf(fp, "%e %9ld", K[iK], N[iK]);
        for (int il = 0; il < Nl; ++il) fprintf(fp, " % e", Pv[(size_t)iK * Nl + il]);
        fprintf(fp, "\n");
    }
    fclose(fp);
    FG_API(leave(grid, false), "Pl()");
    if (!g->quiet) fprintf(stderr, "Pl() %.2fs, saved to %s\n", now_s() - t, file);
}

extern "C" void Pmu(fft_t *grid, gal_t *part, double los[3], double dK, char *file) {
    const double t = now_s();
    Grid *g = G(grid);
    hat(los);
    const int Nmu = 3;
    BinSpec s;
    FG_API(bin_spec_init(&s, grid->Ng, grid->L, dK, los, Nmu), "Pmu()");
    std::vector<double> Pw;
    BinGeometry *geo = nullptr;
    const auto &wc = g->wedge_cache;
    const bool reuse = g->view == FFTGAL_VIEW_LAZY && wc.version == g->version && wc.spec.dK == s.dK &&
                       wc.spec.L == s.L && wc.spec.Nmu == Nmu && wc.spec.los[0] == s.los[0] &&
                       wc.spec.los[1] == s.los[1] && wc.spec.los[2] == s.los[2];
    if (reuse) {
        geo = geometry(g, s);
        if (!geo) die("Pmu()");
        Pw = wc.Pw;
    } else {
        FG_API(enter(grid, true), "Pmu()");
        std::vector<double> Psum;
        FG_API(bin_pass(grid, los, dK, Nmu, &geo, Psum, Pw, 0, 0, 0), "Pmu()");
    }
    const int NK = s.NK;
    std::vector<double> K((size_t)NK * Nmu), Pv((size_t)NK * Nmu);
    std::vector<long> N((size_t)NK * Nmu);
    FG_API(finish_pmu(geo, Pw, K.data(), N.data(), Pv.data()), "Pmu()");
    const double alpha = (part->rand == NULL) ? 0 : (double)part->Np / part->rand->Np;
    FILE *fp = fopen(file, "w");
    if (!fp) {
        set_error(ERR_ARG, "cannot open %s", file);
        die("Pmu()");
    }
    write_header(fp, NK, dK, "Nmu", Nmu, grid, part, alpha, los);
    fprintf(fp, "#");
    for (int imu = 0; imu < Nmu; ++imu) fprintf(fp, " K%d N%d P%d", imu, imu, imu);
    fprintf(fp, "\n");
    for (int iK = 0; iK < NK; ++iK) {
        fprintf(fp, "%e %9ld % e", K[(size_t)iK * Nmu], N[(size_t)iK * Nmu], Pv[(size_t)iK * Nmu]);
        for (int imu = 1; imu < Nmu; ++imu)
            fprintf(fp, " %e %9ld % e", K[(size_t)iK * Nmu + imu], N[(size_t)iK * Nmu + imu],
                    Pv[(size_t)iK * Nmu + imu]);
        fprintf(fp, "\n");
    }
    fclose(fp);
    FG_API(leave(grid, false), "Pmu()");
    if (!g->quiet) fprintf(stderr, "Pmu() %.2fs, saved to %s\n", now_s() - t, file);
}

// ======================================================================================
// extensions: include/fftgal_gb300.h
// ======================================================================================

extern "C" int fftgal_version(void) { return 100; }
extern "C" int fftgal_last_status(void) { return t_status; }
extern "C" const char *fftgal_last_error(void) { return t_msg; }

extern "C" int fftgal_grid_precision(const fft_t *grid) { return grid ? G(grid)->prec : 0; }

extern "C" int fftgal_set_host_view(fft_t *grid, int mode) {
    if (!grid || (mode != FFTGAL_VIEW_SYNC && mode != FFTGAL_VIEW_LAZY))
        return set_error(ERR_ARG, "bad host-view mode");
    Grid *g = G(grid);
    if (g->view == FFTGAL_VIEW_LAZY && mode == FFTGAL_VIEW_SYNC) FG_TRY(device_to_host(g, grid->f, g->pinned));
    g->view = mode;
    return OK;
}

extern "C" int fftgal_sync_host(fft_t *grid) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    return device_to_host(G(grid), grid->f, G(grid)->pinned);
}

extern "C" int fftgal_sync_device(fft_t *grid) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    return host_to_device(G(grid), grid->f, G(grid)->pinned);
}

extern "C" int fftgal_set_stream(fft_t *grid, void *stream) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    FG_CUDA(cudaStreamSynchronize(g->stream));
    g->stream = stream ? (cudaStream_t)stream : g->own_stream;
    return OK;
}

extern "C" int fftgal_fft_columns_f32(int N, void *data, int ncols, long es, long bs, long nbatch, int sign,
                                      int shape, void *stream) {
    if (!data || N < 4 || ncols < 1 || es < 1 || nbatch < 1 || (sign != 1 && sign != -1))
        return set_error(ERR_ARG, "fftgal_fft_columns_f32: bad arguments");
    if (!fft2_supported(N, 4)) return set_error(ERR_UNSUPPORTED, "fftgal_fft_columns_f32: N=%d", N);
    if (shape != -1 && !fft2_valid_shape(N, 1, shape))
        return set_error(ERR_ARG, "fftgal_fft_columns_f32: shape %d invalid for N=%d", shape, N);
    FftPlan p;
    FG_TRY(fft_plan_create(&p, N, 4));
    cudaStream_t st = (cudaStream_t)stream;
    int rc = fft2_cols(N, p.axis.tw, data, data, 1, ncols, es, bs, nbatch, sign, st, shape);
    if (rc == OK) rc = cuda_check(cudaStreamSynchronize(st), "fftgal_fft_columns_f32");
    fft_plan_destroy(&p);
    return rc;
}

extern "C" int fftgal_launch_shapes(fft_t *grid, int shapes[3], int *source, double ms[2]) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    if (shapes) {
        shapes[0] = g->launch.paint_cta > 0 ? g->launch.paint_cta : 2;
        shapes[1] = g->launch.bin_cta > 0 ? g->launch.bin_cta : 3;
        shapes[2] = g->launch.bin_fold > 0 ? g->launch.bin_fold : 0;
    }
    if (source) *source = g->launch_source;
    if (ms) {
        ms[0] = g->launch_ms[0];
        ms[1] = g->launch_ms[1];
    }
    return OK;
}

extern "C" int fftgal_plan_info(fft_t *grid, int tune[3], int *source, double ms[3]) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    for (int w = 0; w < 3; ++w) {
        if (tune) tune[w] = g->fft.tune[w];
        if (ms) ms[w] = g->plan_ms[w];
    }
    if (source) *source = g->plan_source;
    return OK;
}

extern "C" int fftgal_plan_autotune(fft_t *grid, double ms[3]) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    double t[3];
    FG_TRY(fft2_autotune(&g->fft, g->d_f, g->stream, t));
    g->plan_source = FFTGAL_PLAN_MEASURED;
    for (int w = 0; w < 3; ++w) {
        g->plan_ms[w] = t[w];
        if (ms) ms[w] = t[w];
    }
    ++g->version;
    return OK;
}

extern "C" void *fftgal_get_stream(fft_t *grid) { return grid ? (void *)G(grid)->stream : nullptr; }

extern "C" int fftgal_set_quiet(fft_t *grid, int quiet) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    G(grid)->quiet = quiet;
    return OK;
}

extern "C" void *fftgal_device_grid(fft_t *grid) { return grid ? G(grid)->d_f : nullptr; }

extern "C" int fftgal_copy_grid(fft_t *grid, void *buf, int to_grid) {
    if (!grid || !buf) return set_error(ERR_ARG, "null argument");
    Grid *g = G(grid);
    const size_t bytes = (size_t)g->prec * g->Ng3_pad;
    // finish the grid's own work, then copy synchronously on the legacy
    // default stream so the copy also follows the caller's default-stream work
    FG_CUDA(cudaStreamSynchronize(g->stream));
    if (to_grid) {
        FG_CUDA(cudaMemcpy(g->d_f, buf, bytes, cudaMemcpyDefault));
        ++g->version;
    } else {
        FG_CUDA(cudaMemcpy(buf, g->d_f, bytes, cudaMemcpyDefault));
    }
    // a device-to-device cudaMemcpy returns before the copy is done, and the
    // grid's non-blocking stream does not wait for the legacy stream
    FG_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    return OK;
}

extern "C" int fftgal_synchronize(fft_t *grid) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    FG_CUDA(cudaStreamSynchronize(G(grid)->stream));
    return OK;
}

extern "C" int fftgal_nk(int Ng, double L, double dK) {
    BinSpec s;
    const double los[3] = {0, 0, 0};
    if (bin_spec_init(&s, Ng, L, dK, los, 1) != OK) return t_status;
    return s.NK;
}

extern "C" int fftgal_set_timing(fft_t *grid, int on) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    if (on && !g->ev[0])
        for (auto &e : g->ev) FG_CUDA(cudaEventCreate(&e));
    g->timing = on;
    return OK;
}

extern "C" int fftgal_stage_times(fft_t *grid, double out[FFTGAL_NSTAGES]) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    for (int q = 0; q <= kStages; ++q) out[q] = G(grid)->stage_ms[q];
    return OK;
}

namespace fg {
// the fused FP32 pipeline of fftgal_power_f32 / fftgal_power_rsd_f32; vel
// (nullable) displaces every particle along the line of sight while painting
static int power_f32_run(fft_t *grid, const float *x, const float *y, const float *z, const float *const *vel,
                         double aH, long Np, double V, int where, const double los_in[3], double dK, int Nmu,
                         double *K, long *N, double *Plout, double *Kmu, long *Nmu_count, double *Pmuout,
                         bool interlace = true) {
    if (!grid || !x || !y || !z || Np <= 0 || !(V > 0)) return set_error(ERR_ARG, "fftgal_power_f32: bad arguments");
    if (vel && (!vel[0] || !vel[1] || !vel[2] || !(aH != 0)))
        return set_error(ERR_ARG, "fftgal_power_rsd_f32: bad velocities or aH");
    Grid *g = G(grid);
    if (g->prec != 4) return set_error(ERR_STATE, "fftgal_power_f32 needs an FP32 grid");
    if (interlace) FG_TRY(ensure_aux(g));
    FG_TRY(ensure_tables(g));
    const int ngr = interlace ? 2 : 1;
    const bool tm = g->timing != 0;
    cudaStream_t st = g->stream;
    cudaEvent_t *ev = g->ev;
    if (tm) FG_CUDA(cudaEventRecord(ev[0], st));
    const float *px = x, *py = y, *pz = z;
    const float *pv[3] = {vel ? vel[0] : nullptr, vel ? vel[1] : nullptr, vel ? vel[2] : nullptr};
    if (where == FFTGAL_MEM_HOST) {
        const int narr = vel ? 6 : 3;
        const size_t need = (size_t)narr * Np * sizeof(float);
        if (need > g->pos_cap) {
            cudaFree(g->d_pos);
            g->d_pos = nullptr;
            FG_CUDA(cudaMalloc(&g->d_pos, need));
            g->pos_cap = need;
        }
        float *d = (float *)g->d_pos;
        const float *src[6] = {x, y, z, pv[0], pv[1], pv[2]};
        for (int a = 0; a < narr; ++a)
            FG_CUDA(cudaMemcpyAsync(d + a * Np, src[a], sizeof(float) * Np, cudaMemcpyHostToDevice, st));
        px = d;
        py = d + Np;
        pz = d + 2 * Np;
        if (vel)
            for (int a = 0; a < 3; ++a) pv[a] = d + (3 + a) * Np;
    }
    if (tm) FG_CUDA(cudaEventRecord(ev[1], st));
    double los[3] = {los_in[0], los_in[1], los_in[2]};
    hat(los);
    PaintRsd rsd;
    if (vel) {
        for (int a = 0; a < 3; ++a) {
            rsd.v[a] = pv[a];
            rsd.los[a] = los[a];
        }
        rsd.aHinv = 1 / aH;
    }
    const int Ng = grid->Ng;
    const double Hinv = Ng / grid->L;
    const double H3 = H3_of(g);
    const double nbar = Np / V;
    const double Npcinv = 1 / nbar / H3;
    PaintGridSpec spec[2];
    spec[0].out = g->d_f;
    spec[1].out = g->d_aux;
    for (int a = 0; a < 3; ++a) {
        spec[0].offset[a] = 0;
        spec[1].offset[a] = remainder(0.5, Ng);
    }
    spec[0].scale = spec[1].scale = Npcinv;
    FG_TRY(paint(&g->tiling, &g->scratch, 4, px, py, pz, 4, Np, Hinv, spec, ngr, st, tm ? ev + 2 : nullptr,
                 vel ? &rsd : nullptr));
    void *grids[2] = {g->d_f, g->d_aux};
    FG_TRY(fft_pass_k_r2c(&g->fft, grids, ngr, st));
    if (tm) FG_CUDA(cudaEventRecord(ev[6], st));
    FG_TRY(fft_pass_j(&g->fft, grids, ngr, -1, st));
    if (tm) FG_CUDA(cudaEventRecord(ev[7], st));
    FG_TRY(fft_pass_i(&g->fft, grids, ngr, -1, st));
    if (tm) FG_CUDA(cudaEventRecord(ev[8], st));
    for (int a = 0; a < 3; ++a) grid->offset[a] = 0;
    ++g->version;
    BinGeometry *geo = nullptr;
    std::vector<double> Psum, Pw;
    const double Vinv = 1 / V;
    const double Pshot = V / Np;
    // interlacing finish (offset phase, average, deconvolution) fused into the
    // binning pass; the finish stage is timed as part of the binning stage
    BinFinish fin;
    fin.A = g->d_f;
    fin.B = g->d_aux;
    fin.ph32 = dual_tab32(g);
    fin.w32 = winv_tab32(g);
    fin.scale = interlace ? 0.5 * H3 : H3;
    if (!interlace) fin.B = nullptr;
    if (tm) FG_CUDA(cudaEventRecord(ev[9], st));
    // with the lazy host view the finished (or deconvolved) field is binned
    // without being stored (4.3 GB fewer writes at Ng=1024); the grid's
    // contents are then unspecified until the next paint or import
    const bool keep = g->view != FFTGAL_VIEW_LAZY;
    const int bmode = interlace ? (keep ? 2 : 5) : (keep ? 3 : 4);
    FG_TRY(bin_pass(grid, los, dK, Nmu, &geo, Psum, Pw, bmode, Vinv, Pshot, tm ? &ev[10] : nullptr,
                    &fin));
    if (tm) {
        FG_CUDA(cudaEventSynchronize(ev[kStages]));
        float ms;
        for (int q = 0; q < kStages; ++q) {
            FG_CUDA(cudaEventElapsedTime(&ms, ev[q], ev[q + 1]));
            g->stage_ms[q] = ms;
        }
        FG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[kStages]));
        g->stage_ms[kStages] = ms;
    }
    FG_TRY(fft2_tma_check());  // the binning's read-back synchronised the stream
    FG_TRY(finish_pl(geo, Psum, K, N, Plout));
    FG_TRY(finish_pmu(geo, Pw, Kmu, Nmu_count, Pmuout));
    if (g->view == FFTGAL_VIEW_SYNC) FG_TRY(device_to_host(g, grid->f, g->pinned));
    return OK;
}
}  // namespace fg

extern "C" int fftgal_power_f32(fft_t *grid, const float *x, const float *y, const float *z, long Np, double V,
                                int where, const double los[3], double dK, int Nmu, double *K, long *N, double *Pl,
                                double *Kmu, long *Nmu_count, double *Pmu) {
    return power_f32_run(grid, x, y, z, nullptr, 0, Np, V, where, los, dK, Nmu, K, N, Pl, Kmu, Nmu_count, Pmu);
}

extern "C" int fftgal_window_box(fft_t *grid, int Ngsub) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    FG_TRY(enter(grid, true));
    FG_TRY(window_box(g->d_f, grid->Ng, g->prec, Ngsub, g->stream));
    return leave(grid, true);
}

extern "C" int fftgal_window_sphere(fft_t *grid, int Ngsub) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    Grid *g = G(grid);
    FG_TRY(enter(grid, true));
    FG_TRY(window_sphere(g->d_f, grid->Ng, g->prec, Ngsub, g->stream));
    return leave(grid, true);
}

extern "C" int fftgal_dl_sub(fft_t *grid, int sphere, int Nsub, int nlos, const double *los, double bias,
                             double *DeltaL) {
    if (!grid || !los || !DeltaL || nlos < 1 || !(bias != 0)) return set_error(ERR_ARG, "fftgal_dl_sub: bad arguments");
    Grid *g = G(grid);
    const int Ng = grid->Ng;
    if (Nsub < 2 || Ng % Nsub) return set_error(ERR_ARG, "fftgal_dl_sub: Nsub must divide Ng, Nsub >= 2");
    const int Ngsub = Ng / Nsub, nsub3 = Nsub * Nsub * Nsub;
    FG_TRY(enter(grid, true));
    FG_TRY(ensure_aux(g));
    cudaStream_t st = g->stream;
    // the unfiltered k-space field, filtered anew for every (line of sight, multipole)
    FG_CUDA(cudaMemcpyAsync(g->d_aux, g->d_f, (size_t)g->prec * grid->Ng3_pad, cudaMemcpyDeviceToDevice, st));
    // window tables, evaluated on the host like src/app/DLsb.c:44-50 / DLss.c:18-20,78
    std::vector<double> tab;
    if (sphere) {
        const long h = Ng / 2, n2max = 3 * h * h;
        tab.assign((size_t)n2max + 1, 0.0);
        for (long n2 = 1; n2 <= n2max; ++n2) {
            const double Kamp = sqrt((double)n2);
            volatile double KR = Kamp * M_PI * 1.73205080756887729352744634151 / Nsub;  // M_SQRT3
            volatile double KRcos = KR * cos(KR);  // kept separate: no FMA contraction
            tab[n2] = 3 * (sin(KR) - KRcos) / (KR * KR * KR);
        }
    } else {
        tab.assign((size_t)7 * Ng, 0.0);
        tab[0] = 1;
        for (int i = 1; i < Ng; ++i) tab[i] = sin(M_PI * i / Nsub) / sin(M_PI * i / Ng) / Ngsub;
        for (int i = 0; i < 3 * Ng; ++i) {
            tab[Ng + 2 * i] = cos(M_PI * i * (Ngsub - 1) / Ng);
            tab[Ng + 2 * i + 1] = sin(M_PI * i * (Ngsub - 1) / Ng);
        }
    }
    double *d_tab = nullptr, *d_out = nullptr;
    FG_CUDA(cudaMalloc(&d_tab, sizeof(double) * tab.size()));
    cudaError_t e = cudaMalloc(&d_out, sizeof(double) * (size_t)nsub3 * 3 * nlos);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st);
    int rc = cuda_check(e, "fftgal_dl_sub tables");
    const double L3 = grid->L * grid->L * grid->L;
    void *grids[1] = {g->d_f};
    for (int l = 0; l < nlos && rc == OK; ++l) {
        double lh[3] = {los[3 * l], los[3 * l + 1], los[3 * l + 2]};
        hat(lh);
        for (int iL = 0; iL < 3 && rc == OK; ++iL) {
            rc = dl_filter(g->d_f, g->d_aux, Ng, g->prec, sphere, d_tab, lh, iL, st);
            if (rc == OK) rc = fft_c2r(&g->fft, grids, 1, st);
            if (rc == OK) rc = scale_grid(g->d_f, grid->Ng3_pad, g->prec, 1 / L3, st);
            if (rc == OK) rc = dl_sample(g->d_f, Ng, g->prec, Nsub, bias, d_out + (size_t)(3 * l + iL) * nsub3, st);
        }
    }
    if (rc == OK)
        rc = cuda_check(cudaMemcpyAsync(DeltaL, d_out, sizeof(double) * (size_t)nsub3 * 3 * nlos,
                                        cudaMemcpyDeviceToHost, st), "fftgal_dl_sub results");
    if (rc == OK) rc = cuda_check(cudaStreamSynchronize(st), "fftgal_dl_sub");
    cudaFree(d_tab);
    cudaFree(d_out);
    FG_TRY(rc);
    return leave(grid, true);
}

// ---- graph-captured batches ------------------------------------------------------
// The device work of one catalog -- paint key, scan, scatter and tile paint of
// both interlacing grids, the three r2c passes, the fused finish + binning --
// is captured once per upload buffer into a CUDA graph whose kernels read the
// catalog's count and scales from a device block (DevScalars), so one graph
// replays for catalogs of any size.  The host enqueues upload, graph and the
// read-back of the bin sums for every catalog without waiting, and finishes
// all bin tables after one synchronisation.
static void graphs_drop(Grid *g) {
    for (int b = 0; b < 2; ++b)
        if (g->gexec[b]) {
            cudaGraphExecDestroy(g->gexec[b]);
            g->gexec[b] = nullptr;
        }
    g->gkey.clear();
}

static int enqueue_catalog(fft_t *grid, int b, long capNp, BinGeometry *geo, cudaStream_t st) {
    Grid *g = G(grid);
    const float *d = g->d_batch[b];
    const int Ng = grid->Ng;
    PaintGridSpec spec[2];
    spec[0].out = g->d_f;
    spec[1].out = g->d_aux;
    for (int a = 0; a < 3; ++a) {
        spec[0].offset[a] = 0;
        spec[1].offset[a] = remainder(0.5, Ng);
    }
    FG_TRY(paint(&g->tiling, &g->scratch, 4, d, d + capNp, d + 2 * capNp, 4, capNp, Ng / grid->L, spec, 2, st,
                 nullptr, nullptr, g->d_scal + b));
    void *grids[2] = {g->d_f, g->d_aux};
    FG_TRY(fft_pass_k_r2c(&g->fft, grids, 2, st));
    FG_TRY(fft_pass_j(&g->fft, grids, 2, -1, st));
    FG_TRY(fft_pass_i(&g->fft, grids, 2, -1, st));
    BinFinish fin;
    fin.A = g->d_f;
    fin.B = g->d_aux;
    fin.ph32 = dual_tab32(g);
    fin.w32 = winv_tab32(g);
    fin.scale = 0.5 * H3_of(g);
    // the lazy host view bins the finished field without storing it
    return bin_power_launch(geo, g->view == FFTGAL_VIEW_LAZY ? 5 : 2, 0, 0, st, &fin, g->d_scal + b);
}

static int capture_catalog(fft_t *grid, int b, long capNp, BinGeometry *geo, cudaGraphExec_t *exec, int *nkern) {
    Grid *g = G(grid);
    cudaStream_t cs = g->cap_stream;
    FG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    const int rc = enqueue_catalog(grid, b, capNp, geo, cs);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (rc != OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc != OK ? rc : cuda_check(e, "graph capture");
    }
    size_t n = 0;
    e = cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (e == cudaSuccess && n) e = cudaGraphGetNodes(graph, nodes.data(), &n);
    int k = 0;
    for (size_t q = 0; q < n && e == cudaSuccess; ++q) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[q], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    *nkern = k;
    return cuda_check(e, "graph instantiate");
}

template <typename T>
static void key_push(std::vector<uint64_t> &k, T v) {
    uint64_t u = 0;
    memcpy(&u, &v, sizeof(T) < sizeof(u) ? sizeof(T) : sizeof(u));
    k.push_back(u);
}

static int power_batch_graph(fft_t *grid, int ncat, const float *const *x, const float *const *y,
                             const float *const *z, const long *Np, const double *V, const double los_in[3],
                             double dK, int Nmu, double *K, long *N, double *Pl, double *Kmu, long *Nmu_count,
                             double *Pmu) {
    Grid *g = G(grid);
    long maxNp = 0;
    for (int c = 0; c < ncat; ++c) {
        if (!x[c] || !y[c] || !z[c] || Np[c] <= 0 || !(V[c] > 0))
            return set_error(ERR_ARG, "fftgal_power_batch_f32: bad catalog %d", c);
        maxNp = Np[c] > maxNp ? Np[c] : maxNp;
    }
    if (ncat == 0) return OK;
    if (!g->copy_stream) FG_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    if (!g->cap_stream) FG_CUDA(cudaStreamCreateWithFlags(&g->cap_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        if (!g->up_done[b]) FG_CUDA(cudaEventCreateWithFlags(&g->up_done[b], cudaEventDisableTiming));
        if (!g->buf_free[b]) FG_CUDA(cudaEventCreateWithFlags(&g->buf_free[b], cudaEventDisableTiming));
    }
    FG_CUDA(cudaStreamSynchronize(g->stream));
    FG_CUDA(cudaStreamSynchronize(g->copy_stream));
    if ((size_t)3 * maxNp > g->batch_cap) {
        graphs_drop(g);
        for (int b = 0; b < 2; ++b) {
            cudaFree(g->d_batch[b]);
            g->d_batch[b] = nullptr;
        }
        g->batch_cap = 0;
        // 1/8 headroom: a later batch with slightly larger catalogs reuses
        // the buffers (and, with graphs, the captured graphs)
        const size_t room = (size_t)maxNp + (size_t)maxNp / 8 + 1024;
        for (int b = 0; b < 2; ++b) FG_CUDA(cudaMalloc(&g->d_batch[b], sizeof(float) * 3 * room));
        g->batch_cap = 3 * room;
    }
    const long capNp = (long)(g->batch_cap / 3);
    FG_TRY(ensure_aux(g));
    FG_TRY(ensure_tables(g));
    FG_TRY(fft2_prepare());
    FG_TRY(paint_reserve(&g->tiling, &g->scratch, capNp));
    if (!g->d_scal) FG_CUDA(cudaMalloc(&g->d_scal, 2 * sizeof(DevScalars)));
    double los[3] = {los_in[0], los_in[1], los_in[2]};
    hat(los);
    BinSpec spec;
    FG_TRY(bin_spec_init(&spec, grid->Ng, grid->L, dK, los, Nmu));
    BinGeometry *geo = geometry(g, spec);
    if (!geo) return t_status ? t_status : ERR_CUDA;
    if (geo->bad)
        return set_error(ERR_RANGE, "a mode falls beyond the last of NK=%d k bins (dK too small for Ng)", spec.NK);
    if ((size_t)ncat > g->h_scal_cap) {
        if (g->h_scal) cudaFreeHost(g->h_scal);
        g->h_scal = nullptr;
        g->h_scal_cap = 0;
        const size_t cap = (size_t)ncat + (size_t)ncat / 2 + 16;  // headroom for growing batches
        FG_CUDA(cudaMallocHost(&g->h_scal, sizeof(DevScalars) * cap));
        g->h_scal_cap = cap;
    }
    if ((size_t)ncat * geo->acc_len > g->h_acc_cap) {
        if (g->h_acc) cudaFreeHost(g->h_acc);
        g->h_acc = nullptr;
        g->h_acc_cap = 0;
        const size_t cap = ((size_t)ncat + (size_t)ncat / 2 + 16) * geo->acc_len;
        FG_CUDA(cudaMallocHost(&g->h_acc, sizeof(double) * cap));
        g->h_acc_cap = cap;
    }
    // recapture whenever a buffer, table, plan or bin layout the graphs name changed
    std::vector<uint64_t> key;
    const void *ptrs[] = {g->d_batch[0], g->d_batch[1], g->d_f,         g->d_aux,           g->scratch.cursor,
                          g->scratch.sorted, g->scratch.hist, g->scratch.scan_tmp, geo,
                          geo->d_acc,      geo->d_thr,        g->d_tab,       g->d_scal};
    for (const void *q : ptrs) key_push(key, (uintptr_t)q);
    key_push(key, capNp);
    key_push(key, g->view);
    for (int w = 0; w < 3; ++w) key_push(key, g->fft.tune[w]);
    key_push(key, spec.NK);
    key_push(key, Nmu);
    key_push(key, dK);
    for (int a = 0; a < 3; ++a) key_push(key, los[a]);
    if (key != g->gkey) {
        graphs_drop(g);
        for (int b = 0; b < 2; ++b) FG_TRY(capture_catalog(grid, b, capNp, geo, &g->gexec[b], &g->graph_kernels));
        g->gkey = key;
    }
    // per-catalog scalars, formed like power_f32_run forms its launch arguments
    const double H3 = H3_of(g);
    for (int c = 0; c < ncat; ++c) {
        DevScalars &q = g->h_scal[c];
        const double nbar = Np[c] / V[c];
        q.Np = Np[c];
        q.scale[0] = q.scale[1] = 1 / nbar / H3;
        q.Vinv = (float)(1 / V[c]);
        q.Pshot = (float)(V[c] / Np[c]);
    }
    auto upload = [&](int c) -> int {
        const int b = c & 1;
        float *d = g->d_batch[b];
        FG_CUDA(cudaStreamWaitEvent(g->copy_stream, g->buf_free[b], 0));
        const float *src[3] = {x[c], y[c], z[c]};
        for (int a = 0; a < 3; ++a)
            FG_CUDA(cudaMemcpyAsync(d + (size_t)a * capNp, src[a], sizeof(float) * Np[c], cudaMemcpyDefault,
                                    g->copy_stream));
        FG_CUDA(cudaMemcpyAsync(g->d_scal + b, g->h_scal + c, sizeof(DevScalars), cudaMemcpyHostToDevice,
                                g->copy_stream));
        FG_CUDA(cudaEventRecord(g->up_done[b], g->copy_stream));
        return OK;
    };
    for (int b = 0; b < 2; ++b) FG_CUDA(cudaEventRecord(g->buf_free[b], g->stream));
    FG_TRY(upload(0));
    for (int c = 0; c < ncat; ++c) {
        const int b = c & 1;
        if (c + 1 < ncat) FG_TRY(upload(c + 1));
        FG_CUDA(cudaStreamWaitEvent(g->stream, g->up_done[b], 0));
        FG_CUDA(cudaGraphLaunch(g->gexec[b], g->stream));
        note_launches(g->graph_kernels);
        FG_CUDA(cudaEventRecord(g->buf_free[b], g->stream));
        FG_CUDA(cudaMemcpyAsync(g->h_acc + (size_t)c * geo->acc_len, geo->d_acc, sizeof(double) * geo->acc_len,
                                cudaMemcpyDeviceToHost, g->stream));
    }
    FG_CUDA(cudaStreamSynchronize(g->stream));
    FG_CUDA(cudaStreamSynchronize(g->copy_stream));
    FG_TRY(fft2_tma_check());
    for (int a = 0; a < 3; ++a) grid->offset[a] = 0;
    ++g->version;
    const int NK = spec.NK;
    std::vector<double> Psum((size_t)NK * 4), Pw((size_t)NK * (Nmu + 1));
    for (int c = 0; c < ncat; ++c) {
        bin_power_unpack(geo, g->h_acc + (size_t)c * geo->acc_len, Psum.data(), Pw.data());
        const size_t o1 = (size_t)NK * c, o4 = (size_t)NK * 4 * c, om = (size_t)NK * Nmu * c;
        FG_TRY(finish_pl(geo, Psum, K ? K + o1 : nullptr, N ? N + o1 : nullptr, Pl ? Pl + o4 : nullptr));
        FG_TRY(finish_pmu(geo, Pw, Kmu ? Kmu + om : nullptr, Nmu_count ? Nmu_count + om : nullptr,
                          Pmu ? Pmu + om : nullptr));
    }
    if (g->view == FFTGAL_VIEW_SYNC) FG_TRY(device_to_host(g, grid->f, g->pinned));
    return OK;
}

extern "C" int fftgal_set_graphs(fft_t *grid, int on) {
    if (!grid) return set_error(ERR_ARG, "null grid");
    G(grid)->use_graphs = on ? 1 : 0;
    return OK;
}

extern "C" int fftgal_power_batch_f32(fft_t *grid, int ncat, const float *const *x, const float *const *y,
                                      const float *const *z, const long *Np, const double *V,
                                      const double los[3], double dK, int Nmu, double *K, long *N, double *Pl,
                                      double *Kmu, long *Nmu_count, double *Pmu) {
    if (!grid || ncat < 0 || (ncat > 0 && (!x || !y || !z || !Np || !V)))
        return set_error(ERR_ARG, "fftgal_power_batch_f32: bad arguments");
    Grid *g = G(grid);
    if (g->prec != 4) return set_error(ERR_STATE, "fftgal_power_batch_f32 needs an FP32 grid");
    if (g->use_graphs)
        return power_batch_graph(grid, ncat, x, y, z, Np, V, los, dK, Nmu, K, N, Pl, Kmu, Nmu_count, Pmu);
    long maxNp = 0;
    for (int c = 0; c < ncat; ++c) {
        if (!x[c] || !y[c] || !z[c] || Np[c] <= 0 || !(V[c] > 0))
            return set_error(ERR_ARG, "fftgal_power_batch_f32: bad catalog %d", c);
        maxNp = Np[c] > maxNp ? Np[c] : maxNp;
    }
    if (ncat == 0) return OK;
    if (!g->copy_stream) FG_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        if (!g->up_done[b]) FG_CUDA(cudaEventCreateWithFlags(&g->up_done[b], cudaEventDisableTiming));
        if (!g->buf_free[b]) FG_CUDA(cudaEventCreateWithFlags(&g->buf_free[b], cudaEventDisableTiming));
    }
    if ((size_t)3 * maxNp > g->batch_cap) {
        FG_CUDA(cudaStreamSynchronize(g->stream));
        FG_CUDA(cudaStreamSynchronize(g->copy_stream));
        for (int b = 0; b < 2; ++b) {
            cudaFree(g->d_batch[b]);
            g->d_batch[b] = nullptr;
        }
        g->batch_cap = 0;
        // 1/8 headroom: a later batch with slightly larger catalogs reuses
        // the buffers (and, with graphs, the captured graphs)
        const size_t room = (size_t)maxNp + (size_t)maxNp / 8 + 1024;
        for (int b = 0; b < 2; ++b) FG_CUDA(cudaMalloc(&g->d_batch[b], sizeof(float) * 3 * room));
        g->batch_cap = 3 * room;
    }
    const int NK = fftgal_nk(grid->Ng, grid->L, dK);
    if (NK < 1) return set_error(ERR_ARG, "fftgal_power_batch_f32: bad dK");
    // catalog c goes to buffer c % 2: its upload waits until the paint of
    // catalog c - 2 (the buffer's previous user) has read it
    auto upload = [&](int c) -> int {
        const int b = c & 1;
        float *d = g->d_batch[b];
        FG_CUDA(cudaStreamWaitEvent(g->copy_stream, g->buf_free[b], 0));
        const float *src[3] = {x[c], y[c], z[c]};
        for (int a = 0; a < 3; ++a)
            FG_CUDA(cudaMemcpyAsync(d + (size_t)a * Np[c], src[a], sizeof(float) * Np[c], cudaMemcpyDefault,
                                    g->copy_stream));
        FG_CUDA(cudaEventRecord(g->up_done[b], g->copy_stream));
        return OK;
    };
    for (int b = 0; b < 2; ++b) FG_CUDA(cudaEventRecord(g->buf_free[b], g->stream));
    FG_TRY(upload(0));
    for (int c = 0; c < ncat; ++c) {
        const int b = c & 1;
        if (c + 1 < ncat) FG_TRY(upload(c + 1));
        FG_CUDA(cudaStreamWaitEvent(g->stream, g->up_done[b], 0));
        const float *d = g->d_batch[b];
        const size_t o1 = (size_t)NK * c, o4 = (size_t)NK * 4 * c, om = (size_t)NK * Nmu * c;
        FG_TRY(power_f32_run(grid, d, d + Np[c], d + 2 * Np[c], nullptr, 0, Np[c], V[c], FFTGAL_MEM_DEVICE, los,
                             dK, Nmu, K ? K + o1 : nullptr, N ? N + o1 : nullptr, Pl ? Pl + o4 : nullptr,
                             Kmu ? Kmu + om : nullptr, Nmu_count ? Nmu_count + om : nullptr,
                             Pmu ? Pmu + om : nullptr));
        FG_CUDA(cudaEventRecord(g->buf_free[b], g->stream));
    }
    FG_CUDA(cudaStreamSynchronize(g->copy_stream));
    return OK;
}

// ---- catalogs of mixed grid sizes and boxes in one call ----------------------------------
// Grids kept between calls, one per (device, Ng, box length): device state
// only (no host view), released by fftgal_power_mixed_release.
static std::mutex g_mixed_mutex;
static std::map<std::tuple<int, int, double>, fft_t *> g_mixed_grids;

extern "C" int fftgal_power_mixed_release(void) {
    std::lock_guard<std::mutex> lock(g_mixed_mutex);
    int dev = 0;
    cudaGetDevice(&dev);
    for (auto it = g_mixed_grids.begin(); it != g_mixed_grids.end();) {
        if (std::get<0>(it->first) == dev) {
            fft_free(it->second);
            it = g_mixed_grids.erase(it);
        } else {
            ++it;
        }
    }
    return OK;
}

extern "C" int fftgal_power_mixed_f32(int ncat, const float *const *x, const float *const *y, const float *const *z,
                                      const long *Np, const double *V, const int *Ng, const double *L,
                                      const double los[3], const double *dK, int Nmu, double *const *K,
                                      long *const *N, double *const *Pl, double *const *Kmu, long *const *Nmu_count,
                                      double *const *Pmu) {
    if (ncat < 0 || (ncat > 0 && (!x || !y || !z || !Np || !V || !Ng || !L || !dK || !los)))
        return set_error(ERR_ARG, "fftgal_power_mixed_f32: bad arguments");
    if (ncat == 0) return OK;
    int dev = 0;
    FG_CUDA(cudaGetDevice(&dev));
    // groups of catalogs with the same (Ng, box, dK), in order of first appearance
    std::vector<std::tuple<int, double, double>> keys;
    std::vector<std::vector<int>> members;
    for (int c = 0; c < ncat; ++c) {
        if (Ng[c] < 2 || !(L[c] > 0) || !(dK[c] > 0))
            return set_error(ERR_ARG, "fftgal_power_mixed_f32: catalog %d: bad Ng, L or dK", c);
        const auto key = std::make_tuple(Ng[c], L[c], dK[c]);
        size_t q = 0;
        while (q < keys.size() && keys[q] != key) ++q;
        if (q == keys.size()) {
            keys.push_back(key);
            members.emplace_back();
        }
        members[q].push_back(c);
    }
    std::lock_guard<std::mutex> lock(g_mixed_mutex);
    for (size_t q = 0; q < keys.size(); ++q) {
        const int ng = std::get<0>(keys[q]);
        const double box = std::get<1>(keys[q]), dk = std::get<2>(keys[q]);
        fft_t *&grid = g_mixed_grids[std::make_tuple(dev, ng, box)];
        if (!grid) {
            grid = grid_new(ng, box, "FFTW_ESTIMATE", false, true);
            if (!grid) {
                g_mixed_grids.erase(std::make_tuple(dev, ng, box));
                return t_status ? t_status : ERR_CUDA;
            }
        }
        if (G(grid)->prec != 4) return set_error(ERR_STATE, "fftgal_power_mixed_f32 needs FP32 grids");
        const std::vector<int> &m = members[q];
        const int n = (int)m.size();
        const int NK = fftgal_nk(ng, box, dk);
        if (NK < 1) return set_error(ERR_ARG, "fftgal_power_mixed_f32: bad dK for catalog %d", m[0]);
        std::vector<const float *> gx(n), gy(n), gz(n);
        std::vector<long> gn(n);
        std::vector<double> gv(n);
        for (int i = 0; i < n; ++i) {
            gx[i] = x[m[i]];
            gy[i] = y[m[i]];
            gz[i] = z[m[i]];
            gn[i] = Np[m[i]];
            gv[i] = V[m[i]];
        }
        std::vector<double> bK((size_t)n * NK), bPl((size_t)n * NK * 4), bKm((size_t)n * NK * Nmu),
            bPm((size_t)n * NK * Nmu);
        std::vector<long> bN((size_t)n * NK), bNm((size_t)n * NK * Nmu);
        FG_TRY(fftgal_power_batch_f32(grid, n, gx.data(), gy.data(), gz.data(), gn.data(), gv.data(), los, dk, Nmu,
                                      bK.data(), bN.data(), bPl.data(), bKm.data(), bNm.data(), bPm.data()));
        for (int i = 0; i < n; ++i) {
            const int c = m[i];
            const size_t o1 = (size_t)i * NK, o4 = o1 * 4, om = o1 * Nmu;
            if (K && K[c]) memcpy(K[c], &bK[o1], sizeof(double) * NK);
            if (N && N[c]) memcpy(N[c], &bN[o1], sizeof(long) * NK);
            if (Pl && Pl[c]) memcpy(Pl[c], &bPl[o4], sizeof(double) * 4 * NK);
            if (Kmu && Kmu[c]) memcpy(Kmu[c], &bKm[om], sizeof(double) * Nmu * NK);
            if (Nmu_count && Nmu_count[c]) memcpy(Nmu_count[c], &bNm[om], sizeof(long) * Nmu * NK);
            if (Pmu && Pmu[c]) memcpy(Pmu[c], &bPm[om], sizeof(double) * Nmu * NK);
        }
    }
    return OK;
}

extern "C" int fftgal_power_single_f32(fft_t *grid, const float *x, const float *y, const float *z, long Np,
                                       double V, int where, const double los[3], double dK, int Nmu, double *K,
                                       long *N, double *Pl, double *Kmu, long *Nmu_count, double *Pmu) {
    return power_f32_run(grid, x, y, z, nullptr, 0, Np, V, where, los, dK, Nmu, K, N, Pl, Kmu, Nmu_count, Pmu,
                         false);
}

extern "C" int fftgal_power_learned_f32(fft_t *grid, const float *x, const float *y, const float *z, long Np,
                                        double V, int where, const double los[3], double dK, int Nmu,
                                        const float *mlp_params, double *K, long *N, double *Pl, double *Kmu,
                                        long *Nmu_count, double *Pmu) {
    if (!mlp_params) return set_error(ERR_ARG, "fftgal_power_learned_f32: no MLP parameters");
    if (!grid) return set_error(ERR_ARG, "null grid");
    const int NK = fftgal_nk(grid->Ng, grid->L, dK);
    if (NK < 1) return set_error(ERR_ARG, "fftgal_power_learned_f32: bad dK");
    std::vector<double> Kb(NK), Pb((size_t)NK * 4);
    std::vector<long> Nb(NK);
    FG_TRY(power_f32_run(grid, x, y, z, nullptr, 0, Np, V, where, los, dK, Nmu, Kb.data(), Nb.data(), Pb.data(), Kmu,
                         Nmu_count, Pmu, false));
    const double Pshot = V / Np, kNyq = M_PI * grid->Ng / grid->L;
    const int np = fftgal_mlp_nparams();
    std::vector<float> X((size_t)NK * 5), Y((size_t)NK * 3);
    FG_TRY(fftgal_alias_features(NK, Kb.data(), Pb.data(), Pshot, kNyq, X.data()));
    Grid *g = G(grid);
    float *d = nullptr;
    FG_CUDA(cudaMalloc(&d, sizeof(float) * ((size_t)np + X.size() + Y.size())));
    float *dp = d, *dx = d + np, *dy = dx + X.size();
    cudaError_t e = cudaMemcpyAsync(dp, mlp_params, sizeof(float) * np, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, X.data(), sizeof(float) * X.size(), cudaMemcpyHostToDevice, g->stream);
    int rc = cuda_check(e, "fftgal_power_learned_f32 upload");
    if (rc == OK) rc = fftgal_mlp_forward(dp, dx, NK, dy, g->stream);
    if (rc == OK)
        rc = cuda_check(cudaMemcpyAsync(Y.data(), dy, sizeof(float) * Y.size(), cudaMemcpyDeviceToHost, g->stream),
                        "fftgal_power_learned_f32 download");
    if (rc == OK) rc = cuda_check(cudaStreamSynchronize(g->stream), "fftgal_power_learned_f32");
    cudaFree(d);
    FG_TRY(rc);
    // P_l += den e(k / k_Nyq) y_l (l = 0, 2, 4) on bins with modes; l = 6 as measured
    for (int b = 0; b < NK; ++b) {
        if (K) K[b] = Kb[b];
        if (N) N[b] = Nb[b];
        const double den = fabs(Pb[4 * b]) + Pshot;
        const bool ok = std::isfinite(Pb[4 * b]) && Nb[b] > 0;
        const double sc = ok ? den * fftgal_alias_envelope(Kb[b] / kNyq) : 0.0;
        for (int l = 0; l < 4; ++l)
            if (Pl) Pl[4 * b + l] = Pb[4 * b + l] + (l < 3 ? sc * Y[3 * b + l] : 0.0);
    }
    return OK;
}

// Learned mode checked against the interlaced estimator, with fallback: every
// holdout_every-th catalog (0: none) is measured both ways and reported with
// its interlaced result; once a checked catalog's learned estimate differs from
// its interlaced one by more than tol (max over l = 0, 2, 4 and bins with modes
// below 0.8 k_Nyq of |P_l^learned - P_l^interlaced| / (|P_0^interlaced| +
// Pshot)), every later catalog runs interlaced.
extern "C" int fftgal_power_learned_checked_f32(fft_t *grid, int ncat, const float *const *x,
                                                const float *const *y, const float *const *z, const long *Np,
                                                const double *V, int where, const double los[3], double dK,
                                                int Nmu, const float *mlp_params, int holdout_every, double tol,
                                                double *K, long *N, double *Pl, double *Kmu, long *Nmu_count,
                                                double *Pmu, int *used, double *disagreement) {
    if (!grid || ncat < 0 || (ncat > 0 && (!x || !y || !z || !Np || !V || !used)) || !mlp_params ||
        holdout_every < 0 || !(tol >= 0))
        return set_error(ERR_ARG, "fftgal_power_learned_checked_f32: bad arguments");
    const int NK = fftgal_nk(grid->Ng, grid->L, dK);
    if (NK < 1 || Nmu < 1) return set_error(ERR_ARG, "fftgal_power_learned_checked_f32: bad dK or Nmu");
    const double kNyq = M_PI * grid->Ng / grid->L;
    const size_t nw = (size_t)NK * Nmu;
    std::vector<double> Kl(NK), Pll((size_t)NK * 4), Kml(nw), Pml(nw), Ki(NK), Pli((size_t)NK * 4), Kmi(nw), Pmi(nw);
    std::vector<long> Nl(NK), Nml(nw), Ni(NK), Nmi(nw);
    bool fallback = false;
    for (int c = 0; c < ncat; ++c) {
        if (!x[c] || !y[c] || !z[c] || Np[c] <= 0 || !(V[c] > 0))
            return set_error(ERR_ARG, "fftgal_power_learned_checked_f32: bad catalog %d", c);
        if (disagreement) disagreement[c] = NAN;
        const bool check = holdout_every > 0 && c % holdout_every == 0;
        const bool was_fallback = fallback;
        // the estimate reported for catalog c is in (Ki, Ni, Pli, ...) when
        // interlaced, in (Kl, Nl, Pll, ...) when learned
        const bool report_interlaced = was_fallback || check;
        if (!was_fallback)
            FG_TRY(fftgal_power_learned_f32(grid, x[c], y[c], z[c], Np[c], V[c], where, los, dK, Nmu, mlp_params,
                                            Kl.data(), Nl.data(), Pll.data(), Kml.data(), Nml.data(), Pml.data()));
        if (report_interlaced)
            FG_TRY(power_f32_run(grid, x[c], y[c], z[c], nullptr, 0, Np[c], V[c], where, los, dK, Nmu, Ki.data(),
                                 Ni.data(), Pli.data(), Kmi.data(), Nmi.data(), Pmi.data(), true));
        if (check && !was_fallback) {
            const double Pshot = V[c] / Np[c];
            double err = 0;
            for (int b = 0; b < NK; ++b) {
                if (Ni[b] <= 0 || !(Ki[b] < 0.8 * kNyq) || !std::isfinite(Pli[4 * b])) continue;
                const double den = fabs(Pli[4 * b]) + Pshot;
                for (int l = 0; l < 3; ++l) err = std::max(err, fabs(Pll[4 * b + l] - Pli[4 * b + l]) / den);
            }
            if (disagreement) disagreement[c] = err;
            if (err > tol) fallback = true;
        }
        used[c] = was_fallback ? 2 : (check ? 1 : 0);
        const double *Ks = report_interlaced ? Ki.data() : Kl.data();
        const long *Ns = report_interlaced ? Ni.data() : Nl.data();
        const double *Ps = report_interlaced ? Pli.data() : Pll.data();
        const double *Kms = report_interlaced ? Kmi.data() : Kml.data();
        const long *Nms = report_interlaced ? Nmi.data() : Nml.data();
        const double *Pms = report_interlaced ? Pmi.data() : Pml.data();
        const size_t o1 = (size_t)NK * c, o4 = (size_t)NK * 4 * c, om = nw * c;
        if (K) std::copy(Ks, Ks + NK, K + o1);
        if (N) std::copy(Ns, Ns + NK, N + o1);
        if (Pl) std::copy(Ps, Ps + (size_t)NK * 4, Pl + o4);
        if (Kmu) std::copy(Kms, Kms + nw, Kmu + om);
        if (Nmu_count) std::copy(Nms, Nms + nw, Nmu_count + om);
        if (Pmu) std::copy(Pms, Pms + nw, Pmu + om);
    }
    return OK;
}

extern "C" int fftgal_power_rsd_f32(fft_t *grid, const float *x, const float *y, const float *z, const float *vx,
                                    const float *vy, const float *vz, long Np, double V, int where,
                                    const double los[3], double aH, double dK, int Nmu, double *K, long *N,
                                    double *Pl, double *Kmu, long *Nmu_count, double *Pmu) {
    const float *vel[3] = {vx, vy, vz};
    return power_f32_run(grid, x, y, z, vel, aH, Np, V, where, los, dK, Nmu, K, N, Pl, Kmu, Nmu_count, Pmu);
}

extern "C" int fftgal_g2p_sum(fft_t *grid, const gal_t *pos, double *out) {
    if (!grid || !pos || !out) return set_error(ERR_ARG, "null argument");
    FG_TRY(enter(grid, true));
    return g2p_run(grid, pos, 1, out);
}

extern "C" long fftgal_launch_count(void) { return launch_count(); }

extern "C" long fftgal_device_bytes(fft_t *grid) {
    if (!grid) return 0;
    Grid *g = G(grid);
    long b = (long)g->prec * g->Ng3_pad * (g->d_aux ? 2 : 1);
    b += (long)g->pos_cap + (long)g->stage_cap + (long)g->scratch.bytes;
    return b;
}
