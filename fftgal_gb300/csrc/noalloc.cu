// fftgal_power_bins_noalloc: multipoles and wedges of a k-space grid that is
// already in GPU memory, for callers that cannot allocate GPU memory -- code
// running inside a host framework that owns every device allocation (a
// caching allocator, a memory pool shared with other work), or an embedding
// that has handed out all device memory in advance, where a cudaMalloc would
// fail or take memory the framework counts on.
//
// It is a variant of the binning kernels of bins.cu whose scratch (the
// per-bin sums, mode counts, k-bin thresholds and the normalised outputs) is
// one file-scope __device__ array of kNoAllocScratchBytes, held by every GPU
// that loads the library until the process exits.  The data-independent mode
// counts and mean |k| that bins.cu caches per geometry are accumulated here in
// the same pass instead.  Every call shares the array: the accumulators are
// cleared at the start of each call, and calls whose work overlaps on the GPU
// (other host threads, other streams) race on it.  The call waits for its
// stream (cudaStreamSynchronize) before it returns the tables.
//
// Limits: NK <= 2048 k bins (the fixed scratch), Nmu <= 16 wedges, and the
// per-CTA shared accumulators -- FP32 power sums [4 + Nmu + 1][NK], FP64 sums
// of |k| and u32 mode counts [Nmu + 1][NK], the k-bin thresholds [NK + 2] --
// must fit 220 KB: NK * (36 + 16 Nmu) + 8 <= 225280 bytes (NK <= 2048 up to
// Nmu = 5, NK <= 1149 at Nmu = 10, NK <= 771 at Nmu = 16).
#include "internal.h"
#include "common.cuh"
#include "binmath.cuh"

#include "fft.h"
#include "gal.h"
#include "fftgal_gb300.h"

#include <math.h>
#include <mutex>

namespace fg {

constexpr int kNaMaxNK = 2048;   // k bins
constexpr int kNaMaxNmu = 16;    // wedges
constexpr int kNaMaxW = kNaMaxNmu + 1;
constexpr int kNaThreads = 256;
constexpr int kNaChunkRows = 256;  // rows per chunk of FP32 sums
constexpr int kNaSegModes = 16;

// scratch layout for the largest call (bytes, each part 256-aligned)
constexpr size_t na_align(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kNaPsum = na_align(8ull * kNaMaxNK * (4 + kNaMaxW));   // FP64 power sums [4+W][NK]
constexpr size_t kNaKsum = na_align(8ull * kNaMaxNK * kNaMaxW);         // FP64 sum of |k| [W][NK]
constexpr size_t kNaCnt = na_align(8ull * kNaMaxNK * kNaMaxW);          // u64 mode counts [W][NK]
constexpr size_t kNaThr = na_align(4ull * (kNaMaxNK + 2));              // u32 n^2 thresholds
constexpr size_t kNaOut = na_align(8ull * kNaMaxNK * (6 + 3 * kNaMaxNmu));  // normalised outputs
constexpr size_t kNoAllocScratchBytes = kNaPsum + kNaKsum + kNaCnt + kNaThr + kNaOut;  // 1.8 MB

// shared accumulators of na_bin_kernel: NK * (36 + 16 Nmu) + 8 bytes
constexpr size_t kNaSmemMax = 220 * 1024;
constexpr size_t na_smem(int NK, int Nmu) {
    return (size_t)NK * (4 * (4 + Nmu + 1) + 12 * (Nmu + 1)) + 4 * (size_t)(NK + 2);
}

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// device address of g_noalloc_scratch per device (host code must not pass the
// symbol itself to a kernel: on the host it is only a stand-in)
static std::mutex g_na_mutex;
static void *g_na_ptr[64] = {};

static int noalloc_scratch(void **out) {
    int dev = 0;
    FG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_na_ptr[dev] = p;
    }
    *out = g_na_ptr[dev];
    return OK;
}

// thr[b] = smallest n^2 with floor(sqrt(n^2) * dKinv) >= b (src/power.c:58-59
// evaluated in FP64 without contraction); b = 0..NK+1
__global__ void na_thresholds_kernel(uint32_t *thr, int NK, double dKinv, uint32_t n2max) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > NK + 1) return;
    if (b == 0) {
        thr[0] = 0;
        return;
    }
    auto ik = [&](uint32_t n2) { return (int)floor(__dmul_rn(__dsqrt_rn((double)n2), dKinv)); };
    const double x = (double)b / dKinv;
    double s0 = floor(x * x) - 4.0;
    uint32_t n = s0 < 0 ? 0u : (s0 > (double)n2max ? n2max + 1 : (uint32_t)s0);
    for (int it = 0; it < 64 && n > 0 && n <= n2max && ik(n - 1) >= b; ++it) --n;
    for (int it = 0; it < 64 && n <= n2max && ik(n) < b; ++it) ++n;
    thr[b] = n;
}

// bins.cu's segment kernel (mode 1: P = |delta|^2 Vinv - Pshot) plus the
// per-(bin, wedge) mode counts and sums of |k| (double-float sqrt per mode).
// Shared memory holds FP32 power sums (added to the FP64 sums in the scratch
// after every chunk of rows), FP64 sums of |k| and u32 counts (added to the
// scratch once per CTA).
__global__ void __launch_bounds__(kNaThreads)
na_bin_kernel(BinDev d, const float *__restrict__ f, float Vinv, float Pshot, const uint32_t *__restrict__ thr_g,
              double *__restrict__ gP, double *__restrict__ gK, unsigned long long *__restrict__ gN, int Ng_pad) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int NK = d.NK, W = d.W, NQ = 4 + W;
    double *kacc = reinterpret_cast<double *>(smem_raw);                     // [W][NK]
    float *acc32 = reinterpret_cast<float *>(kacc + (size_t)NK * W);         // [NQ][NK]
    uint32_t *cnt = reinterpret_cast<uint32_t *>(acc32 + (size_t)NK * NQ);   // [W][NK]
    uint32_t *thr = cnt + (size_t)NK * W;                                     // [NK + 2]
    const int tid = threadIdx.x;
    for (int e = tid; e < NK * NQ; e += blockDim.x) acc32[e] = 0.f;
    for (int e = tid; e < NK * W; e += blockDim.x) {
        kacc[e] = 0;
        cnt[e] = 0;
    }
    for (int e = tid; e < NK + 2; e += blockDim.x) thr[e] = thr_g[e];
    __syncthreads();

    const int Ng = d.Ng, nh = d.nh;
    const int nrows = Ng * Ng;
    const int nsegr = (nh + kNaSegModes - 1) / kNaSegModes;
    const int nchunks = (nrows + kNaChunkRows - 1) / kNaChunkRows;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int r0 = ch * kNaChunkRows;
        const int nitems = (min(nrows, r0 + kNaChunkRows) - r0) * nsegr;
        for (int it = tid; it < nitems; it += blockDim.x) {
            const int row = r0 + it / nsegr, seg = it % nsegr;
            const int i = row / Ng, j = row - i * Ng;
            const int ki = kval(i, Ng), kj = kval(j, Ng);
            const int n2ij = ki * ki + kj * kj;
            const float2 *frow = reinterpret_cast<const float2 *>(f + (long)row * Ng_pad);
            int cb = -1, cm = -1, cw = -1;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, sw = 0.f;
            uint32_t rc = 0;
            double rk = 0;
            const int k1 = min(nh, (seg + 1) * kNaSegModes);
            for (int k = seg * kNaSegModes; k < k1; ++k) {
                if ((row | k) == 0) continue;  // the k = 0 mode (src/power.c:52-54)
                const int kk = kval(k, Ng);
                const uint32_t n2 = (uint32_t)(n2ij + kk * kk);
                const float2 v = frow[k];
                const float p = (v.x * v.x + v.y * v.y) * Vinv - Pshot;
                const uint32_t count = (k != 0 && 2 * k != Ng) ? 2u : 1u;
                const float pc = count == 2u ? 2.f * p : p;
                const float n2f = (float)n2;
                const float rsq = rsqrtf(n2f);
                int b = kbin_est(n2, n2f * rsq, thr, NK, d.dKinv_f);
                if (b >= NK) b = -1;
                float m2;
                const int imu = wedge_index_r(ki, kj, kk, rsq, d, m2);
                // sqrt(n2) to ~1e-14 as a float pair
                const float sq = sqrtf(n2f);
                const float sq_lo = fmaf(-sq, sq, n2f) / (2.f * sq);
                const int wk = b < 0 ? -1 : b * W + imu;
                if (b != cb) {
                    if (cb >= 0) {
                        atomicAdd(acc32 + 0 * NK + cb, s0);
                        atomicAdd(acc32 + 1 * NK + cb, s1);
                        atomicAdd(acc32 + 2 * NK + cb, s2);
                        atomicAdd(acc32 + 3 * NK + cb, s3);
                    }
                    cb = b;
                    s0 = s1 = s2 = s3 = 0.f;
                }
                if (wk != cw) {
                    if (cw >= 0) {
                        atomicAdd(acc32 + (4 + cm) * NK + cw / W, sw);
                        atomicAdd(kacc + (size_t)cm * NK + cw / W, rk);
                        atomicAdd(cnt + (size_t)cm * NK + cw / W, rc);
                    }
                    cw = wk;
                    cm = imu;
                    sw = 0.f;
                    rk = 0;
                    rc = 0;
                }
                s0 += pc;
                s1 += pc * (1.5f * m2 - 0.5f);
                s2 += pc * ((4.375f * m2 - 3.75f) * m2 + 0.375f);
                s3 += pc * (((14.4375f * m2 - 19.6875f) * m2 + 6.5625f) * m2 - 0.3125f);
                sw += pc;
                rc += count;
                rk += (double)count * ((double)sq + (double)sq_lo);
            }
            if (cb >= 0) {
                atomicAdd(acc32 + 0 * NK + cb, s0);
                atomicAdd(acc32 + 1 * NK + cb, s1);
                atomicAdd(acc32 + 2 * NK + cb, s2);
                atomicAdd(acc32 + 3 * NK + cb, s3);
            }
            if (cw >= 0) {
                atomicAdd(acc32 + (4 + cm) * NK + cw / W, sw);
                atomicAdd(kacc + (size_t)cm * NK + cw / W, rk);
                atomicAdd(cnt + (size_t)cm * NK + cw / W, rc);
            }
        }
        __syncthreads();
        // the chunk's FP32 sums into the FP64 sums of the scratch
        for (int e = tid; e < NK * NQ; e += blockDim.x) {
            const float v = acc32[e];
            if (v != 0.f) atomicAdd(&gP[e], (double)v);
            acc32[e] = 0.f;
        }
        __syncthreads();
    }
    for (int e = tid; e < NK * W; e += blockDim.x) {
        if (kacc[e] != 0) atomicAdd(&gK[e], kacc[e]);
        if (cnt[e] != 0) atomicAdd(&gN[e], (unsigned long long)cnt[e]);
    }
}

// normalisation of src/power.c:69-76 (multipoles) and 139-153 (wedges);
// out = K[NK] | N[NK] | Pl[NK*4] | Kmu[NK*Nmu] | Nmu[NK*Nmu] | Pmu[NK*Nmu]
__global__ void na_finalize_kernel(int NK, int Nmu, double KF, const double *__restrict__ gP,
                                   const double *__restrict__ gK, const unsigned long long *__restrict__ gN,
                                   double *out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= NK) return;
    const int W = Nmu + 1;
    double *K = out, *Pl = out + 2 * (size_t)NK, *Kmu = Pl + 4 * (size_t)NK;
    long long *N = reinterpret_cast<long long *>(out + NK);
    long long *Nm = reinterpret_cast<long long *>(Kmu + (size_t)NK * Nmu);
    double *Pm = Kmu + 2 * (size_t)NK * Nmu;
    long long n = 0;
    double ks = 0;
    for (int m = 0; m < W; ++m) {
        n += (long long)gN[(size_t)m * NK + b];
        ks = __dadd_rn(ks, gK[(size_t)m * NK + b]);
    }
    K[b] = __dmul_rn(ks, __ddiv_rn(KF, (double)n));
    N[b] = n;
    for (int l = 0; l < 4; ++l)
        Pl[(size_t)b * 4 + l] = __dmul_rn(gP[(size_t)l * NK + b], __ddiv_rn(4 * l + 1.0, (double)n));
    for (int m = 0; m < Nmu; ++m) {
        double kk = gK[(size_t)m * NK + b], pp = gP[(size_t)(4 + m) * NK + b];
        long long nn = (long long)gN[(size_t)m * NK + b];
        if (m == Nmu - 1) {  // the mu = 1 slot joins the last wedge (src/power.c:139-143)
            kk = __dadd_rn(kk, gK[(size_t)Nmu * NK + b]);
            pp = __dadd_rn(pp, gP[(size_t)(4 + Nmu) * NK + b]);
            nn += (long long)gN[(size_t)Nmu * NK + b];
        }
        if (nn) {
            kk = __dmul_rn(kk, __ddiv_rn(KF, (double)nn));
            pp = __ddiv_rn(pp, (double)nn);
        }
        Kmu[(size_t)b * Nmu + m] = kk;
        Nm[(size_t)b * Nmu + m] = nn;
        Pm[(size_t)b * Nmu + m] = pp;
    }
}

static int noalloc_run(const float *fk, int Ng, double L, double V, long Np, const double los_in[3], double dK,
                       int Nmu, double *K, long *N, double *Pl, double *Kmu, long *Nmu_count, double *Pmu,
                       cudaStream_t st) {
    if (!fk || Ng < 2 || Ng > 4096 || !(L > 0) || !(V > 0) || Np <= 0 || !(dK > 0))
        return set_error(ERR_ARG, "fftgal_power_bins_noalloc: bad arguments");
    if (Nmu < 1 || Nmu > kNaMaxNmu) return set_error(ERR_ARG, "Nmu must be in [1, %d]", kNaMaxNmu);
    double los[3] = {los_in[0], los_in[1], los_in[2]};
    hat(los);
    BinSpec s;
    FG_TRY(bin_spec_init(&s, Ng, L, dK, los, Nmu));
    const int NK = s.NK, W = Nmu + 1, NQ = 4 + W;
    if (NK > kNaMaxNK)
        return set_error(ERR_RANGE, "fftgal_power_bins_noalloc: NK = %d k bins exceed the %d of its fixed scratch",
                         NK, kNaMaxNK);
    const uint32_t h = Ng / 2, n2max = 3u * h * h;
    if ((int)floor(sqrt((double)n2max) * s.dKinv) >= NK)
        return set_error(ERR_RANGE, "a mode falls beyond the last of NK=%d k bins", NK);
    const size_t smem = na_smem(NK, Nmu);
    if (smem > kNaSmemMax)
        return set_error(ERR_UNSUPPORTED,
                         "fftgal_power_bins_noalloc: NK = %d k bins x Nmu = %d wedges need %zu bytes of shared "
                         "accumulators, more than %zu (NK * (36 + 16 Nmu) + 8)",
                         NK, Nmu, smem, kNaSmemMax);
    void *base = nullptr;
    FG_TRY(noalloc_scratch(&base));
    unsigned char *p = static_cast<unsigned char *>(base);
    double *gP = reinterpret_cast<double *>(p);
    double *gK = reinterpret_cast<double *>(p + kNaPsum);
    unsigned long long *gN = reinterpret_cast<unsigned long long *>(p + kNaPsum + kNaKsum);
    uint32_t *thr = reinterpret_cast<uint32_t *>(p + kNaPsum + kNaKsum + kNaCnt);
    double *out = reinterpret_cast<double *>(p + kNaPsum + kNaKsum + kNaCnt + kNaThr);
    // the previous call's sums are still there: clear what accumulates
    FG_CUDA(cudaMemsetAsync(gP, 0, 8 * (size_t)NK * NQ, st));
    FG_CUDA(cudaMemsetAsync(gK, 0, 8 * (size_t)NK * W, st));
    FG_CUDA(cudaMemsetAsync(gN, 0, 8 * (size_t)NK * W, st));
    na_thresholds_kernel<<<(unsigned)ceil_div(NK + 2, 128), 128, 0, st>>>(thr, NK, s.dKinv, n2max);
    FG_LAUNCHED(1);
    const BinDev d = make_dev(s);
    FG_CUDA(cudaFuncSetAttribute(na_bin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = (int)((220 * 1024) / smem);
    per_sm = per_sm < 1 ? 1 : (per_sm > 8 ? 8 : per_sm);
    long nb = (long)num_sms() * per_sm;
    const long nchunks = ceil_div((long)Ng * Ng, kNaChunkRows);
    if (nb > nchunks) nb = nchunks;
    na_bin_kernel<<<(unsigned)nb, kNaThreads, smem, st>>>(d, fk, (float)(1 / V), (float)(V / Np), thr, gP, gK, gN,
                                                         2 * (Ng / 2 + 1));
    FG_LAUNCHED(1);
    na_finalize_kernel<<<(unsigned)ceil_div(NK, 128), 128, 0, st>>>(NK, Nmu, s.KF, gP, gK, gN, out);
    FG_LAUNCHED(1);
    const size_t nk = NK, nm = (size_t)NK * Nmu;
    double *oK = out, *oPl = out + 2 * nk, *oKm = oPl + 4 * nk, *oPm = oKm + 2 * nm;
    const double *oN = out + nk, *oNm = oKm + nm;
    if (K) FG_CUDA(cudaMemcpyAsync(K, oK, 8 * nk, cudaMemcpyDeviceToHost, st));
    if (N) FG_CUDA(cudaMemcpyAsync(N, oN, 8 * nk, cudaMemcpyDeviceToHost, st));
    if (Pl) FG_CUDA(cudaMemcpyAsync(Pl, oPl, 8 * 4 * nk, cudaMemcpyDeviceToHost, st));
    if (Kmu) FG_CUDA(cudaMemcpyAsync(Kmu, oKm, 8 * nm, cudaMemcpyDeviceToHost, st));
    if (Nmu_count) FG_CUDA(cudaMemcpyAsync(Nmu_count, oNm, 8 * nm, cudaMemcpyDeviceToHost, st));
    if (Pmu) FG_CUDA(cudaMemcpyAsync(Pmu, oPm, 8 * nm, cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (N) {
        long tot = 0;
        for (int b = 0; b < NK; ++b) tot += N[b];
        if (tot != (long)Ng * Ng * Ng - 1) return set_error(ERR_RANGE, "mode count %ld != Ng^3-1", tot);
    }
    return OK;
}

}  // namespace fg

extern "C" int fftgal_power_bins_noalloc(const float *fk, int Ng, double L, double V, long Np, const double los[3],
                                         double dK, int Nmu, double *K, long *N, double *Pl, double *Kmu,
                                         long *Nmu_count, double *Pmu, void *stream) {
    return fg::noalloc_run(fk, Ng, L, V, Np, los, dK, Nmu, K, N, Pl, Kmu, Nmu_count, Pmu,
                           static_cast<cudaStream_t>(stream));
}
