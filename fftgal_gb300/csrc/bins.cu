// k-shell binning of the half spectrum for sm_103a: multipoles l = 0,2,4,6
// (src/power.c:30-101) and mu wedges (src/power.c:104-178) in one pass.
//
// Mode classification is exact with respect to the reference's FP64 code:
//  * the k bin iK = floor(sqrt(n2) * dKinv) depends only on the integer
//    n2 = kx^2 + ky^2 + kz^2, so the host evaluates the reference expression
//    once per n2 and ships the bin thresholds; the kernel finds iK from an FP32
//    estimate corrected against those exact thresholds;
//  * the wedge imu = floor(|mu * Nmu|) is estimated in FP32 and, only when the
//    estimate lies within its error bound of a wedge edge, re-evaluated in FP64
//    with the reference's operation order (explicitly rounded, no FMA).
// Mode counts N and the mean |k| per bin do not depend on the data: they are
// built once per (Ng, L, dK, los, Nmu) from an exact (n2, imu) multiplicity
// histogram and cached; every catalog then only accumulates power sums.
// Power sums: per-warp segmented reductions over runs of equal bins, FP32
// shared-memory accumulators flushed every chunk of rows into FP64 shared
// accumulators, FP64 global atomics once per CTA.
#include "internal.h"
#include "common.cuh"
#include "binmath.cuh"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

namespace fg {

constexpr double kSqrt3 = 1.73205080756887729352744634151;

int bin_spec_init(BinSpec *b, int Ng, double L, double dK, const double los_hat[3], int Nmu) {
    if (!(dK > 0) || !(L > 0)) return set_error(ERR_ARG, "dK and L must be > 0");
    if (Nmu < 1 || Nmu > 64) return set_error(ERR_ARG, "Nmu must be in [1, 64]");
    b->Ng = Ng;
    b->L = L;
    b->dK = dK;
    for (int a = 0; a < 3; ++a) b->los[a] = los_hat[a];
    b->Nmu = Nmu;
    b->KF = 2 * M_PI / L;
    b->dKinv = b->KF / dK;
    // src/power.c:34-36
    b->NK = (int)floor(kSqrt3 * (Ng / 2) * b->dKinv) + 1;
    if (b->NK < 1 || b->NK > (1 << 20)) return set_error(ERR_ARG, "NK = %d out of range", b->NK);
    return OK;
}

// ---- geometry: exact (n2, imu) multiplicities -----------------------------------------------
__global__ void geometry_kernel(BinDev d, uint32_t *__restrict__ hist) {
    const long n = (long)d.Ng * d.Ng * d.nh;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        if (e == 0) continue;  // the k = 0 mode is skipped (src/power.c:52-54)
        const int k = (int)(e % d.nh);
        const long row = e / d.nh;
        const int j = (int)(row % d.Ng), i = (int)(row / d.Ng);
        const int ki = kval(i, d.Ng), kj = kval(j, d.Ng), kk = kval(k, d.Ng);
        const uint32_t n2 = (uint32_t)(ki * ki + kj * kj + kk * kk);
        const uint32_t count = 1 + ((2 * k) % d.Ng > 0);
        float mu2;
        const int imu = wedge_index(ki, kj, kk, sqrtf((float)n2), d, mu2);
        atomicAdd(&hist[(size_t)n2 * d.W + imu], count);
    }
}

void bin_geometry_free(BinGeometry *g) {
    delete[] g->N;
    delete[] g->K;
    delete[] g->Nw;
    delete[] g->Kw;
    cudaFree(g->d_thr);
    cudaFree(g->d_acc);
    *g = BinGeometry();
}

int bin_geometry_build(BinGeometry *g, const BinSpec &s, cudaStream_t st) {
    bin_geometry_free(g);
    g->spec = s;
    const int Ng = s.Ng, NK = s.NK, W = s.Nmu + 1;
    const int h = Ng / 2;
    const uint32_t n2max = (uint32_t)(3L * h * h);
    // exact k-bin thresholds from the reference expression floor(sqrt(n2) * dKinv)
    std::vector<uint32_t> thr(NK + 2, n2max + 1);
    std::vector<int> ik(n2max + 1);
    for (uint32_t n2 = 0; n2 <= n2max; ++n2) {
        volatile double kamp = sqrt((double)n2);
        volatile double t = kamp * s.dKinv;
        ik[n2] = (int)floor(t);
    }
    thr[0] = 0;
    {
        int b = 1;
        for (uint32_t n2 = 0; n2 <= n2max && b <= NK; ++n2)
            while (b <= NK && ik[n2] >= b) thr[b++] = n2;
    }
    FG_CUDA(cudaMalloc(&g->d_thr, sizeof(uint32_t) * (NK + 2)));
    FG_CUDA(cudaMemcpyAsync(g->d_thr, thr.data(), sizeof(uint32_t) * (NK + 2), cudaMemcpyHostToDevice, st));
    // multiplicity histogram over (n2, imu)
    const size_t hlen = (size_t)(n2max + 1) * W;
    uint32_t *d_hist = nullptr;
    FG_CUDA(cudaMalloc(&d_hist, sizeof(uint32_t) * hlen));
    FG_CUDA(cudaMemsetAsync(d_hist, 0, sizeof(uint32_t) * hlen, st));
    const BinDev d = make_dev(s);
    const long nmodes = (long)Ng * Ng * (h + 1);
    long nb = ceil_div(nmodes, 256);
    if (nb > 64L * num_sms()) nb = 64L * num_sms();
    geometry_kernel<<<(unsigned)nb, 256, 0, st>>>(d, d_hist);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    std::vector<uint32_t> hh(hlen);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hh.data(), d_hist, sizeof(uint32_t) * hlen, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_hist);
    if (e != cudaSuccess) return cuda_check(e, "geometry histogram");
    g->N = new long[NK]();
    g->K = new double[NK]();
    g->Nw = new long[(size_t)NK * W]();
    g->Kw = new double[(size_t)NK * W]();
    g->bad = 0;
    for (uint32_t n2 = 1; n2 <= n2max; ++n2) {
        const uint32_t *row = &hh[(size_t)n2 * W];
        long tot = 0;
        for (int m = 0; m < W; ++m) tot += row[m];
        if (!tot) continue;
        const int b = ik[n2];
        if (b < 0 || b >= NK) {
            g->bad = 1;
            continue;
        }
        const double kamp = sqrt((double)n2);
        g->N[b] += tot;
        g->K[b] += (double)tot * kamp;
        for (int m = 0; m < W; ++m)
            if (row[m]) {
                g->Nw[(size_t)b * W + m] += row[m];
                g->Kw[(size_t)b * W + m] += (double)row[m] * kamp;
            }
    }
    g->acc_len = (size_t)NK * (4 + W);
    FG_CUDA(cudaMalloc(&g->d_acc, sizeof(double) * g->acc_len));
    g->valid = true;
    return OK;
}

// ---- power sums ---------------------------------------------------------------------------------

constexpr int kBinThreads = 256;
constexpr int kChunkRows = 64;

// inclusive segmented sum over runs of equal `key` within the warp; returns
// true on the last lane of each run (which then owns the run's sum)
template <int NV>
__device__ __forceinline__ bool warp_segsum(int key, float (&v)[NV], int lane) {
    const unsigned full = 0xffffffffu;
    const int kprev = __shfl_up_sync(full, key, 1);
    const bool head = lane == 0 || kprev != key;
    const unsigned hm = __ballot_sync(full, head);
    const int seg = __popc(hm & (0xffffffffu >> (31 - lane)));
    if (hm != 1u) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int sseg = __shfl_up_sync(full, seg, o);
            float t[NV];
#pragma unroll
            for (int q = 0; q < NV; ++q) t[q] = __shfl_up_sync(full, v[q], o);
            if (lane >= o && sseg == seg) {
#pragma unroll
                for (int q = 0; q < NV; ++q) v[q] += t[q];
            }
        }
        const int snext = __shfl_down_sync(full, seg, 1);
        return lane == 31 || snext != seg;
    }
    // a single run: butterfly reduction, lane 31 owns the total
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] += __shfl_xor_sync(full, v[q], o);
    return lane == 31;
}

// One warp walks one k row (fixed i, j) at a time, 32 modes per step, so the
// k bin is non-decreasing along the step and the row constants are computed
// once.  The CTA advances through chunks of kChunkRows rows and folds its FP32
// partial sums into FP64 after each chunk.
template <typename T, int MODE>
__global__ void __launch_bounds__(kBinThreads)
bin_power_kernel(BinDev d, const T *__restrict__ f, T Vinv, T Pshot,
                 const uint32_t *__restrict__ thr_g, double *__restrict__ gacc, int Ng_pad) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int NK = d.NK, W = d.W, NQ = 4 + W;
    double *acc64 = reinterpret_cast<double *>(smem_raw);               // [NK * NQ]
    float *acc32 = reinterpret_cast<float *>(acc64 + (size_t)NK * NQ);  // [NK * NQ] (FP32 grids)
    uint32_t *thr = reinterpret_cast<uint32_t *>(acc32 + (sizeof(T) == 4 ? (size_t)NK * NQ : 0));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int e = tid; e < NK * NQ; e += blockDim.x) {
        acc64[e] = 0;
        if constexpr (sizeof(T) == 4) acc32[e] = 0.f;
    }
    for (int e = tid; e < NK + 2; e += blockDim.x) thr[e] = thr_g[e];
    __syncthreads();

    const int Ng = d.Ng, nh = d.nh;
    const int nrows = Ng * Ng;
    const int nchunks = (nrows + kChunkRows - 1) / kChunkRows;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int r1 = min(nrows, (ch + 1) * kChunkRows);
        for (int row = ch * kChunkRows + warp; row < r1; row += nwarp) {
            const int i = row / Ng, j = row - i * Ng;
            const int ki = kval(i, Ng), kj = kval(j, Ng);
            const int n2ij = ki * ki + kj * kj;
            const T *frow = f + (long)row * Ng_pad;
            for (int k0 = 0; k0 < nh; k0 += 32) {
                const int k = k0 + lane;
                int b = -1, imu = 0;
                T pc = 0, mu2t = 0;
                if (k < nh && (row | k) != 0) {
                    const int kk = kval(k, Ng);
                    const uint32_t n2 = (uint32_t)(n2ij + kk * kk);
                    const int count = 1 + ((2 * k) % Ng > 0);
                    T p;
                    if constexpr (MODE == 0) {
                        p = frow[2 * k];
                    } else {
                        const T2 v = reinterpret_cast<const T2 *>(frow)[k];
                        if constexpr (sizeof(T) == 8)
                            p = __dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), Vinv), Pshot);
                        else
                            p = (v.x * v.x + v.y * v.y) * Vinv - Pshot;
                    }
                    pc = p * (T)count;
                    b = kbin(n2, thr, NK, d.dKinv_f);
                    if (b >= NK) b = -1;
                    float mu2f;
                    imu = wedge_index(ki, kj, kk, sqrtf((float)n2), d, mu2f);
                    if constexpr (sizeof(T) == 8) {
                        if (!d.zero_los) {
                            const double kamp = __dsqrt_rn((double)n2);
                            const double num = __dadd_rn(__dadd_rn(__dmul_rn((double)ki, d.l0), __dmul_rn((double)kj, d.l1)),
                                                         __dmul_rn((double)kk, d.l2));
                            const double mu = __ddiv_rn(num, kamp);
                            mu2t = __dmul_rn(mu, mu);
                        }
                    } else {
                        mu2t = mu2f;
                    }
                }
                if constexpr (sizeof(T) == 8) {
                    if (b >= 0) {
                        const double m2 = mu2t;
                        double *a = acc64 + (size_t)b * NQ;
                        atomicAdd(a + 0, pc);
                        atomicAdd(a + 1, pc * (1.5 * m2 - 0.5));
                        atomicAdd(a + 2, pc * ((4.375 * m2 - 3.75) * m2 + 0.375));
                        atomicAdd(a + 3, pc * (((14.4375 * m2 - 19.6875) * m2 + 6.5625) * m2 - 0.3125));
                        atomicAdd(a + 4 + imu, pc);
                    }
                } else {
                    const float m2 = mu2t;
                    float v[4] = {pc, pc * (1.5f * m2 - 0.5f), pc * ((4.375f * m2 - 3.75f) * m2 + 0.375f),
                                  pc * (((14.4375f * m2 - 19.6875f) * m2 + 6.5625f) * m2 - 0.3125f)};
                    if (warp_segsum<4>(b, v, lane) && b >= 0) {
                        float *a = acc32 + (size_t)b * NQ;
                        atomicAdd(a + 0, v[0]);
                        atomicAdd(a + 1, v[1]);
                        atomicAdd(a + 2, v[2]);
                        atomicAdd(a + 3, v[3]);
                    }
                    float w[1] = {pc};
                    const int wkey = b < 0 ? -1 : b * W + imu;
                    if (warp_segsum<1>(wkey, w, lane) && wkey >= 0) atomicAdd(acc32 + (size_t)b * NQ + 4 + imu, w[0]);
                }
            }
        }
        if constexpr (sizeof(T) == 4) {
            __syncthreads();
            for (int e = tid; e < NK * NQ; e += blockDim.x) {
                acc64[e] += (double)acc32[e];
                acc32[e] = 0.f;
            }
            __syncthreads();
        }
    }
    __syncthreads();
    for (int e = tid; e < NK * NQ; e += blockDim.x)
        if (acc64[e] != 0) atomicAdd(&gacc[e], acc64[e]);
}

// FP32 grids.  The half spectrum is cut into blocks of 16 (i) x 16 (j) x 32
// (k) modes.  Each warp of a CTA stages one 16 x 32 slab of the block (16
// rows of 32 consecutive k, from coalesced loads) as FP32 powers in shared
// memory, then walks the slab in runs of 16 modes along the grid axis whose
// |n_a| is smallest at the block's centre: along that axis |n| changes
// slowest, so a run crosses the fewest k-bin edges (about 0.3 per mode,
// against 0.55 along a fixed axis).  A thread keeps the run's sums in
// registers and adds them to the CTA's FP32 shared accumulators when the bin
// (or the wedge) changes; every `fold` blocks the CTA adds its FP32
// sums to the FP64 global accumulators.
//   MODE 0: the grid holds P in F_Re (after P()).
//   MODE 1: the grid holds delta; P = |delta|^2 Vinv - Pshot.
//   MODE 2: as 1, with the interlacing finish of the grid fused in: A <-
//           (A + B * phase) * W^-1 * scale is written back and binned.
//   MODE 3: as 2 without an interlacing grid: A <- A * W^-1 * scale (the
//           deconvolution of a single paint, src/fft.c:236-254).
//   MODE 4: as 3 with the deconvolved value binned but not written back.
//   MODE 5: as 2 with the finished value binned but not written back (the
//           fused calls under the lazy host view: 4.3 GB fewer writes at
//           Ng = 1024).
constexpr int kSlabI = 16, kSlabJ = 16, kSlabK = 32, kSlabRow = 33;
constexpr int kSlabThreads = 512;  // one warp per slab of a block
// blocks between folds of the FP32 sums into FP64: FFTGAL_BIN_FOLD, default 8
static int fold_blocks() {
    static const int v = [] {
        const char *e = getenv("FFTGAL_BIN_FOLD");
        const int n = e ? atoi(e) : 0;
        return n >= 1 && n <= 1024 ? n : 8;
    }();
    return v;
}

struct SlabFinish {
    float2 *A = nullptr;
    const float2 *B = nullptr;
    const float2 *ph = nullptr;  // [3][Ng] phase of the interlacing grid (FP32)
    const float *w = nullptr;    // [Ng] PCS window inverse (FP32)
    float scale = 0.f;           // H^3 / 2
};

// The slab blocks cover k < kmain.  When the half spectrum's last k block
// would hold only one or two columns (nh = Ng/2 + 1: the Nyquist column of
// every even Ng that is a multiple of 32), those columns are binned mode by
// mode after the blocks instead, by all threads of the grid, rather than as
// 32-column blocks with one or two columns used (6 % of the lane slots at
// Ng = 1024).
__host__ __device__ __forceinline__ int slab_kmain(int nh) {
    const int r = nh % kSlabK;
    return (nh > kSlabK && r > 0 && r <= 2) ? nh - r : nh;
}

// |delta|^2 Vinv - Pshot of element e.  MODE 2 to 5 finish it first, with the
// phase pf * phr (MODE 2 and 5) and the window inverse wf * wr; MODE 2 and 3
// store the finished value.
template <int MODE>
__device__ __forceinline__ float mode_power(const SlabFinish &fin, const float2 *__restrict__ f, long e, float2 pf,
                                           float2 phr, float wf, float wr, float Vinv, float Pshot) {
    if (MODE == 2 || MODE == 5) {
        const float2 p = cmul(pf, phr);
        const float wk = wf * wr;
        const float2 bv = fin.B[e], av = fin.A[e];
        const float2 dv = cmul(bv, p);
        const float2 v = make_float2((dv.x + av.x) * wk, (dv.y + av.y) * wk);
        if (MODE == 2) fin.A[e] = v;
        return (v.x * v.x + v.y * v.y) * Vinv - Pshot;
    } else if (MODE == 3 || MODE == 4) {
        const float wk = wf * wr;
        const float2 av = fin.A[e];
        const float2 v = make_float2(av.x * wk, av.y * wk);
        if (MODE == 3) fin.A[e] = v;
        return (v.x * v.x + v.y * v.y) * Vinv - Pshot;
    } else if (MODE == 1) {
        const float2 v = f[e];
        return (v.x * v.x + v.y * v.y) * Vinv - Pshot;
    } else {
        return f[e].x;
    }
}

// MINB: CTAs per SM the registers are budgeted for (3: 40 registers with a
// few spills, 2: no spills), chosen by the CTAs per SM that the launch's
// shared memory allows and the tuned launch shape
template <int MODE, int MINB>
__global__ void __launch_bounds__(kSlabThreads, MINB)
bin_power_slab_kernel(BinDev d, const float2 *__restrict__ f, SlabFinish fin, float Vinv, float Pshot,
                      const uint32_t *__restrict__ thr_g, double *__restrict__ gacc, const DevScalars *__restrict__ ds,
                      int fold) {
    if (ds) {
        Vinv = ds->Vinv;
        Pshot = ds->Pshot;
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int NK = d.NK, W = d.W, NQ = 4 + W;
    float *acc32 = reinterpret_cast<float *>(smem_raw);                        // [NQ][NK]
    uint32_t *thr = reinterpret_cast<uint32_t *>(acc32 + (size_t)NK * NQ);     // [NK + 2]
    float *slabs = reinterpret_cast<float *>(thr + ((NK + 2 + 3) & ~3));        // [16][16][kSlabRow]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *slab = slabs + warp * kSlabJ * kSlabRow;
    for (int e = tid; e < NK * NQ; e += blockDim.x) acc32[e] = 0.f;
    for (int e = tid; e < NK + 2; e += blockDim.x) thr[e] = thr_g[e];
    __syncthreads();
    const int Ng = d.Ng, nh = d.nh, kmain = slab_kmain(nh);
    const int nbi = (Ng + kSlabI - 1) / kSlabI, nbj = (Ng + kSlabJ - 1) / kSlabJ, nbk = (kmain + kSlabK - 1) / kSlabK;
    const int nblk = nbi * nbj * nbk;
    int since_fold = 0;
    for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const int bk = blk % nbk, bj = (blk / nbk) % nbj, bi = blk / (nbk * nbj);
        const int i0 = bi * kSlabI, j0 = bj * kSlabJ, k0 = bk * kSlabK;
        const int ci = abs(kval(min(i0 + kSlabI / 2, Ng - 1), Ng));
        const int cj = abs(kval(min(j0 + kSlabJ / 2, Ng - 1), Ng));
        const int ck = min(k0 + kSlabK / 2, nh - 1);
        const int axis = (ck <= ci && ck <= cj) ? 2 : (cj <= ci ? 1 : 0);  // run axis
        // the warp's slab: for runs along i it fixes j and its rows are i,
        // otherwise it fixes i and its rows are j
        const bool rows_i = axis == 0;
        const int fixed = (rows_i ? j0 : i0) + warp;
        const int r0 = rows_i ? i0 : j0;
        const int k = k0 + lane;
        if (fixed < Ng) {
            float2 pfk = make_float2(0.f, 0.f);
            float wfk = 0.f;
            if (MODE >= 2 && k < kmain) {
                if (MODE == 2 || MODE == 5) pfk = cmul(fin.ph[(rows_i ? Ng : 0) + fixed], fin.ph[2 * Ng + k]);
                wfk = fin.w[fixed] * fin.w[k] * fin.scale;
            }
            // the row tables of the slab's 16 rows: lane r holds row r's, the
            // loop takes them by shuffle
            float2 phl = make_float2(0.f, 0.f);
            float wl = 0.f;
            if (MODE >= 2 && lane < kSlabJ && r0 + lane < Ng) {
                if (MODE == 2 || MODE == 5) phl = fin.ph[(rows_i ? 0 : Ng) + r0 + lane];
                wl = fin.w[r0 + lane];
            }
            const long estep = rows_i ? (long)Ng * nh : (long)nh;  // elements between consecutive rows
            long e = (rows_i ? ((long)r0 * Ng + fixed) : ((long)fixed * Ng + r0)) * nh + k;
#pragma unroll 8
            for (int r = 0; r < kSlabJ; ++r, e += estep) {
                float2 phr = make_float2(0.f, 0.f);
                float wr = 0.f;
                if (MODE == 2 || MODE == 5) {
                    phr.x = __shfl_sync(0xffffffffu, phl.x, r);
                    phr.y = __shfl_sync(0xffffffffu, phl.y, r);
                }
                if (MODE >= 2) wr = __shfl_sync(0xffffffffu, wl, r);
                float pv = 0.f;
                if (r0 + r < Ng && k < kmain) pv = mode_power<MODE>(fin, f, e, pfk, phr, wfk, wr, Vinv, Pshot);
                slab[r * kSlabRow + lane] = pv;
            }
        }
        __syncwarp();
        if (fixed < Ng) {
            // runs along k: lane = (row, half of the 32 k); else lane = k
            if (axis == 2) {
                const int r = lane & 15, c = 16 * (lane >> 4), rr = r0 + r, kc = k0 + c;
                const int n = rr < Ng ? min(16, kmain - kc) : 0;
                bin_run<2>(d, thr, acc32, fixed, rr, kc, n, slab + r * kSlabRow + c, 1);
            } else {
                const int kc = k0 + lane;
                const int n = kc < kmain ? min(16, Ng - r0) : 0;
                if (axis == 1)
                    bin_run<1>(d, thr, acc32, fixed, r0, kc, n, slab + lane, kSlabRow);
                else
                    bin_run<0>(d, thr, acc32, r0, fixed, kc, n, slab + lane, kSlabRow);
            }
        }
        __syncwarp();
        if (++since_fold == fold) {
            since_fold = 0;
            __syncthreads();
            bin_fold(acc32, gacc, NK, NQ);
            __syncthreads();
        }
    }
    // the columns k >= kmain, one mode per thread (consecutive threads take
    // consecutive j; the finish takes the phase and window products in the
    // order of the blocks that run along i)
    if (kmain < nh) {
        const int ncol = nh - kmain;
        const long nplane = (long)ncol * Ng * Ng;
        for (long m = (long)blockIdx.x * blockDim.x + tid; m < nplane; m += (long)gridDim.x * blockDim.x) {
            const int kc = kmain + (int)(m % ncol);
            const long ij = m / ncol;
            const int j = (int)(ij % Ng), i = (int)(ij / Ng);
            const long e = ((long)i * Ng + j) * nh + kc;
            float2 pf = make_float2(0.f, 0.f), phr = make_float2(0.f, 0.f);
            float wf = 0.f, wr = 0.f;
            if (MODE == 2 || MODE == 5) {
                pf = cmul(fin.ph[Ng + j], fin.ph[2 * Ng + kc]);
                phr = fin.ph[i];
            }
            if (MODE >= 2) {
                wf = fin.w[j] * fin.w[kc] * fin.scale;
                wr = fin.w[i];
            }
            const float pv = mode_power<MODE>(fin, f, e, pf, phr, wf, wr, Vinv, Pshot);
            BinRun run;
            run.add(d, thr, acc32, kval(i, Ng), kval(j, Ng), kval(kc, Ng), kc, pv);
            run.finish(d, acc32);
        }
    }
    __syncthreads();
    for (int e = tid; e < NK * NQ; e += blockDim.x) {
        const float v = acc32[e];
        if (v != 0.f) {
            const int q = e / NK, b = e - q * NK;
            atomicAdd(&gacc[(size_t)b * NQ + q], (double)v);
        }
    }
}

static size_t slab_smem(int NK, int NQ) {
    return sizeof(float) * (size_t)NK * NQ + sizeof(uint32_t) * (size_t)((NK + 2 + 3) & ~3) +
           sizeof(float) * (kSlabThreads / 32) * kSlabJ * kSlabRow;
}

static int bin_launch(BinGeometry *g, const void *f, int prec, int mode, double Vinv, double Pshot, cudaStream_t st,
                      const BinFinish *fin, const DevScalars *ds);

void bin_power_unpack(const BinGeometry *g, const double *h, double *Psum, double *Pw) {
    const int NK = g->spec.NK, W = g->spec.Nmu + 1, NQ = 4 + W;
    for (int b = 0; b < NK; ++b) {
        for (int l = 0; l < 4; ++l) Psum[b * 4 + l] = h[(size_t)b * NQ + l];
        for (int m = 0; m < W; ++m) Pw[(size_t)b * W + m] = h[(size_t)b * NQ + 4 + m];
    }
}

int bin_power_launch(BinGeometry *g, int mode, double Vinv, double Pshot, cudaStream_t st, const BinFinish *fin,
                     const DevScalars *ds) {
    if (mode < 2 || mode > 5) return set_error(ERR_ARG, "bin_power_launch: modes 2 to 5 only");
    return bin_launch(g, nullptr, 4, mode, Vinv, Pshot, st, fin, ds);
}

int bin_power(BinGeometry *g, const void *f, int prec, int mode, double Vinv, double Pshot,
              double *Psum, double *Pw, cudaStream_t st, cudaEvent_t *ev_end, const BinFinish *fin) {
    FG_TRY(bin_launch(g, f, prec, mode, Vinv, Pshot, st, fin, nullptr));
    if (ev_end) FG_CUDA(cudaEventRecord(*ev_end, st));
    std::vector<double> h(g->acc_len);
    FG_CUDA(cudaMemcpyAsync(h.data(), g->d_acc, sizeof(double) * g->acc_len, cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    bin_power_unpack(g, h.data(), Psum, Pw);
    return OK;
}

static int bin_launch(BinGeometry *g, const void *f, int prec, int mode, double Vinv, double Pshot, cudaStream_t st,
                      const BinFinish *fin, const DevScalars *ds) {
    if (!g->valid) return set_error(ERR_STATE, "bin geometry not built");
    if (mode >= 2 && (prec != 4 || !fin)) return set_error(ERR_ARG, "fused finish needs an FP32 grid");
    const BinSpec &s = g->spec;
    const BinDev d = make_dev(s);
    const int NK = s.NK, W = s.Nmu + 1, NQ = 4 + W;
    const size_t smem = prec == 4 ? slab_smem(NK, NQ) : (size_t)NK * NQ * 8 + sizeof(uint32_t) * (NK + 2);
    if (smem > 220 * 1024)
        return set_error(ERR_UNSUPPORTED, "binning: %d k bins x %d wedges exceed shared memory", NK, s.Nmu);
    FG_CUDA(cudaMemsetAsync(g->d_acc, 0, sizeof(double) * g->acc_len, st));
    if (prec == 4) {
        int per_sm = (int)((224 * 1024) / (smem + 1024));
        per_sm = per_sm < 1 ? 1 : (per_sm > 3 ? 3 : per_sm);
        if (g->cta_per_sm > 0 && g->cta_per_sm < per_sm) per_sm = g->cta_per_sm;  // tuned shape
        const long nblk = ceil_div(s.Ng, kSlabI) * ceil_div(s.Ng, kSlabJ) * ceil_div(slab_kmain(s.Ng / 2 + 1), kSlabK);
        long nb = (long)num_sms() * per_sm;
        if (nb > nblk) nb = nblk;
        SlabFinish sf;
        if (fin) {
            sf.A = static_cast<float2 *>(fin->A);
            sf.B = static_cast<const float2 *>(fin->B);
            sf.ph = static_cast<const float2 *>(fin->ph32);
            sf.w = static_cast<const float *>(fin->w32);
            sf.scale = (float)fin->scale;
        }
        const float2 *fv = static_cast<const float2 *>(mode >= 2 ? fin->A : f);
#define FG_SLAB_LAUNCH2(M, B)                                                                                \
    do {                                                                                                    \
        FG_CUDA(cudaFuncSetAttribute(bin_power_slab_kernel<M, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                                           \
        bin_power_slab_kernel<M, B><<<(unsigned)nb, kSlabThreads, smem, st>>>(                              \
            d, fv, sf, (float)Vinv, (float)Pshot, g->d_thr, g->d_acc, ds, g->fold > 0 ? g->fold : fold_blocks()); \
    } while (0)
#define FG_SLAB_LAUNCH(M)             \
    do {                              \
        if (per_sm >= 3)              \
            FG_SLAB_LAUNCH2(M, 3);    \
        else                          \
            FG_SLAB_LAUNCH2(M, 2);    \
    } while (0)
        if (mode == 0)
            FG_SLAB_LAUNCH(0);
        else if (mode == 1)
            FG_SLAB_LAUNCH(1);
        else if (mode == 2)
            FG_SLAB_LAUNCH(2);
        else if (mode == 3)
            FG_SLAB_LAUNCH(3);
        else if (mode == 4)
            FG_SLAB_LAUNCH(4);
        else
            FG_SLAB_LAUNCH(5);
#undef FG_SLAB_LAUNCH2
#undef FG_SLAB_LAUNCH
    } else {
        const int Ng_pad = 2 * (s.Ng / 2 + 1);
        const long nchunks = ceil_div((long)s.Ng * s.Ng, kChunkRows);
        int per_sm = (int)((220 * 1024) / smem);
        per_sm = per_sm < 1 ? 1 : (per_sm > 8 ? 8 : per_sm);
        long nb = (long)num_sms() * per_sm;
        if (nb > nchunks) nb = nchunks;
#define FG_BIN_LAUNCH(M)                                                                                     \
    do {                                                                                                     \
        FG_CUDA(cudaFuncSetAttribute(bin_power_kernel<double, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                                            \
        bin_power_kernel<double, M><<<(unsigned)nb, kBinThreads, smem, st>>>(                                \
            d, (const double *)f, Vinv, Pshot, g->d_thr, g->d_acc, Ng_pad);                                  \
    } while (0)
        if (mode == 0)
            FG_BIN_LAUNCH(0);
        else
            FG_BIN_LAUNCH(1);
#undef FG_BIN_LAUNCH
    }
    FG_LAUNCHED(1);
    return OK;
}

}  // namespace fg
