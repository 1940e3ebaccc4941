// Two-level FP32 FFT passes for power-of-two lengths up to 2048 (sm_103a).
//
// A length N = N1 * N2 transform along a column (or a packed k row) is done
// as  X[k1 + N1 k2] = sum_n2 W_N2^{n2 k2} W_N^{n2 k1} sum_n1 x[N2 n1 + n2] W_N1^{n1 k1}
// (Cooley-Tukey, N1, N2 <= 32):
//   step 1: each thread loads x[N2 n1 + n2], n1 = 0..N1-1 straight from HBM
//           into registers (lanes cover adjacent columns / adjacent n2, so
//           every load instruction is coalesced), runs an in-register FFT of
//           length N1, applies the twiddle W_N^{n2 k1} and stores to shared;
//   step 2: each thread gathers one k1 across n2 from shared memory, runs an
//           in-register FFT of length N2 and stores X[k1 + N1 k2].
// One shared-memory round trip per pass (the Stockham kernels of fft.cu take
// one per radix pass); the row pitches are padded so both shared-memory
// phases are free of bank conflicts.  Length 2048 on the strided axes is
// 32 x 64 with the 64-point second step split over lane pairs
// (fft2_cols2048_kernel).  Used for the forward r2c k pass and the strided
// j/i passes of FP32 grids; other lengths and FP64 grids use the general
// kernels of fft.cu.
#include "internal.h"
#include "common.cuh"

#include <cuda.h>  // CUtensorMap and its encode function's types; the function comes from the driver at run time

#include <math.h>
#include <stdlib.h>
#include <mutex>

namespace fg {

__constant__ float2 c_w32[32];  // exp(-2 pi i t / 32)

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }
__host__ __device__ constexpr int bitrev(int x, int bits) {
    int r = 0;
    for (int i = 0; i < bits; ++i) r = (r << 1) | ((x >> i) & 1);
    return r;
}

// in-register radix-2 FFT of length M <= 32, natural order in and out
template <int M>
__device__ __forceinline__ void reg_fft(float2 (&v)[M], int sign) {
    if constexpr (M > 1) {
        constexpr int B = ilog2c(M);
        float2 a[M];
#pragma unroll
        for (int i = 0; i < M; ++i) a[bitrev(i, B)] = v[i];
#pragma unroll
        for (int len = 2; len <= M; len <<= 1) {
            const int h = len >> 1;
#pragma unroll
            for (int j = 0; j < h; ++j) {
                const int tix = j * (32 / len);
                float2 w = c_w32[tix];
                if (sign > 0) w.y = -w.y;
#pragma unroll
                for (int s = 0; s < M; s += len) {
                    const float2 u = a[s + j];
                    float2 t = a[s + j + h];
                    if (tix == 8)
                        t = cmul_si(t, sign);
                    else if (tix != 0)
                        t = cmul(t, w);
                    a[s + j] = cadd(u, t);
                    a[s + j + h] = csub(u, t);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < M; ++i) v[i] = a[i];
    }
}

__device__ __forceinline__ float2 twid(const float2 *__restrict__ W, int t, int sign) {
    float2 w = __ldg(&W[t]);
    if (sign > 0) w.y = -w.y;
    return w;
}

// ---- strided axis: C columns per CTA, threads = C * N2 ---------------------------
// element n of column c of batch b: base + b*bs + n*es + c0 + c (complex units)
// One tile: columns c0 .. c0 + C - 1 at `base` (= g + b*bs + c0), `left`
// columns of them valid; threads t < nthr of the CTA (nthr >= C*N2).
template <int N1, int N2>
__device__ __forceinline__ void cols_tile(float2 *base, int left, long es, int logC, const float2 *__restrict__ W,
                                          int sign, float2 *S, int t, int nthr) {
    const int C = 1 << logC;
    const int P = N1 * C + 8;  // shared pitch per n2
    if (t < C * N2) {
        const int c = t & (C - 1), n2 = t >> logC;
        const bool ok = c < left;
        float2 v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) {
            const float2 *src = &base[(long)(N2 * n1 + n2) * es + c];
            v[n1] = ok ? *src : make_float2(0.f, 0.f);
        }
        reg_fft<N1>(v, sign);
        if constexpr (N2 > 1) {
#pragma unroll
            for (int k1 = 1; k1 < N1; ++k1)
                if (n2) v[k1] = cmul(v[k1], twid(W, n2 * k1, sign));
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) S[n2 * P + k1 * C + c] = v[k1];
        } else {
            if (ok)
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1) base[(long)k1 * es + c] = v[k1];
        }
    }
    if constexpr (N2 > 1) {
        __syncthreads();
        for (int s = t; s < C * N1; s += nthr) {
            const int c = s & (C - 1), k1 = s >> logC;
            float2 u[N2];
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2) u[n2] = S[n2 * P + k1 * C + c];
            reg_fft<N2>(u, sign);
            if (c < left)
#pragma unroll
                for (int k2 = 0; k2 < N2; ++k2) base[(long)(k1 + N1 * k2) * es + c] = u[k2];
        }
    }
}

template <int N1, int N2>
__global__ void __launch_bounds__(512)
fft2_cols_kernel(float2 *g0, float2 *g1, int ncols, long es, long bs, int logC,
                 const float2 *__restrict__ W, int sign) {
    extern __shared__ __align__(16) float2 S[];
    const int C = 1 << logC;
    const int ncb = (ncols + C - 1) >> logC;
    const int cb = blockIdx.x % ncb;
    const long batch = blockIdx.x / ncb;
    float2 *g = blockIdx.y == 0 ? g0 : g1;
    const int c0 = cb << logC;
    cols_tile<N1, N2>(g + batch * bs + c0, ncols - c0, es, logC, W, sign, S, threadIdx.x, blockDim.x);
}

// ---- strided axis of length 2048 = 32 x 64 ---------------------------------------------
// Step 1 as fft2_cols_kernel<32, 64> (threads = C * 64).  Step 2's length-64
// transforms would need 64 complex registers per thread; instead each
// (column, k1) is taken by a pair of lanes l and l ^ 16, one transforming the
// even n2 and one the odd n2 with reg_fft<32>, and the final radix-2 step
//   X[k2] = E[k2] + W_64^k2 O[k2],  X[k2 + 32] = E[k2] - W_64^k2 O[k2]
// exchanges E and O through shuffles.  Shared pitch P = 32 C + 16 (= 16 mod 32)
// keeps the step-2 reads of a warp (c, k1 bit, pair half in lane bits 0-4) on
// 32 distinct banks; the step-1 stores then take two wavefronts.
__global__ void __launch_bounds__(512)
fft2_cols2048_kernel(float2 *g0, float2 *g1, int ncols, long es, long bs, int logC, const float2 *__restrict__ W,
                     int sign) {
    constexpr int N1 = 32, N2 = 64;
    extern __shared__ __align__(16) float2 S[];
    const int C = 1 << logC;
    const int P = N1 * C + 16;
    const int ncb = (ncols + C - 1) >> logC;
    const int cb = blockIdx.x % ncb;
    const long batch = blockIdx.x / ncb;
    float2 *g = blockIdx.y == 0 ? g0 : g1;
    const int c0 = cb << logC;
    float2 *base = g + batch * bs + c0;
    const int t = threadIdx.x;
    {
        const int c = t & (C - 1), n2 = t >> logC;
        const bool ok = c0 + c < ncols;
        float2 v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1)
            v[n1] = ok ? base[(long)(N2 * n1 + n2) * es + c] : make_float2(0.f, 0.f);
        reg_fft<N1>(v, sign);
#pragma unroll
        for (int k1 = 1; k1 < N1; ++k1)
            if (n2) v[k1] = cmul(v[k1], twid(W, n2 * k1, sign));
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) S[n2 * P + k1 * C + c] = v[k1];
    }
    __syncthreads();
    // C * N1 tasks for C * N2 / 2 lane pairs: exactly one task per pair
    const int lane = t & 31, h = lane >> 4;
    const int task = (t >> 5) * 16 + (lane & 15);
    const int c = task & (C - 1), k1 = task >> logC;
    float2 u[32];
#pragma unroll
    for (int m = 0; m < 32; ++m) u[m] = S[(2 * m + h) * P + k1 * C + c];
    reg_fft<32>(u, sign);
    const bool ok = c0 + c < ncols;
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2) {
        float2 other;
        other.x = __shfl_xor_sync(0xffffffffu, u[k2].x, 16);
        other.y = __shfl_xor_sync(0xffffffffu, u[k2].y, 16);
        const float2 E = h ? other : u[k2], O = h ? u[k2] : other;
        const float2 wo = cmul(O, twid(W, 32 * k2, sign));  // W_2048^(32 k2) = W_64^k2
        const float2 x = h ? csub(E, wo) : cadd(E, wo);
        if (ok) base[(long)(k1 + N1 * (k2 + 32 * h)) * es + c] = x;
    }
}

// ---- k axis, forward r2c: R rows per CTA, threads = R * N2 ---------------------------
// Each real row of Ng = 2M values is read as M packed complex values
// z[m] = x[2m] + i x[2m+1]; X[k] = E[k] + W_Ng^k O[k] for k = 0..M.
// One tile: rows row0 .. row0 + R - 1 (of nrows) of g; threads t < nthr.
template <int N1, int N2>
__device__ __forceinline__ void kr2c_tile(float *g, long nrows, int Ng_pad, int R, long row0,
                                          const float2 *__restrict__ W, const float2 *__restrict__ rtw, float2 *S,
                                          int t, int nthr) {
    constexpr int M = N1 * N2;
    constexpr int P = N2 * (N1 + 1);  // shared row pitch (step-1 layout, padded)
    {
        const int n2 = t % N2, r = t / N2;
        const bool ok = r < R && row0 + r < nrows;
        const float2 *src = reinterpret_cast<const float2 *>(g + (row0 + r) * Ng_pad);
        float2 v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) v[n1] = ok ? src[N2 * n1 + n2] : make_float2(0.f, 0.f);
        reg_fft<N1>(v, -1);
#pragma unroll
        for (int k1 = 1; k1 < N1; ++k1)
            if (n2) v[k1] = cmul(v[k1], twid(W, n2 * k1, -1));
        if (r < R)
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) S[r * P + n2 * (N1 + 1) + k1] = v[k1];
    }
    __syncthreads();
    // step 2: results in registers until every thread has read its inputs
    constexpr int ROUNDS_MAX = N1 / N2 > 0 ? N1 / N2 : 1;
    float2 res[ROUNDS_MAX][N2];
#pragma unroll
    for (int q = 0; q < ROUNDS_MAX; ++q) {
        const int s = t + q * nthr;
        const int k1 = s % N1, r = s / N1;
        if (r < R) {
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2) res[q][n2] = S[r * P + n2 * (N1 + 1) + k1];
            reg_fft<N2>(res[q], -1);
        }
    }
    __syncthreads();
    constexpr int P2 = M + 1;  // natural-order layout
#pragma unroll
    for (int q = 0; q < ROUNDS_MAX; ++q) {
        const int s = t + q * nthr;
        const int k1 = s % N1, r = s / N1;
        if (r < R)
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) S[r * P2 + k1 + N1 * k2] = res[q][k2];
    }
    __syncthreads();
    // split into the half spectrum and store (lanes over consecutive k): one
    // pass over k = 0 .. M/2 forms X[k] = E + W^k O and, from the same E and
    // W^k O, X[M - k] = conj(E - W^k O) (E[M-k] = conj(E[k]), O[M-k] = conj(O[k])
    // and W^(M-k) = -conj(W^k) for W = exp(-2 pi i / 2M)); k = 0 also gives X[M]
    constexpr int NPAIR = M / 2 + 1;
    for (int e = t; e < R * NPAIR; e += nthr) {
        const int r = e / NPAIR, k = e - r * NPAIR;
        if (row0 + r >= nrows) continue;
        const int km = k == 0 ? 0 : M - k;
        const float2 z1 = S[r * P2 + k];
        const float2 z2 = cconj(S[r * P2 + km]);
        const float2 E = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y + z2.y));
        const float2 D = csub(z1, z2);
        const float2 O = make_float2(0.5f * D.y, -0.5f * D.x);
        const float2 wo = cmul(__ldg(&rtw[k]), O);
        float2 *out = reinterpret_cast<float2 *>(g + (row0 + r) * Ng_pad);
        out[k] = cadd(E, wo);
        if (k < M / 2) out[k == 0 ? M : M - k] = cconj(csub(E, wo));
    }
}

template <int N1, int N2>
__global__ void __launch_bounds__(512)
fft2_k_r2c_kernel(float *g0, float *g1, long nrows, int Ng_pad, int R,
                  const float2 *__restrict__ W, const float2 *__restrict__ rtw) {
    extern __shared__ __align__(16) float2 S[];
    kr2c_tile<N1, N2>(blockIdx.y == 0 ? g0 : g1, nrows, Ng_pad, R, (long)blockIdx.x * R, W, rtw, S, threadIdx.x,
                      blockDim.x);
}

// ---- widely strided axis (the i pass), columns staged by TMA ----------------------------------
// Ng = 512 or 1024 = 32 x N2.  A tile is C = 8 adjacent complex columns at one
// (grid, j) over all Ng rows i: Ng rows of 64 bytes, brought into shared
// memory by cp.async.bulk.tensor (boxes of 256 rows) with an mbarrier per
// stage.  The tensor map views one i plane as a row of Ng * Ng_pad floats and
// the planes as its rows (stride Ng Ng_pad floats, a multiple of 16 bytes);
// a tile starts at float j Ng_pad + 2 kc0 with kc0 = 8 m + (j & 1), which is
// a multiple of 4 floats (16 bytes) for every j (Ng_pad = 2 mod 4).  The
// column each j leaves (kc = Ng/2 for even j, kc = 0 for odd j) is
// transformed by fft2_cols_kernel.
// Persistent, one CTA per SM, three 64 KB stages and two groups of 256
// threads: group (l & 1) transforms the CTA's l-th tile while the loads of the
// next tiles are in flight; as soon as a group has read its stage into
// registers, it issues the load of tile l + 3 into that stage.  Step 1 (a
// 32-point FFT per (column, n2), twiddle) works in place in the stage, step 2
// (an N2-point FFT per (column, k1)) reads it into registers and stores the
// results to HBM.  Every mbarrier wait is bounded: on a time-out the kernel
// sets *err, stops issuing, waits (bounded) for its loads in flight and returns.
constexpr int kTmaCols = 8;
constexpr int kTmaStages = 3;
constexpr int kTmaThreads = 512;   // two groups of 256
constexpr int kTmaBoxRows = 256;
constexpr unsigned kTmaPollLimit = 1u << 24;  // polls of ~32 ns: about half a second

__device__ int g_tma_err;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// true once the phase with the given parity has completed; false after the poll limit
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (unsigned it = 0; it < kTmaPollLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        __nanosleep(32);
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void group_sync(int grp) {
    asm volatile("bar.sync %0, 256;" ::"r"(1 + grp) : "memory");
}

template <int N2>
__global__ void __launch_bounds__(kTmaThreads, 1)
fft2_cols_tma_kernel(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                     float2 *g0, float2 *g1, int ngrids, int Ng, int nh, int Ng_pad, long es,
                     const float2 *__restrict__ W, int sign) {
    constexpr int N1 = 32, N = N1 * N2, C = kTmaCols;
    constexpr uint32_t kTileBytes = N * C * sizeof(float2);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    float2 *stages = reinterpret_cast<float2 *>(smem_raw);  // [kTmaStages][N][C]
    __shared__ __align__(8) uint64_t full[kTmaStages];
    // issued[s]: the last local tile armed on stage s (written after the
    // previous use of the stage completed); consumed[s]: the last one read
    __shared__ volatile long issued[kTmaStages], consumed[kTmaStages];
    __shared__ volatile int group_abort[2];

    const int ntj = (nh - 1) / C;  // tiles per (grid, j)
    const long ntiles = (long)ngrids * Ng * ntj;
    const long nloc = ntiles > (long)blockIdx.x ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const int t = threadIdx.x, grp = t >> 8, gt = t & 255;

    auto tile_of = [&](long l, int &g, int &j, int &kc0) {
        const long q = blockIdx.x + (long)gridDim.x * l;
        g = (int)(q / ((long)Ng * ntj));
        const long r = q - (long)g * Ng * ntj;
        j = (int)(r / ntj);
        kc0 = C * (int)(r - (long)j * ntj) + (j & 1);
    };
    // one thread: arm stage l % 3 and issue the loads of local tile l
    auto issue = [&](long l) {
        int g, j, kc0;
        tile_of(l, g, j, kc0);
        const int s = (int)(l % kTmaStages);
        float2 *dst = stages + (size_t)s * N * C;
        mbar_expect_tx(&full[s], kTileBytes);
        const CUtensorMap *tm = g ? &tm1 : &tm0;
        const int x = j * Ng_pad + 2 * kc0;
#pragma unroll
        for (int y = 0; y < N; y += kTmaBoxRows) tma_load_2d(dst + (size_t)y * C, tm, x, y, &full[s]);
        __threadfence_block();
        issued[s] = l;
    };
    if (t == 0) {
        for (int s = 0; s < kTmaStages; ++s) {
            mbar_init(&full[s], 1);
            issued[s] = consumed[s] = -1;
        }
        group_abort[0] = group_abort[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (t == 0)
        for (long l = 0; l < kTmaStages && l < nloc; ++l) issue(l);

    for (long l = grp; l < nloc; l += 2) {
        const int s = (int)(l % kTmaStages);
        // the parity test below is only meaningful once the stage's previous
        // phase has completed, which its issuer waited for before arming tile l
        bool armed = false;
        for (unsigned it = 0; it < kTmaPollLimit && !armed; ++it) {
            armed = issued[s] >= l;
            if (!armed) __nanosleep(32);
        }
        if (!armed || !mbar_wait(&full[s], (uint32_t)((l / kTmaStages) & 1))) {
            atomicExch(&g_tma_err, 1);
            group_abort[grp] = 1;
        }
        group_sync(grp);
        if (group_abort[grp]) break;  // the group leaves together (the flag is only ever set)
        int g, j, kc0;
        tile_of(l, g, j, kc0);
        float2 *S = stages + (size_t)s * N * C;
        if (gt < C * N2) {  // step 1: x[N2 n1 + n2] -> Y[k1, n2] W_N^(n2 k1), in place
            const int c = gt & (C - 1), n2 = gt >> 3;
            float2 v[N1];
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) v[n1] = S[(N2 * n1 + n2) * C + c];
            reg_fft<N1>(v, sign);
#pragma unroll
            for (int k1 = 1; k1 < N1; ++k1)
                if (n2) v[k1] = cmul(v[k1], twid(W, n2 * k1, sign));
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) S[(N2 * k1 + n2) * C + c] = v[k1];
        }
        group_sync(grp);
        // step 2: one (column, k1) per thread; odd k1 read each pair of rows in
        // swapped order so that a warp's 4 rows fall in both halves of the banks
        const int c = gt & (C - 1), k1 = gt >> 3;
        const bool odd = k1 & 1;
        float2 u[N2];
#pragma unroll
        for (int m = 0; m < N2; m += 2) {
            const float2 a = S[(N2 * k1 + m + (odd ? 1 : 0)) * C + c];
            const float2 b = S[(N2 * k1 + m + (odd ? 0 : 1)) * C + c];
            u[m] = odd ? b : a;
            u[m + 1] = odd ? a : b;
        }
        group_sync(grp);
        if (gt == 0) {
            consumed[s] = l;
            if (l + kTmaStages < nloc) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(l + kTmaStages);
            }
        }
        reg_fft<N2>(u, sign);
        float2 *base = (g ? g1 : g0) + (long)j * nh + kc0 + c;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) base[(long)(k1 + N1 * k2) * es] = u[k2];
    }
    __syncthreads();
    if (t == 0)  // loads still in flight after a time-out land before the CTA exits
        for (int s = 0; s < kTmaStages; ++s)
            if (issued[s] > consumed[s]) mbar_wait(&full[s], (uint32_t)((issued[s] / kTmaStages) & 1));
}

// ---- the i pass of Ng = 1024 by even and odd rows (128-byte rows) ------------------------------
// X[k] = E[k] + W_1024^k O[k], X[k + 512] = E[k] - W_1024^k O[k], with E and O
// the 512-point transforms of the even and the odd rows of a column.  A tile
// is 16 adjacent complex columns at one (grid, j) -- rows of 128 bytes -- and
// is brought in as two half-tiles of 512 rows (64 KB each): the even rows,
// then the odd rows, through a 3D tensor map (plane floats, row parity with
// a stride of one plane, i / 2 with a stride of two planes; boxes of 32 floats
// x 1 x 256).  Three 64 KB stages hold consecutive half-tiles; the CTA (512
// threads, one per SM) transforms one half-tile while the next two are in
// flight, keeping E in registers (16 values per thread) until O arrives.
// A 512-point transform is 32 x 16: step 1 (256 threads, one per (column,
// n2)) a 32-point FFT over n1 in place, twiddled by W_512^(n2 k1); step 2 (512
// threads, one per (column, k1)) a 16-point FFT over n2.  Tiles start at
// kc0 = 16 m + (j & 1) (16-byte aligned for every j); the column each j leaves
// goes to fft2_cols_kernel.  Waits are bounded as in fft2_cols_tma_kernel.
constexpr int kEoCols = 16;
constexpr int kEoThreads = 512;
constexpr int kEoHalfRows = 512;

__global__ void __launch_bounds__(kEoThreads, 1)
fft2_cols_tma_eo_kernel(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                        float2 *g0, float2 *g1, int ngrids, int Ng, int nh, int Ng_pad, long es,
                        const float2 *__restrict__ W, int sign) {
    constexpr int C = kEoCols, N1 = 32, N2 = 16, H = kEoHalfRows;
    constexpr uint32_t kHalfBytes = H * C * sizeof(float2);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    float2 *stages = reinterpret_cast<float2 *>(smem_raw);  // [kTmaStages][H][C]
    __shared__ __align__(8) uint64_t full[kTmaStages];
    __shared__ long issued[kTmaStages], consumed[kTmaStages];

    const int ntj = (nh - 1) / C;  // tiles per (grid, j)
    const long ntiles = (long)ngrids * Ng * ntj;
    const long nloc = ntiles > (long)blockIdx.x ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const long nhalf = 2 * nloc;
    const int t = threadIdx.x;

    auto tile_of = [&](long l, int &g, int &j, int &kc0) {
        const long q = blockIdx.x + (long)gridDim.x * l;
        g = (int)(q / ((long)Ng * ntj));
        const long r = q - (long)g * Ng * ntj;
        j = (int)(r / ntj);
        kc0 = C * (int)(r - (long)j * ntj) + (j & 1);
    };
    auto issue = [&](long h) {  // one thread: half-tile h (tile h / 2, rows of parity h & 1)
        int g, j, kc0;
        tile_of(h >> 1, g, j, kc0);
        const int s = (int)(h % kTmaStages);
        float2 *dst = stages + (size_t)s * H * C;
        mbar_expect_tx(&full[s], kHalfBytes);
        const CUtensorMap *tm = g ? &tm1 : &tm0;
        const int x = j * Ng_pad + 2 * kc0, par = (int)(h & 1);
#pragma unroll
        for (int y = 0; y < H; y += kTmaBoxRows)
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                "%4}], [%5];" ::"r"(smem_addr(dst + (size_t)y * C)),
                "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(par), "r"(y), "r"(smem_addr(&full[s]))
                : "memory");
        issued[s] = h;
    };
    if (t == 0) {
        for (int s = 0; s < kTmaStages; ++s) {
            mbar_init(&full[s], 1);
            issued[s] = consumed[s] = -1;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (long h = 0; h < kTmaStages && h < nhalf; ++h) issue(h);
    }
    __syncthreads();

    float2 E[N2];  // this thread's even-row transform, kept until the odd rows arrive
#pragma unroll
    for (int q = 0; q < N2; ++q) E[q] = make_float2(0.f, 0.f);
    const int c2 = t & (C - 1), k1 = t >> 4;  // step 2 and the output: (column, k1)
    for (long h = 0; h < nhalf; ++h) {
        const int s = (int)(h % kTmaStages);
        const bool ok = mbar_wait(&full[s], (uint32_t)((h / kTmaStages) & 1));
        if (!ok) atomicExch(&g_tma_err, 1);
        if (__syncthreads_or(!ok)) break;  // the CTA leaves together
        float2 *S = stages + (size_t)s * H * C;
        if (t < C * N2) {  // step 1: x[N2 n1 + n2] -> Y[k1, n2] W_512^(n2 k1), in place
            const int c = t & (C - 1), n2 = t >> 4;
            float2 v[N1];
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) v[n1] = S[(N2 * n1 + n2) * C + c];
            reg_fft<N1>(v, sign);
#pragma unroll
            for (int q = 1; q < N1; ++q)
                if (n2) v[q] = cmul(v[q], twid(W, 2 * n2 * q, sign));
#pragma unroll
            for (int q = 0; q < N1; ++q) S[(N2 * q + n2) * C + c] = v[q];
        }
        __syncthreads();
        float2 u[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) u[n2] = S[(N2 * k1 + n2) * C + c2];
        __syncthreads();
        if (t == 0) {
            consumed[s] = h;
            if (h + kTmaStages < nhalf) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(h + kTmaStages);
            }
        }
        reg_fft<N2>(u, sign);  // u[k2] = transform of this parity at k1 + 32 k2
        if ((h & 1) == 0) {
#pragma unroll
            for (int q = 0; q < N2; ++q) E[q] = u[q];
        } else {
            int g, j, kc0;
            tile_of(h >> 1, g, j, kc0);
            float2 *base = (g ? g1 : g0) + (long)j * nh + kc0 + c2;
#pragma unroll
            for (int q = 0; q < N2; ++q) {
                const int k = k1 + N1 * q;
                const float2 wo = cmul(u[q], twid(W, k, sign));
                base[(long)k * es] = cadd(E[q], wo);
                base[(long)(k + N1 * N2) * es] = csub(E[q], wo);
            }
        }
    }
    __syncthreads();
    if (t == 0)  // loads still in flight after a time-out land before the CTA exits
        for (int s = 0; s < kTmaStages; ++s)
            if (issued[s] > consumed[s]) mbar_wait(&full[s], (uint32_t)((issued[s] / kTmaStages) & 1));
}

// ---- host side ----------------------------------------------------------------------------

static bool g_w32_ready = false;

static int ensure_w32() {
    if (g_w32_ready) return OK;
    float2 w[32];
    for (int t = 0; t < 32; ++t) {
        const double a = 2.0 * M_PI * t / 32.0;
        w[t] = make_float2((float)cos(a), (float)-sin(a));
    }
    FG_CUDA(cudaMemcpyToSymbol(c_w32, w, sizeof(w)));
    g_w32_ready = true;
    return OK;
}

// (N1, N2) with N1 >= N2, both <= 32, for power-of-two N <= 1024
static bool split2(int N, int *N1, int *N2) {
    if (N < 1 || N > 1024 || (N & (N - 1))) return false;
    const int b = ilog2c(N);
    const int b2 = b / 2, b1 = b - b2;
    *N1 = 1 << b1;
    *N2 = 1 << b2;
    return true;
}

// strided passes: split2, or 32 x 64 with paired step-2 lanes for N = 2048
static bool cols_split(int N, int *N1, int *N2, bool *paired) {
    *paired = N == 2048;
    if (*paired) {
        *N1 = 32;
        *N2 = 64;
        return true;
    }
    return split2(N, N1, N2);
}

bool fft2_supported(int Ng, int prec) {
    int a, b;
    bool pr;
    return prec == 4 && Ng >= 4 && cols_split(Ng, &a, &b, &pr) && split2(Ng / 2, &a, &b);
}

#define FG_COLS_CASE(A, B)                                                                                 \
    if (N1 == A && N2 == B) {                                                                             \
        FG_CUDA(cudaFuncSetAttribute(fft2_cols_kernel<A, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                     (int)smem));                                                         \
        fft2_cols_kernel<A, B><<<grid, threads, smem, s>>>((float2 *)g0, (float2 *)g1, ncols, es, bs,      \
                                                           logC, (const float2 *)W, sign);                 \
        FG_LAUNCHED(1);                                                                                    \
        return OK;                                                                                         \
    }

// C columns per CTA: threads = C*N2 around 256, C >= 8 for 64-byte rows;
// along a widely strided axis (the i pass) C = 16, so every row access is a
// 128-byte run (measured 15 % faster at Ng = 1024; the j pass is faster with
// C = 8 and two CTAs per SM)
static int cols_default_logC(int N2, bool wide) {
    int logC = wide ? 4 : 3;
    while ((1 << logC) * N2 < 256 && logC < 5) ++logC;
    while ((1 << logC) * N2 > 512 && logC > 0) --logC;
    return logC;
}

static size_t cols_smem(int N1, int N2, int logC, bool paired = false) {
    return (size_t)N2 * (N1 * (1 << logC) + (paired ? 16 : 8)) * sizeof(float2);
}

static int k_default_rows(int N2) {
    int R = 1;  // rows per CTA: threads = R*N2 around 64 (small CTAs, many per SM)
    while (R * N2 < 64 && R < 64) R *= 2;
    return R;
}

static size_t k_smem(int N1, int N2, int R) {
    const int M = N1 * N2, P = N2 * (N1 + 1), P2 = M + 1;
    return (size_t)R * (P > P2 ? P : P2) * sizeof(float2);
}

bool fft2_valid_shape(int Ng, int which, int v) {
    int N1, N2;
    bool paired = false;
    const int N = which == 0 ? Ng / 2 : Ng;
    if (!fft2_supported(Ng, 4) || !(which == 0 ? split2(N, &N1, &N2) : cols_split(N, &N1, &N2, &paired)))
        return false;
    if (which == 0) {  // k pass: R rows per CTA
        if (v < 1 || v > 64 || (v & (v - 1))) return false;
        const int thr = v * N2;
        return thr >= 32 && thr <= 512 && k_smem(N1, N2, v) <= (size_t)device_max_smem();
    }
    if (v < 0 || v > 5) return false;  // j or i pass: log2 columns per CTA
    const int thr = (1 << v) * N2;
    return thr >= 32 && thr <= 512 && cols_smem(N1, N2, v, paired) <= (size_t)device_max_smem();
}

int fft2_default_shape(int Ng, int which) {
    int N1, N2;
    bool paired = false;
    if (!(which == 0 ? split2(Ng / 2, &N1, &N2) : cols_split(Ng, &N1, &N2, &paired))) return -1;
    if (which == 0) return k_default_rows(N2);
    const long es = which == 1 ? (long)(Ng / 2 + 1) : (long)Ng * (Ng / 2 + 1);
    return cols_default_logC(N2, es * (long)sizeof(float2) > (1L << 20));
}

int fft2_prepare() { return ensure_w32(); }

// ---- TMA-staged i pass ------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int tensor_map_encoder(EncodeTiledFn *fn) {
    static std::mutex m;
    static EncodeTiledFn enc = nullptr;
    std::lock_guard<std::mutex> lock(m);
    if (!enc) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
            return set_error(ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available from the driver");
        enc = reinterpret_cast<EncodeTiledFn>(p);
    }
    *fn = enc;
    return OK;
}

// one FP32 grid as [Ng planes i][Ng * Ng_pad floats], boxes of 16 floats x 256 planes
static int plane_tensor_map(CUtensorMap *tm, void *grid, int Ng) {
    EncodeTiledFn enc;
    FG_TRY(tensor_map_encoder(&enc));
    const cuuint64_t Ng_pad = 2 * (cuuint64_t)(Ng / 2 + 1);
    const cuuint64_t dims[2] = {(cuuint64_t)Ng * Ng_pad, (cuuint64_t)Ng};
    const cuuint64_t strides[1] = {(cuuint64_t)Ng * Ng_pad * sizeof(float)};
    const cuuint32_t box[2] = {2 * kTmaCols, (cuuint32_t)(Ng < kTmaBoxRows ? Ng : kTmaBoxRows)};
    const cuuint32_t estr[2] = {1, 1};
    if (reinterpret_cast<uintptr_t>(grid) % 16 || strides[0] % 16)
        return set_error(ERR_UNSUPPORTED, "TMA i pass: grid address or plane stride not 16-byte aligned");
    const CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, grid, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return OK;
}

// one FP32 grid as [Ng/2 plane pairs][2 row parities][Ng * Ng_pad floats],
// boxes of 32 floats x 1 parity x 256 pairs (the even/odd i pass)
static int parity_tensor_map(CUtensorMap *tm, void *grid, int Ng) {
    EncodeTiledFn enc;
    FG_TRY(tensor_map_encoder(&enc));
    const cuuint64_t Ng_pad = 2 * (cuuint64_t)(Ng / 2 + 1), plane = (cuuint64_t)Ng * Ng_pad;
    const cuuint64_t dims[3] = {plane, 2, (cuuint64_t)Ng / 2};
    const cuuint64_t strides[2] = {plane * sizeof(float), 2 * plane * sizeof(float)};
    const cuuint32_t box[3] = {2 * kEoCols, 1, (cuuint32_t)kTmaBoxRows};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (reinterpret_cast<uintptr_t>(grid) % 16 || strides[0] % 16)
        return set_error(ERR_UNSUPPORTED, "TMA i pass: grid address or plane stride not 16-byte aligned");
    const CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, grid, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return OK;
}

bool fft2_tma_supported(int Ng, int prec) {
    // off by default: with 64-byte rows at the plane stride the TMA pass
    // measured 7.8 ms against 4.7 ms for fft2_cols_kernel (16 columns, 128-byte
    // rows) at Ng = 1024; FFTGAL_TMA=1 selects it
    static const int on = [] {
        const char *e = getenv("FFTGAL_TMA");
        return e && e[0] == '1';
    }();
    return on && prec == 4 && (Ng == 512 || Ng == 1024);
}

int fft2_cols_tma(int Ng, const void *W, void *g0, void *g1, int ngrids, int sign, cudaStream_t s) {
    FG_TRY(ensure_w32());
    if (!fft2_tma_supported(Ng, 4)) return set_error(ERR_UNSUPPORTED, "TMA i pass: Ng=%d", Ng);
    const int nh = Ng / 2 + 1, Ng_pad = 2 * nh;
    const long es = (long)Ng * nh;  // complex values between consecutive i
    void *b = ngrids > 1 ? g1 : g0;
    CUtensorMap tm[2];
    FG_TRY(plane_tensor_map(&tm[0], g0, Ng));
    FG_TRY(plane_tensor_map(&tm[1], b, Ng));
    const size_t smem = (size_t)kTmaStages * Ng * kTmaCols * sizeof(float2);
    const long ntiles = (long)ngrids * Ng * ((nh - 1) / kTmaCols);
    const unsigned nb = (unsigned)(ntiles < num_sms() ? ntiles : num_sms());
    if (Ng == 1024) {  // even and odd rows: 16 columns, 128-byte rows
        FG_TRY(parity_tensor_map(&tm[0], g0, Ng));
        FG_TRY(parity_tensor_map(&tm[1], b, Ng));
        const size_t esmem = (size_t)kTmaStages * kEoHalfRows * kEoCols * sizeof(float2);
        const long etiles = (long)ngrids * Ng * ((nh - 1) / kEoCols);
        const unsigned enb = (unsigned)(etiles < num_sms() ? etiles : num_sms());
        FG_CUDA(cudaFuncSetAttribute(fft2_cols_tma_eo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem));
        fft2_cols_tma_eo_kernel<<<enb, kEoThreads, esmem, s>>>(tm[0], tm[1], (float2 *)g0, (float2 *)b, ngrids, Ng,
                                                                nh, Ng_pad, es, (const float2 *)W, sign);
    } else {
        FG_CUDA(cudaFuncSetAttribute(fft2_cols_tma_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fft2_cols_tma_kernel<16><<<nb, kTmaThreads, smem, s>>>(tm[0], tm[1], (float2 *)g0, (float2 *)b, ngrids, Ng,
                                                               nh, Ng_pad, es, (const float2 *)W, sign);
    }
    FG_LAUNCHED(1);
    // the column each j leaves to fft2_cols_kernel: kc = Ng/2 at even j, kc = 0 at odd j
    float2 *a2 = static_cast<float2 *>(g0), *b2 = static_cast<float2 *>(b);
    const int lc = Ng == 512 ? 1 : 0;  // at least 32 threads per CTA
    FG_TRY(fft2_cols(Ng, W, a2 + Ng / 2, b2 + Ng / 2, ngrids, 1, es, 2L * nh, Ng / 2, sign, s, lc));
    FG_TRY(fft2_cols(Ng, W, a2 + nh, b2 + nh, ngrids, 1, es, 2L * nh, Ng / 2, sign, s, lc));
    return OK;
}

int fft2_tma_check() {
    int v = 0;
    FG_CUDA(cudaMemcpyFromSymbol(&v, g_tma_err, sizeof(int)));
    if (v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_tma_err, &zero, sizeof(int));
        return set_error(ERR_CUDA, "TMA column pass: a shared-memory stage never arrived (wait timed out)");
    }
    return OK;
}

int fft2_cols(int N, const void *W, void *g0, void *g1, int ngrids, int ncols, long es, long bs,
              long nbatch, int sign, cudaStream_t s, int logC_req) {
    FG_TRY(ensure_w32());
    int N1, N2;
    bool paired;
    if (!cols_split(N, &N1, &N2, &paired)) return set_error(ERR_UNSUPPORTED, "fft2_cols: N=%d", N);
    int logC = cols_default_logC(N2, es * (long)sizeof(float2) > (1L << 20));
    if (logC_req >= 0) {
        const int thr = (1 << logC_req) * N2;
        if (logC_req > 5 || thr < 32 || thr > 512 ||
            cols_smem(N1, N2, logC_req, paired) > (size_t)device_max_smem())
            return set_error(ERR_ARG, "fft2_cols: %d columns per CTA invalid for N=%d", 1 << logC_req, N);
        logC = logC_req;
    }
    const int C = 1 << logC;
    const int threads = C * N2;
    const size_t smem = cols_smem(N1, N2, logC, paired);
    const long ncb = ceil_div(ncols, C);
    dim3 grid((unsigned)(ncb * nbatch), ngrids);
    if (paired) {
        FG_CUDA(cudaFuncSetAttribute(fft2_cols2048_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fft2_cols2048_kernel<<<grid, threads, smem, s>>>((float2 *)g0, (float2 *)g1, ncols, es, bs, logC,
                                                         (const float2 *)W, sign);
        FG_LAUNCHED(1);
        return OK;
    }
    FG_COLS_CASE(1, 1)
    FG_COLS_CASE(2, 1)
    FG_COLS_CASE(2, 2)
    FG_COLS_CASE(4, 2)
    FG_COLS_CASE(4, 4)
    FG_COLS_CASE(8, 4)
    FG_COLS_CASE(8, 8)
    FG_COLS_CASE(16, 8)
    FG_COLS_CASE(16, 16)
    FG_COLS_CASE(32, 16)
    FG_COLS_CASE(32, 32)
    return set_error(ERR_UNSUPPORTED, "fft2_cols: no kernel for %d x %d", N1, N2);
}
#undef FG_COLS_CASE

#define FG_K_CASE(A, B)                                                                                    \
    if (N1 == A && N2 == B) {                                                                             \
        FG_CUDA(cudaFuncSetAttribute(fft2_k_r2c_kernel<A, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                     (int)smem));                                                         \
        fft2_k_r2c_kernel<A, B><<<grid, threads, smem, s>>>((float *)g0, (float *)g1, nrows, Ng_pad, R,   \
                                                            (const float2 *)W, (const float2 *)rtw);       \
        FG_LAUNCHED(1);                                                                                    \
        return OK;                                                                                         \
    }

int fft2_k_r2c(int Ng, const void *W, const void *rtw, void *g0, void *g1, int ngrids, cudaStream_t s, int R_req) {
    FG_TRY(ensure_w32());
    const int M = Ng / 2;
    int N1, N2;
    if (!split2(M, &N1, &N2)) return set_error(ERR_UNSUPPORTED, "fft2_k_r2c: Ng=%d", Ng);
    const int Ng_pad = 2 * (M + 1);
    const long nrows = (long)Ng * Ng;
    int R = k_default_rows(N2);
    if (R_req > 0) {
        if (!fft2_valid_shape(Ng, 0, R_req))
            return set_error(ERR_ARG, "fft2_k_r2c: %d rows per CTA invalid for Ng=%d", R_req, Ng);
        R = R_req;
    }
    const int threads = R * N2;
    const size_t smem = k_smem(N1, N2, R);
    dim3 grid((unsigned)ceil_div(nrows, R), ngrids);
    FG_K_CASE(1, 1)
    FG_K_CASE(2, 1)
    FG_K_CASE(2, 2)
    FG_K_CASE(4, 2)
    FG_K_CASE(4, 4)
    FG_K_CASE(8, 4)
    FG_K_CASE(8, 8)
    FG_K_CASE(16, 8)
    FG_K_CASE(16, 16)
    FG_K_CASE(32, 16)
    FG_K_CASE(32, 32)
    return set_error(ERR_UNSUPPORTED, "fft2_k_r2c: no kernel for %d x %d", N1, N2);
}
#undef FG_K_CASE

// ---- autotuner ---------------------------------------------------------------------
// Launch shape -> time: two untimed launches, then the median of five timed
// ones (CUDA events on s).  The FFT's arithmetic per row / column does not
// depend on the shape, so every shape gives bit-identical results.
static int time_shape(FftPlan *p, void *grid, cudaStream_t s, int which, int v, cudaEvent_t e0, cudaEvent_t e1,
                      double *ms) {
    const int Ng = p->Ng, nh = p->nh;
    auto launch = [&]() -> int {
        if (which == 0) return fft2_k_r2c(Ng, p->half.tw, p->rtw, grid, grid, 1, s, v);
        const long es = which == 1 ? nh : (long)Ng * nh, bs = which == 1 ? (long)Ng * nh : nh;
        return fft2_cols(Ng, p->axis.tw, grid, grid, 1, nh, es, bs, Ng, -1, s, v);
    };
    for (int r = 0; r < 2; ++r) FG_TRY(launch());
    float t[5];
    for (int r = 0; r < 5; ++r) {
        FG_CUDA(cudaEventRecord(e0, s));
        FG_TRY(launch());
        FG_CUDA(cudaEventRecord(e1, s));
        FG_CUDA(cudaEventSynchronize(e1));
        FG_CUDA(cudaEventElapsedTime(&t[r], e0, e1));
    }
    for (int a = 1; a < 5; ++a)
        for (int b = a; b > 0 && t[b] < t[b - 1]; --b) {
            const float x = t[b];
            t[b] = t[b - 1];
            t[b - 1] = x;
        }
    *ms = t[2];
    return OK;
}

int fft2_autotune(FftPlan *p, void *grid, cudaStream_t s, double ms[3]) {
    if (!fft2_supported(p->Ng, p->prec))
        return set_error(ERR_UNSUPPORTED, "autotune: no tunable launch shapes for Ng=%d (%s grid)", p->Ng,
                         p->prec == 4 ? "FP32" : "FP64");
    const size_t bytes = sizeof(float) * (size_t)p->Ng * p->Ng * 2 * p->nh;
    FG_CUDA(cudaMemsetAsync(grid, 0, bytes, s));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FG_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_check(ce, "autotune events");
    }
    int rc = OK;
    int best[3];
    double best_ms[3];
    for (int which = 0; which < 3 && rc == OK; ++which) {
        const int def = fft2_default_shape(p->Ng, which);
        double def_ms = 0;
        rc = time_shape(p, grid, s, which, def, e0, e1, &def_ms);
        best[which] = def;
        best_ms[which] = def_ms;
        const int lo = which == 0 ? 1 : 0, hi = which == 0 ? 64 : 5;
        for (int v = lo; v <= hi && rc == OK; v = which == 0 ? v * 2 : v + 1) {
            if (v == def || !fft2_valid_shape(p->Ng, which, v)) continue;
            double t = 0;
            rc = time_shape(p, grid, s, which, v, e0, e1, &t);
            // keep the built-in shape unless another is clearly faster (2 %)
            if (rc == OK && t < best_ms[which] && t < 0.98 * def_ms) {
                best[which] = v;
                best_ms[which] = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == OK) rc = cuda_check(cudaMemsetAsync(grid, 0, bytes, s), "autotune clear");
    if (rc == OK) rc = cuda_check(cudaStreamSynchronize(s), "autotune");
    FG_TRY(rc);
    p->tune[0] = best[0];
    p->tune[1] = best[1];
    p->tune[2] = best[2];
    for (int w = 0; w < 3; ++w) ms[w] = best_ms[w];
    return OK;
}

}  // namespace fg
