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

#include <math.h>

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
template <int N1, int N2>
__global__ void __launch_bounds__(512)
fft2_cols_kernel(float2 *g0, float2 *g1, int ncols, long es, long bs, int logC,
                 const float2 *__restrict__ W, int sign) {
    constexpr int N = N1 * N2;
    extern __shared__ __align__(16) float2 S[];
    const int C = 1 << logC;
    const int P = N1 * C + 8;  // shared pitch per n2
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
        for (int s = t; s < C * N1; s += blockDim.x) {
            const int c = s & (C - 1), k1 = s >> logC;
            float2 u[N2];
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2) u[n2] = S[n2 * P + k1 * C + c];
            reg_fft<N2>(u, sign);
            if (c0 + c < ncols)
#pragma unroll
                for (int k2 = 0; k2 < N2; ++k2) base[(long)(k1 + N1 * k2) * es + c] = u[k2];
        }
    }
    (void)N;
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
template <int N1, int N2>
__global__ void __launch_bounds__(512)
fft2_k_r2c_kernel(float *g0, float *g1, long nrows, int Ng_pad, int R,
                  const float2 *__restrict__ W, const float2 *__restrict__ rtw) {
    constexpr int M = N1 * N2;
    constexpr int P = N2 * (N1 + 1);  // shared row pitch (step-1 layout, padded)
    extern __shared__ __align__(16) float2 S[];
    float *g = blockIdx.y == 0 ? g0 : g1;
    const long row0 = (long)blockIdx.x * R;
    const int t = threadIdx.x;
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
    const int nthr = blockDim.x;
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
    // split into the half spectrum and store (lanes over consecutive k)
    const int nh = M + 1;
    for (int e = t; e < R * nh; e += nthr) {
        const int r = e / nh, k = e - r * nh;
        if (row0 + r >= nrows) continue;
        const int k1 = k == M ? 0 : k, k2 = k == 0 ? 0 : M - k;
        const float2 z1 = S[r * P2 + k1];
        const float2 z2 = cconj(S[r * P2 + k2]);
        const float2 E = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y + z2.y));
        const float2 D = csub(z1, z2);
        const float2 O = make_float2(0.5f * D.y, -0.5f * D.x);
        reinterpret_cast<float2 *>(g + (row0 + r) * Ng_pad)[k] = cadd(E, cmul(__ldg(&rtw[k]), O));
    }
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

int fft2_k_r2c(int Ng, const void *W, const void *rtw, void *g0, void *g1, int ngrids, cudaStream_t s, int R_req,
               long row0, long nrows_req) {
    FG_TRY(ensure_w32());
    const int M = Ng / 2;
    int N1, N2;
    if (!split2(M, &N1, &N2)) return set_error(ERR_UNSUPPORTED, "fft2_k_r2c: Ng=%d", Ng);
    const int Ng_pad = 2 * (M + 1);
    const long nrows = nrows_req >= 0 ? nrows_req : (long)Ng * Ng - row0;
    if (row0 < 0 || nrows < 1 || row0 + nrows > (long)Ng * Ng)
        return set_error(ERR_ARG, "fft2_k_r2c: rows [%ld, %ld) outside the grid", row0, row0 + nrows);
    g0 = static_cast<float *>(g0) + row0 * Ng_pad;
    g1 = static_cast<float *>(g1) + row0 * Ng_pad;
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
