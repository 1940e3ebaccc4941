// Full-grid elementwise passes of the reference path, for sm_103a:
//   scale            src/fft.c:128-129, 176-177, 188-189   (f *= H^3, 1/L^3, Npcinv)
//   offset phase     src/fft.c:196-233 (with its Nyquist-table behaviour)
//   deconvolution    src/fft.c:236-254 (PCS window sinc^-4 per axis)
//   interlace mean   src/fft.c:270-271 (f = 0.5 (f_dual + f))
//   power            src/power.c:12-27 (F_Re = |F|^2/V - Pshot, F_Im = 0, DC = 0)
//   precision change (device grid <-> double host view)
// FP64 grids evaluate every product and sum in the reference's order with
// explicitly rounded intrinsics (no FMA contraction), so they reproduce the
// reference's arithmetic; FP32 grids use the same formulas in FP32.
#include "internal.h"
#include "common.cuh"

#include <math.h>
#include <vector>

namespace fg {

static unsigned grid_blocks(long n, int threads) {
    long b = ceil_div(n, threads);
    const long cap = 64L * num_sms();
    return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

// Half-spectrum modes are visited in chunks of kRowChunk rows (row = i*Ng+j)
// so every index is 32-bit: e = chunk offset + q, q < kRowChunk*nh.
constexpr int kRowChunk = 16;

static unsigned chunk_blocks(int Ng) {
    const long nchunks = ceil_div((long)Ng * Ng, kRowChunk);
    const long cap = 32L * num_sms();
    return (unsigned)(nchunks < cap ? nchunks : cap);
}

#define FG_FOR_MODES(Ng, nh)                                                                \
    for (int ch_ = blockIdx.x; ch_ * kRowChunk < (Ng) * (Ng); ch_ += gridDim.x)             \
        for (int q_ = threadIdx.x, row0_ = ch_ * kRowChunk,                                 \
                 qn_ = min(kRowChunk, (Ng) * (Ng) - ch_ * kRowChunk) * (nh);                \
             q_ < qn_; q_ += blockDim.x)                                                   \
            if (const int rl_ = q_ / (nh); true)                                            \
                if (const int k = q_ - rl_ * (nh), row = row0_ + rl_; true)                 \
                    if (const int i = row / (Ng), j = row - i * (Ng); true)                 \
                        if (const long e = (long)row * (nh) + k; true)

// ---- scale -------------------------------------------------------------------
template <typename T>
__global__ void scale_kernel(T *f, long n, T s) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        f[e] = f[e] * s;
}

int scale_grid(void *f, long n, int prec, double s, cudaStream_t st) {
    if (prec == 4)
        scale_kernel<float><<<grid_blocks(n, 256), 256, 0, st>>>((float *)f, n, (float)s);
    else
        scale_kernel<double><<<grid_blocks(n, 256), 256, 0, st>>>((double *)f, n, s);
    FG_LAUNCHED(1);
    return OK;
}

// ---- offset phase ---------------------------------------------------------------
// table: [3][Ng] complex in FP64, built exactly as src/fft.c:201-215 builds it
int build_phase_table(double *tab, int Ng, const double offset[3], int onoff) {
    onoff = onoff > 0 ? 1 : -1;
    for (int a = 0; a < 3; ++a) {
        tab[(a * Ng + 0) * 2 + 0] = 1;
        tab[(a * Ng + 0) * 2 + 1] = 0;
    }
    for (int a = 0; a < 3; ++a)
        for (int n = 1; n <= Ng / 2; ++n) {
            volatile double arg = -onoff * 2 * M_PI * n / Ng * offset[a];
            const double c = cos(arg), s = sin(arg);
            tab[(a * Ng + n) * 2 + 0] = c;
            tab[(a * Ng + n) * 2 + 1] = s;
            tab[(a * Ng + Ng - n) * 2 + 0] = c;
            tab[(a * Ng + Ng - n) * 2 + 1] = -s;
        }
    return OK;
}

template <typename T>
__device__ __forceinline__ void phase_of(const double *__restrict__ tab, int Ng, int i, int j, int k,
                                         T &pr, T &pi) {
    if constexpr (sizeof(T) == 8) {
        const double ar = tab[2 * i], ai = tab[2 * i + 1];
        const double br = tab[2 * (Ng + j)], bi = tab[2 * (Ng + j) + 1];
        const double cr = tab[2 * (2 * Ng + k)], ci = tab[2 * (2 * Ng + k) + 1];
        // src/fft.c:217-228, left to right
        pr = __dsub_rn(__dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(ar, br), cr), __dmul_rn(__dmul_rn(ar, bi), ci)),
                                 __dmul_rn(__dmul_rn(ai, br), ci)),
                       __dmul_rn(__dmul_rn(ai, bi), cr));
        pi = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(ai, br), cr), __dmul_rn(__dmul_rn(ar, bi), cr)),
                                 __dmul_rn(__dmul_rn(ar, br), ci)),
                       __dmul_rn(__dmul_rn(ai, bi), ci));
    } else {
        const float ar = (float)tab[2 * i], ai = (float)tab[2 * i + 1];
        const float br = (float)tab[2 * (Ng + j)], bi = (float)tab[2 * (Ng + j) + 1];
        const float cr = (float)tab[2 * (2 * Ng + k)], ci = (float)tab[2 * (2 * Ng + k) + 1];
        const float xr = ar * br - ai * bi, xi = ar * bi + ai * br;
        pr = xr * cr - xi * ci;
        pi = xr * ci + xi * cr;
    }
}

template <typename T>
__global__ void phase_kernel(T *f, int Ng, const double *__restrict__ tab) {
    using T2 = vec2_t<T>;
    const int nh = Ng / 2 + 1;
    const long n = (long)Ng * Ng * nh;
    T2 *c = reinterpret_cast<T2 *>(f);
    (void)n;
    FG_FOR_MODES(Ng, nh) {
        T pr, pi;
        phase_of<T>(tab, Ng, i, j, k, pr, pi);
        const T2 v = c[e];
        if constexpr (sizeof(T) == 8)
            c[e] = mk2<T2>(__dsub_rn(__dmul_rn(v.x, pr), __dmul_rn(v.y, pi)),
                           __dadd_rn(__dmul_rn(v.x, pi), __dmul_rn(v.y, pr)));
        else
            c[e] = mk2<T2>(v.x * pr - v.y * pi, v.x * pi + v.y * pr);
    }
}

int apply_phase(void *f, int Ng, int prec, const void *d_tab, cudaStream_t st) {
    const long n = (long)Ng * Ng * (Ng / 2 + 1);
    if (prec == 4)
        phase_kernel<float><<<chunk_blocks(Ng), 256, 0, st>>>((float *)f, Ng, (const double *)d_tab);
    else
        phase_kernel<double><<<chunk_blocks(Ng), 256, 0, st>>>((double *)f, Ng, (const double *)d_tab);
    (void)n;
    FG_LAUNCHED(1);
    return OK;
}

// ---- deconvolution ------------------------------------------------------------------
int build_winv_table(double *w, int Ng) {
    w[0] = 1;
    for (int n = 1; n <= Ng / 2; ++n) {
        const double arg = M_PI * n / Ng;
        const double r = arg / sin(arg);
        const double r2 = r * r;
        w[n] = r2 * r2;
        w[Ng - n] = w[n];
    }
    return OK;
}

template <typename T>
__global__ void deconv_kernel(T *f, int Ng, const double *__restrict__ winv) {
    using T2 = vec2_t<T>;
    const int nh = Ng / 2 + 1;
    const long n = (long)Ng * Ng * nh;
    T2 *c = reinterpret_cast<T2 *>(f);
    (void)n;
    FG_FOR_MODES(Ng, nh) {
        const T2 v = c[e];
        if constexpr (sizeof(T) == 8) {
            const double w3 = __dmul_rn(__dmul_rn(winv[i], winv[j]), winv[k]);
            c[e] = mk2<T2>(__dmul_rn(v.x, w3), __dmul_rn(v.y, w3));
        } else {
            const float w3 = (float)(winv[i] * winv[j] * winv[k]);
            c[e] = mk2<T2>(v.x * w3, v.y * w3);
        }
    }
}

int apply_deconv(void *f, int Ng, int prec, const void *d_winv, cudaStream_t st) {
    const long n = (long)Ng * Ng * (Ng / 2 + 1);
    if (prec == 4)
        deconv_kernel<float><<<chunk_blocks(Ng), 256, 0, st>>>((float *)f, Ng, (const double *)d_winv);
    else
        deconv_kernel<double><<<chunk_blocks(Ng), 256, 0, st>>>((double *)f, Ng, (const double *)d_winv);
    (void)n;
    FG_LAUNCHED(1);
    return OK;
}

// ---- interlacing average --------------------------------------------------------------
template <typename T>
__global__ void average_kernel(T *f, const T *__restrict__ g, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        if constexpr (sizeof(T) == 8)
            f[e] = __dmul_rn(0.5, __dadd_rn(g[e], f[e]));
        else
            f[e] = 0.5f * (g[e] + f[e]);
    }
}

int interlace_average(void *f, const void *fdual, long n, int prec, cudaStream_t st) {
    if (prec == 4)
        average_kernel<float><<<grid_blocks(n, 256), 256, 0, st>>>((float *)f, (const float *)fdual, n);
    else
        average_kernel<double><<<grid_blocks(n, 256), 256, 0, st>>>((double *)f, (const double *)fdual, n);
    FG_LAUNCHED(1);
    return OK;
}

// ---- fused interlacing finish ---------------------------------------------------------
// A <- deconv(0.5 * (phase(B * H3) + A * H3)): the tail of src/fft.c:257-276
// (x2k scale of both grids, offset phase of the dual grid, average, PCS
// deconvolution) in one pass that reads both grids and writes one.  FP64
// evaluates each step in the reference's order.
template <typename T>
__global__ void finish_kernel(T *A, const T *__restrict__ B, int Ng, T H3, const double *__restrict__ tab,
                              const double *__restrict__ winv) {
    using T2 = vec2_t<T>;
    const int nh = Ng / 2 + 1;
    T2 *a = reinterpret_cast<T2 *>(A);
    const T2 *b = reinterpret_cast<const T2 *>(B);
    FG_FOR_MODES(Ng, nh) {
        T pr, pi;
        phase_of<T>(tab, Ng, i, j, k, pr, pi);
        const T2 bv = b[e], av = a[e];
        if constexpr (sizeof(T) == 8) {
            const double br = __dmul_rn(bv.x, H3), bi = __dmul_rn(bv.y, H3);
            const double dr = __dsub_rn(__dmul_rn(br, pr), __dmul_rn(bi, pi));
            const double di = __dadd_rn(__dmul_rn(br, pi), __dmul_rn(bi, pr));
            const double mr = __dmul_rn(0.5, __dadd_rn(dr, __dmul_rn(av.x, H3)));
            const double mi = __dmul_rn(0.5, __dadd_rn(di, __dmul_rn(av.y, H3)));
            const double w3 = __dmul_rn(__dmul_rn(winv[i], winv[j]), winv[k]);
            a[e] = mk2<T2>(__dmul_rn(mr, w3), __dmul_rn(mi, w3));
        } else {
            const float dr = bv.x * pr - bv.y * pi, di = bv.x * pi + bv.y * pr;
            const float w3 = (float)(winv[i] * winv[j] * winv[k]) * (0.5f * H3);
            a[e] = mk2<T2>((dr + av.x) * w3, (di + av.y) * w3);
        }
    }
}

// FP32: one warp per k row; the row's i and j factors are formed once and
// the per-axis tables sit in shared memory as FP32
__global__ void __launch_bounds__(256)
finish_f32_kernel(float *A, const float *__restrict__ B, int Ng, float scale, const double *__restrict__ tab,
                  const double *__restrict__ winv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *ph = reinterpret_cast<float2 *>(smem_raw);  // [3][Ng]
    float *w = reinterpret_cast<float *>(ph + 3 * Ng);   // [Ng]
    for (int e = threadIdx.x; e < 3 * Ng; e += blockDim.x)
        ph[e] = make_float2((float)tab[2 * e], (float)tab[2 * e + 1]);
    for (int e = threadIdx.x; e < Ng; e += blockDim.x) w[e] = (float)winv[e];
    __syncthreads();
    const int nh = Ng / 2 + 1, lane = threadIdx.x & 31;
    const int nwarp = blockDim.x >> 5;
    const int nrows = Ng * Ng;
    float2 *a = reinterpret_cast<float2 *>(A);
    const float2 *b = reinterpret_cast<const float2 *>(B);
    for (int row = blockIdx.x * nwarp + (threadIdx.x >> 5); row < nrows; row += gridDim.x * nwarp) {
        const int i = row / Ng, j = row - i * Ng;
        const float2 pij = cmul(ph[i], ph[Ng + j]);
        const float wij = w[i] * w[j] * scale;
        const long base = (long)row * nh;
        for (int k = lane; k < nh; k += 32) {
            const float2 p = cmul(pij, ph[2 * Ng + k]);
            const float wk = wij * w[k];
            const float2 bv = b[base + k], av = a[base + k];
            const float2 dv = cmul(bv, p);
            a[base + k] = make_float2((dv.x + av.x) * wk, (dv.y + av.y) * wk);
        }
    }
}

int interlace_finish(void *A, const void *B, int Ng, int prec, double H3, const void *d_tab,
                     const void *d_winv, cudaStream_t st) {
    if (prec == 4) {
        const size_t smem = sizeof(float2) * 3 * Ng + sizeof(float) * Ng;
        FG_CUDA(cudaFuncSetAttribute(finish_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        long nb = ceil_div((long)Ng * Ng, 8);
        if (nb > 8L * num_sms()) nb = 8L * num_sms();
        finish_f32_kernel<<<(unsigned)nb, 256, smem, st>>>((float *)A, (const float *)B, Ng, (float)(0.5 * H3),
                                                          (const double *)d_tab, (const double *)d_winv);
    } else
        finish_kernel<double><<<chunk_blocks(Ng), 256, 0, st>>>((double *)A, (const double *)B, Ng, H3,
                                                              (const double *)d_tab, (const double *)d_winv);
    FG_LAUNCHED(1);
    return OK;
}

// ---- P(): |delta|^2 / V - Pshot in place ---------------------------------------------------
template <typename T>
__global__ void power_kernel(T *f, int Ng, T Vinv, T Pshot) {
    using T2 = vec2_t<T>;
    const int nh = Ng / 2 + 1;
    const long n = (long)Ng * Ng * nh;
    T2 *c = reinterpret_cast<T2 *>(f);
    (void)n;
    FG_FOR_MODES(Ng, nh) {
        (void)i;
        (void)j;
        if (e == 0) {
            c[0] = mk2<T2>(0, 0);
            continue;
        }
        const T2 v = c[e];
        T p;
        if constexpr (sizeof(T) == 8)
            p = __dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), Vinv), Pshot);
        else
            p = (v.x * v.x + v.y * v.y) * Vinv - Pshot;
        c[e] = mk2<T2>(p, 0);
    }
}

int power_inplace(void *f, int Ng, int prec, double Vinv, double Pshot, cudaStream_t st) {
    const long n = (long)Ng * Ng * (Ng / 2 + 1);
    if (prec == 4)
        power_kernel<float><<<chunk_blocks(Ng), 256, 0, st>>>((float *)f, Ng, (float)Vinv, (float)Pshot);
    else
        power_kernel<double><<<chunk_blocks(Ng), 256, 0, st>>>((double *)f, Ng, Vinv, Pshot);
    (void)n;
    FG_LAUNCHED(1);
    return OK;
}

// ---- sub-volume window deconvolution of the real-space grid ----------------------------------
// Sub-box (src/app/Psb.c:76-83): cells (i, j, k) in (-Ngsub, Ngsub)^3, wrapped
// mod Ng (distinct cells for Ngsub <= Ng/2), times Ngsub^3 / ((Ngsub-|i|)
// (Ngsub-|j|)(Ngsub-|k|)); one thread per (i, j, k).  FP64 grids evaluate the
// factor in the reference's order; FP32 grids as a product of per-axis factors.
template <typename T>
__global__ void window_box_kernel(T *f, int Ng, int Ng_pad, int Ngsub) {
    const long n1 = 2L * Ngsub - 1, n = n1 * n1 * n1;
    const double Ngsub3 = (double)Ngsub * Ngsub * Ngsub;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e / (n1 * n1)) - (Ngsub - 1);
        const int j = (int)((e / n1) % n1) - (Ngsub - 1);
        const int k = (int)(e % n1) - (Ngsub - 1);
        T &v = f[((long)((i + Ng) % Ng) * Ng + (j + Ng) % Ng) * Ng_pad + (k + Ng) % Ng];
        if constexpr (sizeof(T) == 8) {
            const double Winv = __ddiv_rn(Ngsub3, __dmul_rn(__dmul_rn((double)(Ngsub - abs(i)), (double)(Ngsub - abs(j))),
                                                          (double)(Ngsub - abs(k))));
            v = __dmul_rn(v, Winv);
        } else {
            const float s = (float)Ngsub;
            v *= (s / (float)(Ngsub - abs(i))) * (s / (float)(Ngsub - abs(j))) * (s / (float)(Ngsub - abs(k)));
        }
    }
}

// Sub-sphere (src/app/Pss.c:72-84): index range (-Ngbnd, Ngbnd)^3 with Ngbnd =
// ceil(sqrt(3) Ngsub) > Ng/2, so some cells are reached by two images per
// axis and multiplied once per image with d2 < 0.99 D2.  One thread per cell
// applies its images in the reference's loop order (i, then j, then k
// ascending); d2_max is the largest integer d2 below 0.99 D2.
template <typename T>
__global__ void window_sphere_kernel(T *f, int Ng, int Ng_pad, int Ngbnd, double D2, long d2_max) {
    const long n = (long)Ng * Ng * Ng;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int c[3] = {(int)(e / ((long)Ng * Ng)), (int)((e / Ng) % Ng), (int)(e % Ng)};
        int img[3][2], nimg[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {  // images c - Ng, c (ascending) inside the range
            nimg[a] = 0;
            if (c[a] - Ng > -Ngbnd) img[a][nimg[a]++] = c[a] - Ng;
            if (c[a] < Ngbnd) img[a][nimg[a]++] = c[a];
        }
        if (!nimg[0] || !nimg[1] || !nimg[2]) continue;
        T &v = f[((long)c[0] * Ng + c[1]) * Ng_pad + c[2]];
        T x = v;
        for (int p = 0; p < nimg[0]; ++p)
            for (int q = 0; q < nimg[1]; ++q)
                for (int r = 0; r < nimg[2]; ++r) {
                    const long i = img[0][p], j = img[1][q], k = img[2][r];
                    const long d2i = i * i + j * j + k * k;
                    if (d2i > d2_max) continue;
                    if constexpr (sizeof(T) == 8) {
                        const double d2 = __dadd_rn(__dadd_rn((double)(i * i), (double)(j * j)), (double)(k * k));
                        const double dD = __dsqrt_rn(__ddiv_rn(d2, D2));
                        const double u = __dsub_rn(1.0, dD);
                        const double Winv =
                            __ddiv_rn(1.0, __dmul_rn(__dmul_rn(u, u), __dadd_rn(1.0, __dmul_rn(0.5, dD))));
                        x = __dmul_rn(x, Winv);
                    } else {
                        // 1 - dD = (D2 - d2) / (D2 (1 + dD)), free of the cancellation
                        // near the sphere's edge (D2 - d2 is an exact integer)
                        const float fD2 = (float)D2;
                        const float dD = sqrtf((float)d2i / fD2);
                        const float u = (float)((long)D2 - d2i) / (fD2 * (1.f + dD));
                        x *= 1.f / (u * u * (1.f + 0.5f * dD));
                    }
                }
        v = x;
    }
}

// ---- super-sample filters of the k-space field (src/app/DLsb.c:67-85, DLss.c:65-81) -------
// dst <- L_iL(mu^2) W(k) src over the half spectrum, the k = 0 real part
// zeroed and its imaginary part kept.  SPHERE: W = top hat of |n| pi sqrt(3) /
// Nsub, tab[n^2] (host-evaluated); else W = Wamp_i Wamp_j Wamp_k exp(i pi
// (i+j+k)(Ngsub-1)/Ng) from tab = Wamp[Ng] | (cos, sin)[3 Ng].  FP64 grids in
// the reference's operation order.
__device__ __forceinline__ int kval_dl(int i, int Ng) { return 2 * i < Ng ? i : i - Ng; }

template <typename T, bool SPHERE>
__global__ void dl_filter_kernel(T *dst, const T *__restrict__ src, int Ng, const double *__restrict__ tab,
                                 double l0, double l1, double l2, int iL) {
    using T2 = vec2_t<T>;
    const int nh = Ng / 2 + 1;
    const T2 *s2 = reinterpret_cast<const T2 *>(src);
    T2 *d2 = reinterpret_cast<T2 *>(dst);
    FG_FOR_MODES(Ng, nh) {
        const T2 fv = s2[e];
        if (e == 0) {
            d2[0] = mk2<T2>(0, fv.y);
            continue;
        }
        const int ki = kval_dl(i, Ng), kj = kval_dl(j, Ng), kk = kval_dl(k, Ng);
        const double n2 = (double)((long)ki * ki + (long)kj * kj + (long)kk * kk);
        if constexpr (sizeof(T) == 8) {
            const double Kamp = __dsqrt_rn(n2);
            const double num = __dadd_rn(__dadd_rn(__dmul_rn((double)ki, l0), __dmul_rn((double)kj, l1)),
                                         __dmul_rn((double)kk, l2));
            const double q = __ddiv_rn(num, Kamp);
            const double mu2 = __dmul_rn(q, q);
            const double Leg = iL == 0 ? 1.0
                               : iL == 1 ? __dsub_rn(__dmul_rn(1.5, mu2), 0.5)
                                         : __dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(4.375, mu2), 3.75), mu2), 0.375);
            if constexpr (SPHERE) {
                const double LW = __dmul_rn(Leg, tab[(long)n2]);
                d2[e] = mk2<T2>(__dmul_rn(fv.x, LW), __dmul_rn(fv.y, LW));
            } else {
                const double Wamp3 = __dmul_rn(__dmul_rn(tab[i], tab[j]), tab[k]);
                const double *ph = tab + Ng + 2 * (i + j + k);
                const double Wre = __dmul_rn(ph[0], Wamp3), Wim = __dmul_rn(ph[1], Wamp3);
                d2[e] = mk2<T2>(__dmul_rn(Leg, __dsub_rn(__dmul_rn(fv.x, Wre), __dmul_rn(fv.y, Wim))),
                                __dmul_rn(Leg, __dadd_rn(__dmul_rn(fv.x, Wim), __dmul_rn(fv.y, Wre))));
            }
        } else {
            const float q = ((float)ki * (float)l0 + (float)kj * (float)l1 + (float)kk * (float)l2) *
                            rsqrtf((float)n2);
            const float mu2 = q * q;
            const float Leg = iL == 0 ? 1.f : iL == 1 ? 1.5f * mu2 - 0.5f : (4.375f * mu2 - 3.75f) * mu2 + 0.375f;
            if constexpr (SPHERE) {
                const float LW = Leg * (float)tab[(long)n2];
                d2[e] = mk2<T2>(fv.x * LW, fv.y * LW);
            } else {
                const float Wamp3 = (float)tab[i] * (float)tab[j] * (float)tab[k];
                const double *ph = tab + Ng + 2 * (i + j + k);
                const float Wre = (float)ph[0] * Wamp3, Wim = (float)ph[1] * Wamp3;
                d2[e] = mk2<T2>(Leg * (fv.x * Wre - fv.y * Wim), Leg * (fv.x * Wim + fv.y * Wre));
            }
        }
    }
}

int dl_filter(void *dst, const void *src, int Ng, int prec, int sphere, const double *d_tab, const double los[3],
              int iL, cudaStream_t st) {
#define FG_DL(T, S)                                                                                              \
    dl_filter_kernel<T, S><<<chunk_blocks(Ng), 256, 0, st>>>((T *)dst, (const T *)src, Ng, d_tab, los[0], los[1], \
                                                            los[2], iL)
    if (prec == 4) {
        if (sphere) FG_DL(float, true); else FG_DL(float, false);
    } else {
        if (sphere) FG_DL(double, true); else FG_DL(double, false);
    }
#undef FG_DL
    FG_LAUNCHED(1);
    return OK;
}

// out[s] = F(isub*Ngsub, jsub*Ngsub, ksub*Ngsub) / bias, s = (isub*Nsub + jsub)*Nsub + ksub
template <typename T>
__global__ void dl_sample_kernel(const T *__restrict__ f, int Ng, int Nsub, double bias, double *out) {
    const int n = Nsub * Nsub * Nsub;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int Ngsub = Ng / Nsub, Ng_pad = 2 * (Ng / 2 + 1);
    const int is = s / (Nsub * Nsub), js = (s / Nsub) % Nsub, ks = s % Nsub;
    out[s] = __ddiv_rn((double)f[((long)(is * Ngsub) * Ng + js * Ngsub) * Ng_pad + ks * Ngsub], bias);
}

int dl_sample(const void *f, int Ng, int prec, int Nsub, double bias, double *d_out, cudaStream_t st) {
    const int n = Nsub * Nsub * Nsub;
    if (prec == 4)
        dl_sample_kernel<float><<<(unsigned)ceil_div(n, 128), 128, 0, st>>>((const float *)f, Ng, Nsub, bias, d_out);
    else
        dl_sample_kernel<double><<<(unsigned)ceil_div(n, 128), 128, 0, st>>>((const double *)f, Ng, Nsub, bias,
                                                                            d_out);
    FG_LAUNCHED(1);
    return OK;
}

int window_box(void *f, int Ng, int prec, int Ngsub, cudaStream_t st) {
    if (Ngsub < 1 || 2 * Ngsub > Ng) return set_error(ERR_ARG, "window_box: need 1 <= Ngsub <= Ng/2");
    const long n1 = 2L * Ngsub - 1;
    const int Ng_pad = 2 * (Ng / 2 + 1);
    if (prec == 4)
        window_box_kernel<float><<<grid_blocks(n1 * n1 * n1, 256), 256, 0, st>>>((float *)f, Ng, Ng_pad, Ngsub);
    else
        window_box_kernel<double><<<grid_blocks(n1 * n1 * n1, 256), 256, 0, st>>>((double *)f, Ng, Ng_pad, Ngsub);
    FG_LAUNCHED(1);
    return OK;
}

int window_sphere(void *f, int Ng, int prec, int Ngsub, cudaStream_t st) {
    if (Ngsub < 1 || 2 * Ngsub > Ng) return set_error(ERR_ARG, "window_sphere: need 1 <= Ngsub <= Ng/2");
    volatile double D2 = 3.0 * Ngsub * Ngsub;
    const int Ngbnd = (int)ceil(sqrt((double)D2));
    if (Ngbnd >= Ng) return set_error(ERR_ARG, "window_sphere: Ngsub too large for Ng");
    volatile double lim = 0.99 * D2;
    long d2_max = (long)floor((double)lim);
    while (d2_max >= 0 && !((double)d2_max < (double)lim)) --d2_max;  // largest integer d2 < 0.99 D2
    const int Ng_pad = 2 * (Ng / 2 + 1);
    const long n = (long)Ng * Ng * Ng;
    if (prec == 4)
        window_sphere_kernel<float><<<grid_blocks(n, 256), 256, 0, st>>>((float *)f, Ng, Ng_pad, Ngbnd, D2, d2_max);
    else
        window_sphere_kernel<double><<<grid_blocks(n, 256), 256, 0, st>>>((double *)f, Ng, Ng_pad, Ngbnd, D2,
                                                                          d2_max);
    FG_LAUNCHED(1);
    return OK;
}

// ---- precision conversion (device grid <-> pinned host view) ---------------------------------
template <typename D, typename S>
__global__ void convert_kernel(D *d, const S *__restrict__ s, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        d[e] = (D)s[e];
}

int convert_grid(void *dst, int dst_prec, const void *src, int src_prec, long n, cudaStream_t st) {
    if (dst_prec == src_prec) {
        FG_CUDA(cudaMemcpyAsync(dst, src, (size_t)n * dst_prec, cudaMemcpyDefault, st));
        return OK;
    }
    if (dst_prec == 8)
        convert_kernel<double, float><<<grid_blocks(n, 256), 256, 0, st>>>((double *)dst, (const float *)src, n);
    else
        convert_kernel<float, double><<<grid_blocks(n, 256), 256, 0, st>>>((float *)dst, (const double *)src, n);
    FG_LAUNCHED(1);
    return OK;
}

}  // namespace fg
