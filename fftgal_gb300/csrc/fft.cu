// 3D real-to-complex FFT of the in-place padded grid layout used by the
// reference (src/fft.h:10-21: row-major [i][j][k], rows padded to
// 2*(Ng/2+1) reals), written for sm_103a.
//
// Replaces FFTW's r2c/c2r plans (src/fft.c:26-45 planning, src/fft.c:174,186
// execution) with three HBM passes per transform:
//   k axis : each CTA stages a block of contiguous rows in shared memory,
//            runs a length-Ng/2 complex FFT on the packed even/odd samples and
//            splits the result into the Ng/2+1 half-spectrum values;
//   j, i   : each CTA stages a block of C adjacent columns (C complex values
//            per memory row, coalesced) and transforms them along the strided
//            axis in shared memory.
// The in-shared-memory transform is a self-sorting mixed-radix Stockham FFT
// (radices 8, 4, 2 and the odd primes 3..13); butterflies are kept in
// registers between the read and write phases, so one shared buffer suffices.
// Conventions match FFTW: forward = exp(-2 pi i nk/N), unnormalised; the
// backward c2r ignores Im X[0] and Im X[Ng/2] of every k row.
#include "internal.h"
#include "common.cuh"

#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <vector>

namespace fg {

// radices packed 4 bits per pass (no dynamically indexed parameter array)
struct Fft1dDev {
    int n, nrad;
    unsigned long long rads;
    const void *tw;
};

static Fft1dDev to_dev(const Fft1dPlan &p) {
    Fft1dDev d;
    d.n = p.n;
    d.nrad = p.nrad;
    d.rads = 0;
    for (int i = 0; i < p.nrad; ++i) d.rads |= (unsigned long long)p.rad[i] << (4 * i);
    d.tw = p.tw;
    return d;
}

// cos/sin(2 pi m / R) for the odd prime radices, packed: R=3 @0, 5 @3, 7 @8,
// 11 @15, 13 @26
__constant__ double c_dft_cos[39];
__constant__ double c_dft_sin[39];

template <int R> struct DftOff;
template <> struct DftOff<3> { static constexpr int v = 0; };
template <> struct DftOff<5> { static constexpr int v = 3; };
template <> struct DftOff<7> { static constexpr int v = 8; };
template <> struct DftOff<11> { static constexpr int v = 15; };
template <> struct DftOff<13> { static constexpr int v = 26; };

template <typename T2>
__device__ __forceinline__ void dft2(T2 &a, T2 &b) {
    T2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <typename T2>
__device__ __forceinline__ void dft4(T2 &v0, T2 &v1, T2 &v2, T2 &v3, int sign) {
    T2 a = cadd(v0, v2), b = csub(v0, v2);
    T2 c = cadd(v1, v3), d = cmul_si(csub(v1, v3), sign);
    v0 = cadd(a, c);
    v2 = csub(a, c);
    v1 = cadd(b, d);
    v3 = csub(b, d);
}

template <int R, typename T2>
__device__ __forceinline__ void dft(T2 (&v)[R], int sign) {
    using T = decltype(T2::x);
    if constexpr (R == 2) {
        dft2(v[0], v[1]);
    } else if constexpr (R == 4) {
        dft4(v[0], v[1], v[2], v[3], sign);
    } else if constexpr (R == 8) {
        // split into even/odd outputs: a_r = v_r + v_{r+4}, b_r = (v_r - v_{r+4}) w^r
        const T h = (T)0.70710678118654752440;
        T2 a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            a[r] = cadd(v[r], v[r + 4]);
            b[r] = csub(v[r], v[r + 4]);
        }
        // w = exp(sign * 2 pi i / 8)
        b[1] = mk2<T2>(h * (b[1].x - sign * b[1].y), h * (b[1].y + sign * b[1].x));
        b[2] = cmul_si(b[2], sign);
        b[3] = mk2<T2>(h * (-b[3].x - sign * b[3].y), h * (-b[3].y + sign * b[3].x));
        dft4(a[0], a[1], a[2], a[3], sign);
        dft4(b[0], b[1], b[2], b[3], sign);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[2 * q] = a[q];
            v[2 * q + 1] = b[q];
        }
    } else {
        constexpr int off = DftOff<R>::v;
        T2 out[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            T sr = 0, si = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int m = (r * q) % R;
                const T c = (T)c_dft_cos[off + m];
                const T s = (T)(sign * c_dft_sin[off + m]);
                sr += v[r].x * c - v[r].y * s;
                si += v[r].x * s + v[r].y * c;
            }
            out[q] = mk2<T2>(sr, si);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = out[q];
    }
}

// One Stockham pass of radix R over C columns of length N held in shared
// memory at s[n * Cp + c].  Each thread holds up to EMAX/R butterflies.
template <int R, int EMAX, typename T2>
__device__ __forceinline__ void stockham_pass(T2 *s, int N, int C, int Cp, int Ns,
                                              const T2 *__restrict__ W, int sign,
                                              int tid, int nthr) {
    constexpr int NQ = EMAX / R > 0 ? EMAX / R : 1;
    const int m = N / R;
    const int total = m * C;
    const int tstep = N / (Ns * R);
    T2 v[NQ][R];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const int b = tid + q * nthr;
        if (b < total) {
            const int c = b % C, j = b / C;
            const int jm = j % Ns;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                T2 x = s[(j + r * m) * Cp + c];
                if (r > 0 && jm > 0) {
                    T2 w = W[r * jm * tstep];
                    if (sign > 0) w.y = -w.y;
                    x = cmul(x, w);
                }
                v[q][r] = x;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const int b = tid + q * nthr;
        if (b < total) {
            const int c = b % C, j = b / C;
            const int jm = j % Ns;
            dft<R>(v[q], sign);
            const int d = (j / Ns) * Ns * R + jm;
#pragma unroll
            for (int r = 0; r < R; ++r) s[(d + r * Ns) * Cp + c] = v[q][r];
        }
    }
    __syncthreads();
}

// POW2 kernels compile only the radix-8/4/2 passes (the common sizes); the
// general kernels add the odd prime radices with a smaller register budget.
template <typename T, bool POW2> struct Emax;
template <> struct Emax<float, true> { static constexpr int v = 16; };
template <> struct Emax<float, false> { static constexpr int v = 8; };
template <> struct Emax<double, true> { static constexpr int v = 8; };
template <> struct Emax<double, false> { static constexpr int v = 4; };

constexpr int kFftMaxThreads = 512;

template <typename T, bool POW2, typename T2>
__device__ void smem_fft(T2 *s, int C, int Cp, const Fft1dDev &p, int sign) {
    constexpr int EMAX = Emax<T, POW2>::v;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const T2 *W = (const T2 *)p.tw;
    int Ns = 1;
    for (int st = 0; st < p.nrad; ++st) {
        const int R = (int)((p.rads >> (4 * st)) & 15ull);
        if (R == 8) stockham_pass<8, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
        else if (R == 4) stockham_pass<4, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
        else if (R == 2) stockham_pass<2, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
        else if constexpr (!POW2) {
            if (R == 3) stockham_pass<3, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
            else if (R == 5) stockham_pass<5, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
            else if (R == 7) stockham_pass<7, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
            else if (R == 11) stockham_pass<11, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
            else if (R == 13) stockham_pass<13, EMAX>(s, p.n, C, Cp, Ns, W, sign, tid, nthr);
        }
        Ns *= R;
    }
}

// ---- strided-axis (j or i) complex transform ---------------------------------
// Column block (batch, cb) of grid blockIdx.y: columns [cb*C, cb*C + C) of
// the complex half-spectrum rows; element n of column c at
// base + batch*batch_stride + n*elem_stride + c (complex units).
template <typename T, bool POW2>
__global__ void __launch_bounds__(kFftMaxThreads) fft_cols_kernel(vec2_t<T> *g0, vec2_t<T> *g1, int ncols, long elem_stride,
                                long batch_stride, int C, Fft1dDev p, int sign) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *s = reinterpret_cast<T2 *>(smem_raw);
    const int N = p.n;
    const int ncb = (ncols + C - 1) / C;
    const int cb = blockIdx.x % ncb;
    const long batch = blockIdx.x / ncb;
    T2 *g = blockIdx.y == 0 ? g0 : g1;
    const int c0 = cb * C;
    const int cvalid = min(C, ncols - c0);
    T2 *base = g + batch * batch_stride + c0;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int e = tid; e < N * C; e += nthr) {
        const int n = e / C, c = e % C;
        T2 v = mk2<T2>(0, 0);
        if (c < cvalid) v = base[n * elem_stride + c];
        s[n * C + c] = v;
    }
    __syncthreads();
    smem_fft<T, POW2>(s, C, C, p, sign);
    for (int e = tid; e < N * C; e += nthr) {
        const int n = e / C, c = e % C;
        if (c < cvalid) base[n * elem_stride + c] = s[n * C + c];
    }
}

// ---- k axis, forward r2c ---------------------------------------------------------
// R rows per CTA; shared layout s[m * (R+1) + r].  Even Ng: packed length
// Ng/2 transform plus the split X[k] = E[k] + W^k O[k]; odd Ng: full-length
// transform of the real row.
template <typename T, bool POW2>
__global__ void __launch_bounds__(kFftMaxThreads) fft_k_r2c_kernel(T *g0, T *g1, long nrows, int Ng, int Ng_pad, int R,
                                 Fft1dDev p, const vec2_t<T> *__restrict__ rtw) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *s = reinterpret_cast<T2 *>(smem_raw);
    const int Rp = R + 1;
    const bool even = (Ng % 2) == 0;
    const int Nc = p.n;  // Ng/2 (even) or Ng (odd)
    const int nh = Ng / 2 + 1;
    T *g = blockIdx.y == 0 ? g0 : g1;
    const long row0 = (long)blockIdx.x * R;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int e = tid; e < Nc * R; e += nthr) {
        const int r = e / Nc, m = e % Nc;
        T2 v = mk2<T2>(0, 0);
        if (row0 + r < nrows) {
            const T *row = g + (row0 + r) * Ng_pad;
            if (even)
                v = reinterpret_cast<const T2 *>(row)[m];
            else
                v = mk2<T2>(row[m], (T)0);
        }
        s[m * Rp + r] = v;
    }
    __syncthreads();
    smem_fft<T, POW2>(s, R, Rp, p, -1);
    for (int e = tid; e < nh * R; e += nthr) {
        const int r = e / nh, k = e % nh;
        if (row0 + r >= nrows) continue;
        T2 X;
        if (even) {
            const int k1 = k % Nc, k2 = (Nc - k) % Nc;
            const T2 z1 = s[k1 * Rp + r];
            const T2 z2 = cconj(s[k2 * Rp + r]);
            const T2 E = mk2<T2>((T)0.5 * (z1.x + z2.x), (T)0.5 * (z1.y + z2.y));
            const T2 D = csub(z1, z2);
            const T2 O = mk2<T2>((T)0.5 * D.y, (T)-0.5 * D.x);
            X = cadd(E, cmul(rtw[k], O));
        } else {
            X = s[k * Rp + r];
        }
        reinterpret_cast<T2 *>(g + (row0 + r) * Ng_pad)[k] = X;
    }
}

// ---- k axis, backward c2r ------------------------------------------------------------
template <typename T, bool POW2>
__global__ void __launch_bounds__(kFftMaxThreads) fft_k_c2r_kernel(T *g0, T *g1, long nrows, int Ng, int Ng_pad, int R,
                                 Fft1dDev p, const vec2_t<T> *__restrict__ rtw) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *s = reinterpret_cast<T2 *>(smem_raw);
    const int Rp = R + 1;
    const bool even = (Ng % 2) == 0;
    const int Nc = p.n;
    const int nh = Ng / 2 + 1;
    T *g = blockIdx.y == 0 ? g0 : g1;
    const long row0 = (long)blockIdx.x * R;
    const int tid = threadIdx.x, nthr = blockDim.x;
    if (even) {
        for (int e = tid; e < nh * R; e += nthr) {
            const int r = e / nh, k = e % nh;
            T2 v = mk2<T2>(0, 0);
            if (row0 + r < nrows) v = reinterpret_cast<const T2 *>(g + (row0 + r) * Ng_pad)[k];
            s[k * Rp + r] = v;
        }
        __syncthreads();
        // Z[k] = A[k] + i B[k], A = X[k] + X[k+h], B = (X[k] - X[k+h]) e^{+2 pi i k/Ng},
        // X[k+h] = conj X[h-k]; pairs (k, Nc-k) handled by one thread
        const int npair = Nc / 2 + 1;
        for (int e = tid; e < npair * R; e += nthr) {
            const int r = e / npair, k = e % npair;
            const int k2 = Nc - k;
            T2 xa = s[k * Rp + r], xb = s[k2 * Rp + r];
            if (k == 0) { xa.y = 0; xb.y = 0; }
            // Z[k]
            {
                const T2 y = cconj(xb);
                const T2 A = cadd(xa, y);
                const T2 B = cmul(csub(xa, y), cconj(rtw[k]));
                s[k * Rp + r] = mk2<T2>(A.x - B.y, A.y + B.x);
            }
            if (k2 != k && k2 < Nc) {
                const T2 y = cconj(xa);
                const T2 A = cadd(xb, y);
                const T2 B = cmul(csub(xb, y), cconj(rtw[k2]));
                s[k2 * Rp + r] = mk2<T2>(A.x - B.y, A.y + B.x);
            }
        }
    } else {
        for (int e = tid; e < nh * R; e += nthr) {
            const int r = e / nh, k = e % nh;
            T2 v = mk2<T2>(0, 0);
            if (row0 + r < nrows) v = reinterpret_cast<const T2 *>(g + (row0 + r) * Ng_pad)[k];
            if (k == 0) v.y = 0;
            s[k * Rp + r] = v;
            if (k > 0) s[(Ng - k) * Rp + r] = cconj(v);
        }
    }
    __syncthreads();
    smem_fft<T, POW2>(s, R, Rp, p, +1);
    for (int e = tid; e < Nc * R; e += nthr) {
        const int r = e / Nc, m = e % Nc;
        if (row0 + r >= nrows) continue;
        T *row = g + (row0 + r) * Ng_pad;
        const T2 z = s[m * Rp + r];
        if (even)
            reinterpret_cast<T2 *>(row)[m] = z;
        else
            row[m] = z.x;
    }
}

// ---- planner ---------------------------------------------------------------------------

static int factor_radices(int n, int *rad) {
    int k = 0;
    while (n % 8 == 0) { rad[k++] = 8; n /= 8; }
    while (n % 4 == 0) { rad[k++] = 4; n /= 4; }
    while (n % 2 == 0) { rad[k++] = 2; n /= 2; }
    const int odd[] = {3, 5, 7, 11, 13};
    for (int f : odd)
        while (n % f == 0) { rad[k++] = f; n /= f; }
    return n == 1 ? k : -1;
}

static int plan1d(Fft1dPlan *p, int n, int prec) {
    p->n = n;
    p->nrad = factor_radices(n, p->rad);
    if (p->nrad < 0)
        return set_error(ERR_UNSUPPORTED,
                         "FFT length %d has a prime factor above 13 (supported: 2,3,5,7,11,13)", n);
    std::vector<double> tw(2 * (size_t)n);
    for (int t = 0; t < n; ++t) {
        const double a = 2.0 * M_PI * (double)t / (double)n;
        tw[2 * t] = cos(a);
        tw[2 * t + 1] = -sin(a);
    }
    const size_t es = 2 * (size_t)prec;
    FG_CUDA(cudaMalloc(&p->tw, es * n));
    if (prec == 8) {
        FG_CUDA(cudaMemcpy(p->tw, tw.data(), es * n, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(2 * (size_t)n);
        for (size_t i = 0; i < f.size(); ++i) f[i] = (float)tw[i];
        FG_CUDA(cudaMemcpy(p->tw, f.data(), es * n, cudaMemcpyHostToDevice));
    }
    return OK;
}

static bool is_pow2_plan(const Fft1dPlan &p) {
    for (int i = 0; i < p.nrad; ++i)
        if (p.rad[i] != 2 && p.rad[i] != 4 && p.rad[i] != 8) return false;
    return true;
}

static int emax_of(int prec, bool pow2) {
    if (prec == 4) return pow2 ? Emax<float, true>::v : Emax<float, false>::v;
    return pow2 ? Emax<double, true>::v : Emax<double, false>::v;
}

// every radix pass of the plan fits the per-thread register budget
static bool fits(const Fft1dPlan &p, int C, int nthr, int emax) {
    for (int i = 0; i < p.nrad; ++i) {
        const int R = p.rad[i];
        const long need = ceil_div((long)(p.n / R) * C, nthr);
        const int nq = emax / R > 0 ? emax / R : 1;
        if (need > nq) return false;
    }
    return true;
}

// choose (C, threads) for a transform of length n over C columns whose
// shared footprint is (n + extra) * (C + pad) elements
static int choose_shape(const Fft1dPlan &p, int prec, int cmax, int pad, int extra,
                        int *C_out, int *thr_out, size_t *smem_out) {
    const int emax = emax_of(prec, is_pow2_plan(p));
    const size_t es = 2 * (size_t)prec;
    const size_t budget = 200 * 1024;
    int C = cmax;
    while (C > 1 && (size_t)(p.n + extra) * (C + pad) * es > budget) C /= 2;
    int nthr = 64;
    while (nthr < kFftMaxThreads && !fits(p, C, nthr, emax)) nthr *= 2;
    while (!fits(p, C, nthr, emax) && C > 1) C /= 2;
    if (!fits(p, C, nthr, emax) || (size_t)(p.n + extra) * (C + pad) * es > budget)
        return set_error(ERR_UNSUPPORTED, "FFT length %d does not fit one CTA", p.n);
    *C_out = C;
    *thr_out = nthr;
    *smem_out = (size_t)(p.n + extra) * (C + pad) * es;
    return OK;
}

static bool g_const_ready = false;

template <typename T, bool P2>
static int opt_in_smem() {
    FG_CUDA(cudaFuncSetAttribute(fft_cols_kernel<T, P2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    FG_CUDA(cudaFuncSetAttribute(fft_k_r2c_kernel<T, P2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    FG_CUDA(cudaFuncSetAttribute(fft_k_c2r_kernel<T, P2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    return OK;
}

int fft_plan_create(FftPlan *p, int Ng, int prec) {
    if (Ng < 2) return set_error(ERR_ARG, "Ng must be >= 2 (got %d)", Ng);
    if (prec != 4 && prec != 8) return set_error(ERR_ARG, "precision must be 4 or 8");
    if (!g_const_ready) {
        double cs[39], sn[39];
        const int Rs[] = {3, 5, 7, 11, 13};
        int off = 0;
        for (int R : Rs) {
            for (int m = 0; m < R; ++m) {
                cs[off + m] = cos(2.0 * M_PI * m / R);
                sn[off + m] = sin(2.0 * M_PI * m / R);
            }
            off += R;
        }
        FG_CUDA(cudaMemcpyToSymbol(c_dft_cos, cs, sizeof(cs)));
        FG_CUDA(cudaMemcpyToSymbol(c_dft_sin, sn, sizeof(sn)));
        FG_TRY((opt_in_smem<float, true>()));
        FG_TRY((opt_in_smem<float, false>()));
        FG_TRY((opt_in_smem<double, true>()));
        FG_TRY((opt_in_smem<double, false>()));
        g_const_ready = true;
    }
    p->prec = prec;
    p->Ng = Ng;
    p->nh = Ng / 2 + 1;
    p->even = (Ng % 2) == 0;
    FG_TRY(plan1d(&p->axis, Ng, prec));
    if (p->even) FG_TRY(plan1d(&p->half, Ng / 2, prec));
    // r2c split twiddles exp(-2 pi i k / Ng), k <= Ng/2
    const int nr = Ng / 2 + 1;
    std::vector<double> rt(2 * (size_t)nr);
    for (int k = 0; k < nr; ++k) {
        const double a = 2.0 * M_PI * (double)k / (double)Ng;
        rt[2 * k] = cos(a);
        rt[2 * k + 1] = -sin(a);
    }
    const size_t es = 2 * (size_t)prec;
    FG_CUDA(cudaMalloc(&p->rtw, es * nr));
    if (prec == 8) {
        FG_CUDA(cudaMemcpy(p->rtw, rt.data(), es * nr, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(rt.size());
        for (size_t i = 0; i < f.size(); ++i) f[i] = (float)rt[i];
        FG_CUDA(cudaMemcpy(p->rtw, f.data(), es * nr, cudaMemcpyHostToDevice));
    }
    const int cmax = prec == 4 ? 16 : 8;
    FG_TRY(choose_shape(p->axis, prec, cmax, 0, 0, &p->cols, &p->col_threads, &p->col_smem));
    const Fft1dPlan &kp = p->even ? p->half : p->axis;
    FG_TRY(choose_shape(kp, prec, cmax, 1, 1, &p->rows, &p->row_threads, &p->row_smem));
    return OK;
}

void fft_plan_destroy(FftPlan *p) {
    cudaFree(p->axis.tw);
    cudaFree(p->half.tw);
    cudaFree(p->rtw);
    p->axis.tw = p->half.tw = p->rtw = nullptr;
}

template <typename T, bool P2>
static void launch_k(bool forward, dim3 grid, const FftPlan *p, void *g0, void *g1, long nrows,
                     const Fft1dDev &d, cudaStream_t s) {
    using T2 = vec2_t<T>;
    const int Ng = p->Ng, Ng_pad = 2 * p->nh;
    if (forward)
        fft_k_r2c_kernel<T, P2><<<grid, p->row_threads, p->row_smem, s>>>((T *)g0, (T *)g1, nrows, Ng, Ng_pad,
                                                                         p->rows, d, (const T2 *)p->rtw);
    else
        fft_k_c2r_kernel<T, P2><<<grid, p->row_threads, p->row_smem, s>>>((T *)g0, (T *)g1, nrows, Ng, Ng_pad,
                                                                         p->rows, d, (const T2 *)p->rtw);
}

static int k_pass(const FftPlan *p, void *const *grids, int ngrids, bool forward, cudaStream_t s) {
    if (forward && fft2_supported(p->Ng, p->prec))
        return fft2_k_r2c(p->Ng, p->half.tw, p->rtw, grids[0], ngrids > 1 ? grids[1] : grids[0], ngrids, s,
                          p->tune[0]);
    const long nrows = (long)p->Ng * p->Ng;
    const Fft1dPlan &kp = p->even ? p->half : p->axis;
    const Fft1dDev d = to_dev(kp);
    dim3 grid((unsigned)ceil_div(nrows, p->rows), ngrids);
    void *g1 = ngrids > 1 ? grids[1] : grids[0];
    const bool p2 = is_pow2_plan(kp);
    if (p->prec == 4) {
        if (p2) launch_k<float, true>(forward, grid, p, grids[0], g1, nrows, d, s);
        else launch_k<float, false>(forward, grid, p, grids[0], g1, nrows, d, s);
    } else {
        if (p2) launch_k<double, true>(forward, grid, p, grids[0], g1, nrows, d, s);
        else launch_k<double, false>(forward, grid, p, grids[0], g1, nrows, d, s);
    }
    FG_LAUNCHED(1);
    return OK;
}

int fft_pass_k_r2c(const FftPlan *p, void *const *grids, int ngrids, cudaStream_t s) {
    return k_pass(p, grids, ngrids, true, s);
}

template <typename T, bool P2>
static void launch_cols(dim3 grid, const FftPlan *p, void *g0, void *g1, long elem_stride, long batch_stride,
                        const Fft1dDev &d, int sign, cudaStream_t s) {
    using T2 = vec2_t<T>;
    fft_cols_kernel<T, P2><<<grid, p->col_threads, p->col_smem, s>>>((T2 *)g0, (T2 *)g1, p->nh, elem_stride,
                                                                     batch_stride, p->cols, d, sign);
}

static int cols_pass(const FftPlan *p, void *const *grids, int ngrids, int sign,
                     long elem_stride, long batch_stride, cudaStream_t s, int logC) {
    if (fft2_supported(p->Ng, p->prec))
        return fft2_cols(p->Ng, p->axis.tw, grids[0], ngrids > 1 ? grids[1] : grids[0], ngrids, p->nh,
                         elem_stride, batch_stride, p->Ng, sign, s, logC);
    const Fft1dDev d = to_dev(p->axis);
    const long ncb = ceil_div(p->nh, p->cols);
    dim3 grid((unsigned)(ncb * p->Ng), ngrids);
    void *g1 = ngrids > 1 ? grids[1] : grids[0];
    const bool p2 = is_pow2_plan(p->axis);
    if (p->prec == 4) {
        if (p2) launch_cols<float, true>(grid, p, grids[0], g1, elem_stride, batch_stride, d, sign, s);
        else launch_cols<float, false>(grid, p, grids[0], g1, elem_stride, batch_stride, d, sign, s);
    } else {
        if (p2) launch_cols<double, true>(grid, p, grids[0], g1, elem_stride, batch_stride, d, sign, s);
        else launch_cols<double, false>(grid, p, grids[0], g1, elem_stride, batch_stride, d, sign, s);
    }
    FG_LAUNCHED(1);
    return OK;
}

int fft_pass_j(const FftPlan *p, void *const *grids, int ngrids, int sign, cudaStream_t s) {
    return cols_pass(p, grids, ngrids, sign, p->nh, (long)p->Ng * p->nh, s, p->tune[1]);
}

int fft_pass_i(const FftPlan *p, void *const *grids, int ngrids, int sign, cudaStream_t s) {
    if (fft2_tma_supported(p->Ng, p->prec))
        return fft2_cols_tma(p->Ng, p->axis.tw, grids[0], ngrids > 1 ? grids[1] : grids[0], ngrids, sign, s);
    return cols_pass(p, grids, ngrids, sign, (long)p->Ng * p->nh, p->nh, s, p->tune[2]);
}

int fft_r2c(const FftPlan *p, void *const *grids, int ngrids, cudaStream_t s) {
    FG_TRY(fft_pass_k_r2c(p, grids, ngrids, s));
    FG_TRY(fft_pass_j(p, grids, ngrids, -1, s));
    FG_TRY(fft_pass_i(p, grids, ngrids, -1, s));
    return OK;
}

int fft_c2r(const FftPlan *p, void *const *grids, int ngrids, cudaStream_t s) {
    FG_TRY(fft_pass_i(p, grids, ngrids, +1, s));
    FG_TRY(fft_pass_j(p, grids, ngrids, +1, s));
    return k_pass(p, grids, ngrids, false, s);
}

}  // namespace fg
