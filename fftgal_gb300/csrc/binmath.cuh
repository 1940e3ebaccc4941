// Per-mode classification shared by the binning kernels (bins.cu) and the
// allocation-free binning entry point (noalloc.cu): the k bin from exact n^2
// thresholds, the wedge from an FP32 estimate with an FP64 fallback inside its
// error band.  Both files use these same functions, so their mode counts agree.
#pragma once

#include "internal.h"
#include "common.cuh"

namespace fg {

struct BinDev {
    int Ng, nh, NK, Nmu, W;     // W = Nmu + 1 wedge slots
    float dKinv_f;
    double l0, l1, l2;
    float l0f, l1f, l2f;
    bool zero_los;
};

// signed wavenumber index of grid index i: the reference's Kval table
// (src/power.c:46-51), where the even-Ng Nyquist entry ends up as -Ng/2
__device__ __forceinline__ int kval(int i, int Ng) { return 2 * i < Ng ? i : i - Ng; }

__device__ __forceinline__ int kbin(uint32_t n2, const uint32_t *thr, int NK, float dKinv_f) {
    int b = (int)(sqrtf((float)n2) * dKinv_f);
    b = b < 0 ? 0 : (b > NK ? NK : b);
    while (b > 0 && n2 < thr[b]) --b;
    while (b < NK && n2 >= thr[b + 1]) ++b;
    return b;  // == NK means beyond the last bin
}

// exact wedge index, reference expression (src/power.c:131-134)
__device__ __forceinline__ int wedge_exact(int ki, int kj, int kk, const BinDev &d) {
    const double a = (double)ki, b = (double)kj, c = (double)kk;
    const double kamp = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c)));
    const double num = __dadd_rn(__dadd_rn(__dmul_rn(a, d.l0), __dmul_rn(b, d.l1)), __dmul_rn(c, d.l2));
    const double mu = __ddiv_rn(num, kamp);
    return (int)floor(fabs(__dmul_rn(mu, (double)d.Nmu)));
}

// wedge index and mu^2 (FP32) for one mode
__device__ __forceinline__ int wedge_index(int ki, int kj, int kk, float kamp, const BinDev &d,
                                           float &mu2) {
    if (d.zero_los) {
        mu2 = 0.f;
        return 0;
    }
    const float num = (float)ki * d.l0f + (float)kj * d.l1f + (float)kk * d.l2f;
    const float mu = num / kamp;
    mu2 = mu * mu;
    const float t = fabsf(mu * (float)d.Nmu);
    const float eps = 2e-6f * (float)(d.Nmu + 1);
    const float r = rintf(t);
    if (r >= 1.f && fabsf(t - r) < eps) return wedge_exact(ki, kj, kk, d);
    return (int)t;
}

// the same with mu = num * rsqrt(n2), num = k . los in FP32 in any order of
// its three terms (a few ulp of the largest term; the tie band of
// wedge_index covers it)
__device__ __forceinline__ int wedge_num_r(float num, int ki, int kj, int kk, float rkamp, const BinDev &d,
                                           float &mu2) {
    if (d.zero_los) {
        mu2 = 0.f;
        return 0;
    }
    const float mu = num * rkamp;
    mu2 = mu * mu;
    const float t = fabsf(mu * (float)d.Nmu);
    const float eps = 2e-6f * (float)(d.Nmu + 1);
    const float r = rintf(t);
    if (r >= 1.f && fabsf(t - r) < eps) return wedge_exact(ki, kj, kk, d);
    return (int)t;
}

__device__ __forceinline__ int wedge_index_r(int ki, int kj, int kk, float rkamp, const BinDev &d, float &mu2) {
    const float num = (float)ki * d.l0f + (float)kj * d.l1f + (float)kk * d.l2f;
    return wedge_num_r(num, ki, kj, kk, rkamp, d, mu2);
}

__device__ __forceinline__ int kbin_est(uint32_t n2, float kamp, const uint32_t *thr, int NK, float dKinv_f) {
    int b = (int)(kamp * dKinv_f);
    b = b < 0 ? 0 : (b > NK ? NK : b);
    while (b > 0 && n2 < thr[b]) --b;
    while (b < NK && n2 >= thr[b + 1]) ++b;
    return b;
}

// One thread's run of modes whose k bin changes rarely (a run along the
// grid axis with the smallest |n_a|): the run's sums of P L_l(mu^2), l = 0, 2,
// 4, 6, and of P per wedge stay in registers and are added to the CTA's FP32
// shared accumulators acc32 [4 + W][NK] when the bin or the wedge changes.
struct BinRun {
    int cb = -1, cm = -1;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, sw = 0.f;

    __device__ __forceinline__ void flush_bin(float *acc32, int NK) {
        if (cb >= 0) {
            atomicAdd(acc32 + 0 * NK + cb, s0);
            atomicAdd(acc32 + 1 * NK + cb, s1);
            atomicAdd(acc32 + 2 * NK + cb, s2);
            atomicAdd(acc32 + 3 * NK + cb, s3);
            atomicAdd(acc32 + (4 + cm) * NK + cb, sw);
        }
    }
    // mode (ki, kj, kk) of the half spectrum, raw k index kraw (its count is
    // 1 + (2 kraw % Ng > 0), src/power.c:57), power p; not the k = 0 mode
    __device__ __forceinline__ void add(const BinDev &d, const uint32_t *thr, float *acc32, int ki, int kj, int kk,
                                        int kraw, float p) {
        const uint32_t n2 = (uint32_t)(ki * ki + kj * kj + kk * kk);
        const float pc = (kraw != 0 && 2 * kraw != d.Ng) ? 2.f * p : p;
        const float num = (float)ki * d.l0f + (float)kj * d.l1f + (float)kk * d.l2f;
        add_mode(d, thr, acc32, n2, num, pc, ki, kj, kk);
    }
    // the same with n^2, k . los (FP32) and the counted power pc given
    __device__ __forceinline__ void add_mode(const BinDev &d, const uint32_t *thr, float *acc32, uint32_t n2,
                                             float num, float pc, int ki, int kj, int kk) {
        const int NK = d.NK;
        const float n2f = (float)n2;
        const float rk = rsqrtf(n2f);
        int b = kbin_est(n2, n2f * rk, thr, NK, d.dKinv_f);
        if (b >= NK) b = -1;
        float m2;
        const int imu = wedge_num_r(num, ki, kj, kk, rk, d, m2);
        // one flush block for a new bin (all five sums) and a new wedge (its
        // sum), so a warp whose lanes see both runs it once
        const bool newbin = b != cb;
        if (newbin || imu != cm) {
            if (cb >= 0) {
                if (newbin) {
                    atomicAdd(acc32 + 0 * NK + cb, s0);
                    atomicAdd(acc32 + 1 * NK + cb, s1);
                    atomicAdd(acc32 + 2 * NK + cb, s2);
                    atomicAdd(acc32 + 3 * NK + cb, s3);
                }
                atomicAdd(acc32 + (4 + cm) * NK + cb, sw);
            }
            if (newbin) {
                cb = b;
                s0 = s1 = s2 = s3 = 0.f;
            }
            cm = imu;
            sw = 0.f;
        }
        s0 += pc;
        s1 += pc * (1.5f * m2 - 0.5f);
        s2 += pc * ((4.375f * m2 - 3.75f) * m2 + 0.375f);
        s3 += pc * (((14.4375f * m2 - 19.6875f) * m2 + 6.5625f) * m2 - 0.3125f);
        sw += pc;
    }
    __device__ __forceinline__ void finish(const BinDev &d, float *acc32) { flush_bin(acc32, d.NK); }
};

// One thread's run of up to 16 modes along grid axis AX (0: i, 1: j, 2: k)
// from mode (i, j, kc) (grid indices; kc < Ng/2 + 1), the t-th of whose
// powers is p[t * ps]; the first n lie inside the half spectrum.  The two
// fixed coordinates' parts of n^2 and of k . los are formed once per run.
template <int AX>
__device__ __forceinline__ void bin_run(const BinDev &d, const uint32_t *thr, float *acc32, int i, int j, int kc,
                                        int n, const float *p, int ps) {
    const int Ng = d.Ng;
    BinRun run;
    if (AX == 2) {
        const int ki = kval(i, Ng), kj = kval(j, Ng);
        const uint32_t n2c = (uint32_t)(ki * ki + kj * kj);
        const float numc = (float)ki * d.l0f + (float)kj * d.l1f;
        for (int t = 0; t < n; ++t) {
            const int kr = kc + t, kk = kval(kr, Ng);
            const uint32_t n2 = n2c + (uint32_t)(kk * kk);
            if (n2 == 0) continue;  // the k = 0 mode (src/power.c:52-54)
            const float pv = p[t * ps];
            const float pc = (kr != 0 && 2 * kr != Ng) ? 2.f * pv : pv;
            run.add_mode(d, thr, acc32, n2, numc + (float)kk * d.l2f, pc, ki, kj, kk);
        }
    } else {
        const int kk = kval(kc, Ng), kf = kval(AX == 0 ? j : i, Ng);  // the fixed k and the other fixed index
        const float fac = (kc != 0 && 2 * kc != Ng) ? 2.f : 1.f;
        const uint32_t n2c = (uint32_t)(kk * kk + kf * kf);
        const float numc = (float)kf * (AX == 0 ? d.l1f : d.l0f) + (float)kk * d.l2f;
        const float lv = AX == 0 ? d.l0f : d.l1f;
        const int v0 = AX == 0 ? i : j;
        for (int t = 0; t < n; ++t) {
            const int kv = kval(v0 + t, Ng);
            const uint32_t n2 = n2c + (uint32_t)(kv * kv);
            if (n2 == 0) continue;
            run.add_mode(d, thr, acc32, n2, numc + (float)kv * lv, fac * p[t * ps], AX == 0 ? kv : kf,
                         AX == 0 ? kf : kv, kk);
        }
    }
    run.finish(d, acc32);
}

// fold a CTA's FP32 shared sums [NQ][NK] into the FP64 global sums [NK][NQ]
// and clear them (every thread of the CTA takes part; the caller synchronises)
__device__ __forceinline__ void bin_fold(float *acc32, double *gacc, int NK, int NQ) {
    for (int e = threadIdx.x; e < NK * NQ; e += blockDim.x) {
        const float v = acc32[e];
        if (v != 0.f) {
            const int q = e / NK, b = e - q * NK;
            atomicAdd(&gacc[(size_t)b * NQ + q], (double)v);
            acc32[e] = 0.f;
        }
    }
}

static inline BinDev make_dev(const BinSpec &s) {
    BinDev d;
    d.Ng = s.Ng;
    d.nh = s.Ng / 2 + 1;
    d.NK = s.NK;
    d.Nmu = s.Nmu;
    d.W = s.Nmu + 1;
    d.dKinv_f = (float)s.dKinv;
    d.l0 = s.los[0];
    d.l1 = s.los[1];
    d.l2 = s.los[2];
    d.l0f = (float)s.los[0];
    d.l1f = (float)s.los[1];
    d.l2f = (float)s.los[2];
    d.zero_los = (s.los[0] == 0 && s.los[1] == 0 && s.los[2] == 0);
    return d;
}

}  // namespace fg
