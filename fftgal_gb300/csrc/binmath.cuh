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

// the same with mu = num * rsqrt(n2) (a few ulp; the tie band of
// wedge_index covers it)
__device__ __forceinline__ int wedge_index_r(int ki, int kj, int kk, float rkamp, const BinDev &d, float &mu2) {
    if (d.zero_los) {
        mu2 = 0.f;
        return 0;
    }
    const float num = (float)ki * d.l0f + (float)kj * d.l1f + (float)kk * d.l2f;
    const float mu = num * rkamp;
    mu2 = mu * mu;
    const float t = fabsf(mu * (float)d.Nmu);
    const float eps = 2e-6f * (float)(d.Nmu + 1);
    const float r = rintf(t);
    if (r >= 1.f && fabsf(t - r) < eps) return wedge_exact(ki, kj, kk, d);
    return (int)t;
}

__device__ __forceinline__ int kbin_est(uint32_t n2, float kamp, const uint32_t *thr, int NK, float dKinv_f) {
    int b = (int)(kamp * dKinv_f);
    b = b < 0 ? 0 : (b > NK ? NK : b);
    while (b > 0 && n2 < thr[b]) --b;
    while (b < NK && n2 >= thr[b + 1]) ++b;
    return b;
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
