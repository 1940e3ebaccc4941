// Learned aliasing correction: a 5 -> 64 -> 64 -> 64 -> 3 perceptron (tanh
// hidden units, linear output, FP32) that maps the single-paint multipoles of
// a k bin to the interlaced ones, and its training kernels (mean squared
// error, batch gradients, Adam).  No counterpart in the reference: the
// interlaced estimator (fft_p2k, src/fft.c:257-276) is the training target and the measure of its error.
//
// Features of bin b (fftgal_alias_features), den = |P0| + Pshot:
//   k / k_Nyq, Pshot / den, P2 / den, P4 / den, d ln den / d ln k (neighbours);
// outputs y_l with P_l^interlaced - P_l^single = den e(k / k_Nyq) y_l for
// l = 0, 2, 4, e(u) = u^6 / (1 + u^6) (fftgal_alias_envelope).  The envelope
// takes out the steep rise of the aliased power towards k_Nyq (the measured
// differences grow about as u^6 below u = 1), so one squared error weighs
// every k range alike.
//
// Parameter layout (floats): W1[5][64] b1[64] W2[64][64] b2[64] W3[64][64]
// b3[64] W4[64][3] b4[3].
#include "internal.h"
#include "common.cuh"
#include "fftgal_gb300.h"

#include <cmath>
#include <math.h>
#include <vector>

namespace fg {

constexpr int kIn = 5, kHid = 64, kOut = 3;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kIn * kHid, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid,
              kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kHid, kOffW4 = kOffB3 + kHid,
              kOffB4 = kOffW4 + kHid * kOut, kNParams = kOffB4 + kOut;
constexpr int kMlpThreads = 256, kMlpS = 32;  // samples per CTA round

// a[s][j] = act(b[j] + sum_i x[s][i] W[i][j]) for S samples, cooperatively
template <bool TANH>
__device__ __forceinline__ void mlp_layer(const float *x, int nin, const float *W, const float *b, float *a, int nout,
                                          int S) {
    for (int e = threadIdx.x; e < S * nout; e += blockDim.x) {
        const int s = e / nout, j = e - s * nout;
        float z = b[j];
        for (int i = 0; i < nin; ++i) z = fmaf(x[s * nin + i], W[i * nout + j], z);
        a[e] = TANH ? tanhf(z) : z;
    }
}

// delta of a hidden layer: d[s][i] = (sum_j dn[s][j] Wn[i][j]) (1 - a[s][i]^2)
__device__ __forceinline__ void mlp_back(const float *dn, int nn, const float *Wn, const float *a, float *d, int S) {
    for (int e = threadIdx.x; e < S * kHid; e += blockDim.x) {
        const int s = e / kHid, i = e - s * kHid;
        float g = 0.f;
        for (int j = 0; j < nn; ++j) g = fmaf(dn[s * nn + j], Wn[i * nn + j], g);
        d[e] = g * (1.f - a[e] * a[e]);
    }
}

// gW[i][j] += sum_s x[s][i] d[s][j], gb[j] += sum_s d[s][j]
__device__ __forceinline__ void mlp_accum(const float *x, int nin, const float *d, int nout, float *gW, float *gb,
                                          int S) {
    for (int e = threadIdx.x; e < nin * nout; e += blockDim.x) {
        const int i = e / nout, j = e - i * nout;
        float g = 0.f;
        for (int s = 0; s < S; ++s) g = fmaf(x[s * nin + i], d[s * nout + j], g);
        atomicAdd(&gW[e], g);
    }
    for (int j = threadIdx.x; j < nout; j += blockDim.x) {
        float g = 0.f;
        for (int s = 0; s < S; ++s) g += d[s * nout + j];
        atomicAdd(&gb[j], g);
    }
}

// grad += d/dparams of sum_s scale * |y_s - t_s|^2 (scale = 1/n for the mean), loss += that sum
__global__ void __launch_bounds__(kMlpThreads)
mlp_grad_kernel(const float *__restrict__ params, const float *__restrict__ X, const float *__restrict__ T, long n,
                float scale, float *__restrict__ grad, float *__restrict__ loss) {
    extern __shared__ __align__(16) float sm[];
    float *P = sm;                       // kNParams
    float *x0 = P + kNParams;            // [S][kIn]
    float *a1 = x0 + kMlpS * kIn;        // [S][kHid]
    float *a2 = a1 + kMlpS * kHid;
    float *a3 = a2 + kMlpS * kHid;
    float *y = a3 + kMlpS * kHid;        // [S][kOut] -> output deltas
    float *d3 = y + kMlpS * kOut;        // [S][kHid]
    float *d2 = d3 + kMlpS * kHid;
    float *d1 = d2 + kMlpS * kHid;
    __shared__ float lsum;
    for (int e = threadIdx.x; e < kNParams; e += blockDim.x) P[e] = params[e];
    if (threadIdx.x == 0) lsum = 0.f;
    __syncthreads();
    for (long s0 = (long)blockIdx.x * kMlpS; s0 < n; s0 += (long)gridDim.x * kMlpS) {
        const int S = n - s0 < kMlpS ? (int)(n - s0) : kMlpS;
        for (int e = threadIdx.x; e < S * kIn; e += blockDim.x) x0[e] = X[s0 * kIn + e];
        __syncthreads();
        mlp_layer<true>(x0, kIn, P + kOffW1, P + kOffB1, a1, kHid, S);
        __syncthreads();
        mlp_layer<true>(a1, kHid, P + kOffW2, P + kOffB2, a2, kHid, S);
        __syncthreads();
        mlp_layer<true>(a2, kHid, P + kOffW3, P + kOffB3, a3, kHid, S);
        __syncthreads();
        mlp_layer<false>(a3, kHid, P + kOffW4, P + kOffB4, y, kOut, S);
        __syncthreads();
        for (int e = threadIdx.x; e < S * kOut; e += blockDim.x) {
            const float r = y[e] - T[s0 * kOut + e];
            atomicAdd(&lsum, scale * r * r);
            y[e] = 2.f * scale * r;  // output delta
        }
        __syncthreads();
        mlp_back(y, kOut, P + kOffW4, a3, d3, S);
        __syncthreads();
        mlp_back(d3, kHid, P + kOffW3, a2, d2, S);
        __syncthreads();
        mlp_back(d2, kHid, P + kOffW2, a1, d1, S);
        __syncthreads();
        mlp_accum(a3, kHid, y, kOut, grad + kOffW4, grad + kOffB4, S);
        mlp_accum(a2, kHid, d3, kHid, grad + kOffW3, grad + kOffB3, S);
        mlp_accum(a1, kHid, d2, kHid, grad + kOffW2, grad + kOffB2, S);
        mlp_accum(x0, kIn, d1, kHid, grad + kOffW1, grad + kOffB1, S);
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, lsum);
}

__global__ void mlp_adam_kernel(float *__restrict__ params, const float *__restrict__ grad, float *__restrict__ m,
                                float *__restrict__ v, float lr, float beta1, float beta2, float eps, float c1,
                                float c2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kNParams) return;
    const float g = grad[e];
    const float mm = beta1 * m[e] + (1.f - beta1) * g;
    const float vv = beta2 * v[e] + (1.f - beta2) * g * g;
    m[e] = mm;
    v[e] = vv;
    params[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// one thread per sample: y = f(x)
__global__ void __launch_bounds__(128)
mlp_forward_kernel(const float *__restrict__ params, const float *__restrict__ X, long n, float *__restrict__ Y) {
    __shared__ float P[kNParams];
    for (int e = threadIdx.x; e < kNParams; e += blockDim.x) P[e] = params[e];
    __syncthreads();
    const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (s >= n) return;
    float a[kHid], b[kHid];
    for (int j = 0; j < kHid; ++j) {
        float z = P[kOffB1 + j];
        for (int i = 0; i < kIn; ++i) z = fmaf(X[s * kIn + i], P[kOffW1 + i * kHid + j], z);
        a[j] = tanhf(z);
    }
    for (int j = 0; j < kHid; ++j) {
        float z = P[kOffB2 + j];
        for (int i = 0; i < kHid; ++i) z = fmaf(a[i], P[kOffW2 + i * kHid + j], z);
        b[j] = tanhf(z);
    }
    for (int j = 0; j < kHid; ++j) {
        float z = P[kOffB3 + j];
        for (int i = 0; i < kHid; ++i) z = fmaf(b[i], P[kOffW3 + i * kHid + j], z);
        a[j] = tanhf(z);
    }
    for (int o = 0; o < kOut; ++o) {
        float z = P[kOffB4 + o];
        for (int i = 0; i < kHid; ++i) z = fmaf(a[i], P[kOffW4 + i * kOut + o], z);
        Y[s * kOut + o] = z;
    }
}

static size_t grad_smem() {
    return sizeof(float) * ((size_t)kNParams + kMlpS * kIn + 3 * kMlpS * kHid + kMlpS * kOut + 3 * kMlpS * kHid);
}

}  // namespace fg

using namespace fg;

extern "C" int fftgal_mlp_nparams(void) { return kNParams; }

extern "C" int fftgal_mlp_grad(const float *params, const float *X, const float *T, long n, float *grad,
                               float *loss, void *stream) {
    if (!params || !X || !T || !grad || !loss || n < 1) return set_error(ERR_ARG, "fftgal_mlp_grad: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t smem = grad_smem();
    FG_CUDA(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    long nb = ceil_div(n, kMlpS);
    if (nb > 2L * num_sms()) nb = 2L * num_sms();
    mlp_grad_kernel<<<(unsigned)nb, kMlpThreads, smem, st>>>(params, X, T, n, 1.0f / (float)n, grad, loss);
    FG_LAUNCHED(1);
    return OK;
}

extern "C" int fftgal_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr,
                               void *stream) {
    if (!params || !grad || !m || !v || step < 1) return set_error(ERR_ARG, "fftgal_mlp_adam: bad arguments");
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    mlp_adam_kernel<<<(unsigned)ceil_div(kNParams, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, grad, m, v, lr, b1, b2, 1e-8f, c1, c2);
    FG_LAUNCHED(1);
    return OK;
}

extern "C" int fftgal_mlp_forward(const float *params, const float *X, long n, float *Y, void *stream) {
    if (!params || !X || !Y || n < 1) return set_error(ERR_ARG, "fftgal_mlp_forward: bad arguments");
    mlp_forward_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(params, X, n, Y);
    FG_LAUNCHED(1);
    return OK;
}

extern "C" double fftgal_alias_envelope(double u) {
    const double u2 = u * u, u6 = u2 * u2 * u2;
    return u6 / (1.0 + u6);
}

extern "C" int fftgal_alias_features(int NK, const double *K, const double *P, double Pshot, double kNyq,
                                     float *X) {
    if (NK < 1 || !K || !P || !X || !(kNyq > 0)) return set_error(ERR_ARG, "fftgal_alias_features: bad arguments");
    std::vector<double> lden(NK), lk(NK);
    std::vector<char> ok(NK);
    for (int b = 0; b < NK; ++b) {
        const double den = fabs(P[4 * b]) + Pshot;
        ok[b] = std::isfinite(P[4 * b]) && std::isfinite(K[b]) && K[b] > 0 && den > 0;
        lden[b] = ok[b] ? log(den) : 0;
        lk[b] = ok[b] ? log(K[b]) : 0;
    }
    for (int b = 0; b < NK; ++b) {
        float *x = X + (size_t)kIn * b;
        if (!ok[b]) {
            for (int i = 0; i < kIn; ++i) x[i] = 0.f;
            continue;
        }
        const double den = fabs(P[4 * b]) + Pshot;
        int lo = b - 1, hi = b + 1;
        while (lo >= 0 && !ok[lo]) --lo;
        while (hi < NK && !ok[hi]) ++hi;
        if (lo < 0) lo = b;
        if (hi >= NK) hi = b;
        double slope = 0;
        if (hi != lo && lk[hi] != lk[lo]) slope = (lden[hi] - lden[lo]) / (lk[hi] - lk[lo]);
        slope = slope < -5 ? -5 : (slope > 5 ? 5 : slope);
        x[0] = (float)(K[b] / kNyq);
        x[1] = (float)(Pshot / den);
        x[2] = (float)(P[4 * b + 1] / den);
        x[3] = (float)(P[4 * b + 2] / den);
        x[4] = (float)slope;
    }
    return OK;
}
