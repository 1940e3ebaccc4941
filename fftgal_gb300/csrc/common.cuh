// Device-side helpers shared by the kernels of libfftgal_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fg {

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };
template <typename T> using vec2_t = typename Vec2<T>::type;

template <typename T2>
__device__ __forceinline__ T2 mk2(decltype(T2::x) a, decltype(T2::x) b) {
    T2 r;
    r.x = a;
    r.y = b;
    return r;
}

template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) { return mk2<T2>(a.x + b.x, a.y + b.y); }
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) { return mk2<T2>(a.x - b.x, a.y - b.y); }
template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    return mk2<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T2>
__device__ __forceinline__ T2 cconj(T2 a) { return mk2<T2>(a.x, -a.y); }
// multiply by (sign * i)
template <typename T2>
__device__ __forceinline__ T2 cmul_si(T2 a, int sign) {
    return sign < 0 ? mk2<T2>(a.y, -a.x) : mk2<T2>(-a.y, a.x);
}

__host__ __device__ __forceinline__ long ceil_div(long a, long b) { return (a + b - 1) / b; }

}  // namespace fg
