// Arithmetic shared by the 2D and 3D elastic SPML propagators
// (src/fwdTimeSpmlFor2dEw.m, src/fwdTimeSpmlFor3dEw.m): the staggered
// derivative of diffOperator in its rounding order, the elementary operations
// of the strict (no fused multiply-add) and fused forms, and the damping
// factors the files form from dampPml.
#pragma once

#include <cmath>

#include "divide.cuh"
#include "sssi_gb300.h"

namespace sssi {
namespace elastic {

// sum_k c_k (f(q + s1 k + o1) - f(q - s1 k - o2)) / d in the file's rounding
// (strict) or as fused multiply-adds with w_k = c_k / d.  s1: the axis stride,
// forward (D+): f(q+(1+k)s) - f(q-ks); backward (D-): f(q+ks) - f(q-(1+k)s).
template <typename T, int N, int kMode, bool kForward>
__device__ __forceinline__ T el_diff(const T* __restrict__ f, int64_t q, int64_t s, const T* c, const T* w,
                                     const Divisor<T>& d) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const T a = __ldg(f + q + (kForward ? (1 + k) : k) * s);
        const T b = __ldg(f + q - (kForward ? k : (1 + k)) * s);
        if constexpr (kMode == SSSI_MODE_FP64_STRICT)
            acc = __dadd_rn(acc, div_rn(__dmul_rn(c[k], __dsub_rn(a, b)), d));
        else
            acc = fma(w[k], a - b, acc);
    }
    return acc;
}

template <typename T, int kMode>
__device__ __forceinline__ T el_mul(T a, T b) {
    if constexpr (kMode == SSSI_MODE_FP64_STRICT)
        return __dmul_rn(a, b);
    else
        return a * b;
}
template <typename T, int kMode>
__device__ __forceinline__ T el_add(T a, T b) {
    if constexpr (kMode == SSSI_MODE_FP64_STRICT)
        return __dadd_rn(a, b);
    else
        return a + b;
}
template <typename T, int kMode>
__device__ __forceinline__ T el_sub(T a, T b) {
    if constexpr (kMode == SSSI_MODE_FP64_STRICT)
        return __dsub_rn(a, b);
    else
        return a - b;
}
// r * x + s * y: two roundings and a sum in strict mode, one multiply-add fused
template <typename T, int kMode>
__device__ __forceinline__ T el_axpby(T r, T x, T s, T y) {
    if constexpr (kMode == SSSI_MODE_FP64_STRICT)
        return __dadd_rn(__dmul_rn(r, x), __dmul_rn(s, y));
    else
        return fma(s, y, r * x);
}
// r * x for a damping factor r that is exactly 1 outside its band: there the
// product is x itself, and the FP64 forms (bound by the FP64 pipe) do not form
// it; FP32 forms it unless kSkip32 (the same value either way: measured, the 2D
// FP32 step gains from skipping it, the 3D one loses)
template <typename T, int kMode, bool kSkip32 = false>
__device__ __forceinline__ T el_rx(bool damped, T r, T x) {
    if constexpr (kMode == SSSI_MODE_FP32 && !kSkip32)
        return r * x;
    else
        return damped ? el_mul<T, kMode>(r, x) : x;
}
// el_axpby with r = 1 outside the band (see el_rx)
template <typename T, int kMode, bool kSkip32 = false>
__device__ __forceinline__ T el_raxpby(bool damped, T r, T x, T s, T y) {
    if constexpr (kMode == SSSI_MODE_FP64_STRICT)
        return __dadd_rn(el_rx<T, kMode>(damped, r, x), __dmul_rn(s, y));
    else
        return fma(s, y, el_rx<T, kMode, kSkip32>(damped, r, x));
}
template <typename T, int kMode>
__device__ __forceinline__ T el_div(T a, T b) {
    if constexpr (kMode == SSSI_MODE_FP64_STRICT)
        return __ddiv_rn(a, b);
    else
        return a / b;
}

// The damping profile of src/dampPml.m:16-18 in its operation order,
// d = (-(3 v) / (2 L) * log(R)) * (u / L)^2, and the factors the file forms
// from it: den = 1 + 0.5 d dt, r = (1 - 0.5 d dt) / den, s = dt / den.
inline void el_band(double v, double u, double L, double dt, double& r, double& s, double& den) {
    const double d0 = -(3.0 * v) / (2.0 * L) * std::log(1e-6);
    const double qq = u / L;
    const double d = d0 * (qq * qq);
    den = 1.0 + 0.5 * d * dt;
    r = (1.0 - 0.5 * d * dt) / den;
    s = dt / den;
}

}  // namespace elastic
}  // namespace sssi
