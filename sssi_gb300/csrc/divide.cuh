// Correctly rounded division by a divisor that stays fixed over a whole run
// (a grid spacing), as used by the strict FP64 forms, which divide every
// stencil term by the spacing (finiteDifference.c:116-117,
// diffOperator_mex.c:120-213, fwdTimeSpmlFor2dEw.m through diffOperator).
//
// With r = RN(1/d) rounded once on the host, Markstein's correction step
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1):111-119, 1990; see also
// J.-M. Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed., 2018,
// on division with a fused multiply-add) gives a candidate quotient
//     q0 = RN(a r),   e0 = a - d q0 (one FMA),   q1 = RN(q0 + e0 r).
// q1 is then checked, not trusted: its remainder e1 = RN(a - d q1) (one FMA)
// must be smaller than |d| times half the distance from q1 to the next double
// on the side of the exact quotient (a quarter of q1's spacing below a power
// of two).  That bound is a power-of-two multiple of |d|, an exact double, and
// rounding is monotonic, so a remainder at or beyond it never passes; a
// remainder below it puts a / d strictly inside q1's rounding interval, so
// q1 = RN(a / d).  A zero dividend gives its signed zero directly; every
// other case (a tie, non-finite or extreme operands) takes the IEEE division.
// The result is always the IEEE quotient, bit for bit; only the work differs
// (one multiply and three FMAs in the common case).
#pragma once

#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

namespace sssi {

template <typename T>
struct Divisor;

// FP32 has no strict form: the divisor only travels with the parameters.
template <>
struct Divisor<float> {
    float d;
};

template <>
struct Divisor<double> {
    double d, r;        // divisor and RN(1/d)
    unsigned dmant_hi;  // high word of d without sign and exponent
    unsigned dlo;       // low word of d
    int dexp;           // biased exponent of d
    int dsign;          // sign bit of d (as the high word's sign)
    int qlo, qhi;       // biased exponents of q1 whose check bounds are normal doubles (empty: no fast path)
    int zero_ok;        // d is neither zero nor NaN: a zero dividend gives a signed zero
};

inline Divisor<float> make_divisor_f32(double d) { return {static_cast<float>(d)}; }

inline Divisor<double> make_divisor_f64(double d) {
    Divisor<double> v{};
    v.d = d;
    v.r = 1.0 / d;  // IEEE division on the host: correctly rounded
    uint64_t bits;
    std::memcpy(&bits, &d, sizeof bits);
    const int e = static_cast<int>((bits >> 52) & 0x7ff);
    v.dexp = e;
    v.dmant_hi = static_cast<unsigned>(bits >> 32) & 0x000fffffu;
    v.dlo = static_cast<unsigned>(bits);
    v.dsign = static_cast<int>(static_cast<unsigned>(bits >> 32) & 0x80000000u);
    v.zero_ok = d != 0.0 && d == d;
    // the bound |d| 2^(eq - 1076) (half of q1's spacing; one less for a quarter)
    // has biased exponent dexp + eq - 1076: keep it in [2, 2046]
    if (e > 0 && e < 0x7ff) {
        v.qlo = 1078 - e > 1 ? 1078 - e : 1;
        v.qhi = 3122 - e < 2046 ? 3122 - e : 2046;
    } else {
        v.qlo = 1;
        v.qhi = 0;
    }
    return v;
}

template <typename T>
inline Divisor<T> make_divisor(double d);
template <>
inline Divisor<float> make_divisor<float>(double d) {
    return make_divisor_f32(d);
}
template <>
inline Divisor<double> make_divisor<double>(double d) {
    return make_divisor_f64(d);
}

#ifdef __CUDACC__
// RN(a / v.d), equal to __ddiv_rn(a, v.d) for every a.
__device__ __forceinline__ double div_rn(double a, const Divisor<double>& v) {
    const long long abits = __double_as_longlong(a);
    if ((abits << 1) == 0 && v.zero_ok) {  // a = +-0: zero with the sign of a times that of d
        const unsigned long long sign = (static_cast<unsigned long long>(abits) ^
                                         (static_cast<unsigned long long>(static_cast<unsigned>(v.dsign)) << 32)) &
                                        (1ULL << 63);
        return __longlong_as_double(static_cast<long long>(sign));
    }
    const double q0 = __dmul_rn(a, v.r);
    const double e0 = __fma_rn(-q0, v.d, a);
    const double q1 = __fma_rn(e0, v.r, q0);
    const double e1 = __fma_rn(-q1, v.d, a);
    const int hi = __double2hiint(q1);
    const int eq = (hi >> 20) & 0x7ff;
    if (eq >= v.qlo && eq <= v.qhi) {
        // the exact quotient lies toward zero from q1 when sign(e1) sign(d) differs
        // from sign(q1); below a power of two the next double is half as far
        const bool pow2 = ((hi & 0x000fffff) | __double2loint(q1)) == 0;
        const bool down = (__double2hiint(e1) ^ hi ^ v.dsign) < 0;
        const int tb = v.dexp + eq - 1076 - ((pow2 && down) ? 1 : 0);
        const long long bound = (static_cast<long long>((tb << 20) | static_cast<int>(v.dmant_hi)) << 32) |
                                static_cast<long long>(v.dlo);
        // |e1| < bound, compared as bit patterns of non-negative doubles
        if ((__double_as_longlong(e1) & 0x7fffffffffffffffLL) < bound) return q1;
    }
    return __ddiv_rn(a, v.d);
}
#endif

}  // namespace sssi
