// Outward-rounded scalar arithmetic on the device.
//
// GB300-native restatement of the reference's floating_point_bounds.hpp
// (src/algorithms/mathematics/floating_point_bounds.hpp:35-401).  The
// reference forms each bound in long double and then rounds it outward with
// one extra nextafter step; here the hardware's directed-rounding
// instructions (__dadd_ru, __dmul_rd, __dsqrt_ru, ...) give the correctly
// rounded bound and one extra step keeps the same safety margin.  Every
// function returns a valid outward bound for binary64 inputs; the results can
// differ from the reference's in the last bit only.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace amfls_gpu {
namespace fpb {

constexpr double kInf = __builtin_huge_val();
constexpr double kDenormMin = 4.9406564584124654e-324;
constexpr double kDblMax = 1.7976931348623157e308;
constexpr double kUnitRoundoff = 1.1102230246251565e-16;  // 2^-53

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

__device__ __forceinline__ double next_up(double v) {
    if (isnan(v) || v == kInf) return v;
    if (v == 0.0) return kDenormMin;
    long long bits = __double_as_longlong(v);
    bits += v > 0.0 ? 1 : -1;
    return __longlong_as_double(bits);
}

__device__ __forceinline__ double next_down(double v) {
    if (isnan(v) || v == -kInf) return v;
    if (v == 0.0) return -kDenormMin;
    long long bits = __double_as_longlong(v);
    bits += v > 0.0 ? -1 : 1;
    return __longlong_as_double(bits);
}

// Upward bound of a nonnegative exact value already rounded up: one more step.
__device__ __forceinline__ double widen_up(double ru) {
    if (!(ru >= 0.0) || !isfinite(ru) || ru > kDblMax) return kInf;
    if (ru == 0.0) return 0.0;
    return next_up(ru);
}

__device__ __forceinline__ double widen_down(double rd) {
    if (!(rd > 0.0) || !isfinite(rd)) return 0.0;
    const double d = next_down(rd);
    return d > 0.0 ? d : 0.0;
}

// gamma_k = k u / (1 - k u), rounded outward (floating_point_bounds.hpp:123-135).
__device__ __forceinline__ double gamma(long long ops, double unit = kUnitRoundoff) {
    if (ops < 0) return kInf;
    const double num = __dmul_ru(static_cast<double>(ops), unit);
    if (!(num < 1.0)) return kInf;
    const double den = __dadd_rd(1.0, -num);
    return widen_up(__ddiv_ru(num, den));
}

__device__ __forceinline__ double up_add(double a, double b) {
    return widen_up(__dadd_ru(a, b));
}

__device__ __forceinline__ double up_mul(double a, double b) {
    if (a < 0.0 || b < 0.0) return kInf;
    const double p = __dmul_ru(a, b);
    if (a > 0.0 && b > 0.0 && p == 0.0) return kDenormMin;
    return widen_up(p);
}

__device__ __forceinline__ double down_add(double a, double b) {
    if (a < 0.0 || b < 0.0 || !isfinite(a) || !isfinite(b)) return 0.0;
    return widen_down(__dadd_rd(a, b));
}

__device__ __forceinline__ double down_mul(double a, double b) {
    if (a < 0.0 || b < 0.0 || !isfinite(a) || !isfinite(b)) return 0.0;
    return widen_down(__dmul_rd(a, b));
}

__device__ __forceinline__ double down_div(double a, double b) {
    if (!(a > 0.0) || !(b > 0.0) || !isfinite(a) || !isfinite(b)) return 0.0;
    return widen_down(__ddiv_rd(a, b));
}

__device__ __forceinline__ double down_diff(double a, double b) {
    if (!(a > b) || !isfinite(a) || b < 0.0 || !isfinite(b)) return 0.0;
    return widen_down(__dadd_rd(a, -b));
}

__device__ __forceinline__ double up_div(double a, double b) {
    if (a == 0.0) return 0.0;
    if (!(b > 0.0) || a < 0.0 || !isfinite(a) || !isfinite(b)) return kInf;
    const double q = __ddiv_ru(a, b);
    if (q == 0.0) return kDenormMin;
    return widen_up(q);
}

__device__ __forceinline__ double up_sqrt(double v) {
    if (v < 0.0 || !isfinite(v)) return v == kInf ? v : kInf;
    return widen_up(__dsqrt_ru(v));
}

__device__ __forceinline__ double down_sqrt(double v) {
    if (!(v > 0.0) || !isfinite(v)) return 0.0;
    return widen_down(__dsqrt_rd(v));
}

// k * denorm_min rounded up (exact unless k is huge).
__device__ __forceinline__ double denorm_multiple(double k) {
    return widen_up(__dmul_ru(k, kDenormMin));
}

// Upper bound of an exact nonnegative sum from its stored value after `ops`
// rounded operations (floating_point_bounds.hpp:216-259).
__device__ __forceinline__ double sum_upper(double stored, long long ops, bool zero_exact) {
    if (stored < 0.0 || !isfinite(stored) || ops < 0) return kInf;
    if (zero_exact && stored == 0.0) return 0.0;
    const double g = gamma(ops);
    const double den = down_diff(1.0, g);
    if (!(den > 0.0)) return kInf;
    return up_div(up_add(stored, denorm_multiple(static_cast<double>(ops))), den);
}

__device__ __forceinline__ double sum_lower(double stored, long long ops) {
    if (!(stored > 0.0) || !isfinite(stored) || ops < 0) return 0.0;
    const double g = gamma(ops);
    const double den = up_add(1.0, g);
    if (!isfinite(den)) return 0.0;
    return down_div(down_diff(stored, denorm_multiple(static_cast<double>(ops))), den);
}

__device__ __forceinline__ double scale_up_pow2(double v, int e) {
    if (v == 0.0) return 0.0;
    if (!(v > 0.0) || !isfinite(v)) return kInf;
    const double s = scalbn(v, e);
    if (isinf(s)) return s;
    if (s == 0.0) return kDenormMin;
    return next_up(s);
}

__device__ __forceinline__ double scale_down_pow2(double v, int e) {
    if (!(v > 0.0) || !isfinite(v)) return 0.0;
    const double s = scalbn(v, e);
    if (isinf(s)) return kDblMax;
    if (s == 0.0) return 0.0;
    const double d = next_down(s);
    return d > 0.0 ? d : 0.0;
}

struct Interval {
    double lower;
    double upper;
};

// Norm interval from the two passes of norm_interval
// (floating_point_bounds.hpp:325-376): `max_abs` is max |v_i|, `exponent`
// its frexp exponent, `scaled_square_sum` the FMA sum of (|v_i| 2^-e)^2 over
// `count` terms (any summation tree: its depth is at most `count`).
__device__ inline Interval norm_interval_from(double max_abs, int exponent,
                                              double scaled_square_sum, long long count,
                                              bool all_finite) {
    if (!all_finite) return {0.0, kInf};
    if (max_abs == 0.0) return {0.0, 0.0};
    const double lo2 = sum_lower(scaled_square_sum, count);
    const double hi2 = sum_upper(scaled_square_sum, count, true);
    const double lo = down_sqrt(lo2);
    const double hi = up_sqrt(hi2);
    const double serr = widen_up(__dmul_ru(__dsqrt_ru(static_cast<double>(count)), kDenormMin));
    return {scale_down_pow2(down_diff(lo, serr), exponent),
            scale_up_pow2(up_add(hi, serr), exponent)};
}

}  // namespace fpb
}  // namespace amfls_gpu
