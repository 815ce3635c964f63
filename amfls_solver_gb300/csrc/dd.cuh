// Double-double (unevaluated sum of two binary64) arithmetic for the
// validation refinement products.
//
// Error-free transformations after Knuth (TwoSum), Dekker/FMA (TwoProd) and
// the accurate pair addition of Joldes, Muller and Popescu (2017,
// "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic", Alg. 6 AccurateDWPlusDW, relative error <= 3u^2 + O(u^3);
// Alg. 9 DWTimesFP, relative error <= 2u^2).  The certified validator charges
// each accumulated term with unit roundoff kDDUnit = 2^-100, a factor of
// 16 above 2^-104 (~3u^2), so gamma_k(kDDUnit) bounds the accumulation.
#pragma once

#include <cuda_runtime.h>

namespace amfls_gpu {

constexpr double kDDUnit = 7.888609052210118e-31;  // 2^-100

struct dd {
    double hi;
    double lo;
};

__device__ __forceinline__ dd two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    const double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

__device__ __forceinline__ dd fast_two_sum(double a, double b) {
    const double s = a + b;
    const double e = b - (s - a);
    return {s, e};
}

__device__ __forceinline__ dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}

// (x.hi + x.lo) * b
__device__ __forceinline__ dd dd_mul_d(dd x, double b) {
    const double p = x.hi * b;
    double e = fma(x.hi, b, -p);
    e = fma(x.lo, b, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ dd dd_shfl_xor(dd v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

}  // namespace amfls_gpu
