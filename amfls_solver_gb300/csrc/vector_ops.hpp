// Multi-vector norm passes used by initialisation and validation.
//
// The reference's norm_interval (floating_point_bounds.hpp:325-376) makes two
// passes: max |v_i| (with a finiteness check), then an FMA sum of squares of
// v_i scaled by the power of two 2^-e that puts the largest entry in
// [1/2, 1).  NormPasses runs both passes for up to kMaxVectors vectors in two
// launches; the scaled sum also gives the Euclidean norm 2^e sqrt(sum) that
// stands in for the reference's dnrm2.
#pragma once

#include <cuda_runtime.h>

namespace amfls_gpu {

constexpr int kMaxVectors = 6;

struct NormResult {
    double max_abs[kMaxVectors];
    double scaled_sumsq[kMaxVectors];
    int exponent[kMaxVectors];
    int nonfinite[kMaxVectors];
    long long count[kMaxVectors];
};

struct VectorSet {
    const double* v[kMaxVectors];
    long long n[kMaxVectors];
    int count;
};

// Both passes; results land in device `out`.  `partials` must hold
// 2 * kMaxVectors * kMaxGridCap doubles and `counter` one zeroed unsigned.
void norm_passes(const VectorSet& set, NormResult* out, double* partials, unsigned* counter,
                 cudaStream_t stream);

// Host-side Euclidean norm from a NormResult entry (scaled sum times 2^e).
double euclid_from(const NormResult& r, int i);

}  // namespace amfls_gpu
