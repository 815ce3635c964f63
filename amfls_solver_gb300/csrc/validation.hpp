// Certified validation of a candidate solution on the device.
//
// Restates validate_original_candidate and its helpers
// (src/algorithms/mathematics/krylov/candidate_validation.cpp:67-1378):
// the base pair A x - b, A^T r + lambda x; the nominal contract; the
// outward-rounded envelope and certified contract; the extended-precision
// repeat when the gradient's rounding radius dominates (double-double here,
// long double in the reference); and the one-step ridge correction for
// lambda > 0.  Vector passes are device kernels; the scalar envelope runs in
// one device thread with directed-rounding intrinsics.
#pragma once

#include <cuda_runtime.h>

#include "device_operator.hpp"

namespace amfls_gpu {

struct ValidationOutput {
    double objective, residual_norm, augmented_residual_norm, normal_residual_norm;
    double solution_norm, solution_energy_norm, operator_norm_lower_bound;
    double augmented_operator_norm_lower_bound;
    double compatible_backward_error_upper_bound;
    double least_squares_backward_error_upper_bound;
    double backward_error_upper_bound;
    double relative_normal_residual_upper_bound;
    double energy_error_upper_bound, relative_energy_error_upper_bound;
    double objective_gap_upper_bound;
    double ridge_base_energy_error_upper_bound;
    double ridge_corrected_energy_error_upper_bound;
    double ridge_correction_gamma, ridge_correction_z_h_z;
    double ridge_correction_two_abs_z_t_q, ridge_correction_q_norm_squared;
    int status, stop_reason, ridge_correction_disposition;
    // operator calls: base A, base A^T, refinement A, refinement A^T,
    // correction A, correction A^T
    int calls[6];
    double seconds[6];  // device time of those calls
};

class Validator {
public:
    Validator(const DeviceOperator& op, const double* d_b, double regularization,
              cudaStream_t stream);
    ~Validator();
    Validator(const Validator&) = delete;
    Validator& operator=(const Validator&) = delete;

    // Full validation of the device candidate d_x (n); synchronous.
    ValidationOutput validate(const double* d_x, double tolerance);

private:
    struct Impl;
    Impl* impl_;
};

}  // namespace amfls_gpu
