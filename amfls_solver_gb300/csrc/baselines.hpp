// Scalar LSQR and LSMR baselines on the device operators (host C++20 over
// device vectors).
#pragma once

#include <cuda_runtime.h>

#include "controller.hpp"
#include "device_operator.hpp"

namespace amfls_gpu {

// LsqrOptions (include/amfls/lsqr.hpp:8-12) and LsmrOptions
// (include/amfls/lsmr.hpp): the same three fields.
struct BaselineOptions {
    double regularization = 0.0;
    double tolerance = 1e-8;
    int maximum_iterations = 0;  // 0: min(rows, cols)
};

// solve_lsqr (src/algorithms/lsqr/lsqr.cpp:84-281) and solve_lsmr
// (src/algorithms/lsmr/lsmr.cpp:112-351): the reference's recurrences and
// checkpoint protocol, each candidate certified by the device validation.
// The solution is written to d_solution (cols doubles).
SolveResult solve_lsqr(const DeviceOperator& op, const double* d_b, const BaselineOptions& o,
                       double* d_solution, cudaStream_t stream);
SolveResult solve_lsmr(const DeviceOperator& op, const double* d_b, const BaselineOptions& o,
                       double* d_solution, cudaStream_t stream);

}  // namespace amfls_gpu
