// Batched AMFLS (batch.cu): independent problems solved concurrently.
#pragma once

#include <string>
#include <vector>

#include "controller.hpp"

namespace amfls_gpu {

struct BatchItem {
    const DeviceOperator* op = nullptr;
    const double* b = nullptr;  // device, op->rows()
    SolveOptions options;
    double* x = nullptr;        // device, op->cols()
};

struct BatchOutcome {
    SolveResult result;
    bool ok = false;
    std::string error;     // why the solve raised (ok == false)
    double seconds = 0.0;  // wall time of this problem's solve
    double finished = 0.0; // completion time since the batch started
    int worker = -1;
};

// Solves every item with solve_amfls on `workers` host threads, each with
// its own CUDA stream, largest problems first.  Synchronous; per-problem
// failures are reported in the outcomes, not thrown.
std::vector<BatchOutcome> solve_amfls_batch(const std::vector<BatchItem>& items, int workers,
                                            double* wall_seconds);

}  // namespace amfls_gpu
