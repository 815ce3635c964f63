// AMFLS controller (host C++20) over the device workspace.
#pragma once

#include <cstdint>
#include <vector>

#include "device_operator.hpp"
#include "validation.hpp"
#include "width_policy.hpp"

namespace amfls_gpu {

// AmflsOptions (include/amfls/amfls.hpp:10-20) plus FixedRbgkOptions'
// fields (include/amfls/fixed_rbgk.hpp:8-18) and GB300 switches.
struct SolveOptions {
    double regularization = 0.0;
    double tolerance = 1e-8;
    double failure_probability = 1e-6;
    int maximum_epochs = 0;
    int maximum_basis_size = 0;
    std::uint64_t seed = 0;
    std::uint64_t stream = 0;
    int maximum_depth = 0;
    int maximum_auxiliary_width = 0;
    int auxiliary_width = 4;  // fixed RBGK only
    bool stop_early = true;   // fixed RBGK only
    bool time_operators = true;
    bool use_graphs = true;
    // At a work or basis limit return the latest checkpoint's candidate even
    // for lambda = 0 (the reference returns the one with the smallest
    // backward error there, amfls.cpp:156-163).  Not part of the reference's
    // options: the mixed form's restarted inner solves use it, because the
    // latest least-squares iterate has the smallest error in the normal
    // equations' energy norm while the backward error need not be monotone.
    bool latest_at_limit = false;
    // 1 (FP32) or 2 (FP16): width-one levels keep a reduced copy of the
    // right basis and run their first reorthogonalisation pass on it,
    // redoing it in FP64 when the coefficients are not small (see the
    // reduced-basis sweeps in workspace.cu); 0 keeps every sweep FP64.  Not
    // part of the reference's options: the mixed-precision form's reduced
    // sweeps.
    int reduced_basis = 0;
};

// RunStatistics (include/amfls/least_squares_result.hpp:57-109).
struct Statistics {
    long long a_columns = 0, at_columns = 0, a_block_calls = 0, at_block_calls = 0;
    long long search_a_columns = 0, search_at_columns = 0;
    long long validation_a_columns = 0, validation_at_columns = 0;
    long long sketch_a_columns = 0, sketch_at_columns = 0, sketch_a_block_calls = 0,
              sketch_at_block_calls = 0;
    long long iterative_a_columns = 0, iterative_at_columns = 0, iterative_a_block_calls = 0,
              iterative_at_block_calls = 0;
    long long gaussian_random_columns = 0, gaussian_random_values = 0;
    double total_seconds = 0.0, a_seconds = 0.0, at_seconds = 0.0;
    double orthogonalization_seconds = 0.0, projected_solve_seconds = 0.0, validation_seconds = 0.0;
    long long search_a_block_calls = 0, search_at_block_calls = 0;
    long long validation_a_block_calls = 0, validation_at_block_calls = 0;
    long long base_validation_a_columns = 0, base_validation_at_columns = 0;
    long long base_validation_a_block_calls = 0, base_validation_at_block_calls = 0;
    long long ridge_correction_a_columns = 0, ridge_correction_at_columns = 0;
    long long ridge_correction_a_block_calls = 0, ridge_correction_at_block_calls = 0;
    double base_validation_seconds = 0.0, ridge_correction_validation_seconds = 0.0;
    long long gaussian_random_block_requests = 0;
    // GB300 extras (not in the reference's tensors)
    long long projected_rank_flags = 0;
    long long kernel_launches = 0;  // kernels this solve ran on the GPU
    long long reduced_levels = 0;     // levels projected on the reduced copy of V
    long long reduced_fallbacks = 0;  // of those, levels redone in FP64
};

struct TraceRow {
    double f[29];
    long long i[4];
};

// LeastSquaresResult (include/amfls/least_squares_result.hpp:162-229); the
// solution is written to the caller's device buffer.
struct SolveResult {
    int rows = 0, cols = 0, iterations = 0, depth = 0, auxiliary_width = 0, basis_rank = 0;
    ValidationOutput v{};
    int status = 1, stop_reason = 3;
    Statistics statistics;
    std::vector<TraceRow> trace;
};

// Optional control of the width decisions (no counterpart in the
// reference): a learned policy that replaces the heuristic's choice, random
// exploration (with probability `exploration` the choice is a fair coin),
// and a log of every decision with its features and the certificate's rate
// of decrease until the next decision.  Without it (or with all fields
// empty) solve_amfls is the reference's controller.
//
// Schedule replay: with replay_count >= 0 the heuristic's candidate bit at
// the n-th decision site (amfls.cpp:323-354) is replaced by replay[n]; sites
// beyond the list keep the heuristic's bit and are counted in *overrun.  The
// bit is the only part of a width decision that depends on measured seconds,
// so replaying the reference's recorded bits reproduces its widening solve
// whatever the timings.  `sites` (if set) receives every site's bit in order.
struct WidthControl {
    const WidthPolicy* policy = nullptr;
    double exploration = 0.0;
    std::uint64_t exploration_seed = 0;
    std::vector<DecisionRecord>* log = nullptr;
    const int* replay = nullptr;
    int replay_count = -1;
    std::vector<int>* sites = nullptr;
    long long* overrun = nullptr;
};

SolveResult solve_amfls(const DeviceOperator& op, const double* d_b, const SolveOptions& options,
                        double* d_solution, cudaStream_t stream,
                        const WidthControl* control = nullptr);

SolveResult solve_fixed_rbgk(const DeviceOperator& op, const double* d_b,
                             const SolveOptions& options, double* d_solution, cudaStream_t stream);

// One outer step of the mixed-precision solve: the inner solve's outcome and
// the FP64 certificate of the refined x.
struct RefinementStep {
    int inner_status, inner_stop_reason, inner_depth, inner_basis_rank;
    double certificate;
};

// Mixed-precision form (mixed.cu): inner AMFLS solves on `reduced` (an FP32
// or BF16 copy of `op`, or any operator of its shape) to `inner_tolerance`,
// refined in FP64 until op's certified validation meets options.tolerance.
// The result's validation fields, status and stop reason are those of the
// last FP64 validation; depth and iterations add up the inner solves.
SolveResult solve_amfls_mixed(const DeviceOperator& op, const DeviceOperator& reduced,
                              const double* d_b, const SolveOptions& options,
                              double inner_tolerance, int maximum_refinements,
                              double* d_solution, cudaStream_t stream,
                              std::vector<RefinementStep>* steps = nullptr);

// Result tensors in the torch binding's layout (bindings/torch/result_tensors.hpp:12-156).
void pack_metrics(const SolveResult& r, double out[21]);
void pack_counters(const SolveResult& r, long long out[36]);
void pack_timings(const SolveResult& r, double out[9]);

}  // namespace amfls_gpu
