// Test infrastructure only: a C-callable driver around the reference
// implementation of AMFLS (doloMing/amfls_solver), compiled from the
// reference sources where they lie by oracle/Makefile into oracle/_ref/.
// Nothing in the product links or loads this file; tests and the fixture
// generator under tests/golden/ call it through ctypes to pin the oracle.
//
// Entry points mirror the reference's own call sites:
//   solve_amfls          include/amfls/amfls.hpp:22-25
//   solve_fixed_rbgk     include/amfls/fixed_rbgk.hpp:22-25 (FixedRbgkOptions :8-18)
//   solve_lsqr           include/amfls/lsqr.hpp:8-18 (LsqrOptions)
//   solve_lsmr           include/amfls/lsmr.hpp (LsmrOptions, the same three fields)
//   SparseCsrOperator    src/algorithms/mathematics/operators/sparse_csr_operator.hpp:13-58
//   RowMajorDenseOperator / DenseOperator (validation_error_model, apply)
//   gaussian_matrix      src/algorithms/mathematics/random/gaussian.cpp:39-55
//   fp::norm_interval    src/algorithms/mathematics/floating_point_bounds.hpp:325-376
//   width decisions      amfls.cpp:323-354 (recorded / replayed through ref_hooks.hpp)
// The result packing follows the layout of bindings/torch/result_tensors.hpp:24-156
// (21 metrics, 36 counters, 9 timings, 29 + 4 trace columns).
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <span>
#include <string>
#include <vector>

#include "amfls/amfls.hpp"
#include "amfls/fixed_rbgk.hpp"
#include "amfls/lsmr.hpp"
#include "amfls/lsqr.hpp"
#include "algorithms/mathematics/floating_point_bounds.hpp"
#include "algorithms/mathematics/operators/dense_operator.hpp"
#include "algorithms/mathematics/operators/row_major_dense_operator.hpp"
#include "algorithms/mathematics/operators/sparse_csr_operator.hpp"
#include "algorithms/mathematics/random/gaussian.hpp"

namespace {

thread_local std::string g_error;

// Width decisions of the last AMFLS solve (candidate bit, matched horizon)
// and, when g_replay_active, the candidate bits to substitute in order.
std::vector<int> g_decisions;
std::vector<int> g_horizons;
std::vector<int> g_replay;
bool g_replay_active = false;
std::size_t g_replay_position = 0;
long long g_replay_overrun = 0;

}  // namespace

amfls::detail::WidthDecision amfls::detail::ref_hook_width_decision(WidthDecision decision) {
    if (g_replay_active) {
        if (g_replay_position < g_replay.size()) {
            decision.candidate = g_replay[g_replay_position] != 0;
        } else {
            ++g_replay_overrun;  // more decision sites than recorded: keep the reference's
        }
        ++g_replay_position;
    }
    g_decisions.push_back(decision.candidate ? 1 : 0);
    g_horizons.push_back(decision.matched_horizon);
    return decision;
}

namespace {

struct OperatorSpec {
    int kind;  // 0 CSR, 1 row-major dense, 2 column-major dense, 3 CSR behind a custom operator
    int rows;
    int cols;
    const std::int64_t* row_offsets;
    const std::int64_t* column_indices;
    const double* values;
    std::int64_t nonzeros;
};

// A user's custom MatrixOperator over a CSR matrix: it forwards the products
// and the validation error model of a SparseCsrOperator and keeps the
// interface defaults for everything else (block cost, no extended-precision
// validation products, matrix_operator.hpp:45-88).
class ForwardingOperator final : public amfls::MatrixOperator {
public:
    explicit ForwardingOperator(std::unique_ptr<amfls::MatrixOperator> inner)
        : inner_(std::move(inner)) {}
    int rows() const override { return inner_->rows(); }
    int cols() const override { return inner_->cols(); }
    void apply(const double* x, int block_cols, double* y) const override {
        inner_->apply(x, block_cols, y);
    }
    void apply_transpose(const double* y, int block_cols, double* x) const override {
        inner_->apply_transpose(y, block_cols, x);
    }
    amfls::MatrixOperatorValidationErrorModel validation_error_model() const noexcept override {
        return inner_->validation_error_model();
    }

private:
    std::unique_ptr<amfls::MatrixOperator> inner_;
};

std::unique_ptr<amfls::MatrixOperator> make_operator(const OperatorSpec& s) {
    using namespace amfls::math;
    if (s.kind == 3) {
        return std::make_unique<ForwardingOperator>(std::make_unique<SparseCsrOperator>(
            s.rows, s.cols, s.row_offsets, s.column_indices, s.values, s.nonzeros));
    }
    if (s.kind == 0) {
        return std::make_unique<SparseCsrOperator>(
            s.rows, s.cols, s.row_offsets, s.column_indices, s.values,
            s.nonzeros);
    }
    if (s.kind == 1) {
        return std::make_unique<RowMajorDenseOperator>(s.rows, s.cols, s.values);
    }
    return std::make_unique<DenseOperator>(s.rows, s.cols, s.values);
}

// Packs one LeastSquaresResult in the torch binding's tensor layout.
void pack_result(
    const amfls::LeastSquaresResult& r,
    double* solution,
    double* metrics,
    std::int64_t* counters,
    double* timings,
    double* trace_float,
    std::int64_t* trace_int,
    int trace_capacity,
    int* trace_rows,
    int* status,
    int* stop_reason) {
    std::memcpy(solution, r.solution.data(), sizeof(double) * r.solution.size());
    const double m[21] = {
        r.objective, r.residual_norm, r.augmented_residual_norm,
        r.normal_residual_norm, r.solution_norm, r.solution_energy_norm,
        r.operator_norm_lower_bound, r.augmented_operator_norm_lower_bound,
        r.compatible_backward_error_upper_bound,
        r.least_squares_backward_error_upper_bound,
        r.backward_error_upper_bound, r.relative_normal_residual_upper_bound,
        r.energy_error_upper_bound, r.relative_energy_error_upper_bound,
        r.objective_gap_upper_bound, r.ridge_base_energy_error_upper_bound,
        r.ridge_corrected_energy_error_upper_bound, r.ridge_correction_gamma,
        r.ridge_correction_z_h_z, r.ridge_correction_two_abs_z_t_q,
        r.ridge_correction_q_norm_squared};
    std::memcpy(metrics, m, sizeof(m));
    const auto& s = r.statistics;
    const std::int64_t c[36] = {
        s.a_columns, s.at_columns, s.a_block_calls, s.at_block_calls,
        s.search_a_columns, s.search_at_columns, s.validation_a_columns,
        s.validation_at_columns, r.iterations, r.depth, r.auxiliary_width,
        r.basis_rank, s.sketch_a_columns, s.sketch_at_columns,
        s.sketch_a_block_calls, s.sketch_at_block_calls, s.iterative_a_columns,
        s.iterative_at_columns, s.iterative_a_block_calls,
        s.iterative_at_block_calls, s.gaussian_random_columns,
        s.gaussian_random_values, s.search_a_block_calls,
        s.search_at_block_calls, s.validation_a_block_calls,
        s.validation_at_block_calls, s.base_validation_a_columns,
        s.base_validation_at_columns, s.base_validation_a_block_calls,
        s.base_validation_at_block_calls, s.ridge_correction_a_columns,
        s.ridge_correction_at_columns, s.ridge_correction_a_block_calls,
        s.ridge_correction_at_block_calls, s.gaussian_random_block_requests,
        static_cast<std::int64_t>(r.ridge_correction_disposition)};
    std::memcpy(counters, c, sizeof(c));
    double other = s.total_seconds - s.a_seconds - s.at_seconds -
        s.orthogonalization_seconds - s.projected_solve_seconds;
    if (!(other > 0.0)) other = 0.0;
    const double t[9] = {
        s.total_seconds, s.a_seconds, s.at_seconds,
        s.orthogonalization_seconds, s.projected_solve_seconds,
        s.validation_seconds, other, s.base_validation_seconds,
        s.ridge_correction_validation_seconds};
    std::memcpy(timings, t, sizeof(t));
    const int rows = static_cast<int>(r.trace.size());
    *trace_rows = rows;
    for (int i = 0; i < rows && i < trace_capacity; ++i) {
        const auto& e = r.trace[static_cast<std::size_t>(i)];
        const double f[29] = {
            double(e.epoch), double(e.depth), double(e.auxiliary_width),
            double(e.basis_rank), double(e.a_columns), double(e.at_columns),
            double(e.a_block_calls), double(e.at_block_calls), e.objective,
            e.residual_norm, e.augmented_residual_norm, e.normal_residual_norm,
            e.operator_norm_lower_bound,
            e.compatible_backward_error_upper_bound,
            e.least_squares_backward_error_upper_bound,
            e.backward_error_upper_bound,
            e.relative_normal_residual_upper_bound,
            e.relative_energy_error_upper_bound, e.solution_norm,
            e.solution_energy_norm, e.augmented_operator_norm_lower_bound,
            e.energy_error_upper_bound, e.objective_gap_upper_bound,
            e.ridge_base_energy_error_upper_bound,
            e.ridge_corrected_energy_error_upper_bound,
            e.ridge_correction_gamma, e.ridge_correction_z_h_z,
            e.ridge_correction_two_abs_z_t_q,
            e.ridge_correction_q_norm_squared};
        std::memcpy(trace_float + 29 * i, f, sizeof(f));
        const std::int64_t g[4] = {
            static_cast<std::int64_t>(e.contract_status),
            static_cast<std::int64_t>(e.contract_stop_reason),
            e.contract_passed ? 1 : 0,
            static_cast<std::int64_t>(e.ridge_correction_disposition)};
        std::memcpy(trace_int + 4 * i, g, sizeof(g));
    }
    *status = static_cast<int>(r.status);
    *stop_reason = static_cast<int>(r.stop_reason);
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

// Replay list for the next AMFLS solves (count < 0 switches replay off).
void ref_set_width_replay(const int* decisions, int count) {
    g_replay_active = count >= 0;
    g_replay.assign(decisions, decisions + (count > 0 ? count : 0));
}

// Decisions of the last solve: candidate bits and matched horizons (up to
// `capacity` each); returns the number of decision sites, and the count of
// sites beyond the replay list in *overrun.
int ref_width_decisions(int* decisions, int* horizons, int capacity, long long* overrun) {
    const int n = static_cast<int>(g_decisions.size());
    for (int i = 0; i < n && i < capacity; ++i) {
        decisions[i] = g_decisions[i];
        horizons[i] = g_horizons[i];
    }
    *overrun = g_replay_overrun;
    return n;
}

// Returns 0 on success, -1 on an exception (message in ref_last_error()).
int ref_solve(
    int algorithm,  // 0 AMFLS, 1 fixed RBGK, 2 LSQR, 3 LSMR (maximum_depth: maximum_iterations)
    int kind, int rows, int cols, const std::int64_t* row_offsets,
    const std::int64_t* column_indices, const double* values,
    std::int64_t nonzeros, const double* b, double regularization,
    double tolerance, double failure_probability, int maximum_epochs,
    int maximum_depth, int maximum_auxiliary_width, int maximum_basis_size,
    std::uint64_t seed, std::uint64_t stream, int fixed_auxiliary_width,
    double* solution, double* metrics, std::int64_t* counters,
    double* timings, double* trace_float, std::int64_t* trace_int,
    int trace_capacity, int* trace_rows, int* status, int* stop_reason) {
    try {
        g_decisions.clear();
        g_horizons.clear();
        g_replay_position = 0;
        g_replay_overrun = 0;
        const OperatorSpec spec{kind, rows, cols, row_offsets, column_indices,
                                values, nonzeros};
        auto op = make_operator(spec);
        amfls::LeastSquaresResult r;
        if (algorithm == 0) {
            amfls::AmflsOptions o;
            o.regularization = regularization;
            o.tolerance = tolerance;
            o.failure_probability = failure_probability;
            o.maximum_epochs = maximum_epochs;
            o.maximum_depth = maximum_depth;
            o.maximum_auxiliary_width = maximum_auxiliary_width;
            o.maximum_basis_size = maximum_basis_size;
            o.seed = seed;
            o.stream = stream;
            r = amfls::solve_amfls(*op, b, o);
        } else if (algorithm == 2) {
            amfls::LsqrOptions o;
            o.regularization = regularization;
            o.tolerance = tolerance;
            o.maximum_iterations = maximum_depth;
            r = amfls::solve_lsqr(*op, b, o);
        } else if (algorithm == 3) {
            amfls::LsmrOptions o;
            o.regularization = regularization;
            o.tolerance = tolerance;
            o.maximum_iterations = maximum_depth;
            r = amfls::solve_lsmr(*op, b, o);
        } else {
            amfls::FixedRbgkOptions o;
            o.regularization = regularization;
            o.tolerance = tolerance;
            o.failure_probability = failure_probability;
            o.auxiliary_width = fixed_auxiliary_width;
            o.maximum_depth = maximum_depth;
            o.maximum_basis_size = maximum_basis_size;
            o.seed = seed;
            o.stream = stream;
            r = amfls::solve_fixed_rbgk(*op, b, o);
        }
        pack_result(r, solution, metrics, counters, timings, trace_float,
                    trace_int, trace_capacity, trace_rows, status, stop_reason);
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Y = A X or X = A^T Y for a block of `block_cols` column-major columns.
int ref_apply(int kind, int rows, int cols, const std::int64_t* row_offsets,
              const std::int64_t* column_indices, const double* values,
              std::int64_t nonzeros, int transpose, const double* input,
              int block_cols, double* output) {
    try {
        auto op = make_operator({kind, rows, cols, row_offsets, column_indices,
                                 values, nonzeros});
        if (transpose) {
            op->apply_transpose(input, block_cols, output);
        } else {
            op->apply(input, block_cols, output);
        }
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// model[0] = ||A|| upper, model[1] = ||A|| lower; steps[0] apply, steps[1] transpose.
int ref_validation_model(int kind, int rows, int cols,
                         const std::int64_t* row_offsets,
                         const std::int64_t* column_indices,
                         const double* values, std::int64_t nonzeros,
                         double* model, std::int64_t* steps) {
    try {
        auto op = make_operator({kind, rows, cols, row_offsets, column_indices,
                                 values, nonzeros});
        const auto v = op->validation_error_model();
        model[0] = v.operator_norm_upper_bound;
        model[1] = v.operator_norm_lower_bound;
        steps[0] = v.apply_rounding_steps;
        steps[1] = v.apply_transpose_rounding_steps;
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

int ref_gaussian_matrix(int rows, int cols, std::uint64_t seed,
                        std::uint64_t stream, std::uint64_t first_column,
                        double* output) {
    try {
        auto g = amfls::math::gaussian_matrix(rows, cols, seed, stream,
                                              first_column);
        std::memcpy(output, g.data(), sizeof(double) * std::size_t(rows) * cols);
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

void ref_norm_interval(const double* values, std::int64_t size, double* out) {
    const auto v = amfls::math::fp::norm_interval(
        std::span<const double>(values, static_cast<std::size_t>(size)));
    out[0] = v.lower;
    out[1] = v.upper;
}

}  // extern "C"
