// C ABI layer (include/amfls_gpu.h): exceptions become error codes and the
// message is kept per thread, mirroring the reference's exception types
// (std::invalid_argument, std::length_error, std::logic_error, ...).
#include <cstring>
#include <memory>
#include <vector>
#include <stdexcept>
#include <string>

#include "../../include/amfls_gpu.h"
#include "baselines.hpp"
#include "batch.hpp"
#include "callback_operator.hpp"
#include "common.cuh"
#include "workspace.hpp"
#include "controller.hpp"
#include "csr_operator.hpp"
#include "dense_operator.hpp"
#include "reduced_operator.hpp"
#include "width_policy.hpp"

struct amfls_gpu_operator {
    std::unique_ptr<amfls_gpu::DeviceOperator> impl;
};

struct amfls_gpu_policy {
    std::unique_ptr<amfls_gpu::WidthPolicy> impl;
};

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F&& f) {
    try {
        f();
        g_last_error.clear();
        return AMFLS_GPU_OK;
    } catch (const std::invalid_argument& e) {
        g_last_error = e.what();
        return AMFLS_GPU_INVALID_ARGUMENT;
    } catch (const std::length_error& e) {
        g_last_error = e.what();
        return AMFLS_GPU_LENGTH_ERROR;
    } catch (const std::overflow_error& e) {
        g_last_error = e.what();
        return AMFLS_GPU_LENGTH_ERROR;
    } catch (const std::logic_error& e) {
        g_last_error = e.what();
        return AMFLS_GPU_LOGIC_ERROR;
    } catch (const amfls_gpu::CudaError& e) {
        g_last_error = e.what();
        return AMFLS_GPU_CUDA_ERROR;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return AMFLS_GPU_RUNTIME_ERROR;
    } catch (...) {
        g_last_error = "unknown error";
        return AMFLS_GPU_RUNTIME_ERROR;
    }
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

amfls_gpu::SolveOptions to_options(const amfls_gpu_options* o) {
    if (o == nullptr) throw std::invalid_argument("options must not be null");
    amfls_gpu::SolveOptions s;
    s.regularization = o->regularization;
    s.tolerance = o->tolerance;
    s.failure_probability = o->failure_probability;
    s.maximum_epochs = o->maximum_epochs;
    s.maximum_basis_size = o->maximum_basis_size;
    s.seed = o->seed;
    s.stream = o->stream;
    s.maximum_depth = o->maximum_depth;
    s.maximum_auxiliary_width = o->maximum_auxiliary_width;
    s.auxiliary_width = o->auxiliary_width;
    s.stop_early = o->stop_early != 0;
    s.time_operators = o->time_operators != 0;
    s.use_graphs = o->use_graphs != 0;
    if (o->reduced_basis < 0 || o->reduced_basis > 2)
        throw std::invalid_argument("options.reduced_basis must be 0 (off), 1 (FP32) or 2 (FP16)");
    s.reduced_basis = o->reduced_basis;
    return s;
}

void export_result(const amfls_gpu::SolveResult& r, amfls_gpu_result* out, double* tf,
                   int64_t* ti, int cap) {
    if (out == nullptr) throw std::invalid_argument("result must not be null");
    out->rows = r.rows;
    out->cols = r.cols;
    out->iterations = r.iterations;
    out->depth = r.depth;
    out->auxiliary_width = r.auxiliary_width;
    out->basis_rank = r.basis_rank;
    out->status = r.status;
    out->stop_reason = r.stop_reason;
    amfls_gpu::pack_metrics(r, out->metrics);
    amfls_gpu::pack_counters(r, out->counters);
    amfls_gpu::pack_timings(r, out->timings);
    out->trace_rows = static_cast<int>(r.trace.size());
    out->kernel_launches = r.statistics.kernel_launches;
    out->reduced_basis_levels = r.statistics.reduced_levels;
    out->reduced_basis_fallbacks = r.statistics.reduced_fallbacks;
    const int rows = std::min<int>(cap, static_cast<int>(r.trace.size()));
    for (int i = 0; i < rows; ++i) {
        if (tf) std::memcpy(tf + 29 * i, r.trace[i].f, sizeof(double) * 29);
        if (ti)
            for (int j = 0; j < 4; ++j) ti[4 * i + j] = r.trace[i].i[j];
    }
}

const amfls_gpu::DeviceOperator& deref(const amfls_gpu_operator* op) {
    if (op == nullptr || !op->impl) throw std::invalid_argument("operator must not be null");
    return *op->impl;
}

}  // namespace

namespace amfls_gpu {
void set_last_error(const std::string& message) { g_last_error = message; }
}  // namespace amfls_gpu

extern "C" {

void amfls_gpu_default_options(amfls_gpu_options* o) {
    if (o == nullptr) return;
    std::memset(o, 0, sizeof(*o));
    o->regularization = 0.0;
    o->tolerance = 1e-8;
    o->failure_probability = 1e-6;
    o->auxiliary_width = 4;
    o->maximum_depth = 0;
    o->stop_early = 1;
    o->time_operators = 1;
    o->use_graphs = 1;
}

void amfls_gpu_default_baseline_options(amfls_gpu_baseline_options* o) {
    if (o == nullptr) return;
    std::memset(o, 0, sizeof(*o));
    o->regularization = 0.0;
    o->tolerance = 1e-8;
    o->maximum_iterations = 0;
}

const char* amfls_gpu_last_error(void) { return g_last_error.c_str(); }

int amfls_gpu_csr_operator_create(int rows, int cols, const int64_t* d_row_offsets,
                                  const int64_t* d_column_indices, const double* d_values,
                                  int64_t nonzeros, void* stream, amfls_gpu_operator** out) {
    return guarded([&] {
        if (out == nullptr) throw std::invalid_argument("output handle must not be null");
        *out = nullptr;
        auto h = std::make_unique<amfls_gpu_operator>();
        h->impl = std::make_unique<amfls_gpu::CsrOperator>(
            rows, cols, reinterpret_cast<const long long*>(d_row_offsets),
            reinterpret_cast<const long long*>(d_column_indices), d_values, nonzeros,
            as_stream(stream));
        *out = h.release();
    });
}

int amfls_gpu_dense_operator_create(int rows, int cols, const double* d_values, int column_major,
                                    void* stream, amfls_gpu_operator** out) {
    return guarded([&] {
        if (out == nullptr) throw std::invalid_argument("output handle must not be null");
        *out = nullptr;
        auto h = std::make_unique<amfls_gpu_operator>();
        h->impl = std::make_unique<amfls_gpu::DenseOperator>(rows, cols, d_values,
                                                             column_major != 0, as_stream(stream));
        *out = h.release();
    });
}

int amfls_gpu_callback_operator_create(int rows, int cols,
                                       const amfls_gpu_operator_callbacks* callbacks, void* stream,
                                       amfls_gpu_operator** out) {
    return guarded([&] {
        if (out == nullptr) throw std::invalid_argument("output handle must not be null");
        *out = nullptr;
        if (callbacks == nullptr) throw std::invalid_argument("callbacks must not be null");
        amfls_gpu::Callbacks cb;
        cb.context = callbacks->context;
        cb.apply = callbacks->apply;
        cb.apply_transpose = callbacks->apply_transpose;
        cb.relative_block_product_cost = callbacks->relative_block_product_cost;
        cb.has_model = callbacks->has_validation_model != 0;
        cb.model.norm_upper = callbacks->validation_model.operator_norm_upper_bound;
        cb.model.norm_lower = callbacks->validation_model.operator_norm_lower_bound;
        cb.model.apply_steps = callbacks->validation_model.apply_rounding_steps;
        cb.model.transpose_steps = callbacks->validation_model.apply_transpose_rounding_steps;
        auto h = std::make_unique<amfls_gpu_operator>();
        h->impl = std::make_unique<amfls_gpu::CallbackOperator>(rows, cols, cb, as_stream(stream));
        *out = h.release();
    });
}

int amfls_gpu_operator_destroy(amfls_gpu_operator* op) {
    return guarded([&] { delete op; });
}

int amfls_gpu_operator_rows(const amfls_gpu_operator* op) {
    return op && op->impl ? op->impl->rows() : -1;
}

int amfls_gpu_operator_cols(const amfls_gpu_operator* op) {
    return op && op->impl ? op->impl->cols() : -1;
}

int amfls_gpu_operator_apply(const amfls_gpu_operator* op, const double* d_x, int block_cols,
                             double* d_y, void* stream) {
    return guarded([&] {
        if (d_x == nullptr || d_y == nullptr || block_cols <= 0)
            throw std::invalid_argument("apply block is invalid");
        deref(op).apply(d_x, block_cols, d_y, as_stream(stream));
    });
}

int amfls_gpu_operator_apply_transpose(const amfls_gpu_operator* op, const double* d_y,
                                       int block_cols, double* d_x, void* stream) {
    return guarded([&] {
        if (d_x == nullptr || d_y == nullptr || block_cols <= 0)
            throw std::invalid_argument("transpose block is invalid");
        deref(op).apply_transpose(d_y, block_cols, d_x, as_stream(stream));
    });
}

double amfls_gpu_operator_relative_block_product_cost(const amfls_gpu_operator* op,
                                                      int block_cols) {
    if (op == nullptr || !op->impl) return __builtin_huge_val();
    return op->impl->relative_block_product_cost(block_cols);
}

int amfls_gpu_operator_validation_error_model(const amfls_gpu_operator* op,
                                              amfls_gpu_validation_error_model* out) {
    return guarded([&] {
        if (out == nullptr) throw std::invalid_argument("output must not be null");
        const auto m = deref(op).validation_error_model();
        out->operator_norm_upper_bound = m.norm_upper;
        out->operator_norm_lower_bound = m.norm_lower;
        out->apply_rounding_steps = m.apply_steps;
        out->apply_transpose_rounding_steps = m.transpose_steps;
    });
}

int amfls_gpu_solve_amfls(const amfls_gpu_operator* op, const double* d_b,
                          const amfls_gpu_options* options, double* d_solution,
                          amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                          int trace_capacity, void* stream) {
    return guarded([&] {
        const auto opts = to_options(options);  // option errors before any device work
        if (d_solution == nullptr) throw std::invalid_argument("solution must not be null");
        const auto r = amfls_gpu::solve_amfls(deref(op), d_b, opts, d_solution, as_stream(stream));
        export_result(r, result, trace_float, trace_int, trace_capacity);
    });
}

int amfls_gpu_solve_fixed_rbgk(const amfls_gpu_operator* op, const double* d_b,
                               const amfls_gpu_options* options, double* d_solution,
                               amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                               int trace_capacity, void* stream) {
    return guarded([&] {
        const auto opts = to_options(options);
        if (d_solution == nullptr) throw std::invalid_argument("solution must not be null");
        const auto r = amfls_gpu::solve_fixed_rbgk(deref(op), d_b, opts, d_solution,
                                                   as_stream(stream));
        export_result(r, result, trace_float, trace_int, trace_capacity);
    });
}

static amfls_gpu::BaselineOptions to_baseline_options(const amfls_gpu_baseline_options* o) {
    if (o == nullptr) throw std::invalid_argument("options must not be null");
    amfls_gpu::BaselineOptions b;
    b.regularization = o->regularization;
    b.tolerance = o->tolerance;
    b.maximum_iterations = o->maximum_iterations;
    return b;
}

int amfls_gpu_solve_lsqr(const amfls_gpu_operator* op, const double* d_b,
                         const amfls_gpu_baseline_options* options, double* d_solution,
                         amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                         int trace_capacity, void* stream) {
    return guarded([&] {
        if (d_solution == nullptr) throw std::invalid_argument("solution must not be null");
        const auto r = amfls_gpu::solve_lsqr(deref(op), d_b, to_baseline_options(options),
                                             d_solution, as_stream(stream));
        export_result(r, result, trace_float, trace_int, trace_capacity);
    });
}

int amfls_gpu_solve_lsmr(const amfls_gpu_operator* op, const double* d_b,
                         const amfls_gpu_baseline_options* options, double* d_solution,
                         amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                         int trace_capacity, void* stream) {
    return guarded([&] {
        if (d_solution == nullptr) throw std::invalid_argument("solution must not be null");
        const auto r = amfls_gpu::solve_lsmr(deref(op), d_b, to_baseline_options(options),
                                             d_solution, as_stream(stream));
        export_result(r, result, trace_float, trace_int, trace_capacity);
    });
}

int amfls_gpu_reduced_operator_create(const amfls_gpu_operator* source, int value_type,
                                      void* stream, amfls_gpu_operator** out) {
    return guarded([&] {
        if (out == nullptr) throw std::invalid_argument("output handle must not be null");
        *out = nullptr;
        if (value_type != AMFLS_GPU_VALUES_FP32 && value_type != AMFLS_GPU_VALUES_BF16)
            throw std::invalid_argument("value_type must be FP32 (1) or BF16 (2)");
        const auto type = value_type == AMFLS_GPU_VALUES_FP32 ? amfls_gpu::ValueType::fp32
                                                              : amfls_gpu::ValueType::bf16;
        const amfls_gpu::DeviceOperator& src = deref(source);
        auto h = std::make_unique<amfls_gpu_operator>();
        if (const auto* csr = dynamic_cast<const amfls_gpu::CsrOperator*>(&src))
            h->impl = std::make_unique<amfls_gpu::ReducedCsrOperator>(*csr, type, as_stream(stream));
        else if (const auto* dense = dynamic_cast<const amfls_gpu::DenseOperator*>(&src))
            h->impl =
                std::make_unique<amfls_gpu::ReducedDenseOperator>(*dense, type, as_stream(stream));
        else
            throw std::invalid_argument("the source must be an FP64 CSR or dense operator");
        *out = h.release();
    });
}

int amfls_gpu_solve_amfls_mixed(const amfls_gpu_operator* op, const amfls_gpu_operator* reduced,
                                const double* d_b, const amfls_gpu_options* options,
                                double inner_tolerance, int maximum_refinements,
                                double* d_solution, amfls_gpu_result* result,
                                double* trace_float, int64_t* trace_int, int trace_capacity,
                                void* stream) {
    return guarded([&] {
        const auto opts = to_options(options);
        const auto r = amfls_gpu::solve_amfls_mixed(deref(op), deref(reduced), d_b, opts,
                                                    inner_tolerance,
                                                    maximum_refinements, d_solution,
                                                    as_stream(stream));
        export_result(r, result, trace_float, trace_int, trace_capacity);
    });
}

static_assert(amfls_gpu::kPolicyParams == AMFLS_GPU_POLICY_PARAMS, "policy size");
static_assert(amfls_gpu::kPolicyInputs == AMFLS_GPU_POLICY_INPUTS, "policy inputs");
static_assert(amfls_gpu::kPolicyFeatures == AMFLS_GPU_POLICY_FEATURES, "policy features");
static_assert(AMFLS_GPU_DECISION_COLUMNS == AMFLS_GPU_POLICY_FEATURES + 4, "decision row");

namespace {
std::vector<double> policy_params(const double* params, int count) {
    if (params == nullptr || count != AMFLS_GPU_POLICY_PARAMS)
        throw std::invalid_argument("policy parameters must be AMFLS_GPU_POLICY_PARAMS doubles");
    return std::vector<double>(params, params + count);
}
void check_batch(const double* inputs, int n) {
    if (inputs == nullptr || n <= 0) throw std::invalid_argument("policy batch is empty");
}
}  // namespace

int amfls_gpu_policy_initial_params(uint64_t seed, double* params, int count) {
    return guarded([&] {
        if (params == nullptr || count != AMFLS_GPU_POLICY_PARAMS)
            throw std::invalid_argument("policy parameters must be AMFLS_GPU_POLICY_PARAMS doubles");
        const auto p = amfls_gpu::policy_initial_params(seed);
        std::memcpy(params, p.data(), sizeof(double) * p.size());
    });
}

int amfls_gpu_policy_create(const double* params, int count, amfls_gpu_policy** out) {
    return guarded([&] {
        if (out == nullptr) throw std::invalid_argument("output handle must not be null");
        *out = nullptr;
        auto h = std::make_unique<amfls_gpu_policy>();
        h->impl = std::make_unique<amfls_gpu::WidthPolicy>(policy_params(params, count));
        *out = h.release();
    });
}

int amfls_gpu_policy_destroy(amfls_gpu_policy* policy) {
    return guarded([&] { delete policy; });
}

int amfls_gpu_policy_forward(const double* params, int count, const double* inputs, int n,
                             double* out, void* stream) {
    return guarded([&] {
        check_batch(inputs, n);
        if (out == nullptr) throw std::invalid_argument("output must not be null");
        amfls_gpu::policy_forward(policy_params(params, count), inputs, n, out, as_stream(stream));
    });
}

int amfls_gpu_policy_gradient(const double* params, int count, const double* inputs,
                              const double* targets, int n, double* grad, double* loss,
                              void* stream) {
    return guarded([&] {
        check_batch(inputs, n);
        if (targets == nullptr || grad == nullptr || loss == nullptr)
            throw std::invalid_argument("targets, grad and loss must not be null");
        *loss = amfls_gpu::policy_gradient(policy_params(params, count), inputs, targets, n, grad,
                                           as_stream(stream));
    });
}

int amfls_gpu_policy_train(double* params, int count, const double* inputs, const double* targets,
                           int n, int epochs, double learning_rate, double* loss_first,
                           double* loss_last, void* stream) {
    return guarded([&] {
        check_batch(inputs, n);
        if (targets == nullptr) throw std::invalid_argument("targets must not be null");
        auto p = policy_params(params, count);
        const auto r = amfls_gpu::policy_train(p, inputs, targets, n, epochs, learning_rate,
                                               as_stream(stream));
        std::memcpy(params, p.data(), sizeof(double) * p.size());
        if (loss_first) *loss_first = r.loss_first;
        if (loss_last) *loss_last = r.loss_last;
    });
}

int amfls_gpu_solve_amfls_controlled(const amfls_gpu_operator* op, const double* d_b,
                                     const amfls_gpu_options* options,
                                     const amfls_gpu_policy* policy, double exploration,
                                     uint64_t exploration_seed, double* decisions,
                                     int decision_capacity, int* decision_rows,
                                     double* d_solution, amfls_gpu_result* result,
                                     double* trace_float, int64_t* trace_int, int trace_capacity,
                                     void* stream) {
    return guarded([&] {
        if (d_solution == nullptr) throw std::invalid_argument("solution must not be null");
        if (!(exploration >= 0.0 && exploration <= 1.0))
            throw std::invalid_argument("exploration must lie in [0, 1]");
        if (decision_capacity < 0 || (decision_capacity > 0 && decisions == nullptr))
            throw std::invalid_argument("decision log buffer is invalid");
        std::vector<amfls_gpu::DecisionRecord> log;
        amfls_gpu::WidthControl ctl;
        ctl.policy = policy && policy->impl ? policy->impl.get() : nullptr;
        ctl.exploration = exploration;
        ctl.exploration_seed = exploration_seed;
        ctl.log = &log;
        const auto opts = to_options(options);
        const auto r = amfls_gpu::solve_amfls(deref(op), d_b, opts, d_solution,
                                              as_stream(stream), &ctl);
        export_result(r, result, trace_float, trace_int, trace_capacity);
        const int rows = std::min<int>(decision_capacity, (int)log.size());
        for (int i = 0; i < rows; ++i) {
            double* row = decisions + (long long)i * AMFLS_GPU_DECISION_COLUMNS;
            for (int j = 0; j < amfls_gpu::kPolicyFeatures; ++j) row[j] = log[i].features[j];
            row[11] = log[i].action;
            row[12] = log[i].heuristic;
            row[13] = log[i].rate;
            row[14] = log[i].valid;
        }
        if (decision_rows) *decision_rows = (int)log.size();
    });
}

int amfls_gpu_solve_amfls_replay(const amfls_gpu_operator* op, const double* d_b,
                                 const amfls_gpu_options* options, const int* replay,
                                 int replay_count, int* decisions, int decision_capacity,
                                 int* decision_count, long long* replay_overrun,
                                 double* d_solution, amfls_gpu_result* result,
                                 double* trace_float, int64_t* trace_int, int trace_capacity,
                                 void* stream) {
    return guarded([&] {
        const auto opts = to_options(options);
        if (d_solution == nullptr) throw std::invalid_argument("solution must not be null");
        if (replay_count > 0 && replay == nullptr)
            throw std::invalid_argument("replay list must not be null");
        if (decision_capacity < 0 || (decision_capacity > 0 && decisions == nullptr))
            throw std::invalid_argument("decision buffer is invalid");
        std::vector<int> sites;
        long long overrun = 0;
        amfls_gpu::WidthControl ctl;
        ctl.replay = replay;
        ctl.replay_count = replay_count < 0 ? -1 : replay_count;
        ctl.sites = &sites;
        ctl.overrun = &overrun;
        const auto r = amfls_gpu::solve_amfls(deref(op), d_b, opts, d_solution,
                                              as_stream(stream), &ctl);
        export_result(r, result, trace_float, trace_int, trace_capacity);
        const int n = std::min<int>(decision_capacity, (int)sites.size());
        for (int i = 0; i < n; ++i) decisions[i] = sites[i];
        if (decision_count) *decision_count = (int)sites.size();
        if (replay_overrun) *replay_overrun = overrun;
    });
}

int amfls_gpu_probe_reorthogonalization(int n, int k, int reps, void* stream,
                                        double* seconds) {
    return guarded([&] {
        if (seconds == nullptr) throw std::invalid_argument("seconds must not be null");
        amfls_gpu::probe_reorthogonalization(n, k, reps, as_stream(stream), seconds);
    });
}

int amfls_gpu_probe_reorthogonalization_reduced(int n, int k, int reps, int storage,
                                                void* stream, double* seconds,
                                                double* max_rel_error) {
    return guarded([&] {
        if (seconds == nullptr) throw std::invalid_argument("seconds must not be null");
        amfls_gpu::probe_reorthogonalization_reduced(n, k, reps, storage, as_stream(stream),
                                                     seconds, max_rel_error);
    });
}

int amfls_gpu_csr_operator_schedule(const amfls_gpu_operator* op, int* chains,
                                    double* microseconds) {
    return guarded([&] {
        if (chains == nullptr || microseconds == nullptr)
            throw std::invalid_argument("schedule buffers must not be null");
        const auto* csr = dynamic_cast<const amfls_gpu::CsrOperator*>(&deref(op));
        if (csr == nullptr) throw std::invalid_argument("operator is not a CSR operator");
        csr->single_column_schedule(chains, microseconds);
    });
}

int amfls_gpu_solve_amfls_batch(int count, const amfls_gpu_operator* const* ops,
                                const double* const* d_b, const amfls_gpu_options* options,
                                double* const* d_solutions, amfls_gpu_result* results,
                                double* seconds, int workers, double* wall_seconds) {
    return guarded([&] {
        if (count < 0) throw std::invalid_argument("count must be nonnegative");
        if (count > 0 && (ops == nullptr || d_b == nullptr || options == nullptr ||
                          d_solutions == nullptr || results == nullptr))
            throw std::invalid_argument("batch arrays must not be null");
        std::vector<amfls_gpu::BatchItem> items(count);
        for (int i = 0; i < count; ++i) {
            items[i].options = to_options(&options[i]);
            items[i].op = &deref(ops[i]);
            items[i].b = d_b[i];
            items[i].x = d_solutions[i];
        }
        const auto out = amfls_gpu::solve_amfls_batch(items, workers, wall_seconds);
        std::string first_error;
        for (int i = 0; i < count; ++i) {
            if (seconds) seconds[i] = out[i].seconds;
            if (out[i].ok)
                export_result(out[i].result, &results[i], nullptr, nullptr, 0);
            else if (first_error.empty())
                first_error = "problem " + std::to_string(i) + ": " + out[i].error;
        }
        if (!first_error.empty()) throw std::runtime_error(first_error);
    });
}

}  // extern "C"
