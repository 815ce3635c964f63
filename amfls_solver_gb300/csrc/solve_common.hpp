// Pieces shared by the solvers' host loops (AMFLS, fixed RBGK, LSQR, LSMR):
// the certificate checkpoint cadence, the numerical-failure test, the
// bookkeeping of one validation and its trace row.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include "controller.hpp"
#include "validation.hpp"

namespace amfls_gpu {

// Iterations at which the certificate is evaluated regardless of prediction
// (certificate_checkpoint_schedule.hpp:15-35): 1, powers of two and, for
// least squares, three times a power of two.
inline bool is_certificate_checkpoint(int it, double reg) {
    if (it <= 1) return true;
    int odd = it;
    while (odd % 2 == 0) odd /= 2;
    return odd == 1 || (reg == 0.0 && odd == 3);
}

// CertificateCheckpointSchedule (certificate_checkpoint_schedule.hpp:37-131):
// besides the fixed checkpoints, at most one predicted log-linear crossing
// of the tolerance per interval.
class CheckpointSchedule {
public:
    CheckpointSchedule(double reg, double tol) : reg_(reg), tol_(tol) {}
    bool should_evaluate(int it) const {
        return is_certificate_checkpoint(it, reg_) || it >= predicted_;
    }
    void record(int it, const ValidationOutput& r) {
        predicted_ = kNone;
        if (is_certificate_checkpoint(it, reg_) && has_prev_ && it > prev_it_) {
            if (reg_ > 0.0) {
                predicted_ = crossing(prev_energy_, r.relative_energy_error_upper_bound, prev_it_, it);
            } else {
                predicted_ = std::min(
                    crossing(prev_compat_, r.compatible_backward_error_upper_bound, prev_it_, it),
                    crossing(prev_ls_, r.least_squares_backward_error_upper_bound, prev_it_, it));
            }
        }
        prev_it_ = it;
        prev_compat_ = r.compatible_backward_error_upper_bound;
        prev_ls_ = r.least_squares_backward_error_upper_bound;
        prev_energy_ = r.relative_energy_error_upper_bound;
        has_prev_ = true;
    }

private:
    using LD = long double;
    static constexpr int kNone = std::numeric_limits<int>::max();
    int crossing(double prev, double cur, int prev_it, int cur_it) const {
        if (!(prev > cur) || !(cur > tol_) || !(tol_ > 0.0) || !std::isfinite(prev) ||
            !std::isfinite(cur) || !std::isfinite(tol_))
            return kNone;
        const LD dist = std::log(static_cast<LD>(cur)) - std::log(static_cast<LD>(tol_));
        const LD contraction = std::log(static_cast<LD>(prev)) - std::log(static_cast<LD>(cur));
        const LD offset = std::ceil(static_cast<LD>(cur_it - prev_it) * dist / contraction);
        if (!(offset > 0.0L) || !std::isfinite(offset) ||
            offset > static_cast<LD>(kNone - cur_it))
            return kNone;
        return cur_it + static_cast<int>(offset);
    }
    double reg_, tol_;
    int predicted_ = kNone;
    int prev_it_ = 0;
    double prev_compat_ = 0.0, prev_ls_ = 0.0, prev_energy_ = 0.0;
    bool has_prev_ = false;
};

// candidate_validation_failed_numerically (candidate_validation.hpp:27-29).
inline bool failed_numerically(const ValidationOutput& v) {
    return v.status == 4 || v.stop_reason == 7;
}

// The operator calls of one validation in the run statistics (base pair and
// refinement, ridge correction), as validate_original_candidate counts them.
inline void account_validation(Statistics& s, const ValidationOutput& v) {
    const int base_a = v.calls[0] + v.calls[2], base_at = v.calls[1] + v.calls[3];
    const int corr_a = v.calls[4], corr_at = v.calls[5];
    s.a_columns += base_a + corr_a;
    s.at_columns += base_at + corr_at;
    s.a_block_calls += base_a + corr_a;
    s.at_block_calls += base_at + corr_at;
    s.validation_a_columns += base_a + corr_a;
    s.validation_at_columns += base_at + corr_at;
    s.validation_a_block_calls += base_a + corr_a;
    s.validation_at_block_calls += base_at + corr_at;
    s.base_validation_a_columns += base_a;
    s.base_validation_at_columns += base_at;
    s.base_validation_a_block_calls += base_a;
    s.base_validation_at_block_calls += base_at;
    s.ridge_correction_a_columns += corr_a;
    s.ridge_correction_at_columns += corr_at;
    s.ridge_correction_a_block_calls += corr_a;
    s.ridge_correction_at_block_calls += corr_at;
    const double ta = v.seconds[0] + v.seconds[2] + v.seconds[4];
    const double tat = v.seconds[1] + v.seconds[3] + v.seconds[5];
    s.a_seconds += ta;
    s.at_seconds += tat;
    s.base_validation_seconds += v.seconds[0] + v.seconds[1] + v.seconds[2] + v.seconds[3];
    s.ridge_correction_validation_seconds += v.seconds[4] + v.seconds[5];
    s.validation_seconds = s.base_validation_seconds + s.ridge_correction_validation_seconds;
}

// make_iteration_record (krylov_workspace.cpp:1206-1260) in the trace
// tensor's column order (result_tensors.hpp:80-156).
inline void fill_trace_row(TraceRow& t, const ValidationOutput& v, const Statistics& s, int epoch,
                           int depth, int auxiliary_width, int basis_rank) {
    const double f[29] = {
        double(epoch), double(depth), double(auxiliary_width), double(basis_rank),
        double(s.a_columns), double(s.at_columns), double(s.a_block_calls),
        double(s.at_block_calls), v.objective, v.residual_norm,
        v.augmented_residual_norm, v.normal_residual_norm, v.operator_norm_lower_bound,
        v.compatible_backward_error_upper_bound, v.least_squares_backward_error_upper_bound,
        v.backward_error_upper_bound, v.relative_normal_residual_upper_bound,
        v.relative_energy_error_upper_bound, v.solution_norm, v.solution_energy_norm,
        v.augmented_operator_norm_lower_bound, v.energy_error_upper_bound,
        v.objective_gap_upper_bound, v.ridge_base_energy_error_upper_bound,
        v.ridge_corrected_energy_error_upper_bound, v.ridge_correction_gamma,
        v.ridge_correction_z_h_z, v.ridge_correction_two_abs_z_t_q,
        v.ridge_correction_q_norm_squared};
    std::memcpy(t.f, f, sizeof(f));
    t.i[0] = v.status;
    t.i[1] = v.stop_reason;
    t.i[2] = v.status == 0 ? 1 : 0;
    t.i[3] = v.ridge_correction_disposition;
}

}  // namespace amfls_gpu
