// Device-resident state of the block Golub-Kahan process.
//
// The reference keeps this state in host members of BlockGolubKahanWorkspace
// (src/algorithms/mathematics/krylov/krylov_workspace.hpp:154-188) and its
// per-step audit in BlockGolubKahanStepAudit (krylov_workspace.hpp:22-43).
// Here the scalar part lives in device memory so that a run of levels can be
// enqueued without host round trips: every level's first kernel decides on
// the device whether the level runs (the reference's can_advance() and the
// depth target), and every rank decision is taken by a device kernel.  The
// host reads this struct back only at checkpoints.
#pragma once

namespace amfls_gpu {

struct StepAudit {
    int requested_injected_columns;
    int retained_injected_columns;
    int left_input_width;
    int retained_right_width;
    int retained_next_left_width;
    int basis_rank_before;
    int basis_rank_after;
    int right_rank_loss;
    int left_rank_loss;
    int right_positive_finite_below_cutoff;
    int left_positive_finite_below_cutoff;
    int right_nonfinite_residual;
    int left_nonfinite_residual;
    int right_basis_cap_truncation;
    int left_basis_cap_truncation;
    int pad;
    double right_rank_cutoff;
    double right_discarded_residual_norm;
    double right_active_discarded_residual_norm;
    double left_rank_cutoff;
    double left_discarded_residual_norm;
};

struct DevState {
    // process state (krylov_workspace.hpp:154-188)
    int k;                 // right basis rank = V columns
    int depth;             // completed levels
    int reliable;          // continuation_reliable_
    int left_width;        // physical active left columns (U)
    int pending;           // pending P*Omega columns
    int rows_t;            // logical T rows = g entries
    int active_first;      // active_left_.first
    int prev_right_first;  // previous_right_
    int prev_right_width;
    int basis_limit;
    // per-level control
    int go;           // the current level runs
    int second_pass;  // DGKS second projection needed (right or left side)
    int right_rank;   // retained right width of the current level
    int left_rank;    // retained next left width of the current level
    int level_ok;     // advance_level's return value for the last run level
    int coeff_nonfinite;
    int target_depth;     // depth at which the enqueued run of levels stops
    int iterations_left;  // hard cap on loop iterations of the enqueued run
    int sub_col;          // V column subtracted by the coupling (0 when none)
    int sweep_fp64;       // reduced-basis level: redo the projection in FP64
    // device time of search operator calls (globaltimer, ns)
    unsigned long long a_ns;
    unsigned long long at_ns;
    unsigned long long t_mark;
    long long body_runs;   // executions of the captured level body
    // operator call counters of executed search levels
    long long search_a_columns;
    long long search_at_columns;
    long long search_a_calls;
    long long search_at_calls;
    long long levels_run;
    long long reduced_levels;    // levels projected on the reduced copy of V
    long long reduced_fallbacks; // of those, levels redone in FP64
    // scalars of the current level
    double coupling;       // frontier coupling (1x1 at width one)
    double coupling_eff;   // coupling actually subtracted (0 when none applies)
    double right_scale;
    double norm_before;
    double norm_after;
    double right_factor;   // retained right factor (= residual norm)
    double left_scale;
    double left_coeff;     // accumulated left projection coefficient
    double pass_coeff;     // coefficient of the pending second left pass
    double b_dot;          // (unnormalised next left vector) . b
    double inv_right;      // 1 / retained right factor
    double inv_left;       // 1 / retained left factor
    double left_norm;      // left residual norm after projection
    StepAudit audit;
};

}  // namespace amfls_gpu
