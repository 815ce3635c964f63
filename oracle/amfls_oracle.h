/* Test infrastructure: the C half of the AMFLS oracle (a CPU restatement of the
 * reference's arithmetic, used only by tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg as the checker).  Parity pinned against the
 * reference's own outputs through the fixtures in tests/golden/.
 */
#ifndef AMFLS_ORACLE_H
#define AMFLS_ORACLE_H
#include <stdint.h>

/* Operator description: kind 0 = CSR (int64 offsets / indices), 1 = row-major
 * dense, 2 = column-major dense, 3 = CSR behind a custom MatrixOperator (no
 * extended-precision validation products). */
typedef struct {
    int kind;
    int rows;
    int cols;
    const int64_t* row_offsets;
    const int64_t* column_indices;
    const double* values;
    int64_t nonzeros;
} orc_operator;

typedef struct {
    double norm_upper;
    double norm_lower;
    long long apply_steps;
    long long transpose_steps;
} orc_model;

/* Validation output: the LeastSquaresResult scalar fields. */
typedef struct {
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
    /* operator calls made: base A, base At, refinement A, refinement At,
     * correction A, correction At */
    int calls[6];
} orc_validation;

void orc_apply(const orc_operator* op, const double* x, int block_cols, double* y);
void orc_apply_transpose(const orc_operator* op, const double* y, int block_cols, double* x);
int orc_model_of(const orc_operator* op, orc_model* out);
void orc_gaussian_matrix(int rows, int cols, uint64_t seed, uint64_t stream,
                         uint64_t first_column, double* out);
void orc_norm_interval(const double* v, int64_t n, double* lower, double* upper);
double orc_binary64_gamma(long long operations);
void orc_validate(const orc_operator* op, const orc_model* model, const double* b,
                  const double* x, double regularization, double tolerance,
                  orc_validation* out);
#endif
