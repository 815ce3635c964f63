/* Test infrastructure: the C half of the AMFLS oracle.
 *
 * A CPU restatement of the reference's scalar and elementwise arithmetic,
 * written independently from its description in doloMing/amfls_solver and
 * used only as the checker (tests/, __graft_entry__.smoke(), bench.py's
 * cpu_baseline leg).  The product never links it.  Parity is pinned against
 * the reference's own outputs through tests/golden/ (see test_oracle.py).
 *
 * Contents and the reference code each part follows:
 *   directed rounding via long double   floating_point_bounds.hpp:35-210, 383-401
 *   norm_interval                       floating_point_bounds.hpp:325-376
 *   CSR products (sequential FMA)       sparse_csr_operator.cpp:203-269
 *   CSR norm model                      sparse_csr_operator.cpp:14-149
 *   dense norm models                   dense_operator.cpp:20-115,
 *                                       row_major_dense_operator.cpp:20-115
 *   long-double validation products     sparse_csr_operator.cpp:155-201 (and dense analogues)
 *   counter Gaussian (splitmix64 + Box-Muller)  gaussian.cpp:13-55
 *   validate_original_candidate         candidate_validation.cpp:67-1378
 */
#include "amfls_oracle.h"

/* kind 3 is a CSR matrix behind a custom MatrixOperator: the same products
 * and model, but no extended-precision validation products (the interface
 * defaults, matrix_operator.hpp:62-88), so validation never refines. */
#define IS_CSR(op) ((op)->kind == 0 || (op)->kind == 3)

#include <fenv.h>
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define INF_D ((double)INFINITY)

/* ---------------------------------------------------------------- fp ---- */

static int subnormals_survive(void) {
    volatile double tiny = 4.9406564584124654e-324;
    volatile double one = 1.0;
    volatile double kept = tiny * one;
    volatile double smallest = DBL_MIN;
    volatile double half = 0.5;
    volatile double made = smallest * half;
    return kept == 4.9406564584124654e-324 && made > 0.0;
}

static int binary64_environment(void) {
    return fegetround() == FE_TONEAREST && subnormals_survive();
}

/* Round a nonnegative long double up to a binary64, then one more step up. */
static double up_ld(long double v) {
    if (!(v >= 0.0L) || !isfinite(v) || v > (long double)DBL_MAX) return INF_D;
    if (v == 0.0L) return 0.0;
    double r = (double)v;
    if ((long double)r < v) r = nextafter(r, INF_D);
    return nextafter(r, INF_D);
}

static double down_ld(long double v) {
    if (!(v > 0.0L) || !isfinite(v)) return 0.0;
    if (v > (long double)DBL_MAX) return DBL_MAX;
    double r = (double)v;
    if ((long double)r > v) r = nextafter(r, 0.0);
    return nextafter(r, 0.0);
}

double orc_binary64_gamma(long long ops) {
    if (ops < 0) return INF_D;
    long double t = (long double)ops * (0.5L * (long double)DBL_EPSILON);
    if (!(t < 1.0L)) return INF_D;
    return up_ld(t / (1.0L - t));
}

static double up_add(double a, double b) {
    return up_ld((long double)a + (long double)b);
}

static double up_mul(double a, double b) {
    if (a < 0.0 || b < 0.0) return INF_D;
    long double p = (long double)a * (long double)b;
    if (a > 0.0 && b > 0.0 && p == 0.0L) return 4.9406564584124654e-324;
    return up_ld(p);
}

static double down_add(double a, double b) {
    if (a < 0.0 || b < 0.0 || !isfinite(a) || !isfinite(b)) return 0.0;
    return down_ld((long double)a + (long double)b);
}

static double down_mul(double a, double b) {
    if (a < 0.0 || b < 0.0 || !isfinite(a) || !isfinite(b)) return 0.0;
    return down_ld((long double)a * (long double)b);
}

static double down_div(double a, double b) {
    if (!(a > 0.0) || !(b > 0.0) || !isfinite(a) || !isfinite(b)) return 0.0;
    return down_ld((long double)a / (long double)b);
}

static double down_diff(double a, double b) {
    if (!(a > b) || !isfinite(a) || b < 0.0 || !isfinite(b)) return 0.0;
    return down_ld((long double)a - (long double)b);
}

static double up_div(double a, double b) {
    if (a == 0.0) return 0.0;
    if (!(b > 0.0) || a < 0.0 || !isfinite(a) || !isfinite(b)) return INF_D;
    long double q = (long double)a / (long double)b;
    if (q == 0.0L) return 4.9406564584124654e-324;
    return up_ld(q);
}

static double up_sqrt(double v) {
    if (v < 0.0 || !isfinite(v)) return v == INF_D ? v : INF_D;
    return up_ld(sqrtl((long double)v) * (1.0L + 2.0L * LDBL_EPSILON));
}

static double down_sqrt(double v) {
    if (!(v > 0.0) || !isfinite(v)) return 0.0;
    return down_ld(sqrtl((long double)v) * (1.0L - 2.0L * LDBL_EPSILON));
}

/* Upper bound of an exact nonnegative sum given its stored binary64 value
 * after `ops` rounded operations (gamma_k plus k denorm_min). */
static double sum_upper(double stored, long long ops, int zero_is_exact) {
    if (stored < 0.0 || !isfinite(stored) || ops < 0) return INF_D;
    if (zero_is_exact && stored == 0.0) return 0.0;
    double g = orc_binary64_gamma(ops);
    double den = down_diff(1.0, g);
    if (!(den > 0.0)) return INF_D;
    double absr = up_ld((long double)ops * (long double)4.9406564584124654e-324);
    return up_div(up_add(stored, absr), den);
}

static double sum_lower(double stored, long long ops) {
    if (!(stored > 0.0) || !isfinite(stored) || ops < 0) return 0.0;
    double g = orc_binary64_gamma(ops);
    double den = up_add(1.0, g);
    if (!isfinite(den)) return 0.0;
    double absr = up_ld((long double)ops * (long double)4.9406564584124654e-324);
    return down_div(down_diff(stored, absr), den);
}

static double scale_up_pow2(double v, int e) {
    if (v == 0.0) return 0.0;
    if (!(v > 0.0) || !isfinite(v)) return INF_D;
    double s = scalbn(v, e);
    if (isinf(s)) return s;
    if (s == 0.0) return 4.9406564584124654e-324;
    return nextafter(s, INF_D);
}

static double scale_down_pow2(double v, int e) {
    if (!(v > 0.0) || !isfinite(v)) return 0.0;
    double s = scalbn(v, e);
    if (isinf(s)) return DBL_MAX;
    if (s == 0.0) return 0.0;
    return nextafter(s, 0.0);
}

void orc_norm_interval(const double* v, int64_t n, double* lower, double* upper) {
    *lower = 0.0;
    *upper = INF_D;
    if (!binary64_environment()) return;
    double mx = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        if (!isfinite(v[i])) return;
        double a = fabs(v[i]);
        if (a > mx) mx = a;
    }
    if (mx == 0.0) {
        *lower = 0.0;
        *upper = 0.0;
        return;
    }
    int e = 0;
    (void)frexp(mx, &e);
    double acc = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double s = scalbn(fabs(v[i]), -e);
        acc = fma(s, s, acc);
    }
    double lo2 = sum_lower(acc, (long long)n);
    double hi2 = sum_upper(acc, (long long)n, 1);
    double lo = down_sqrt(lo2);
    double hi = up_sqrt(hi2);
    double serr = up_ld(sqrtl((long double)n) * (long double)4.9406564584124654e-324);
    *lower = scale_down_pow2(down_diff(lo, serr), e);
    *upper = scale_up_pow2(up_add(hi, serr), e);
}

/* --------------------------------------------------------- operators ---- */

void orc_apply(const orc_operator* op, const double* x, int s, double* y) {
    const int64_t m = op->rows, n = op->cols;
    memset(y, 0, sizeof(double) * (size_t)(m * s));
    if (IS_CSR(op)) {
        for (int64_t r = 0; r < m; ++r)
            for (int64_t e = op->row_offsets[r]; e < op->row_offsets[r + 1]; ++e) {
                const int64_t c = op->column_indices[e];
                const double a = op->values[e];
                for (int k = 0; k < s; ++k)
                    y[k * m + r] = fma(a, x[k * n + c], y[k * m + r]);
            }
    } else if (op->kind == 1) {
        for (int k = 0; k < s; ++k)
            for (int64_t r = 0; r < m; ++r) {
                double acc = 0.0;
                const double* row = op->values + r * n;
                for (int64_t c = 0; c < n; ++c) acc = fma(row[c], x[k * n + c], acc);
                y[k * m + r] = acc;
            }
    } else {
        for (int k = 0; k < s; ++k)
            for (int64_t c = 0; c < n; ++c) {
                const double xc = x[k * n + c];
                const double* col = op->values + c * m;
                for (int64_t r = 0; r < m; ++r) y[k * m + r] = fma(col[r], xc, y[k * m + r]);
            }
    }
}

void orc_apply_transpose(const orc_operator* op, const double* y, int s, double* x) {
    const int64_t m = op->rows, n = op->cols;
    memset(x, 0, sizeof(double) * (size_t)(n * s));
    if (IS_CSR(op)) {
        for (int64_t r = 0; r < m; ++r)
            for (int64_t e = op->row_offsets[r]; e < op->row_offsets[r + 1]; ++e) {
                const int64_t c = op->column_indices[e];
                const double a = op->values[e];
                for (int k = 0; k < s; ++k)
                    x[k * n + c] = fma(a, y[k * m + r], x[k * n + c]);
            }
    } else if (op->kind == 1) {
        for (int k = 0; k < s; ++k)
            for (int64_t r = 0; r < m; ++r) {
                const double yr = y[k * m + r];
                const double* row = op->values + r * n;
                for (int64_t c = 0; c < n; ++c) x[k * n + c] = fma(row[c], yr, x[k * n + c]);
            }
    } else {
        for (int k = 0; k < s; ++k)
            for (int64_t c = 0; c < n; ++c) {
                double acc = 0.0;
                const double* col = op->values + c * m;
                for (int64_t r = 0; r < m; ++r) acc = fma(col[r], y[k * m + r], acc);
                x[k * n + c] = acc;
            }
    }
}

/* Extended-precision validation products: long double multiply/add over the
 * stored binary64 entries (row sums for A, row-ordered scatter for A^T). */
static int apply_ld(const orc_operator* op, const long double* x, long double* y) {
    const int64_t m = op->rows, n = op->cols;
    if (IS_CSR(op)) {
        for (int64_t r = 0; r < m; ++r) {
            long double acc = 0.0L;
            for (int64_t e = op->row_offsets[r]; e < op->row_offsets[r + 1]; ++e)
                acc += (long double)op->values[e] * x[op->column_indices[e]];
            if (!isfinite(acc)) return 0;
            y[r] = acc;
        }
        return 1;
    }
    if (op->kind == 1) {
        for (int64_t r = 0; r < m; ++r) {
            long double acc = 0.0L;
            for (int64_t c = 0; c < n; ++c) acc += (long double)op->values[r * n + c] * x[c];
            if (!isfinite(acc)) return 0;
            y[r] = acc;
        }
        return 1;
    }
    for (int64_t r = 0; r < m; ++r) y[r] = 0.0L;
    for (int64_t c = 0; c < n; ++c) {
        if (!isfinite(x[c])) return 0;
        for (int64_t r = 0; r < m; ++r) y[r] += (long double)op->values[c * m + r] * x[c];
    }
    for (int64_t r = 0; r < m; ++r)
        if (!isfinite(y[r])) return 0;
    return 1;
}

static int apply_transpose_ld(const orc_operator* op, const long double* y, long double* x) {
    const int64_t m = op->rows, n = op->cols;
    if (op->kind == 2) {
        for (int64_t c = 0; c < n; ++c) {
            long double acc = 0.0L;
            for (int64_t r = 0; r < m; ++r) acc += (long double)op->values[c * m + r] * y[r];
            if (!isfinite(acc)) return 0;
            x[c] = acc;
        }
        return 1;
    }
    for (int64_t c = 0; c < n; ++c) x[c] = 0.0L;
    for (int64_t r = 0; r < m; ++r) {
        const long double yr = y[r];
        if (!isfinite(yr)) return 0;
        if (IS_CSR(op)) {
            for (int64_t e = op->row_offsets[r]; e < op->row_offsets[r + 1]; ++e)
                x[op->column_indices[e]] += (long double)op->values[e] * yr;
        } else {
            for (int64_t c = 0; c < n; ++c) x[c] += (long double)op->values[r * n + c] * yr;
        }
    }
    for (int64_t c = 0; c < n; ++c)
        if (!isfinite(x[c])) return 0;
    return 1;
}

/* Norm bounds: ||A||_2 <= min(sqrt(||A||_1 ||A||_inf), ||A||_F) and
 * ||A||_2 >= max(max |a_ij|, max row/column 2-norm), all outward rounded. */
int orc_model_of(const orc_operator* op, orc_model* out) {
    const int64_t m = op->rows, n = op->cols;
    out->norm_upper = INF_D;
    out->norm_lower = 0.0;
    double max_row_sum = 0.0, max_col_sum = 0.0, max_two_lower = 0.0, max_entry = 0.0;
    double frob2 = 0.0;
    int certifiable = 1;
    if (IS_CSR(op)) {
        int64_t max_row_nnz = 0, max_col_nnz = 0;
        int64_t* col_nnz = calloc((size_t)n, sizeof(int64_t));
        double* col_sum = calloc((size_t)n, sizeof(double));
        double* col_sq = calloc((size_t)n, sizeof(double));
        for (int64_t r = 0; r < m; ++r) {
            const int64_t len = op->row_offsets[r + 1] - op->row_offsets[r];
            if (len > max_row_nnz) max_row_nnz = len;
            double rs = 0.0, rq = 0.0;
            for (int64_t e = op->row_offsets[r]; e < op->row_offsets[r + 1]; ++e) {
                const int64_t c = op->column_indices[e];
                const double a = fabs(op->values[e]);
                if (++col_nnz[c] > max_col_nnz) max_col_nnz = col_nnz[c];
                if (a > max_entry) max_entry = a;
                rs += a;
                col_sum[c] += a;
                rq = fma(a, a, rq);
                col_sq[c] = fma(a, a, col_sq[c]);
            }
            double u = sum_upper(rs, len, 1);
            if (u > max_row_sum) max_row_sum = u;
            double l = down_sqrt(sum_lower(rq, len));
            if (l > max_two_lower) max_two_lower = l;
        }
        for (int64_t c = 0; c < n; ++c) {
            double u = sum_upper(col_sum[c], col_nnz[c], 1);
            if (u > max_col_sum) max_col_sum = u;
            double l = down_sqrt(sum_lower(col_sq[c], col_nnz[c]));
            if (l > max_two_lower) max_two_lower = l;
            frob2 = up_add(frob2, sum_upper(col_sq[c], col_nnz[c], 0));
        }
        free(col_nnz);
        free(col_sum);
        free(col_sq);
        out->apply_steps = 2LL * max_row_nnz + 2LL;
        out->transpose_steps = 2LL * max_col_nnz + 2LL;
    } else {
        /* outer loop runs over the storage-major index like the reference */
        const int row_major = op->kind == 1;
        const int64_t outer = row_major ? m : n, inner = row_major ? n : m;
        double* in_sum = calloc((size_t)inner, sizeof(double));
        double* in_sq = calloc((size_t)inner, sizeof(double));
        double max_outer_sum = 0.0, max_inner_sum = 0.0;
        for (int64_t o = 0; o < outer; ++o) {
            double os = 0.0, oq = 0.0;
            for (int64_t i = 0; i < inner; ++i) {
                const double a = fabs(op->values[o * inner + i]);
                if (!isfinite(a)) {
                    certifiable = 0;
                    continue;
                }
                if (a > max_entry) max_entry = a;
                in_sum[i] += a;
                in_sq[i] = fma(a, a, in_sq[i]);
                os += a;
                oq = fma(a, a, oq);
            }
            double u = sum_upper(os, inner, 1);
            if (u > max_outer_sum) max_outer_sum = u;
            double l = down_sqrt(sum_lower(oq, inner));
            if (l > max_two_lower) max_two_lower = l;
            if (!row_major) frob2 = up_add(frob2, sum_upper(oq, inner, 0));
        }
        for (int64_t i = 0; i < inner; ++i) {
            double u = sum_upper(in_sum[i], outer, 1);
            if (u > max_inner_sum) max_inner_sum = u;
        }
        for (int64_t i = 0; i < inner; ++i) {
            double l = down_sqrt(sum_lower(in_sq[i], outer));
            if (l > max_two_lower) max_two_lower = l;
            if (row_major) frob2 = up_add(frob2, sum_upper(in_sq[i], outer, 0));
        }
        free(in_sum);
        free(in_sq);
        max_row_sum = row_major ? max_outer_sum : max_inner_sum;
        max_col_sum = row_major ? max_inner_sum : max_outer_sum;
        out->apply_steps = 2LL * n + 2LL;
        out->transpose_steps = 2LL * m + 2LL;
    }
    if (certifiable && binary64_environment()) {
        double one_inf = up_mul(up_sqrt(max_col_sum), up_sqrt(max_row_sum));
        double frob = up_sqrt(frob2);
        out->norm_upper = one_inf < frob ? one_inf : frob;
        out->norm_lower = max_entry > max_two_lower ? max_entry : max_two_lower;
    }
    if (!isfinite(out->norm_upper) || out->norm_lower > out->norm_upper) {
        out->norm_upper = INF_D;
        out->norm_lower = 0.0;
    }
    return 0;
}

/* ---------------------------------------------------------- gaussian ---- */

static uint64_t mix64(uint64_t v) {
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

static double unit_open(uint64_t bits) {
    return (double)((bits >> 11) + 1U) * (1.0 / 9007199254740992.0);
}

void orc_gaussian_matrix(int rows, int cols, uint64_t seed, uint64_t stream,
                         uint64_t first_column, double* out) {
    const uint64_t key = mix64(seed) ^ mix64(stream + 0xd2b74407b1ce6e93ULL);
    const double two_pi = 6.283185307179586476925286766559;
    for (int c = 0; c < cols; ++c)
        for (int r = 0; r < rows; ++r) {
            const uint64_t idx = (first_column + (uint64_t)c) * (uint64_t)rows + (uint64_t)r;
            const double u1 = unit_open(mix64(key ^ (2U * idx)));
            const double u2 = unit_open(mix64(key ^ (2U * idx + 1U)));
            out[(size_t)c * rows + r] = sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
        }
}

/* -------------------------------------------------------- validation ---- */

typedef struct {
    double lower, upper;
} interval;

typedef struct {
    int certified;
    double op_upper, op_lower;
    double res_lower, res_upper, grad_upper, sol_lower, sol_upper, b_lower;
    double energy_lower, grad_radius;
} envelope;

static int model_ok(const orc_model* m) {
    return binary64_environment() && isfinite(m->norm_upper) && m->norm_upper >= 0.0 &&
           isfinite(m->norm_lower) && m->norm_lower >= 0.0 && m->norm_lower <= m->norm_upper &&
           m->apply_steps > 0 && m->transpose_steps > 0;
}

static double underflow_radius(long long ops, int64_t size) {
    if (ops <= 0 || size <= 0) return 0.0;
    return up_ld((long double)ops * sqrtl((long double)size) * (long double)4.9406564584124654e-324);
}

static double callback_radius(const orc_model* m, int transpose, double in_upper, int64_t out_size) {
    if (!model_ok(m) || !isfinite(in_upper) || in_upper < 0.0) return INF_D;
    if (m->norm_upper == 0.0 || in_upper == 0.0) return 0.0;
    const long long ops = transpose ? m->transpose_steps : m->apply_steps;
    return up_add(up_mul(orc_binary64_gamma(ops), up_mul(m->norm_upper, in_upper)),
                  underflow_radius(ops, out_size));
}

static double one_op_radius(double stored_upper, int can_underflow, int64_t size) {
    if (!isfinite(stored_upper) || stored_upper < 0.0) return INF_D;
    double r = up_mul(orc_binary64_gamma(2), stored_upper);
    if (can_underflow) r = up_add(r, underflow_radius(1, size));
    return r;
}

static double ld_gamma(long long ops) {
    if (ops < 0) return INF_D;
    long double t = (long double)ops * (0.5L * LDBL_EPSILON);
    if (!(t < 1.0L)) return INF_D;
    return up_ld(t / (1.0L - t));
}

static double ld_underflow_radius(long long ops, int64_t size) {
    if (ops <= 0 || size <= 0) return 0.0;
    return up_ld((long double)ops * sqrtl((long double)size) * LDBL_TRUE_MIN);
}

static double ld_callback_radius(const orc_model* m, long long dot_length, double in_upper, int64_t out_size) {
    if (!model_ok(m) || dot_length <= 0 || !isfinite(in_upper) || in_upper < 0.0) return INF_D;
    if (m->norm_upper == 0.0 || in_upper == 0.0) return 0.0;
    const long long ops = 2 * dot_length;
    return up_add(up_mul(ld_gamma(ops), up_mul(m->norm_upper, in_upper)),
                  ld_underflow_radius(ops, out_size));
}

static double ld_one_op_radius(double stored_upper, int can_underflow, int64_t size) {
    if (!isfinite(stored_upper) || stored_upper < 0.0) return INF_D;
    double r = up_mul(ld_gamma(2), stored_upper);
    if (can_underflow) r = up_add(r, ld_underflow_radius(1, size));
    return r;
}

static interval enlarge(interval s, double radius) {
    interval out = {0.0, INF_D};
    if (!isfinite(radius) || radius < 0.0) return out;
    out.lower = down_diff(s.lower, radius);
    out.upper = up_add(s.upper, radius);
    return out;
}

static interval augmented(interval p, interval s, double reg) {
    interval out;
    out.lower = down_sqrt(down_add(down_mul(p.lower, p.lower), down_mul(reg, down_mul(s.lower, s.lower))));
    out.upper = up_sqrt(up_add(up_mul(p.upper, p.upper), up_mul(reg, up_mul(s.upper, s.upper))));
    return out;
}

static interval nint(const double* v, int64_t n) {
    interval i;
    orc_norm_interval(v, n, &i.lower, &i.upper);
    return i;
}

static double norm2(const double* v, int64_t n) {
    /* accurate Euclidean norm with scaling (stands in for dnrm2) */
    double mx = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        if (isnan(v[i])) return NAN;
        double a = fabs(v[i]);
        if (a > mx) mx = a;
    }
    if (mx == 0.0 || isinf(mx)) return mx;
    long double acc = 0.0L;
    for (int64_t i = 0; i < n; ++i) {
        long double s = (long double)v[i] / (long double)mx;
        acc += s * s;
    }
    return (double)((long double)mx * sqrtl(acc));
}

static double dot(const double* a, const double* b, int64_t n) {
    long double acc = 0.0L;
    for (int64_t i = 0; i < n; ++i) acc += (long double)a[i] * (long double)b[i];
    return (double)acc;
}

static int all_finite(const double* v, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (!isfinite(v[i])) return 0;
    return 1;
}

static double ratio_cert(double num, double den) {
    if (!isfinite(num)) return INF_D;
    if (num == 0.0) return 0.0;
    if (!isfinite(den) || den <= 0.0) return INF_D;
    return num / den;
}

static double rel_energy(double abs_bound, double energy) {
    if (!isfinite(energy)) return INF_D;
    if (abs_bound == 0.0) return 0.0;
    if (!isfinite(abs_bound) || energy <= 0.0) return INF_D;
    double s = abs_bound / energy;
    if (!isfinite(s) || s >= 1.0) return INF_D;
    return s / (1.0 - s);
}

enum { ST_SUCCESS = 0, ST_WORK = 1, ST_BREAKDOWN = 4 };
enum { SR_EXACT = 1, SR_DEPTH = 3, SR_BREAKDOWN = 7, SR_COMPAT = 8, SR_LS = 9, SR_ENERGY = 10 };

static void nominal_contract(orc_validation* r, double bnorm, double reg, double tol,
                             int has_ridge, double ridge_bound) {
    const double rr = sqrt(reg);
    r->augmented_residual_norm = hypot(r->residual_norm, rr * r->solution_norm);
    r->augmented_operator_norm_lower_bound = hypot(r->operator_norm_lower_bound, rr);
    r->compatible_backward_error_upper_bound = ratio_cert(
        r->augmented_residual_norm,
        r->augmented_operator_norm_lower_bound * r->solution_norm + bnorm);
    r->least_squares_backward_error_upper_bound = ratio_cert(
        r->normal_residual_norm,
        r->augmented_operator_norm_lower_bound * r->augmented_residual_norm);
    r->backward_error_upper_bound = fmin(r->compatible_backward_error_upper_bound,
                                         r->least_squares_backward_error_upper_bound);
    const double opl = r->operator_norm_lower_bound;
    r->relative_normal_residual_upper_bound = ratio_cert(
        r->normal_residual_norm, (opl * opl + reg) * r->solution_norm + opl * bnorm);
    if (reg > 0.0) {
        double req = has_ridge ? ridge_bound : r->normal_residual_norm / rr;
        r->energy_error_upper_bound = req >= 0.0 ? req : INF_D;
        r->objective_gap_upper_bound = r->energy_error_upper_bound * r->energy_error_upper_bound;
        r->relative_energy_error_upper_bound = rel_energy(r->energy_error_upper_bound,
                                                          r->solution_energy_norm);
    } else if (r->normal_residual_norm == 0.0) {
        r->energy_error_upper_bound = r->relative_energy_error_upper_bound = 0.0;
        r->objective_gap_upper_bound = 0.0;
    } else {
        r->energy_error_upper_bound = r->relative_energy_error_upper_bound = INF_D;
        r->objective_gap_upper_bound = INF_D;
    }
#define FIN(v) (isfinite(v) && (v) >= 0.0)
    if (!(FIN(bnorm) && FIN(r->residual_norm) && FIN(r->augmented_residual_norm) &&
          FIN(r->normal_residual_norm) && FIN(r->solution_norm) &&
          FIN(r->solution_energy_norm) && FIN(r->objective) &&
          FIN(r->operator_norm_lower_bound) && FIN(r->augmented_operator_norm_lower_bound))) {
        r->status = ST_BREAKDOWN;
        r->stop_reason = SR_BREAKDOWN;
        return;
    }
#undef FIN
    const int passed = reg > 0.0 ? r->relative_energy_error_upper_bound <= tol
                                 : r->backward_error_upper_bound <= tol;
    r->status = passed ? ST_SUCCESS : ST_WORK;
    if (r->normal_residual_norm == 0.0) r->stop_reason = SR_EXACT;
    else if (passed && reg > 0.0) r->stop_reason = SR_ENERGY;
    else if (passed && r->compatible_backward_error_upper_bound <=
                           r->least_squares_backward_error_upper_bound)
        r->stop_reason = SR_COMPAT;
    else if (passed) r->stop_reason = SR_LS;
    else r->stop_reason = SR_DEPTH;
}

static void certified_contract(orc_validation* r, const envelope* e, double reg, double tol,
                               int has_ridge, double ridge_bound) {
    if (!e->certified) {
        r->compatible_backward_error_upper_bound = INF_D;
        r->least_squares_backward_error_upper_bound = INF_D;
        r->backward_error_upper_bound = INF_D;
        r->relative_normal_residual_upper_bound = INF_D;
        r->energy_error_upper_bound = INF_D;
        r->relative_energy_error_upper_bound = INF_D;
        r->objective_gap_upper_bound = INF_D;
        r->status = ST_WORK;
        r->stop_reason = SR_DEPTH;
        return;
    }
    interval sol = {e->sol_lower, e->sol_upper};
    interval res = {e->res_lower, e->res_upper};
    interval aug = augmented(res, sol, reg);
    const double opl = r->operator_norm_lower_bound;
    r->augmented_operator_norm_lower_bound = down_sqrt(down_add(down_mul(opl, opl), reg));
    const double aopl = r->augmented_operator_norm_lower_bound;
    r->compatible_backward_error_upper_bound =
        up_div(aug.upper, down_add(down_mul(aopl, e->sol_lower), e->b_lower));
    r->least_squares_backward_error_upper_bound =
        up_div(e->grad_upper, down_mul(aopl, aug.lower));
    r->backward_error_upper_bound = fmin(r->compatible_backward_error_upper_bound,
                                         r->least_squares_backward_error_upper_bound);
    r->relative_normal_residual_upper_bound = up_div(
        e->grad_upper,
        down_add(down_mul(down_add(down_mul(opl, opl), reg), e->sol_lower), down_mul(opl, e->b_lower)));
    if (reg > 0.0) {
        double base = up_div(e->grad_upper, down_sqrt(reg));
        r->energy_error_upper_bound = has_ridge ? ridge_bound : base;
        r->objective_gap_upper_bound = up_mul(r->energy_error_upper_bound, r->energy_error_upper_bound);
        r->relative_energy_error_upper_bound = up_div(
            r->energy_error_upper_bound, down_diff(e->energy_lower, r->energy_error_upper_bound));
    } else if (e->grad_upper == 0.0) {
        r->energy_error_upper_bound = r->relative_energy_error_upper_bound = 0.0;
        r->objective_gap_upper_bound = 0.0;
    } else {
        r->energy_error_upper_bound = r->relative_energy_error_upper_bound = INF_D;
        r->objective_gap_upper_bound = INF_D;
    }
    const int passed = e->grad_upper == 0.0 ||
                       (reg > 0.0 ? r->relative_energy_error_upper_bound <= tol
                                  : r->backward_error_upper_bound <= tol);
    r->status = passed ? ST_SUCCESS : ST_WORK;
    if (e->grad_upper == 0.0) r->stop_reason = SR_EXACT;
    else if (passed && reg > 0.0) r->stop_reason = SR_ENERGY;
    else if (passed && r->compatible_backward_error_upper_bound <=
                           r->least_squares_backward_error_upper_bound)
        r->stop_reason = SR_COMPAT;
    else if (passed) r->stop_reason = SR_LS;
    else r->stop_reason = SR_DEPTH;
}

static void fill_norms(orc_validation* r, const double* x, const double* ax, const double* res,
                       const double* g, int64_t m, int64_t n, double reg) {
    const double an = norm2(ax, m);
    r->residual_norm = norm2(res, m);
    r->normal_residual_norm = norm2(g, n);
    r->solution_norm = norm2(x, n);
    r->solution_energy_norm = hypot(an, sqrt(reg) * r->solution_norm);
    r->objective = r->residual_norm * r->residual_norm + reg * r->solution_norm * r->solution_norm;
}

static envelope base_envelope(const orc_model* mdl, const double* b, const double* x,
                              const double* ax, const double* res, const double* atr,
                              const double* g, int64_t m, int64_t n, double reg) {
    envelope e;
    memset(&e, 0, sizeof(e));
    e.op_upper = mdl->norm_upper;
    e.res_upper = e.grad_upper = e.sol_upper = e.grad_radius = INF_D;
    if (!model_ok(mdl)) return e;
    interval bn = nint(b, m), xn = nint(x, n), an = nint(ax, m), rn = nint(res, m);
    interval tn = nint(atr, n), gn = nint(g, n);
    const double apply_err = callback_radius(mdl, 0, xn.upper, m);
    const double sub_err = one_op_radius(rn.upper, an.upper > 0.0 || bn.upper > 0.0, m);
    const double res_err = up_add(apply_err, sub_err);
    interval true_res = enlarge(rn, res_err);
    const double t_err = callback_radius(mdl, 1, rn.upper, n);
    const double ridge_err = one_op_radius(gn.upper, reg > 0.0 && xn.upper > 0.0, n);
    const double prop = up_mul(e.op_upper, res_err);
    const double g_err = up_add(up_add(t_err, prop), ridge_err);
    interval true_g = enlarge(gn, g_err);
    interval true_a = enlarge(an, apply_err);
    double opl = mdl->norm_lower;
    if (xn.upper > 0.0) opl = fmax(opl, down_div(down_diff(an.lower, apply_err), xn.upper));
    if (rn.upper > 0.0) opl = fmax(opl, down_div(down_diff(tn.lower, t_err), rn.upper));
    interval energy = augmented(true_a, xn, reg);
    e.res_lower = true_res.lower;
    e.res_upper = true_res.upper;
    e.grad_upper = true_g.upper;
    e.sol_lower = xn.lower;
    e.sol_upper = xn.upper;
    e.b_lower = fmax(0.0, bn.lower);
    e.energy_lower = energy.lower;
    e.grad_radius = g_err;
    e.certified = isfinite(e.res_upper) && isfinite(e.grad_upper) && isfinite(e.sol_upper) &&
                  isfinite(e.op_upper);
    e.op_lower = opl;
    return e;
}

/* Extended-precision repeat of the base chain; returns 1 with replaced vectors. */
static int refine(const orc_operator* op, const orc_model* mdl, const double* b, const double* x,
                  double reg, double* ax, double* res, double* atr, double* g, envelope* out,
                  orc_validation* r) {
    const int64_t m = op->rows, n = op->cols;
    if (!model_ok(mdl)) return 0;
    if (LDBL_MANT_DIG <= DBL_MANT_DIG) return 0;
    interval bn = nint(b, m), xn = nint(x, n);
    if (!isfinite(bn.upper) || !isfinite(xn.upper)) return 0;
    int ok = 0;
    long double* lx = malloc(sizeof(long double) * (size_t)n);
    long double* la = malloc(sizeof(long double) * (size_t)m);
    long double* lr = malloc(sizeof(long double) * (size_t)m);
    long double* lt = malloc(sizeof(long double) * (size_t)n);
    double *a2 = malloc(sizeof(double) * (size_t)m), *r2 = malloc(sizeof(double) * (size_t)m);
    double *t2 = malloc(sizeof(double) * (size_t)n), *g2 = malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) lx[i] = x[i];
    r->calls[2]++;
    if (!apply_ld(op, lx, la)) goto done;
    for (int64_t i = 0; i < m; ++i) {
        a2[i] = (double)la[i];
        if (!isfinite(a2[i])) goto done;
    }
    interval san = nint(a2, m);
    const double a_cast = one_op_radius(san.upper, 1, m);
    const double a_acc = ld_callback_radius(mdl, n, xn.upper, m);
    const double a_err = up_add(a_acc, a_cast);
    for (int64_t i = 0; i < m; ++i) {
        lr[i] = la[i] - (long double)b[i];
        if (!isfinite(lr[i])) goto done;
        r2[i] = (double)lr[i];
        if (!isfinite(r2[i])) goto done;
    }
    interval srn = nint(r2, m);
    const double r_cast = one_op_radius(srn.upper, 1, m);
    const double lr_up = up_add(srn.upper, r_cast);
    const double r_sub = ld_one_op_radius(lr_up, san.upper > 0.0 || bn.upper > 0.0, m);
    const double lr_err = up_add(a_acc, r_sub);
    const double sr_err = up_add(lr_err, r_cast);
    r->calls[3]++;
    if (!apply_transpose_ld(op, lr, lt)) goto done;
    for (int64_t i = 0; i < n; ++i) {
        t2[i] = (double)lt[i];
        if (!isfinite(t2[i])) goto done;
    }
    interval stn = nint(t2, n);
    const double t_cast = one_op_radius(stn.upper, 1, n);
    const double t_acc = ld_callback_radius(mdl, m, lr_up, n);
    for (int64_t i = 0; i < n; ++i) {
        long double lg = fmal((long double)reg, lx[i], lt[i]);
        if (!isfinite(lg)) goto done;
        g2[i] = (double)lg;
        if (!isfinite(g2[i])) goto done;
    }
    interval sgn = nint(g2, n);
    const double g_cast = one_op_radius(sgn.upper, 1, n);
    const double lg_up = up_add(sgn.upper, g_cast);
    const double rs_err = ld_one_op_radius(lg_up, reg > 0.0 && xn.upper > 0.0, n);
    const double prop = up_mul(mdl->norm_upper, lr_err);
    const double g_err = up_add(up_add(t_acc, prop), up_add(rs_err, g_cast));
    interval ta = enlarge(san, a_err), tr = enlarge(srn, sr_err), tg = enlarge(sgn, g_err);
    double opl = mdl->norm_lower;
    if (xn.upper > 0.0) opl = fmax(opl, down_div(down_diff(san.lower, a_err), xn.upper));
    if (srn.upper > 0.0) {
        const double conv = up_mul(mdl->norm_upper, r_cast);
        const double terr = up_add(up_add(t_acc, t_cast), conv);
        opl = fmax(opl, down_div(down_diff(stn.lower, terr), srn.upper));
    }
    interval energy = augmented(ta, xn, reg);
    envelope e;
    memset(&e, 0, sizeof(e));
    e.op_upper = mdl->norm_upper;
    e.op_lower = opl;
    e.res_lower = tr.lower;
    e.res_upper = tr.upper;
    e.grad_upper = tg.upper;
    e.sol_lower = xn.lower;
    e.sol_upper = xn.upper;
    e.b_lower = fmax(0.0, bn.lower);
    e.energy_lower = energy.lower;
    e.grad_radius = g_err;
    e.certified = isfinite(e.res_upper) && isfinite(e.grad_upper) && isfinite(e.sol_upper) &&
                  isfinite(e.op_upper);
    if (!e.certified) goto done;
    memcpy(ax, a2, sizeof(double) * (size_t)m);
    memcpy(res, r2, sizeof(double) * (size_t)m);
    memcpy(atr, t2, sizeof(double) * (size_t)n);
    memcpy(g, g2, sizeof(double) * (size_t)n);
    *out = e;
    ok = 1;
done:
    free(lx); free(la); free(lr); free(lt); free(a2); free(r2); free(t2); free(g2);
    return ok;
}

enum {
    RC_NA = 0, RC_SKIP_PASS = 1, RC_SKIP_ZERO = 2, RC_SKIP_NONFINITE = 3, RC_IMPROVED = 4,
    RC_NOT_IMPROVED = 5, RC_BAD_CURVATURE = 6, RC_PARTIAL = 7, RC_NONFINITE = 8
};

static void ridge_correction(const orc_operator* op, const orc_model* mdl, const double* g,
                             double gnorm, double reg, const envelope* env, orc_validation* r) {
    const int64_t m = op->rows, n = op->cols;
    r->ridge_correction_disposition = RC_NONFINITE;
    if (!(gnorm > 0.0) || !isfinite(gnorm) || !all_finite(g, n)) {
        r->ridge_correction_disposition = RC_SKIP_NONFINITE;
        return;
    }
    double* d = malloc(sizeof(double) * (size_t)n);
    double* ad = malloc(sizeof(double) * (size_t)m);
    double* h = malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) d[i] = g[i] / gnorm;
    if (!all_finite(d, n)) {
        r->ridge_correction_disposition = RC_SKIP_NONFINITE;
        goto done;
    }
    interval dn = nint(d, n);
    r->calls[4]++;
    orc_apply(op, d, 1, ad);
    if (!all_finite(ad, m)) {
        r->ridge_correction_disposition = RC_PARTIAL;
        goto done;
    }
    interval adn = nint(ad, m);
    const double ad_err = callback_radius(mdl, 0, dn.upper, m);
    r->calls[5]++;
    orc_apply_transpose(op, ad, 1, h);
    const double t_err = callback_radius(mdl, 1, adn.upper, n);
    for (int64_t i = 0; i < n; ++i) h[i] = fma(reg, d[i], h[i]);
    if (!all_finite(h, n)) goto done;
    interval hn = nint(h, n);
    const double prop = up_mul(env->op_upper, ad_err);
    const double hsum = one_op_radius(hn.upper, reg > 0.0 && dn.upper > 0.0, n);
    const double herr = up_add(up_add(t_err, prop), hsum);
    const double curv = dot(d, h, n);
    if (!isfinite(curv)) goto done;
    if (!(curv > 0.0)) {
        r->ridge_correction_disposition = RC_BAD_CURVATURE;
        goto done;
    }
    const double step = gnorm / curv;
    if (!(step > 0.0) || !isfinite(step)) goto done;
    for (int64_t i = 0; i < n; ++i) h[i] = fma(-step, h[i], g[i]);
    if (!all_finite(h, n)) goto done;
    interval qn = nint(h, n);
    const double axpy_err = one_op_radius(qn.upper, gnorm > 0.0 && hn.upper > 0.0, n);
    const double q_err = up_add(up_add(env->grad_radius, up_mul(step, herr)), axpy_err);
    const double q_up = up_add(qn.upper, q_err);
    const double ad_true = up_add(adn.upper, ad_err);
    const double step2 = up_mul(step, step);
    const double de2 = up_add(up_mul(ad_true, ad_true), up_mul(reg, up_mul(dn.upper, dn.upper)));
    const double zhz = up_mul(step2, de2);
    const double two_cross = up_mul(2.0, up_mul(step, up_mul(dn.upper, q_up)));
    const double qsq = up_mul(q_up, q_up);
    const double corrected = up_sqrt(up_add(zhz, up_add(two_cross, up_div(qsq, reg))));
    if (isnan(corrected)) goto done;
    r->ridge_corrected_energy_error_upper_bound = corrected;
    r->ridge_correction_gamma = 1.0 / curv;
    r->ridge_correction_z_h_z = zhz;
    r->ridge_correction_two_abs_z_t_q = two_cross;
    r->ridge_correction_q_norm_squared = qsq;
    r->ridge_correction_disposition = RC_NOT_IMPROVED;
done:
    free(d); free(ad); free(h);
}

void orc_validate(const orc_operator* op, const orc_model* mdl, const double* b, const double* x,
                  double reg, double tol, orc_validation* r) {
    const int64_t m = op->rows, n = op->cols;
    memset(r, 0, sizeof(*r));
    r->ridge_base_energy_error_upper_bound = NAN;
    r->ridge_corrected_energy_error_upper_bound = NAN;
    r->ridge_correction_gamma = NAN;
    r->ridge_correction_z_h_z = NAN;
    r->ridge_correction_two_abs_z_t_q = NAN;
    r->ridge_correction_q_norm_squared = NAN;
    r->ridge_correction_disposition = RC_NA;
    r->status = ST_WORK;
    r->stop_reason = SR_DEPTH;
    double* ax = malloc(sizeof(double) * (size_t)m);
    double* res = malloc(sizeof(double) * (size_t)m);
    double* atr = malloc(sizeof(double) * (size_t)n);
    double* g = malloc(sizeof(double) * (size_t)n);
    r->calls[0]++;
    orc_apply(op, x, 1, ax);
    for (int64_t i = 0; i < m; ++i) res[i] = ax[i] - b[i];
    r->calls[1]++;
    orc_apply_transpose(op, res, 1, atr);
    for (int64_t i = 0; i < n; ++i) g[i] = fma(reg, x[i], atr[i]);
    fill_norms(r, x, ax, res, g, m, n, reg);
    const double bnorm = norm2(b, m);
    nominal_contract(r, bnorm, reg, tol, 0, 0.0);
    const int finite = all_finite(x, n) && all_finite(ax, m) && all_finite(res, m) &&
                       all_finite(atr, n) && all_finite(g, n);
    if (!finite || r->status == ST_BREAKDOWN || r->stop_reason == SR_BREAKDOWN) {
        r->status = ST_BREAKDOWN;
        r->stop_reason = SR_BREAKDOWN;
    } else {
        envelope e = base_envelope(mdl, b, x, ax, res, atr, g, m, n, reg);
        r->operator_norm_lower_bound = e.op_lower;
        certified_contract(r, &e, reg, tol, 0, 0.0);
        if (op->kind != 3 && r->status != ST_SUCCESS && e.certified &&
            e.grad_radius >= r->normal_residual_norm) {
            envelope e2;
            if (refine(op, mdl, b, x, reg, ax, res, atr, g, &e2, r)) {
                e = e2;
                fill_norms(r, x, ax, res, g, m, n, reg);
                nominal_contract(r, bnorm, reg, tol, 0, 0.0);
                r->operator_norm_lower_bound = e.op_lower;
                certified_contract(r, &e, reg, tol, 0, 0.0);
            }
        }
        if (reg > 0.0) {
            r->ridge_base_energy_error_upper_bound = r->energy_error_upper_bound;
            if (r->status == ST_SUCCESS) r->ridge_correction_disposition = RC_SKIP_PASS;
            else if (!e.certified) r->ridge_correction_disposition = RC_SKIP_NONFINITE;
            else if (e.energy_lower == 0.0) r->ridge_correction_disposition = RC_SKIP_ZERO;
            else if (!(e.grad_upper > 0.0) || !isfinite(e.grad_upper))
                r->ridge_correction_disposition = RC_SKIP_NONFINITE;
            else {
                ridge_correction(op, mdl, g, r->normal_residual_norm, reg, &e, r);
                if (r->ridge_correction_disposition == RC_NOT_IMPROVED &&
                    isfinite(r->ridge_corrected_energy_error_upper_bound) &&
                    r->ridge_corrected_energy_error_upper_bound < r->energy_error_upper_bound) {
                    r->ridge_correction_disposition = RC_IMPROVED;
                    certified_contract(r, &e, reg, tol, 1, r->ridge_corrected_energy_error_upper_bound);
                }
            }
        }
    }
    if (reg > 0.0 && r->status == ST_BREAKDOWN) {
        r->ridge_base_energy_error_upper_bound = isnan(r->normal_residual_norm) ? NAN : INF_D;
        r->energy_error_upper_bound = r->ridge_base_energy_error_upper_bound;
        r->relative_energy_error_upper_bound = INF_D;
        r->objective_gap_upper_bound = INF_D;
        r->ridge_correction_disposition = RC_SKIP_NONFINITE;
    }
    free(ax); free(res); free(atr); free(g);
}
