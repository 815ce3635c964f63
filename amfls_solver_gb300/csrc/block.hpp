// Block kernels for the block Golub-Kahan path (width > 1); see block.cu.
#pragma once

#include <cuda_runtime.h>

namespace amfls_gpu {

// ------------------------------------------------------------ products ----

// C (a x b, column-major, ld a) = X^T Y;  X (m x a, ld ldx), Y (m x b, ld ldy).
// `partials` must hold ts_tn_partial_doubles(m, a, b) doubles.  When
// `nonfinite` is not null it is set to 1 if an entry of C is not finite.
long long ts_tn_partial_doubles(long long m, int a, int b);
void ts_tn(const double* X, long long ldx, const double* Y, long long ldy, long long m, int a,
           int b, double* C, double* partials, int* nonfinite, cudaStream_t s);

// Y (m x b, ld ldy) = beta Y + alpha X C;  X (m x a, ld ldx), C (a x b, ld a).
// Y must not overlap X.
void ts_nn(const double* X, long long ldx, const double* C, long long m, int a, int b, double* Y,
           long long ldy, double alpha, double beta, cudaStream_t s);

// Basis V stored as row-major 32-column panels (panel p holds columns
// 32p..32p+31; entry (i, j) at panels[j / 32][i * 32 + j % 32]).
//
// C (k x c, ld k) = V[:, 0:k]^T R;  R (n x c, ld ldr).
long long panel_tn_partial_doubles(long long n, int k, int c);
void panel_tn(double* const* panels, long long n, int k, const double* R, long long ldr, int c,
              double* C, double* partials, int* nonfinite, cudaStream_t s);

// R (n x c, ld ldr) += alpha V[:, first:first+w] C;  C (w x c, ld w).
void panel_nn(double* const* panels, long long n, int first, int w, const double* C, int c,
              double* R, long long ldr, double alpha, cudaStream_t s);

// V[:, k0 + j] = Q[:, j] for j < r (Q column-major n x r).
void panel_append(double* const* panels, long long n, int k0, const double* Q, int r,
                  cudaStream_t s);

// ----------------------------------------------------- factorisations ----

// R factor (c x c, column-major, upper triangular) of the tall block B
// (rows x c, ld ldb) by Householder TSQR; `work` must hold
// tsqr_work_doubles(rows, c) doubles.
long long tsqr_work_doubles(long long rows, int c);
void tsqr_r(const double* B, long long rows, int c, long long ldb, double* R, double* work,
            cudaStream_t s);

// One-sided Jacobi SVD of the c x c matrix R (column-major): sigma (c,
// descending) and right singular vectors W (c x c, column i pairs sigma i).
// `work` must hold jacobi_work_doubles(c) doubles.
long long jacobi_work_doubles(int c);
void jacobi_svd(const double* R, int c, double* sigma, double* W, double* work, cudaStream_t s);

// Upper Cholesky factor U of the symmetric c x c matrix G (G = U^T U) and
// U^{-1}; flag[0] = 1 when G is not numerically positive definite.
void cholesky_upper(const double* G, int c, double* U, double* Uinv, int* flag, cudaStream_t s);

// ------------------------------------------------ projected solve ----

// Level records of the block lower-bidiagonal projected operator T.  Level j
// adds r_j columns; its rows couple to the aw_j rows of the previous left
// block (G_j, aw_j x r_j) and to the nlw_j rows of the new left block
// (N_j, nlw_j x r_j), whose projected right-hand side entries are g_j (nlw_j).
// meta per level: r, aw, nlw, value offset, state offset (5 ints).
struct LevelRecords {
    const int* meta;
    const double* vals;  // G (aw x r) | N (nlw x r) | g (nlw) at the value offset
};
constexpr int kLevelMeta = 5;

// state-area doubles level j needs (r_prev = r_{j-1}, 0 for j = 0)
long long level_state_doubles(int r, int nlw, int r_prev);
// carry / work doubles for levels up to width w
long long projected_carry_doubles(int w);
long long projected_work_doubles(int w);

// Reduce levels [first, last) of [T; sqrt(lambda) I] by Householder QR,
// continuing from the carry left by the previous call (first == 0 starts
// from the first row block, g0 = ||b||), then back-substitute all levels
// into y (k).  w bounds every r, aw and nlw of the levels (carry and work
// are sized for it).  flags: bit 0 zero pivot, bit 1 pivot ratio below
// rcond (lambda == 0 only), bit 2 inconsistent level records.
void block_projected_solve(const LevelRecords& rec, int first, int last, int w, double lambda,
                           double g0, double* state, double* carry, double* work, double* y,
                           int k, double rcond, int* flags, cudaStream_t s);

}  // namespace amfls_gpu
