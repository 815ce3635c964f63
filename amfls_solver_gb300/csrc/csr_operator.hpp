// FP64 CSR operator on the device (see csr_operator.cu).
#pragma once

#include <vector>

#include <memory>

#include "device_operator.hpp"

namespace amfls_gpu {

class ReducedCsrOperator;

class CsrOperator final : public DeviceOperator {
public:
    // The CSR arrays are device pointers in the reference's layout: int64 row
    // offsets (rows+1), int64 column indices and FP64 values (nnz).  They are
    // copied and validated; the caller may free them afterwards.
    // `elems_per_lane` sets the row-length binning (lanes per row ~ len / it).
    CsrOperator(int rows, int cols, const long long* d_offsets, const long long* d_indices,
                const double* d_values, long long nnz, cudaStream_t stream,
                int elems_per_lane = 4);
    ~CsrOperator() override;
    CsrOperator(const CsrOperator&) = delete;
    CsrOperator& operator=(const CsrOperator&) = delete;

    int rows() const override { return rows_; }
    int cols() const override { return cols_; }
    int kind() const override { return 0; }
    long long nonzeros() const { return nnz_; }
    long long max_row_nonzeros() const { return max_row_nnz_; }
    long long max_col_nonzeros() const { return max_col_nnz_; }

    void apply(const double* x, int block_cols, double* y, cudaStream_t s) const override;
    void apply_transpose(const double* y, int block_cols, double* x,
                         cudaStream_t s) const override;
    ValidationModel validation_error_model() const override { return model_; }
    bool supports_validation_refinement() const override { return true; }
    void apply_refined(const double* x_hi, const double* x_lo, double* y_hi, double* y_lo,
                       int* finite, cudaStream_t s) const override;
    void apply_transpose_refined(const double* y_hi, const double* y_lo, double* x_hi,
                                 double* x_lo, int* finite, cudaStream_t s) const override;
    bool product1(bool transpose, const double* x, const Epilogue& ep,
                  cudaStream_t s) const override;
    // Tiling of the single-column products per side (A, then the stored
    // transpose): 1 = chain groups, 0 = row blocks; the autotuner's timings
    // (microseconds per product, row blocks then chain groups, 0 = not timed).
    void single_column_schedule(int chains[2], double microseconds[4]) const;

private:
    friend class ReducedCsrOperator;
    struct Side;
    void build(const long long* d_off, const long long* d_idx, const double* d_val,
               cudaStream_t stream);
    void build_bins(Side& s, const int* d_bins, cudaStream_t stream);
    void tune_single_column(Side& s, const std::vector<long long>& host_off,
                            cudaStream_t stream);
    void fill_ids(int* ids, long long n, cudaStream_t stream);
    void product(bool transpose, const double* x, int block_cols, double* y,
                 cudaStream_t stream) const;
    void refined(bool transpose, const double* x_hi, const double* x_lo, double* y_hi,
                 double* y_lo, int* finite, cudaStream_t stream) const;
    void release();

    int rows_;
    int cols_;
    long long nnz_;
    int elems_per_lane_;
    long long max_row_nnz_ = 0;
    long long max_col_nnz_ = 0;
    ValidationModel model_;
    std::unique_ptr<Side> a_;
    std::unique_ptr<Side> t_;
    double* scratch_ = nullptr;
    unsigned* counter_ = nullptr;
    // row-major staging of a multi-column input block (max(rows, cols) x 8);
    // multi-column products on one operator are therefore stream-ordered
    double* xrows_ = nullptr;
};

// The matrix of a CsrOperator with its values rounded to FP32 or BF16 (one
// rounding per entry, round to nearest): products read the stored values,
// round x to FP32 and accumulate in FP32.  It shares the source operator's
// structure, so the source must outlive it.  Its validation model is the
// source's widened for the rounded values and FP32 accumulation (see
// reduced_model), so certificates computed with it describe the rounded
// matrix.  Part of the mixed-precision form; no counterpart in the reference.
class ReducedCsrOperator final : public DeviceOperator {
public:
    ReducedCsrOperator(const CsrOperator& src, ValueType type, cudaStream_t stream);
    ~ReducedCsrOperator() override;
    ReducedCsrOperator(const ReducedCsrOperator&) = delete;
    ReducedCsrOperator& operator=(const ReducedCsrOperator&) = delete;

    int rows() const override { return src_.rows(); }
    int cols() const override { return src_.cols(); }
    int kind() const override { return 0; }
    ValueType value_type() const { return type_; }
    void apply(const double* x, int block_cols, double* y, cudaStream_t s) const override;
    void apply_transpose(const double* y, int block_cols, double* x,
                         cudaStream_t s) const override;
    ValidationModel validation_error_model() const override { return model_; }
    bool product1(bool transpose, const double* x, const Epilogue& ep,
                  cudaStream_t s) const override;
    // Tiling of the single-column products per side (A, then the stored
    // transpose): 1 = chain groups, 0 = row blocks; the autotuner's timings
    // (microseconds per product, row blocks then chain groups, 0 = not timed).
    void single_column_schedule(int chains[2], double microseconds[4]) const;

private:
    void product(bool transpose, const double* x, int block_cols, double* y,
                 cudaStream_t s) const;
    void release();
    const CsrOperator& src_;
    ValueType type_;
    void* vals_[2] = {nullptr, nullptr};  // A side, transpose side
    double* xrows_ = nullptr;
    double* scratch_ = nullptr;
    unsigned* counter_ = nullptr;
    ValidationModel model_;
};

}  // namespace amfls_gpu
