// Operators of the mixed-precision form (no counterpart in the reference).
//
//   ReducedDenseOperator   the matrix of a DenseOperator rounded once to FP32
//                          or BF16, products in FP32;
//   AugmentedOperator      [A; sqrt(lambda) I] over any operator, so that a
//                          ridge correction step is a plain least-squares
//                          solve (lambda = 0) on it.
// ReducedCsrOperator lives beside CsrOperator (csr_operator.hpp).
#pragma once

#include "dense_operator.hpp"
#include "device_operator.hpp"

namespace amfls_gpu {

// Products read the rounded values, round x to FP32 and accumulate in FP32;
// chunk partial sums are added in FP64 in a fixed order.  The copy has the
// source's layout with the contiguous dimension padded to a multiple of 8
// (16-byte vector loads).  Independent of the source after construction.
class ReducedDenseOperator final : public DeviceOperator {
public:
    ReducedDenseOperator(const DenseOperator& src, ValueType type, cudaStream_t stream);
    ~ReducedDenseOperator() override;
    ReducedDenseOperator(const ReducedDenseOperator&) = delete;
    ReducedDenseOperator& operator=(const ReducedDenseOperator&) = delete;

    int rows() const override { return rows_; }
    int cols() const override { return cols_; }
    int kind() const override { return column_major_ ? 2 : 1; }
    ValueType value_type() const { return type_; }
    void apply(const double* x, int block_cols, double* y, cudaStream_t s) const override;
    void apply_transpose(const double* y, int block_cols, double* x,
                         cudaStream_t s) const override;
    double relative_block_product_cost(int block_cols) const override {
        return block_cols > 0 ? 1.0 : __builtin_huge_val();
    }
    ValidationModel validation_error_model() const override { return model_; }
    bool product1(bool transpose, const double* x, const Epilogue& ep,
                  cudaStream_t s) const override;

private:
    void product(bool transpose, const double* x, int block_cols, double* y,
                 cudaStream_t s) const;
    int rows_, cols_;
    bool column_major_;
    ValueType type_;
    long long ld_ = 0;  // padded contiguous extent of the copy
    void* a_ = nullptr;
    ValidationModel model_;
    double* partials_ = nullptr;
    long long partial_cap_ = 0;
    double* tmp_ = nullptr;
    double* scratch_ = nullptr;
    unsigned* counter_ = nullptr;
};

// [A; sqrt(lambda) I] (rows + cols) x cols over a non-owned operator A.
class AugmentedOperator final : public DeviceOperator {
public:
    AugmentedOperator(const DeviceOperator& a, double lambda, cudaStream_t stream);
    ~AugmentedOperator() override;
    AugmentedOperator(const AugmentedOperator&) = delete;
    AugmentedOperator& operator=(const AugmentedOperator&) = delete;

    int rows() const override { return a_.rows() + a_.cols(); }
    int cols() const override { return a_.cols(); }
    int kind() const override { return 3; }
    bool graph_safe() const override { return a_.graph_safe(); }
    void apply(const double* x, int block_cols, double* y, cudaStream_t s) const override;
    void apply_transpose(const double* y, int block_cols, double* x,
                         cudaStream_t s) const override;
    double relative_block_product_cost(int block_cols) const override {
        return a_.relative_block_product_cost(block_cols);
    }
    ValidationModel validation_error_model() const override { return model_; }
    bool product1(bool transpose, const double* x, const Epilogue& ep,
                  cudaStream_t s) const override;

private:
    const DeviceOperator& a_;
    double root_;
    ValidationModel model_;
    double* top_ = nullptr;  // rows x 8 staging of the A part of a block
    double* tmp_ = nullptr;  // rows + cols product vector for the fused path
    double* scratch_ = nullptr;
    unsigned* counter_ = nullptr;
};

}  // namespace amfls_gpu
