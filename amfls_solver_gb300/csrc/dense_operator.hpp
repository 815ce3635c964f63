// FP64 dense operator on the device (see dense_operator.cu).
#pragma once

#include "device_operator.hpp"

namespace amfls_gpu {

class DenseOperator final : public DeviceOperator {
public:
    // d_values: rows x cols FP64 in device memory, row-major unless
    // column_major; not copied (the caller keeps it alive, as in the
    // reference's non-owning DenseOperator / RowMajorDenseOperator).
    DenseOperator(int rows, int cols, const double* d_values, bool column_major,
                  cudaStream_t stream);
    ~DenseOperator() override;
    DenseOperator(const DenseOperator&) = delete;
    DenseOperator& operator=(const DenseOperator&) = delete;

    int rows() const override { return rows_; }
    int cols() const override { return cols_; }
    int kind() const override { return column_major_ ? 2 : 1; }
    const double* values() const { return a_; }
    void apply(const double* x, int block_cols, double* y, cudaStream_t s) const override;
    void apply_transpose(const double* y, int block_cols, double* x,
                         cudaStream_t s) const override;
    // one shared pass over the matrix per block (dense_operator.cpp:100-105)
    double relative_block_product_cost(int block_cols) const override {
        return block_cols > 0 ? 1.0 : __builtin_huge_val();
    }
    ValidationModel validation_error_model() const override { return model_; }
    bool supports_validation_refinement() const override { return true; }
    void apply_refined(const double* x_hi, const double* x_lo, double* y_hi, double* y_lo,
                       int* finite, cudaStream_t s) const override;
    void apply_transpose_refined(const double* y_hi, const double* y_lo, double* x_hi,
                                 double* x_lo, int* finite, cudaStream_t s) const override;
    bool product1(bool transpose, const double* x, const Epilogue& ep,
                  cudaStream_t s) const override;

private:
    void release() noexcept;  // frees the operator's device buffers
    void product(bool transpose, const double* x, double* y, const int* guard,
                 cudaStream_t s) const;
    void block_product(bool transpose, const double* x, int block_cols, double* y,
                       cudaStream_t s) const;
    int rows_, cols_;
    const double* a_;
    bool column_major_;
    ValidationModel model_;
    double* partials_ = nullptr;  // chunk partial sums
    long long partial_cap_ = 0;
    double* tmp_ = nullptr;       // product vector for the fused path
    double* scratch_ = nullptr;
    unsigned* counter_ = nullptr;
};

// Applies an Epilogue to a computed product vector t (length n) with the
// reductions; shared by operators without an in-kernel epilogue.
void run_epilogue(const double* t, long long n, const Epilogue& ep, double* partials,
                  unsigned* counter, cudaStream_t s);

}  // namespace amfls_gpu
