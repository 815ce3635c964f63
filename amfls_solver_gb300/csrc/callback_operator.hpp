// Matrix-free operator over user callbacks (the reference's custom
// MatrixOperator, include/amfls/matrix_operator.hpp:29-89, on device blocks).
#pragma once

#include "device_operator.hpp"

namespace amfls_gpu {

struct Callbacks {
    void* context = nullptr;
    // y (rows x s) = A x (cols x s), column-major device blocks; work is
    // enqueued on `stream`; nonzero return = failure
    int (*apply)(void* context, const double* x, int s, double* y, void* stream) = nullptr;
    int (*apply_transpose)(void* context, const double* y, int s, double* x, void* stream) = nullptr;
    // optional; the interface default (s) when null
    double (*relative_block_product_cost)(void* context, int s) = nullptr;
    bool has_model = false;  // without a model no solve can certify success
    ValidationModel model;
};

class CallbackOperator final : public DeviceOperator {
public:
    CallbackOperator(int rows, int cols, const Callbacks& cb, cudaStream_t stream);
    ~CallbackOperator() override;
    CallbackOperator(const CallbackOperator&) = delete;
    CallbackOperator& operator=(const CallbackOperator&) = delete;

    int rows() const override { return rows_; }
    int cols() const override { return cols_; }
    int kind() const override { return 3; }
    bool graph_safe() const override { return false; }
    void apply(const double* x, int block_cols, double* y, cudaStream_t s) const override;
    void apply_transpose(const double* y, int block_cols, double* x,
                         cudaStream_t s) const override;
    double relative_block_product_cost(int block_cols) const override;
    ValidationModel validation_error_model() const override {
        return cb_.has_model ? cb_.model : ValidationModel{};
    }
    // the fused single-column product: the callback, then the epilogue
    bool product1(bool transpose, const double* x, const Epilogue& ep,
                  cudaStream_t s) const override;

private:
    int rows_, cols_;
    Callbacks cb_;
    double* tmp_ = nullptr;
    double* scratch_ = nullptr;
    unsigned* counter_ = nullptr;
};

}  // namespace amfls_gpu
