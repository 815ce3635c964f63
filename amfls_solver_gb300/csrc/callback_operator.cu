// Matrix-free operator over user callbacks (see callback_operator.hpp).
//
// The reference accepts any MatrixOperator subclass
// (include/amfls/matrix_operator.hpp:29-89); across a C ABI that becomes a
// table of function pointers with a context.  The callbacks receive
// column-major device blocks and a CUDA stream and must leave the result
// there in stream order.  Because they run user code, the solve launches
// width-one levels one by one instead of capturing them into a graph
// (graph_safe() is false).  Validation uses the model the caller supplies;
// without one the norm bounds stay (inf, 0) and no solve certifies success,
// as in the reference (matrix_operator.hpp:17-20).
#include <cmath>
#include <stdexcept>
#include <string>

#include "callback_operator.hpp"
#include "common.cuh"
#include "dense_operator.hpp"

namespace amfls_gpu {

CallbackOperator::CallbackOperator(int rows, int cols, const Callbacks& cb, cudaStream_t stream)
    : rows_(rows), cols_(cols), cb_(cb) {
    if (rows <= 0 || cols <= 0) throw std::invalid_argument("operator dimensions must be positive");
    if (cb.apply == nullptr || cb.apply_transpose == nullptr)
        throw std::invalid_argument("custom operator needs apply and apply_transpose callbacks");
    if (cb.has_model) {
        const ValidationModel& m = cb.model;
        if (!(m.norm_lower >= 0.0) || !(m.norm_upper >= m.norm_lower) || m.apply_steps < 0 ||
            m.transpose_steps < 0)
            throw std::invalid_argument("custom operator validation model is invalid");
    }
    try {
        AMFLS_CUDA(cudaMalloc(&tmp_, sizeof(double) * (size_t)std::max(rows, cols)));
        AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * 6 * kMaxGridCap + 64));
        counter_ = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(scratch_) +
                                               sizeof(double) * 6 * kMaxGridCap);
        AMFLS_CUDA(cudaMemsetAsync(counter_, 0, 64, stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
    } catch (...) {  // free what was allocated before the failure
        cudaFree(tmp_);
        cudaFree(scratch_);
        throw;
    }
}

CallbackOperator::~CallbackOperator() {
    cudaFree(tmp_);
    cudaFree(scratch_);
}

void CallbackOperator::apply(const double* x, int block_cols, double* y, cudaStream_t s) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("custom operator block is invalid");
    const int rc = cb_.apply(cb_.context, x, block_cols, y, s);
    if (rc != 0) throw std::runtime_error("custom operator apply failed (" + std::to_string(rc) + ")");
}

void CallbackOperator::apply_transpose(const double* y, int block_cols, double* x,
                                       cudaStream_t s) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("custom operator block is invalid");
    const int rc = cb_.apply_transpose(cb_.context, y, block_cols, x, s);
    if (rc != 0)
        throw std::runtime_error("custom operator apply_transpose failed (" + std::to_string(rc) + ")");
}

double CallbackOperator::relative_block_product_cost(int block_cols) const {
    if (cb_.relative_block_product_cost == nullptr)
        return DeviceOperator::relative_block_product_cost(block_cols);
    const double c = cb_.relative_block_product_cost(cb_.context, block_cols);
    return std::isfinite(c) && c > 0.0 ? c : __builtin_huge_val();
}

bool CallbackOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                                cudaStream_t s) const {
    if (transpose)
        apply_transpose(x, 1, tmp_, s);
    else
        apply(x, 1, tmp_, s);
    run_epilogue(tmp_, transpose ? cols_ : rows_, ep, ep.partials ? ep.partials : scratch_,
                 ep.counter ? ep.counter : counter_, s);
    return true;
}

}  // namespace amfls_gpu
