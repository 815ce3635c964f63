// Device-side MatrixOperator contract.
//
// Mirrors include/amfls/matrix_operator.hpp:29-89 of the reference with
// device pointers: apply / apply_transpose act on column-major blocks
// X (cols x s) and Y (rows x s) resident in GPU memory, asynchronously on a
// CUDA stream.  relative_block_product_cost and validation_error_model keep
// their meaning; the extended-precision validation products of the
// reference (long double, matrix_operator.hpp:70-88) become double-double
// products here (apply_refined / apply_transpose_refined).
//
// Built-in operators also implement `product1`, a single-column product with
// a fused epilogue and a device-side guard flag.  The solver uses it so that
// an enqueued level does no work once the device state says the process
// must stop, and so that the norms and dot products the level needs come
// out of the same pass over the operator.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <limits>

namespace amfls_gpu {

struct ValidationModel {
    double norm_upper = std::numeric_limits<double>::infinity();
    double norm_lower = 0.0;
    long long apply_steps = 0;
    long long transpose_steps = 0;
};

// Reductions produced by a fused epilogue (written by the last block).
struct RedResult {
    double sq_t;       // sum t_i^2
    double sq_out;     // sum out_i^2
    double dot;        // sum out_i * dot_vec_i
    double max_t;      // max |t_i|
    double max_out;    // max |out_i|
    int nonfinite;     // count of nonfinite t_i or out_i
    int pad;
};

// t_i is the i-th entry of the product.  Then
//   out_i = t_i - (*coef) * sub[i * sub_stride]         if sub != nullptr
//   out_i = t_i - (*coef) * panel(*sub_col)[i]           if sub_table != nullptr
//   out_i = fma(lambda, fma_vec[i], t_i)                 if fma_vec != nullptr
//   out_i = t_i - minus_vec[i]                           if minus_vec != nullptr
//   out_i = t_i                                          otherwise
struct Epilogue {
    double* t_out = nullptr;
    double* out = nullptr;
    const double* sub = nullptr;
    long long sub_stride = 1;
    // alternatively the subtracted vector is column *sub_col of a table of
    // row-major 32-column panels (read on the device at run time)
    double* const* sub_table = nullptr;
    const int* sub_col = nullptr;
    const double* coef = nullptr;
    const double* fma_vec = nullptr;
    double lambda = 0.0;
    const double* minus_vec = nullptr;
    const double* dot_vec = nullptr;
    RedResult* red = nullptr;
    const int* guard = nullptr;  // skip the launch's work when *guard == 0
    // Scratch for the cross-block reduction (one slot of 6 doubles per block
    // and a ticket counter that must start at zero).  When null the operator
    // uses its own, which serialises fused products on one operator.
    double* partials = nullptr;
    unsigned* counter = nullptr;
};

// Storage precision of an operator's values.
enum class ValueType { fp64 = 0, fp32 = 1, bf16 = 2 };

// Validation model of a matrix whose entries are those of a source matrix
// rounded once to `type` (relative change at most u_t: 2^-24 FP32, 2^-8
// BF16), with products that round x to FP32 and accumulate in FP32.  The
// norm bounds widen by the factor (1 +- u_t); the rounding-step counts are
// expressed in units of the FP64 unit roundoff 2^-53 that the validation
// formulas use: an FP32 step is 2^29 FP64 steps, and the rounding of x adds
// one step.
inline ValidationModel reduced_model(const ValidationModel& m, ValueType type) {
    const double u = type == ValueType::bf16 ? 0x1p-8 : 0x1p-24;
    ValidationModel r;
    r.norm_upper = m.norm_upper * (1.0 + 2.0 * u);
    r.norm_lower = m.norm_lower * (1.0 - 2.0 * u);
    constexpr long long kScale = 1LL << 29;
    r.apply_steps = (m.apply_steps + 1) * kScale;
    r.transpose_steps = (m.transpose_steps + 1) * kScale;
    return r;
}

class DeviceOperator {
public:
    virtual ~DeviceOperator() = default;
    virtual int rows() const = 0;
    virtual int cols() const = 0;
    virtual void apply(const double* x, int block_cols, double* y, cudaStream_t s) const = 0;
    virtual void apply_transpose(const double* y, int block_cols, double* x,
                                 cudaStream_t s) const = 0;
    virtual double relative_block_product_cost(int block_cols) const {
        return block_cols > 0 ? static_cast<double>(block_cols)
                              : std::numeric_limits<double>::infinity();
    }
    virtual ValidationModel validation_error_model() const { return {}; }
    virtual bool supports_validation_refinement() const { return false; }
    // Double-double validation products.  Inputs and outputs are (hi, lo)
    // pairs; `finite` receives 0 when a nonfinite value appeared.
    virtual void apply_refined(const double* x_hi, const double* x_lo, double* y_hi,
                               double* y_lo, int* finite, cudaStream_t s) const {
        (void)x_hi; (void)x_lo; (void)y_hi; (void)y_lo; (void)finite; (void)s;
    }
    virtual void apply_transpose_refined(const double* y_hi, const double* y_lo, double* x_hi,
                                         double* x_lo, int* finite, cudaStream_t s) const {
        (void)y_hi; (void)y_lo; (void)x_hi; (void)x_lo; (void)finite; (void)s;
    }
    // Fused single-column product; returns false when the operator has none.
    virtual bool product1(bool transpose, const double* x, const Epilogue& ep,
                          cudaStream_t s) const {
        (void)transpose; (void)x; (void)ep; (void)s;
        return false;
    }
    // Storage kind for diagnostics: 0 CSR, 1 row-major dense, 2 column-major
    // dense, 3 custom callbacks or a composition.
    virtual int kind() const = 0;
    // Whether the products only enqueue device work on the stream they are
    // given (no host synchronisation, no allocation), so that they may be
    // captured into a CUDA graph.  The built-in operators are; operators
    // that call user code are not assumed to be.
    virtual bool graph_safe() const { return true; }
};

}  // namespace amfls_gpu
