// Reduced-precision dense operator and the augmented ridge operator of the
// mixed-precision form (see reduced_operator.hpp).
//
// Dense products in FP32 are HBM-bound at every block width the solver uses
// (4 or 2 bytes per element against 2 flops per element and column), so the
// kernels stream the copy once per pass with 16-byte vector loads:
//   dot    A(o, i) at a[o * ld + i], i contiguous: a warp owns two outputs,
//          lanes stride i by one vector (4 FP32 or 8 BF16 values);
//   across A(i, o) at a[i * ld + o], o contiguous: a thread owns one vector of
//          consecutive outputs and walks i.
// Both split the summed dimension into chunks; chunk partial sums (FP64)
// are added in chunk order by a second kernel, so results are deterministic.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <type_traits>

#include "common.cuh"
#include "epilogue.cuh"
#include "reduced_operator.hpp"

namespace amfls_gpu {
namespace {

constexpr int kThreads = 256;
// blocks that fill the GPU (eight per SM)
inline int target_blocks() { return grid_cap(); }
constexpr int kMaxCols = 8;  // columns per pass over the matrix

int grid_1d(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + kThreads - 1) / kThreads,
                                                           target_blocks()));
}

// 16 bytes of T as FP32 values
template <typename T>
struct Vec;
template <>
struct Vec<float> {
    static constexpr int N = 4;
    __device__ static void load(const float* p, float (&v)[4]) {
        const float4 q = __ldcs(reinterpret_cast<const float4*>(p));
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
        v[3] = q.w;
    }
};
template <>
struct Vec<__nv_bfloat16> {
    static constexpr int N = 8;
    __device__ static void load(const __nv_bfloat16* p, float (&v)[8]) {
        const uint4 q = __ldcs(reinterpret_cast<const uint4*>(p));
        const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // a BF16 value is the upper half of an FP32 bit pattern
            v[2 * k] = __uint_as_float(w[k] << 16);
            v[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
        }
    }
};

template <typename T, int S>
__global__ void __launch_bounds__(kThreads)
rdot_kernel(const T* __restrict__ a, long long ld, int outer, int inner, int chunk,
            const double* __restrict__ x, long long ldx, double* partial, const int* guard) {
    constexpr int N = Vec<T>::N;
    if (guard && *guard == 0) return;
    const int lane = threadIdx.x & 31;
    const long long o0 = ((long long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5)) * 2;
    if (o0 >= outer) return;
    const int ch = blockIdx.y;
    const int i0 = ch * chunk, i1 = min(inner, i0 + chunk);
    const T* rows[2] = {a + o0 * ld, a + min(o0 + 1, (long long)outer - 1) * ld};
    float acc[2][S];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int c = 0; c < S; ++c) acc[j][c] = 0.0f;
    for (int i = i0 + lane * N; i < i1; i += 32 * N) {
        float xv[S][N];
#pragma unroll
        for (int c = 0; c < S; ++c)
#pragma unroll
            for (int k = 0; k < N; ++k)
                xv[c][k] = i + k < i1 ? (float)__ldg(x + i + k + c * ldx) : 0.0f;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            float av[N];
            Vec<T>::load(rows[j] + i, av);  // padding beyond `inner` is zero
#pragma unroll
            for (int k = 0; k < N; ++k)
#pragma unroll
                for (int c = 0; c < S; ++c) acc[j][c] = fmaf(av[k], xv[c][k], acc[j][c]);
        }
    }
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int c = 0; c < S; ++c) {
            float v = acc[j][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && o0 + j < outer)
                partial[((long long)ch * S + c) * outer + o0 + j] = (double)v;
        }
}

template <typename T, int S>
__global__ void __launch_bounds__(kThreads)
racross_kernel(const T* __restrict__ a, long long ld, int outer, int inner, int chunk,
               const double* __restrict__ x, long long ldx, double* partial, const int* guard) {
    constexpr int N = Vec<T>::N;
    if (guard && *guard == 0) return;
    const long long o = (blockIdx.x * (long long)blockDim.x + threadIdx.x) * N;
    if (o >= outer) return;
    const int ch = blockIdx.y;
    const int i0 = ch * chunk, i1 = min(inner, i0 + chunk);
    float acc[N][S];
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int c = 0; c < S; ++c) acc[k][c] = 0.0f;
    for (int i = i0; i < i1; ++i) {
        float av[N];
        Vec<T>::load(a + (long long)i * ld + o, av);
#pragma unroll
        for (int c = 0; c < S; ++c) {
            const float xv = (float)__ldg(x + i + c * ldx);
#pragma unroll
            for (int k = 0; k < N; ++k) acc[k][c] = fmaf(av[k], xv, acc[k][c]);
        }
    }
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int c = 0; c < S; ++c)
            if (o + k < outer) partial[((long long)ch * S + c) * outer + o + k] = (double)acc[k][c];
}

__global__ void rreduce_kernel(const double* partial, int chunks, int S, int outer, double* y,
                               long long ldy, const int* guard) {
    if (guard && *guard == 0) return;
    const long long total = (long long)S * outer;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / outer);
        const long long o = t % outer;
        double s = 0.0;
        for (int ch = 0; ch < chunks; ++ch) s += partial[((long long)ch * S + c) * outer + o];
        y[o + c * ldy] = s;
    }
}

// Rounded copy of the source (contiguous extent `inner`, padded to `ld`).
template <typename T>
__global__ void narrow_matrix_kernel(const double* src, int outer, int inner, T* dst,
                                     long long ld) {
    const long long total = (long long)outer * ld;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long o = t / ld, i = t % ld;
        const double v = i < inner ? src[o * inner + i] : 0.0;
        if constexpr (std::is_same_v<T, float>)
            dst[t] = __double2float_rn(v);
        else
            dst[t] = __double2bfloat16(v);
    }
}

// Launch shape of one pass: dot products need about one warp per output pair
// and chunk, across products one thread per output vector and chunk; chunks
// are sized so that the grid covers the GPU.
struct Shape {
    int bx, chunks, chunk;
};

Shape shape_of(bool dot, int outer, int inner, int vec) {
    Shape s{};
    if (dot) {
        s.bx = (int)ceil_div(outer, 2 * (kThreads / 32));
        s.chunks = (int)std::max<long long>(1, std::min<long long>(target_blocks() / std::max(1, s.bx),
                                                                   ceil_div(inner, 32LL * vec)));
        s.chunk = (int)(ceil_div(ceil_div(inner, s.chunks), 32LL * vec) * 32 * vec);
    } else {
        s.bx = (int)ceil_div(ceil_div(outer, vec), kThreads);
        s.chunks = (int)std::max<long long>(1, std::min<long long>(target_blocks() / std::max(1, s.bx),
                                                                   inner));
        s.chunk = (int)ceil_div(inner, s.chunks);
    }
    s.chunks = (int)ceil_div(inner, s.chunk);
    return s;
}

template <typename T, int S>
void launch_pass(bool dot, const T* a, long long ld, int outer, int inner, const double* x,
                 long long ldx, double* partial, double* y, long long ldy, int ncols,
                 const int* guard, cudaStream_t s) {
    const Shape sh = shape_of(dot, outer, inner, Vec<T>::N);
    const dim3 grid(sh.bx, sh.chunks);
    if (dot)
        rdot_kernel<T, S><<<grid, kThreads, 0, s>>>(a, ld, outer, inner, sh.chunk, x, ldx,
                                                    partial, guard);
    else
        racross_kernel<T, S><<<grid, kThreads, 0, s>>>(a, ld, outer, inner, sh.chunk, x, ldx,
                                                       partial, guard);
    AMFLS_LAUNCHED();
    rreduce_kernel<<<grid_1d((long long)S * outer), kThreads, 0, s>>>(partial, sh.chunks, S, outer,
                                                                    y, ldy, guard);
    AMFLS_LAUNCHED();
    (void)ncols;
}

template <typename T>
void dense_pass(bool dot, const T* a, long long ld, int outer, int inner, const double* x,
                long long ldx, int ncols, double* partial, double* y, long long ldy,
                const int* guard, cudaStream_t s) {
    switch (ncols) {
        case 1: launch_pass<T, 1>(dot, a, ld, outer, inner, x, ldx, partial, y, ldy, 1, guard, s); break;
        case 2: launch_pass<T, 2>(dot, a, ld, outer, inner, x, ldx, partial, y, ldy, 2, guard, s); break;
        case 3: launch_pass<T, 3>(dot, a, ld, outer, inner, x, ldx, partial, y, ldy, 3, guard, s); break;
        case 4: launch_pass<T, 4>(dot, a, ld, outer, inner, x, ldx, partial, y, ldy, 4, guard, s); break;
        default:
            // 5..8 columns: one pass of 8 would write partial columns beyond
            // ncols into y, so split into 4 + the rest
            launch_pass<T, 4>(dot, a, ld, outer, inner, x, ldx, partial, y, ldy, 4, guard, s);
            dense_pass<T>(dot, a, ld, outer, inner, x + 4 * ldx, ldx, ncols - 4, partial,
                          y + 4 * ldy, ldy, guard, s);
    }
}

__global__ void augment_apply_kernel(const double* top, long long m, const double* x, long long n,
                                     double root, double* y, long long ldy, int ncols) {
    const long long total = (m + n) * ncols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / (m + n));
        const long long r = t % (m + n);
        y[r + c * ldy] = r < m ? top[r + c * m] : root * x[(r - m) + c * n];
    }
}

__global__ void augment_split_kernel(const double* y, long long m, long long n, long long ldy,
                                     int ncols, double* top) {
    const long long total = m * ncols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / m);
        const long long r = t % m;
        top[r + c * m] = y[r + c * ldy];
    }
    (void)n;
}

__global__ void augment_add_kernel(const double* y, long long m, long long n, long long ldy,
                                   int ncols, double root, double* x) {
    const long long total = n * ncols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / n);
        const long long i = t % n;
        x[i + c * n] = fma(root, y[m + i + c * ldy], x[i + c * n]);
    }
}

__global__ void augment_tail_kernel(const double* x, long long n, double root, double* out,
                                    const int* guard) {
    if (guard && *guard == 0) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = root * x[i];
}

}  // namespace

// --------------------------------------------------- reduced dense ----

ReducedDenseOperator::ReducedDenseOperator(const DenseOperator& src, ValueType type,
                                           cudaStream_t stream)
    : rows_(src.rows()), cols_(src.cols()), column_major_(src.kind() == 2), type_(type) {
    if (type != ValueType::fp32 && type != ValueType::bf16)
        throw std::invalid_argument("reduced dense values must be FP32 or BF16");
    const int outer = column_major_ ? cols_ : rows_;
    const int inner = column_major_ ? rows_ : cols_;
    ld_ = (inner + 7) / 8 * 8;
    const size_t eb = type == ValueType::fp32 ? 4 : 2;
    try {
        AMFLS_CUDA(cudaMalloc(&a_, eb * (size_t)outer * ld_));
        if (type == ValueType::fp32)
            narrow_matrix_kernel<float><<<grid_1d((long long)outer * ld_), kThreads, 0, stream>>>(
                src.values(), outer, inner, static_cast<float*>(a_), ld_);
        else
            narrow_matrix_kernel<__nv_bfloat16>
                <<<grid_1d((long long)outer * ld_), kThreads, 0, stream>>>(
                    src.values(), outer, inner, static_cast<__nv_bfloat16*>(a_), ld_);
        AMFLS_LAUNCHED();
        const int vec = type == ValueType::fp32 ? 4 : 8;
        for (int tr = 0; tr < 2; ++tr) {
            const int on = tr ? cols_ : rows_, inn = tr ? rows_ : cols_;
            const bool dot = column_major_ == (tr == 1);
            const Shape sh = shape_of(dot, on, inn, vec);
            partial_cap_ = std::max(partial_cap_, 4LL * sh.chunks * on);
        }
        AMFLS_CUDA(cudaMalloc(&partials_, sizeof(double) * partial_cap_));
        AMFLS_CUDA(cudaMalloc(&tmp_, sizeof(double) * std::max(rows_, cols_)));
        AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * 6 * kMaxGridCap + 64));
        counter_ = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(scratch_) +
                                               sizeof(double) * 6 * kMaxGridCap);
        AMFLS_CUDA(cudaMemsetAsync(counter_, 0, 64, stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
    } catch (...) {
        cudaFree(a_);
        cudaFree(partials_);
        cudaFree(tmp_);
        cudaFree(scratch_);
        throw;
    }
    model_ = reduced_model(src.validation_error_model(), type);
}

ReducedDenseOperator::~ReducedDenseOperator() {
    cudaFree(a_);
    cudaFree(partials_);
    cudaFree(tmp_);
    cudaFree(scratch_);
}

void ReducedDenseOperator::product(bool transpose, const double* x, int block_cols, double* y,
                                   cudaStream_t s) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("dense product block is invalid");
    const int out = transpose ? cols_ : rows_, in = transpose ? rows_ : cols_;
    const bool dot = column_major_ == transpose;  // the summed dimension is contiguous
    for (int c0 = 0; c0 < block_cols; c0 += kMaxCols) {
        const int nc = std::min(kMaxCols, block_cols - c0);
        const double* xc = x + (long long)c0 * in;
        double* yc = y + (long long)c0 * out;
        if (type_ == ValueType::fp32)
            dense_pass(dot, static_cast<const float*>(a_), ld_, out, in, xc, in, nc, partials_, yc,
                       out, nullptr, s);
        else
            dense_pass(dot, static_cast<const __nv_bfloat16*>(a_), ld_, out, in, xc, in, nc,
                       partials_, yc, out, nullptr, s);
    }
}

void ReducedDenseOperator::apply(const double* x, int block_cols, double* y,
                                 cudaStream_t s) const {
    product(false, x, block_cols, y, s);
}

void ReducedDenseOperator::apply_transpose(const double* y, int block_cols, double* x,
                                           cudaStream_t s) const {
    product(true, y, block_cols, x, s);
}

bool ReducedDenseOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                                    cudaStream_t s) const {
    const int out = transpose ? cols_ : rows_, in = transpose ? rows_ : cols_;
    const bool dot = column_major_ == transpose;
    if (type_ == ValueType::fp32)
        dense_pass(dot, static_cast<const float*>(a_), ld_, out, in, x, in, 1, partials_, tmp_, out,
                   ep.guard, s);
    else
        dense_pass(dot, static_cast<const __nv_bfloat16*>(a_), ld_, out, in, x, in, 1, partials_,
                   tmp_, out, ep.guard, s);
    run_epilogue(tmp_, out, ep, ep.partials ? ep.partials : scratch_,
                 ep.counter ? ep.counter : counter_, s);
    return true;
}

// ------------------------------------------------------- augmented ----

AugmentedOperator::AugmentedOperator(const DeviceOperator& a, double lambda, cudaStream_t stream)
    : a_(a), root_(std::sqrt(lambda)) {
    if (!(lambda >= 0.0) || !std::isfinite(lambda))
        throw std::invalid_argument("augmented operator needs a finite lambda >= 0");
    const long long m = a.rows(), n = a.cols();
    try {
        AMFLS_CUDA(cudaMalloc(&top_, sizeof(double) * m * kMaxCols));
        AMFLS_CUDA(cudaMalloc(&tmp_, sizeof(double) * (m + n)));
        AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * 6 * kMaxGridCap + 64));
        counter_ = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(scratch_) +
                                               sizeof(double) * 6 * kMaxGridCap);
        AMFLS_CUDA(cudaMemsetAsync(counter_, 0, 64, stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
    } catch (...) {
        cudaFree(top_);
        cudaFree(tmp_);
        cudaFree(scratch_);
        throw;
    }
    // ||[A; r I]||^2 = ||A^T A + r^2 I|| = ||A||^2 + r^2 (rounded outward)
    const ValidationModel am = a.validation_error_model();
    model_.norm_upper = std::nextafter(
        std::sqrt(std::nextafter(am.norm_upper * am.norm_upper + lambda, HUGE_VAL) * (1.0 + 0x1p-52)),
        HUGE_VAL);
    model_.norm_lower = std::max(
        0.0, std::nextafter(std::sqrt(am.norm_lower * am.norm_lower + lambda) * (1.0 - 0x1p-51), 0.0));
    if (!std::isfinite(am.norm_upper)) {
        model_.norm_upper = HUGE_VAL;
        model_.norm_lower = 0.0;
    }
    // the sqrt(lambda) x rows add one rounding; A^T y + r y_bottom adds one
    model_.apply_steps = std::max(am.apply_steps, 1LL);
    model_.transpose_steps = am.transpose_steps + 1;
}

AugmentedOperator::~AugmentedOperator() {
    cudaFree(top_);
    cudaFree(tmp_);
    cudaFree(scratch_);
}

void AugmentedOperator::apply(const double* x, int block_cols, double* y, cudaStream_t s) const {
    const long long m = a_.rows(), n = a_.cols();
    for (int c0 = 0; c0 < block_cols; c0 += kMaxCols) {
        const int nc = std::min(kMaxCols, block_cols - c0);
        a_.apply(x + c0 * n, nc, top_, s);
        augment_apply_kernel<<<grid_1d((m + n) * nc), kThreads, 0, s>>>(
            top_, m, x + c0 * n, n, root_, y + c0 * (m + n), m + n, nc);
        AMFLS_LAUNCHED();
    }
}

void AugmentedOperator::apply_transpose(const double* y, int block_cols, double* x,
                                        cudaStream_t s) const {
    const long long m = a_.rows(), n = a_.cols();
    for (int c0 = 0; c0 < block_cols; c0 += kMaxCols) {
        const int nc = std::min(kMaxCols, block_cols - c0);
        augment_split_kernel<<<grid_1d(m * nc), kThreads, 0, s>>>(y + c0 * (m + n), m, n, m + n,
                                                                  nc, top_);
        AMFLS_LAUNCHED();
        a_.apply_transpose(top_, nc, x + c0 * n, s);
        augment_add_kernel<<<grid_1d(n * nc), kThreads, 0, s>>>(y + c0 * (m + n), m, n, m + n, nc,
                                                                root_, x + c0 * n);
        AMFLS_LAUNCHED();
    }
}

bool AugmentedOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                                 cudaStream_t s) const {
    const long long m = a_.rows(), n = a_.cols();
    Epilogue inner;
    inner.out = tmp_;
    inner.guard = ep.guard;
    if (transpose) {
        // A^T y_top + sqrt(lambda) y_bottom in one fused pass over A
        inner.fma_vec = x + m;
        inner.lambda = root_;
        if (!a_.product1(true, x, inner, s)) return false;
    } else {
        if (!a_.product1(false, x, inner, s)) return false;
        augment_tail_kernel<<<grid_1d(n), kThreads, 0, s>>>(x, n, root_, tmp_ + m, ep.guard);
        AMFLS_LAUNCHED();
    }
    run_epilogue(tmp_, transpose ? n : m + n, ep, ep.partials ? ep.partials : scratch_,
                 ep.counter ? ep.counter : counter_, s);
    return true;
}

}  // namespace amfls_gpu
